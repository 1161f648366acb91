// textio.h -- the reference's whitespace text format for fields and records,
// and a binary form of the same arrays.
//
// Text layout as mimo-io.cuh:6-45: for each l, for each k, for each j, one line
// of the nx values of row j ("v " each), a blank line after every k-slice and
// one more after every l-block; each value printed as the shortest decimal that
// reads back as the same float (std::to_chars), so values round-trip exactly.
// Reading accepts any whitespace and any number strtof accepts; plain decimal
// tokens go through std::from_chars (the same correctly rounded value as
// strtof, about three times faster on the reference's 75 MB side files).
//
// Binary layout (files named *.bin): the 8 bytes "TOMOF32\n", four
// little-endian int32 dims (nx, ny, nz, nw), then nx*ny*nz*nw little-endian
// IEEE float32 values in the text format's order (i fastest).  read_floats
// recognises it by the magic, so either form can be read wherever the other
// was written.
#pragma once

#include <charconv>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace textio {

constexpr char kMagic[8] = {'T', 'O', 'M', 'O', 'F', '3', '2', '\n'};

inline uint32_t le32(const unsigned char* b) {
    return (uint32_t)b[0] | ((uint32_t)b[1] << 8) | ((uint32_t)b[2] << 16) | ((uint32_t)b[3] << 24);
}

inline void put_le32(unsigned char* b, uint32_t v) {
    b[0] = (unsigned char)(v & 0xffu); b[1] = (unsigned char)((v >> 8) & 0xffu);
    b[2] = (unsigned char)((v >> 16) & 0xffu); b[3] = (unsigned char)((v >> 24) & 0xffu);
}

inline bool is_binary_name(const std::string& path) {
    return path.size() >= 4 && path.compare(path.size() - 4, 4, ".bin") == 0;
}

// Reads exactly n floats (text or binary form); returns false if the file is missing or short.
inline bool read_floats(const std::string& path, float* out, size_t n) {
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) return false;
    unsigned char head[24];
    const size_t h = std::fread(head, 1, sizeof head, f);
    if (h == sizeof head && std::memcmp(head, kMagic, 8) == 0) {
        const uint64_t count = (uint64_t)le32(head + 8) * le32(head + 12) * le32(head + 16) * le32(head + 20);
        if (count != n) { std::fclose(f); return false; }
        std::vector<unsigned char> raw(n * 4);
        const bool ok = std::fread(raw.data(), 1, raw.size(), f) == raw.size();
        std::fclose(f);
        if (!ok) return false;
        for (size_t q = 0; q < n; ++q) {
            const uint32_t u = le32(&raw[q * 4]);
            std::memcpy(&out[q], &u, 4);
        }
        return true;
    }
    std::string text;
    if (std::fseek(f, 0, SEEK_END) == 0) {
        const long size = std::ftell(f);
        if (size > 0) text.reserve((size_t)size);
    }
    std::rewind(f);
    std::vector<char> buf(1 << 20);
    size_t r;
    while ((r = std::fread(buf.data(), 1, buf.size(), f)) > 0) text.append(buf.data(), r);
    std::fclose(f);
    const char* p = text.c_str();
    const char* const end = p + text.size();
    auto space = [](char c) { return c == ' ' || c == '\n' || c == '\t' || c == '\r' || c == '\v' || c == '\f'; };
    size_t got = 0;
    while (got < n) {
        while (p < end && space(*p)) ++p;
        if (p == end) break;
        float v = 0.f;
        const std::from_chars_result fc = std::from_chars(p, end, v);
        if (fc.ec == std::errc() && (fc.ptr == end || space(*fc.ptr))) {
            p = fc.ptr;
        } else {
            // tokens from_chars does not take whole ('+1', hex, out of range): strtof decides
            char* e = nullptr;
            v = std::strtof(p, &e);
            if (e == p) break;   // a non-number
            p = e;
        }
        out[got++] = v;
    }
    return got == n;
}

// Binary form of write_floats.
inline bool write_binary(const std::string& path, const float* a, int nx, int ny, int nz = 1, int nw = 1) {
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) return false;
    unsigned char head[24];
    std::memcpy(head, kMagic, 8);
    put_le32(head + 8, (uint32_t)nx); put_le32(head + 12, (uint32_t)ny);
    put_le32(head + 16, (uint32_t)nz); put_le32(head + 20, (uint32_t)nw);
    bool ok = std::fwrite(head, 1, sizeof head, f) == sizeof head;
    const size_t n = (size_t)nx * ny * nz * nw;
    std::vector<unsigned char> raw(n * 4);
    for (size_t q = 0; q < n; ++q) {
        uint32_t u;
        std::memcpy(&u, &a[q], 4);
        put_le32(&raw[q * 4], u);
    }
    ok = ok && std::fwrite(raw.data(), 1, raw.size(), f) == raw.size();
    return std::fclose(f) == 0 && ok;
}

// Writes dims (nx, ny, nz, nw) with i fastest, as mimo-io.cuh write(); a path
// ending in ".bin" gets the binary form.
inline bool write_floats(const std::string& path, const float* a, int nx, int ny, int nz = 1, int nw = 1) {
    if (is_binary_name(path)) return write_binary(path, a, nx, ny, nz, nw);
    FILE* f = std::fopen(path.c_str(), "w");
    if (!f) return false;
    std::string out;
    out.reserve((1 << 20) + 64 * (size_t)nx);
    bool ok = true;
    auto flush = [&] {
        ok = ok && std::fwrite(out.data(), 1, out.size(), f) == out.size();
        out.clear();
    };
    char num[32];
    size_t q = 0;
    for (int l = 0; l < nw; ++l) {
        for (int k = 0; k < nz; ++k) {
            for (int j = 0; j < ny; ++j) {
                for (int i = 0; i < nx; ++i) {
                    const std::to_chars_result tc = std::to_chars(num, num + sizeof num, a[q++]);
                    out.append(num, tc.ptr);
                    out.push_back(' ');
                }
                out.push_back('\n');
                if (out.size() >= (1u << 20)) flush();
            }
            out.push_back('\n');
        }
        out.push_back('\n');
    }
    flush();
    return std::fclose(f) == 0 && ok;
}

}  // namespace textio
