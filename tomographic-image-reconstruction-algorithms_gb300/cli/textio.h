// textio.h -- the reference's whitespace text format for fields and records.
//
// Layout as mimo-io.cuh:6-45: for each l, for each k, for each j, one line of
// the nx values of row j ("v " each), a blank line after every k-slice and one
// more after every l-block; values printed with max_digits10 so float values
// round-trip exactly.  Reading accepts any whitespace.
#pragma once

#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

namespace textio {

// Reads exactly n floats; returns false if the file is missing or short.
inline bool read_floats(const std::string& path, float* out, size_t n) {
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) return false;
    std::string text;
    std::vector<char> buf(1 << 20);
    size_t r;
    while ((r = std::fread(buf.data(), 1, buf.size(), f)) > 0) text.append(buf.data(), r);
    std::fclose(f);
    const char* p = text.c_str();
    size_t got = 0;
    while (got < n) {
        char* e = nullptr;
        const float v = std::strtof(p, &e);
        if (e == p) break;   // end of input or a non-number
        out[got++] = v;
        p = e;
    }
    return got == n;
}

// Writes dims (nx, ny, nz, nw) with i fastest, as mimo-io.cuh write().
inline bool write_floats(const std::string& path, const float* a, int nx, int ny, int nz = 1, int nw = 1) {
    FILE* f = std::fopen(path.c_str(), "w");
    if (!f) return false;
    size_t q = 0;
    for (int l = 0; l < nw; ++l) {
        for (int k = 0; k < nz; ++k) {
            for (int j = 0; j < ny; ++j) {
                for (int i = 0; i < nx; ++i) std::fprintf(f, "%.9g ", (double)a[q++]);
                std::fputc('\n', f);
            }
            std::fputc('\n', f);
        }
        std::fputc('\n', f);
    }
    return std::fclose(f) == 0;
}

}  // namespace textio
