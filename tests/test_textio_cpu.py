"""Host checks of the CLI's file formats (cli/textio.h), compiled with g++ on the CPU.

The text writer prints each float as its shortest round-trip decimal and the reader takes
plain decimal tokens through std::from_chars and everything else strtof accepts through
strtof; both must give back the exact bits, read files written by the reference's
`ofstream << float` layout and by an earlier `%.9g` writer, and fail (return false) on a
short, missing or non-numeric file.  The binary form must round-trip as well.
"""
import os
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(REPO, "tomographic-image-reconstruction-algorithms_gb300", "cli")

HARNESS = r"""
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <random>
#include "textio.h"

static int fails = 0;
#define CHECK(c) do { if (!(c)) { std::printf("FAIL line %d: %s\n", __LINE__, #c); ++fails; } } while (0)

static bool same_bits(const std::vector<float>& a, const std::vector<float>& b) {
    return a.size() == b.size() && std::memcmp(a.data(), b.data(), a.size() * 4) == 0;
}
static void put(const char* path, const char* text) {
    FILE* f = std::fopen(path, "wb"); std::fputs(text, f); std::fclose(f);
}

int main() {
    // values: random normals at several scales, subnormals, signed zeros, extremes, inf, nan
    std::vector<float> a;
    std::mt19937 r(7);
    std::normal_distribution<float> d(0.f, 1.f);
    for (int s = -40; s <= 38; s += 6)
        for (int q = 0; q < 200; ++q) a.push_back(d(r) * std::ldexp(1.f, s));
    const float lim[] = {0.f, -0.f, std::numeric_limits<float>::denorm_min(), -std::numeric_limits<float>::denorm_min(),
                         std::numeric_limits<float>::min(), std::numeric_limits<float>::max(),
                         -std::numeric_limits<float>::max(), std::numeric_limits<float>::infinity(),
                         -std::numeric_limits<float>::infinity(), std::numeric_limits<float>::quiet_NaN(),
                         1.f, 0.1f, 1e-5f, 3.3333e-07f};
    for (float v : lim) a.push_back(v);
    while (a.size() % 12) a.push_back(0.5f);
    const int nx = 4, ny = 3, nz = (int)(a.size() / 12);
    std::vector<float> b(a.size());
    CHECK(textio::write_floats("t.txt", a.data(), nx, ny, nz));
    CHECK(textio::read_floats("t.txt", b.data(), b.size()));
    CHECK(same_bits(a, b));
    CHECK(textio::write_floats("t.bin", a.data(), nx, ny, nz));
    std::fill(b.begin(), b.end(), 0.f);
    CHECK(textio::read_floats("t.bin", b.data(), b.size()));
    CHECK(same_bits(a, b));
    // the layout: nx values and a space each per row, a blank line after each slice and block
    {
        std::vector<float> s = {1.f, 2.f, 3.f, 4.f};
        CHECK(textio::write_floats("s.txt", s.data(), 2, 2, 1, 1));
        FILE* f = std::fopen("s.txt", "rb"); char buf[64] = {0}; size_t n = std::fread(buf, 1, 63, f); std::fclose(f);
        CHECK(n == 12 && std::strcmp(buf, "1 2 \n3 4 \n\n\n") == 0);
    }
    // earlier writers: the reference's default-precision stream output and %.9g
    {
        put("ref.txt", "0.03 0 -1.5e-05 \n4.2e+06 7 0.000123457 \n\n\n");
        std::vector<float> v(6);
        CHECK(textio::read_floats("ref.txt", v.data(), 6));
        CHECK(v[0] == 0.03f && v[1] == 0.f && v[2] == -1.5e-05f && v[3] == 4.2e+06f && v[4] == 7.f && v[5] == 0.000123457f);
        FILE* f = std::fopen("g9.txt", "wb");
        for (size_t q = 0; q < a.size(); ++q) std::fprintf(f, "%.9g ", (double)a[q]);
        std::fclose(f);
        std::fill(b.begin(), b.end(), 0.f);
        CHECK(textio::read_floats("g9.txt", b.data(), b.size()));
        bool eq = true;
        for (size_t q = 0; q < a.size(); ++q) eq = eq && (std::isnan(a[q]) ? std::isnan(b[q]) : a[q] == b[q]);
        CHECK(eq);
    }
    // tokens strtof takes and from_chars does not take whole, and separators
    {
        put("odd.txt", "+1.5\t0x1p3\r\n1e50 -1e50\n\n nan  inf 1e-46 2.5");
        std::vector<float> v(8);
        CHECK(textio::read_floats("odd.txt", v.data(), 8));
        CHECK(v[0] == 1.5f && v[1] == 8.f && std::isinf(v[2]) && v[2] > 0 && std::isinf(v[3]) && v[3] < 0);
        CHECK(std::isnan(v[4]) && std::isinf(v[5]) && v[6] == 0.f && v[7] == 2.5f);
    }
    // failures: short file, non-number, missing file, binary header of another size
    {
        std::vector<float> v(4);
        put("short.txt", "1 2 3");
        CHECK(!textio::read_floats("short.txt", v.data(), 4));
        put("bad.txt", "1 2 x 4");
        CHECK(!textio::read_floats("bad.txt", v.data(), 4));
        put("comma.txt", "1,2,3,4");
        CHECK(!textio::read_floats("comma.txt", v.data(), 4));
        CHECK(!textio::read_floats("missing.txt", v.data(), 4));
        CHECK(!textio::read_floats("t.bin", v.data(), 4));
        put("empty.txt", "");
        CHECK(!textio::read_floats("empty.txt", v.data(), 1));
        CHECK(textio::read_floats("empty.txt", v.data(), 0));
    }
    std::printf(fails ? "FAILED %d\n" : "OK\n", fails);
    return fails ? 1 : 0;
}
"""


def test_text_and_binary_formats(tmp_path):
    src = tmp_path / "textio_check.cpp"
    src.write_text(HARNESS)
    exe = tmp_path / "textio_check"
    r = subprocess.run(["g++", "-O2", "-std=c++17", "-Wall", "-I" + CLI, str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    if r.returncode != 0:
        pytest.fail("harness does not compile:\n" + r.stderr)
    out = subprocess.run([str(exe)], cwd=tmp_path, capture_output=True, text=True, timeout=120)
    assert out.returncode == 0 and out.stdout.strip().endswith("OK"), out.stdout + out.stderr
