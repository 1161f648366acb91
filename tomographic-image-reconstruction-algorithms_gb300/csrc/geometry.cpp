// geometry.cpp -- problem set-up on the host: transducers, emitter groups,
// receivers, update mask, source wavelets, phantoms and record noise.
//
// REF profile follows the reference program's compile-time problem:
//   transducers   Position_Transducers (sirt-mimo.cu:438-466), generalised to a
//                 ring of side hi-lo between sensor lines lo and hi
//   groups        g*gs .. g*gs+gs-1, emission over the bounding box of the first
//                 and last transducer (sirt-mimo.cu:543-554)
//   wavelet       v^2 dt^2 cos(wc t) exp(-t^2/2tau^2), t = k dt - tt, k+1 <= 24
//                 (sirt-mimo.cu:553-561)
//   receivers     the four sensor lines, i in (lo, hi) (sirt-mimo.cu:629-647)
//   mask          [lo+1, hi)^2 (sirt-mimo.cu:870)
//   phantom       field_setup (generate-field.cu:117-172)
// CFG profile: transducers on a circle, point emitters and receivers, Ricker
// wavelet, quadratic sponge (parameters in tomo_config).
#include <algorithm>
#include <cmath>
#include <cstring>

#include "internal.h"

namespace tomo {

double Rng::normal() {
    // Box-Muller on two uniforms in (0, 1]
    const double u1 = 1.0 - uniform(), u2 = uniform();
    return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
}

tomo_status build_geometry(const tomo_config& c, Geometry& geo, std::string& why) {
    geo = Geometry{};
    geo.cfg = c;
    geo.nx = c.nx; geo.ny = c.ny; geo.nt = c.nt;
    geo.N = (int64_t)c.nx * c.ny;
    geo.gs = c.group_size;
    geo.ref = c.profile == TOMO_PROFILE_REF;
    if (c.profile != TOMO_PROFILE_REF && c.profile != TOMO_PROFILE_CFG) { why = "unknown profile"; return TOMO_ERR_ARG; }
    if (c.nx < 8 || c.ny < 8 || c.nt < 4) { why = "grid must be at least 8x8 with nt >= 4"; return TOMO_ERR_ARG; }
    if ((int64_t)c.nx * c.ny > (int64_t)1 << 30) { why = "grid larger than 2^30 cells"; return TOMO_ERR_ARG; }
    if (c.group_size < 1) { why = "group_size must be >= 1"; return TOMO_ERR_ARG; }
    const int nx = c.nx, ny = c.ny;

    if (geo.ref) {
        geo.lo = c.ring_lo; geo.hi = c.ring_hi;
        if (geo.lo < 2 || geo.hi < geo.lo + 2 || geo.hi > std::min(nx, ny) - 3) {
            why = "ring_lo/ring_hi must satisfy 2 <= lo, lo+2 <= hi <= min(nx,ny)-3";
            return TOMO_ERR_ARG;
        }
        const int side = geo.hi - geo.lo;
        geo.ns = 4 * side;
        geo.ii.resize(geo.ns); geo.jj.resize(geo.ns);
        // Walk the ring: bottom row left to right, right column bottom to top,
        // top row right to left, left column top to bottom (1-based cells).
        int p = 0;
        for (int q = 1; q <= side; ++q, ++p) { geo.ii[p] = geo.lo + 1 + q; geo.jj[p] = geo.hi + 1; }
        for (int q = 1; q <= side; ++q, ++p) { geo.ii[p] = geo.hi + 1; geo.jj[p] = geo.hi + 1 - q; }
        for (int q = 1; q <= side; ++q, ++p) { geo.ii[p] = geo.hi + 1 - q; geo.jj[p] = geo.lo + 1; }
        for (int q = 1; q <= side; ++q, ++p) { geo.ii[p] = geo.lo + 1; geo.jj[p] = geo.lo + 1 + q; }
        geo.nch = 4 * nx;
        geo.rcv.assign(geo.nch, -1);
        for (int t = geo.lo + 1; t < geo.hi; ++t) {
            geo.rcv[t] = geo.hi * nx + t;               // bottom line j = hi
            geo.rcv[nx + t] = t * nx + geo.hi;          // right line  i = hi
            geo.rcv[2 * nx + t] = geo.lo * nx + t;      // top line    j = lo
            geo.rcv[3 * nx + t] = t * nx + geo.lo;      // left line   i = lo
        }
        geo.mask.assign(geo.N, 0);
        for (int j = geo.lo + 1; j < geo.hi; ++j)
            std::memset(geo.mask.data() + (int64_t)j * nx + geo.lo + 1, 1, geo.hi - geo.lo - 1);
        // Source (sirt-mimo.cu:553-561), emitted while k + 1 <= 24: the kernel forms
        // v v DT DT cos(wc t) exp(-t^2 / 2 tau^2) per cell in FP32, in that order; the two
        // transcendental factors are evaluated here in FP32 (t = k DT - TT) and tabled as
        // src[k] = cos(wc t) and src[n + k] = exp(-t^2 / 2 tau^2), n = n_src_steps.
        geo.n_src_steps = std::min(24, c.nt - 1);
        const int n = geo.n_src_steps;
        geo.src.assign(std::max(c.nt, 2 * n), 0.f);
        for (int k = 0; k < n; ++k) {
            const float t = (float)k * kRefDT - kRefTT;
            geo.src[k] = std::cos(kRefOmegaC * t);
            geo.src[n + k] = std::exp(-(t * t) / (2.f * kRefTao * kRefTao));
        }
        const float hh = kRefH * kRefH;
        geo.corr_scale = 1.0 / (double)hh;
    } else {
        geo.ns = c.n_transducers;
        const double R = c.radius, C = c.courant, cx = 0.5 * nx, cy = 0.5 * ny;
        if (geo.ns < 1 || !(R > 1.0) || R + 2.0 > 0.5 * std::min(nx, ny)) {
            why = "circle must fit inside the grid with a 2-cell margin"; return TOMO_ERR_ARG;
        }
        if (!(C > 0.0) || C > 0.70710678) { why = "courant must be in (0, 1/sqrt(2)]"; return TOMO_ERR_ARG; }
        if (!(c.cells_per_wavelength >= 2.0f)) { why = "cells_per_wavelength must be >= 2"; return TOMO_ERR_ARG; }
        if (c.sponge_width < 0 || c.sponge_width > 64 || c.sponge_max < 0.f || c.sponge_max >= 1.f) {
            why = "bad sponge (width 0..64, 0 <= max < 1)";
            return TOMO_ERR_ARG;
        }
        geo.ii.resize(geo.ns); geo.jj.resize(geo.ns);
        for (int p = 0; p < geo.ns; ++p) {
            const double th = 2.0 * M_PI * p / geo.ns;
            geo.ii[p] = (int)std::floor(cx + R * std::cos(th) + 0.5);
            geo.jj[p] = (int)std::floor(cy + R * std::sin(th) + 0.5);
        }
        geo.nch = geo.ns;
        geo.rcv.resize(geo.nch);
        geo.rid.assign(geo.N, -1);
        for (int p = 0; p < geo.ns; ++p) {
            const int cell = geo.jj[p] * nx + geo.ii[p];
            if (geo.rid[cell] >= 0) { why = "two transducers fall on one cell; use fewer transducers"; return TOMO_ERR_ARG; }
            geo.rcv[p] = cell;
            geo.rid[cell] = p;
        }
        geo.mask.assign(geo.N, 0);
        const double rm = R - 1.5;
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                const double dx = i - cx, dy = j - cy;
                if (dx * dx + dy * dy < rm * rm) geo.mask[(int64_t)j * nx + i] = 1;
            }
        // Ricker at peak wavelength cells_per_wavelength (c0 = h = 1), delayed by
        // 1.5 periods, amplitude C^2; emitted while t <= t0.
        const double fp = 1.0 / c.cells_per_wavelength, t0 = 1.5 / fp;
        geo.src.assign(c.nt, 0.f);
        geo.n_src_steps = 0;
        for (int n = 0; n < c.nt; ++n) {
            const double t = n * C - t0;
            if (t > t0) break;
            const double a = (M_PI * fp * t) * (M_PI * fp * t);
            geo.src[n] = (float)(C * C * (1.0 - 2.0 * a) * std::exp(-a));
            geo.n_src_steps = n + 1;
        }
        geo.n_src_steps = std::min(geo.n_src_steps, c.nt - 1);
        geo.corr_scale = C * C;
    }
    geo.G = geo.ns / geo.gs;
    if (geo.G < 1) { why = "group_size larger than the number of transducers"; return TOMO_ERR_ARG; }
    if (geo.ref) {
        geo.box.resize(4 * (size_t)geo.G);
        for (int g = 0; g < geo.G; ++g) {
            const int a = g * geo.gs, b = a + geo.gs - 1;
            // 1-based bounding box -> 0-based cells
            geo.box[4 * g + 0] = std::min(geo.ii[a], geo.ii[b]) - 1;
            geo.box[4 * g + 1] = std::max(geo.ii[a], geo.ii[b]) - 1;
            geo.box[4 * g + 2] = std::min(geo.jj[a], geo.jj[b]) - 1;
            geo.box[4 * g + 3] = std::max(geo.jj[a], geo.jj[b]) - 1;
        }
    } else {
        geo.emit.resize((size_t)geo.G * geo.gs);
        for (int t = 0; t < geo.G * geo.gs; ++t) geo.emit[t] = geo.jj[t] * nx + geo.ii[t];
    }
    return TOMO_OK;
}

tomo_status phantom_ref(int nx, int ny, float* fo) {
    if (nx < 1 || ny < 1 || !fo) return TOMO_ERR_ARG;
    // A 15 mm-radius disc of 0.03 with three 5 mm discs of 0.05 on the circle of
    // radius 15 mm at -30, 210 and 270 degrees; cell centres x = -0.1 + i h.
    const float big_r = 0.015f, small_r = 0.005f;
    const float deg = 3.14159265f / 180.f;
    const float ox = big_r * std::cos(30.f * deg), oy = big_r * std::sin(30.f * deg);
    const float centres[3][2] = {{ox, oy}, {-ox, oy}, {0.f, -big_r}};
    for (int j = 0; j < ny; ++j) {
        const float y = -0.1f + (float)j * kRefH;
        for (int i = 0; i < nx; ++i) {
            const float x = -0.1f + (float)i * kRefH;
            float v = (x * x + y * y <= big_r * big_r) ? 0.03f : 0.f;
            for (const auto& cc : centres) {
                const float dx = x - cc[0], dy = y - cc[1];
                if (dx * dx + dy * dy <= small_r * small_r) v = 0.05f;
            }
            fo[(int64_t)j * nx + i] = v;
        }
    }
    return TOMO_OK;
}

tomo_status phantom_cfg(int nx, int ny, int kind, int n, float rmin, float rmax, float vmax, float noise_sigma,
                        float support, uint64_t seed, float* fo) {
    if (nx < 1 || ny < 1 || !fo || n < 0 || !(rmax >= rmin) || rmin < 0.f || !(support > 0.f)) return TOMO_ERR_ARG;
    if (kind != 0 && kind != 1) return TOMO_ERR_ARG;
    Rng rng(seed);
    const double cx = 0.5 * nx, cy = 0.5 * ny;
    std::vector<double> f((size_t)nx * ny, 0.0);
    for (int e = 0; e < n; ++e) {
        double a, b, th = 0.0;
        if (kind == 0) {  // disc of radius U[rmin, rmax]
            a = b = rmin + (rmax - rmin) * rng.uniform();
        } else {          // ellipse with axes (diameters) U[rmin, rmax], random orientation
            a = 0.5 * (rmin + (rmax - rmin) * rng.uniform());
            b = 0.5 * (rmin + (rmax - rmin) * rng.uniform());
            th = M_PI * rng.uniform();
        }
        const double val = vmax * (2.0 * rng.uniform() - 1.0);
        const double reach = std::max(0.0, (double)support - std::max(a, b));
        const double rad = reach * std::sqrt(rng.uniform()), ang = 2.0 * M_PI * rng.uniform();
        const double ex = cx + rad * std::cos(ang), ey = cy + rad * std::sin(ang);
        const double ct = std::cos(th), st = std::sin(th);
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                const double dx = i - ex, dy = j - ey;
                const double u = (dx * ct + dy * st) / a, v = (-dx * st + dy * ct) / b;
                if (u * u + v * v <= 1.0) f[(size_t)j * nx + i] += val;
            }
    }
    if (noise_sigma > 0.f) {
        // white N(0,1) -> separable Gaussian blur (sigma 2 cells) -> rescaled to
        // standard deviation noise_sigma inside the support circle.
        std::vector<double> w((size_t)nx * ny), t((size_t)nx * ny);
        for (auto& x : w) x = rng.normal();
        const int R = 6;
        double ker[2 * R + 1], ks = 0.0;
        for (int d = -R; d <= R; ++d) ks += (ker[d + R] = std::exp(-0.5 * d * d / 4.0));
        for (auto& k : ker) k /= ks;
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                double acc = 0.0;
                for (int d = -R; d <= R; ++d) acc += ker[d + R] * w[(size_t)j * nx + std::min(std::max(i + d, 0), nx - 1)];
                t[(size_t)j * nx + i] = acc;
            }
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                double acc = 0.0;
                for (int d = -R; d <= R; ++d) acc += ker[d + R] * t[(size_t)std::min(std::max(j + d, 0), ny - 1) * nx + i];
                w[(size_t)j * nx + i] = acc;
            }
        double s2 = 0.0;
        int64_t cnt = 0;
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                const double dx = i - cx, dy = j - cy;
                if (dx * dx + dy * dy <= (double)support * support) { s2 += w[(size_t)j * nx + i] * w[(size_t)j * nx + i]; ++cnt; }
            }
        const double sc = cnt ? noise_sigma / std::sqrt(s2 / cnt) : 0.0;
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                const double dx = i - cx, dy = j - cy;
                if (dx * dx + dy * dy <= (double)support * support) f[(size_t)j * nx + i] += sc * w[(size_t)j * nx + i];
            }
    }
    for (size_t q = 0; q < f.size(); ++q) fo[q] = (float)f[q];
    return TOMO_OK;
}

void add_record_noise(float* rec, int G, int nt, int nch, float level, uint64_t seed) {
    Rng rng(seed);
    for (int g = 0; g < G; ++g)
        for (int c = 0; c < nch; ++c) {
            double s = 0.0, s2 = 0.0;
            for (int k = 0; k < nt; ++k) {
                const double v = rec[((int64_t)g * nt + k) * nch + c];
                s += v; s2 += v * v;
            }
            const double mean = s / nt, var = std::max(0.0, s2 / nt - mean * mean);
            const double amp = level * std::sqrt(var);
            for (int k = 0; k < nt; ++k) {
                const double z = rng.normal();
                if (amp > 0.0) rec[((int64_t)g * nt + k) * nch + c] += (float)(amp * z);
            }
        }
}

void mul_record_noise(float* rec, int G, int nt, int nch, float level, uint64_t seed) {
    for (int g = 0; g < G; ++g)
        for (int k = 0; k < nt; ++k)
            for (int c = 0; c < nch; ++c) rec[((int64_t)g * nt + k) * nch + c] *= noise_factor(seed, level, g, k, c);
}

void fill_damp(DevGeo& g) {
    for (int dd = 0; dd < 64; ++dd) {
        const double x = dd < g.sponge_w ? (double)(g.sponge_w - dd) / (double)g.sponge_w : 0.0;
        g.damp[dd] = (float)(1.0 - (double)g.sponge_max * x * x);
    }
}

}  // namespace tomo
