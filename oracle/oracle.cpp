/*
 * oracle.cpp -- CPU restatement of the reference's reconstruction hot path.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle.h).  The product never links this file.
 *
 * What it restates, in the reference's launch order (all paths relative to the
 * reference project):
 *   Position_Transducers            sirt-mimo.cu:438-466
 *   field_setup                     generate-field.cu:117-172
 *   propagation (+ source, edges)   sirt-mimo.cu:511-593
 *   propagation_at_corners          sirt-mimo.cu:595-615
 *   initial_signal                  sirt-mimo.cu:617-649 (generate-data.cu:364-396)
 *   difference_signal               sirt-mimo.cu:651-684
 *   backpropagation1 / 2            sirt-mimo.cu:686-774
 *   laplace / laplace_corners       sirt-mimo.cu:776-831
 *   update_differential             sirt-mimo.cu:833-856 (per group: sirt-mimo-norm.cu:845-871)
 *   update_field                    sirt-mimo.cu:858-877, sirt-mimo-io.cu:774-795
 *   normalised weights              sirt-mimo-norm.cu:56-118,440-453
 *   intermediate-field rules        sirt-mimo-weight.cu:786-839, sirt-mimo-avg.cu,
 *                                   sirt-mimo-avg-weight.cu:130-203
 *   ART loop                        art-mimo.cu:683-736
 *   epsilon                         sirt-mimo.cu:342-344,427-436
 *
 * Two deliberate restatements, both exact in real arithmetic:
 *   - the correlation sum_k z(k)*Lu(k) is accumulated while the adjoint runs
 *     instead of after it from stored z and Lu histories (the reference's
 *     float atomics make its own summation order undefined anyway);
 *   - the corner mean in backpropagation2 (sirt-mimo.cu:756-772) reads edge
 *     cells that other threads of the same launch write; it is taken here after
 *     the edge copies, i.e. in program order.
 *
 * The CFG profile (synthetic workloads) keeps the same method with documented
 * choices: sponge u <- (1-sigma) u with sigma(d) = smax*((W-d)/W)^2 over the
 * outer W cells, zero field outside the grid, point Ricker emitters and point
 * receivers on a circle, and the exact discrete adjoint of that forward
 * recurrence (so its gradient equals -dJ/df of J = 1/2 sum |P u - meas|^2).
 */
#include "oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// Reference constants as the float values the reference uses (sirt-mimo.cu:26-35).
const float RH = 0.001f;
const float RDT = 3.3333e-07f;
const float ROMEGAC = 7.8540e+05f;
const float RTAO = 4.0000e-06f;
const float RTT = 8.1573e-06f;
const double PI = 3.14159265358979323846;

struct Problem {
    tomo_config c{};
    bool ref = true;
    int nx = 0, ny = 0, nt = 0, N = 0, G = 0, gs = 0, NS = 0, nch = 0;
    int lo = 0, hi = 0;
    std::vector<int> ii, jj;                  // transducers
    std::vector<int> ip1, ip2, jp1, jp2;      // REF: group emission boxes (1-based, inclusive)
    std::vector<int> emit;                    // CFG: G*gs emitter cells
    std::vector<int> rcv;                     // receiver cell per channel (-1: none)
    std::vector<double> damp;                 // CFG: 1 - sigma
    std::vector<double> src;                  // CFG: source amplitude added at step n
    std::vector<uint8_t> mask;                // update mask
    double corr_scale = 1.0;                  // REF: 1/h^2; CFG: C^2
};

int nthreads(int threads) {
#ifdef _OPENMP
    return threads > 0 ? threads : omp_get_max_threads();
#else
    (void)threads;
    return 1;
#endif
}

int setup(const tomo_config* cfg, Problem& P) {
    if (!cfg) return TOMO_ERR_ARG;
    P.c = *cfg;
    P.ref = cfg->profile == TOMO_PROFILE_REF;
    P.nx = cfg->nx; P.ny = cfg->ny; P.nt = cfg->nt; P.N = P.nx * P.ny;
    P.gs = cfg->group_size;
    if (P.nx < 8 || P.ny < 8 || P.nt < 4 || P.gs < 1) return TOMO_ERR_ARG;
    if (cfg->profile != TOMO_PROFILE_REF && cfg->profile != TOMO_PROFILE_CFG) return TOMO_ERR_ARG;
    if (P.ref) {
        P.lo = cfg->ring_lo; P.hi = cfg->ring_hi;
        // Sensor lines keep one row/column away from the edge-copy rows 1 and n-2, where the
        // reference's backpropagation2 would otherwise race (sirt-mimo.cu:742-754).
        if (P.lo < 2 || P.hi < P.lo + 2 || P.hi > std::min(P.nx, P.ny) - 3) return TOMO_ERR_ARG;
        const int L = P.hi - P.lo;
        P.NS = 4 * L;
        P.ii.resize(P.NS); P.jj.resize(P.NS);
        // Position_Transducers (sirt-mimo.cu:438-466) on a ring of side L.
        for (int p = 0; p < P.NS; ++p) {
            const int s = p / L, q = p % L;
            if (s == 0)      { P.ii[p] = P.lo + 2 + q; P.jj[p] = P.hi + 1; }
            else if (s == 1) { P.ii[p] = P.hi + 1;     P.jj[p] = P.hi - q; }
            else if (s == 2) { P.ii[p] = P.hi - q;     P.jj[p] = P.lo + 1; }
            else             { P.ii[p] = P.lo + 1;     P.jj[p] = P.lo + 2 + q; }
        }
        P.nch = 4 * P.nx;
        P.rcv.assign(P.nch, -1);
        for (int i = P.lo + 1; i < P.hi; ++i) {      // initial_signal (sirt-mimo.cu:629-647)
            P.rcv[0 * P.nx + i] = P.hi * P.nx + i;   // bottom  u(i, 180)
            P.rcv[1 * P.nx + i] = i * P.nx + P.hi;   // right   u(180, i)
            P.rcv[2 * P.nx + i] = P.lo * P.nx + i;   // top     u(i, 20)
            P.rcv[3 * P.nx + i] = i * P.nx + P.lo;   // left    u(20, i)
        }
        P.mask.assign(P.N, 0);                        // update_field mask [21,180)^2
        for (int j = P.lo + 1; j < P.hi; ++j)
            for (int i = P.lo + 1; i < P.hi; ++i) P.mask[j * P.nx + i] = 1;
        const float hh = RH * RH;
        P.corr_scale = 1.0 / (double)hh;
    } else {
        P.NS = cfg->n_transducers;
        const double R = cfg->radius, C = cfg->courant;
        const double cx = 0.5 * P.nx, cy = 0.5 * P.ny;
        if (P.NS < 1 || !(R > 1.0) || R + 2.0 > 0.5 * std::min(P.nx, P.ny)) return TOMO_ERR_ARG;
        if (!(C > 0.0) || C > 0.70710678 || !(cfg->cells_per_wavelength >= 2.0f)) return TOMO_ERR_ARG;
        if (cfg->sponge_width < 0 || cfg->sponge_max < 0.0f || cfg->sponge_max >= 1.0f) return TOMO_ERR_ARG;
        P.ii.resize(P.NS); P.jj.resize(P.NS);
        for (int p = 0; p < P.NS; ++p) {
            const double th = 2.0 * PI * p / P.NS;
            P.ii[p] = (int)std::floor(cx + R * std::cos(th) + 0.5);
            P.jj[p] = (int)std::floor(cy + R * std::sin(th) + 0.5);
        }
        P.nch = P.NS;
        P.rcv.resize(P.nch);
        for (int p = 0; p < P.NS; ++p) P.rcv[p] = P.jj[p] * P.nx + P.ii[p];
        P.mask.assign(P.N, 0);
        const double rm = R - 1.5;
        for (int j = 0; j < P.ny; ++j)
            for (int i = 0; i < P.nx; ++i) {
                const double dx = i - cx, dy = j - cy;
                P.mask[j * P.nx + i] = (dx * dx + dy * dy < rm * rm) ? 1 : 0;
            }
        const int W = cfg->sponge_width;
        P.damp.assign(P.N, 1.0);
        for (int j = 0; j < P.ny; ++j)
            for (int i = 0; i < P.nx; ++i) {
                const int d = std::min(std::min(i, j), std::min(P.nx - 1 - i, P.ny - 1 - j));
                if (d < W) {
                    const double x = (double)(W - d) / W;
                    P.damp[j * P.nx + i] = 1.0 - cfg->sponge_max * x * x;
                }
            }
        // Ricker wavelet, peak wavelength cells_per_wavelength at c0 = h = 1,
        // delayed by 1.5 periods; amplitude C^2 (the dt^2 c0^2 / h^2 factor).
        const double fp = 1.0 / cfg->cells_per_wavelength, t0 = 1.5 / fp;
        P.src.assign(P.nt, 0.0);
        for (int n = 0; n < P.nt; ++n) {
            const double t = n * C - t0;
            if (t > t0) break;
            const double a = (PI * fp * t) * (PI * fp * t);
            P.src[n] = C * C * (1.0 - 2.0 * a) * std::exp(-a);
        }
        P.corr_scale = C * C;
    }
    P.G = P.NS / P.gs;
    if (P.G < 1) return TOMO_ERR_ARG;
    if (P.ref) {
        P.ip1.resize(P.G); P.ip2.resize(P.G); P.jp1.resize(P.G); P.jp2.resize(P.G);
        for (int g = 0; g < P.G; ++g) {          // sirt-mimo.cu:543-551
            const int p = g * P.gs;
            int a = P.jj[p], b = P.jj[p + P.gs - 1], c = P.ii[p], d = P.ii[p + P.gs - 1];
            if (a > b) std::swap(a, b);
            if (c > d) std::swap(c, d);
            P.jp1[g] = a; P.jp2[g] = b; P.ip1[g] = c; P.ip2[g] = d;
        }
    } else {
        P.emit.resize((size_t)P.G * P.gs);
        for (int g = 0; g < P.G; ++g)
            for (int q = 0; q < P.gs; ++q) {
                const int p = g * P.gs + q;
                P.emit[(size_t)g * P.gs + q] = P.jj[p] * P.nx + P.ii[p];
            }
    }
    return TOMO_OK;
}

// ---------------------------------------------------------------------------
// Per-cell coefficients from f.
template <typename T>
struct Coef {
    std::vector<T> v, r, onef;   // REF: v = 1500 sqrt(1+f), r = v dt / h, 1+f
    std::vector<T> c;            // CFG: C^2 (1+f)
};

template <typename T>
void make_coef(const Problem& P, const double* f, Coef<T>& K) {
    if (P.ref) {
        K.v.resize(P.N); K.r.resize(P.N); K.onef.resize(P.N);
        for (int q = 0; q < P.N; ++q) {
            const T fq = (T)f[q];
            K.v[q] = T(1500) * std::sqrt(T(1) + fq);            // sirt-mimo.cu:525
            K.r[q] = K.v[q] * T(RDT) / T(RH);                    // sirt-mimo.cu:526
            K.onef[q] = T(1) + fq;
        }
    } else {
        const T C2 = (T)P.c.courant * (T)P.c.courant;
        K.c.resize(P.N);
        for (int q = 0; q < P.N; ++q) K.c[q] = C2 * (T(1) + (T)f[q]);
    }
}

// ---------------------------------------------------------------------------
// REF forward of group g into the full history u (nt*N, zeroed by caller).
template <typename T>
void forward_ref(const Problem& P, const Coef<T>& K, int g, T* u, int nth) {
    const int nx = P.nx, ny = P.ny, N = P.N, nt = P.nt;
    const int ip1 = P.ip1[g], ip2 = P.ip2[g], jp1 = P.jp1[g], jp2 = P.jp2[g];
    const T* r = K.r.data();
    const T* v = K.v.data();
#pragma omp parallel num_threads(nth)
    for (int k = 1; k < nt - 1; ++k) {
        const T* uc = u + (size_t)k * N;
        const T* up = u + (size_t)(k - 1) * N;
        T* un = u + (size_t)(k + 1) * N;
#pragma omp for schedule(static)
        for (int j = 0; j < ny; ++j) {
            for (int i = 0; i < nx; ++i) {
                const int q = j * nx + i;
                const T rq = r[q];
                const T s = T(2) - T(4) * rq * rq;
                T val;
                if (i != 0 && i != nx - 1 && j != 0 && j != ny - 1) {       // sirt-mimo.cu:532-541
                    val = rq * rq * (uc[q + 1] + uc[q - 1] + uc[q - nx] + uc[q + nx]) + s * uc[q] - up[q];
                    if (j + 1 >= jp1 && j + 1 <= jp2 && i + 1 >= ip1 && i + 1 <= ip2 && k + 1 <= 24) {
                        const T t = (T)k * T(RDT) - T(RTT);                  // sirt-mimo.cu:553-561
                        val += v[q] * v[q] * T(RDT) * T(RDT) * std::cos(T(ROMEGAC) * t) *
                               std::exp(-(t * t) / (T(2) * T(RTAO) * T(RTAO)));
                    }
                } else {                                                    // sirt-mimo.cu:565-587
                    const bool top = (j == 0), bottom = (j == ny - 1);
                    const bool left = (i == 0), right = (i == nx - 1);
                    const int ja = top ? j + 1 : bottom ? j - 1 : j;
                    const int jb = top ? j + 2 : bottom ? j - 2 : j;
                    const int ia = left ? i + 1 : right ? i - 1 : i;
                    const int ib = left ? i + 2 : right ? i - 2 : i;
                    const int qa = ja * nx + ia, qb = jb * nx + ib;
                    val = (T(2) - T(2) * rq - rq * rq) * uc[q] + T(2) * rq * (T(1) + rq) * uc[qa] -
                          rq * rq * uc[qb] + (T(2) * rq - T(1)) * up[q] - T(2) * rq * up[qa];
                }
                un[q] = val;
            }
        }
    }
    // propagation_at_corners for every k (sirt-mimo.cu:595-615)
    for (int k = 0; k < nt; ++k) {
        T* a = u + (size_t)k * N;
        a[0] = T(1) / T(2) * (a[1 * nx + 0] + a[0 * nx + 1]);
        a[nx - 1] = T(1) / T(2) * (a[nx - 2] + a[1 * nx + nx - 1]);
        a[(ny - 1) * nx] = T(1) / T(2) * (a[(ny - 2) * nx] + a[(ny - 1) * nx + 1]);
        a[(ny - 1) * nx + nx - 1] = T(1) / T(2) * (a[(ny - 1) * nx + nx - 2] + a[(ny - 2) * nx + nx - 1]);
    }
}

// CFG forward of group g into the full history u (nt*N, zeroed by caller).
template <typename T>
void forward_cfg(const Problem& P, const Coef<T>& K, int g, T* u, int nth) {
    const int nx = P.nx, ny = P.ny, N = P.N, nt = P.nt;
    const T* c = K.c.data();
    std::vector<T> d(P.damp.begin(), P.damp.end());
#pragma omp parallel num_threads(nth)
    for (int k = 1; k < nt - 1; ++k) {
        const T* uc = u + (size_t)k * N;
        const T* up = u + (size_t)(k - 1) * N;
        T* un = u + (size_t)(k + 1) * N;
#pragma omp for schedule(static)
        for (int j = 0; j < ny; ++j) {
            for (int i = 0; i < nx; ++i) {
                const int q = j * nx + i;
                const T e = i + 1 < nx ? uc[q + 1] : T(0);
                const T w = i > 0 ? uc[q - 1] : T(0);
                const T s = j > 0 ? uc[q - nx] : T(0);
                const T n = j + 1 < ny ? uc[q + nx] : T(0);
                const T lap = (e + w + s + n) - T(4) * uc[q];
                un[q] = d[q] * ((T(2) * uc[q] - up[q]) + c[q] * lap);
            }
        }
#pragma omp single
        {
            const T a = (T)P.src[k];
            if (a != T(0))
                for (int q = 0; q < P.gs; ++q) un[P.emit[(size_t)g * P.gs + q]] += a;
        }
    }
}

// Records of group g from its history, and the residual meas - rec.
template <typename T>
void record(const Problem& P, const T* u, float* rec_g, const float* meas_g, T* rr, double* resid2) {
    const int nch = P.nch;
    double acc = 0.0;
    for (int k = 0; k < P.nt; ++k)
        for (int ch = 0; ch < nch; ++ch) {
            const int cell = P.rcv[ch];
            const bool on = cell >= 0 && k > 1;                          // k > 1 (sirt-mimo.cu:629)
            const T val = on ? u[(size_t)k * P.N + cell] : T(0);
            if (rec_g) rec_g[(size_t)k * nch + ch] = (float)val;
            if (rr) {
                const T e = on ? (T)meas_g[(size_t)k * nch + ch] - val : T(0);   // sirt-mimo.cu:670-682
                rr[(size_t)k * nch + ch] = e;
                acc += (double)e * (double)e;
            }
        }
    if (resid2) *resid2 += acc;
}

// REF adjoint of group g with on-the-fly correlation; corr += sum_k z(k) Lu(k)
// (Lu without the 1/h^2 factor, which is applied with corr_scale).
template <typename T>
void adjoint_ref(const Problem& P, const Coef<T>& K, const T* u, const T* rr, double* corr, int nth) {
    const int nx = P.nx, ny = P.ny, N = P.N, nt = P.nt, nch = P.nch, lo = P.lo, hi = P.hi;
    std::vector<T> zb((size_t)3 * N, T(0));
    std::vector<T> Lu(N);
    const T* of = K.onef.data();
    const T A = T(1500) * T(1500) * (T(RDT) * T(RDT));
    const T HH = T(RH) * T(RH);
#pragma omp parallel num_threads(nth)
    for (int k = nt - 2; k > 0; --k) {
        T* zk = zb.data() + (size_t)(k % 3) * N;
        const T* z1 = zb.data() + (size_t)((k + 1) % 3) * N;
        const T* z2 = zb.data() + (size_t)((k + 2) % 3) * N;
        const T* uk = u + (size_t)k * N;
        const T* rk = rr + (size_t)k * nch;
        // backpropagation1 (sirt-mimo.cu:686-710)
#pragma omp for schedule(static)
        for (int j = 1; j < ny - 1; ++j)
            for (int i = 1; i < nx - 1; ++i) {
                const int q = j * nx + i;
                zk[q] = A * (of[q - nx] * z1[q - nx] + of[q + nx] * z1[q + nx] + of[q - 1] * z1[q - 1] +
                             of[q + 1] * z1[q + 1] - T(4) * of[q] * z1[q]) / HH +
                        T(2) * z1[q] - z2[q];
            }
#pragma omp single
        {
            // backpropagation2 (sirt-mimo.cu:712-774): sensor lines (z + (rr H) 1000, the
            // reference's order), then edges, then corners.
            for (int i = lo + 1; i < hi; ++i) {
                zk[hi * nx + i] = zk[(hi - 1) * nx + i] + rk[0 * nx + i] * T(RH) * T(1000);
                zk[lo * nx + i] = zk[(lo + 1) * nx + i] + rk[2 * nx + i] * T(RH) * T(1000);
                zk[i * nx + hi] = zk[i * nx + hi - 1] + rk[1 * nx + i] * T(RH) * T(1000);
                zk[i * nx + lo] = zk[i * nx + lo + 1] + rk[3 * nx + i] * T(RH) * T(1000);
            }
            for (int i = 1; i < nx - 1; ++i) {
                zk[i] = zk[nx + i];
                zk[(ny - 1) * nx + i] = zk[(ny - 2) * nx + i];
            }
            for (int j = 1; j < ny - 1; ++j) {
                zk[j * nx] = zk[j * nx + 1];
                zk[j * nx + nx - 1] = zk[j * nx + nx - 2];
            }
            zk[0] = (zk[1] + zk[nx]) / T(2);
            zk[nx - 1] = (zk[nx - 2] + zk[nx + nx - 1]) / T(2);
            zk[(ny - 1) * nx] = (zk[(ny - 1) * nx + 1] + zk[(ny - 2) * nx]) / T(2);
            zk[(ny - 1) * nx + nx - 1] = (zk[(ny - 1) * nx + nx - 2] + zk[(ny - 2) * nx + nx - 1]) / T(2);
        }
        // laplace (sirt-mimo.cu:776-804) with clamped edges, unscaled
#pragma omp for schedule(static)
        for (int j = 0; j < ny; ++j) {
            const int ja = j > 0 ? j - 1 : j, jb = j < ny - 1 ? j + 1 : j;
            for (int i = 0; i < nx; ++i) {
                const int ia = i > 0 ? i - 1 : i, ib = i < nx - 1 ? i + 1 : i;
                Lu[j * nx + i] = uk[ja * nx + i] + uk[jb * nx + i] + uk[j * nx + ia] + uk[j * nx + ib] -
                                 T(4) * uk[j * nx + i];
            }
        }
#pragma omp single
        {
            // laplace_corners (sirt-mimo.cu:806-831)
            Lu[0] = (Lu[1] + Lu[nx]) / T(2);
            Lu[nx - 1] = (Lu[nx - 2] + Lu[nx + nx - 1]) / T(2);
            Lu[(ny - 1) * nx] = (Lu[(ny - 1) * nx + 1] + Lu[(ny - 2) * nx]) / T(2);
            Lu[(ny - 1) * nx + nx - 1] = (Lu[(ny - 1) * nx + nx - 2] + Lu[(ny - 2) * nx + nx - 1]) / T(2);
        }
        // update_differential (sirt-mimo.cu:833-856)
#pragma omp for schedule(static)
        for (int q = 0; q < N; ++q) corr[q] += (double)zk[q] * (double)Lu[q];
    }
    (void)HH;
}

// CFG exact adjoint of group g; corr += sum_m z(m) * Lap u(m-1).
template <typename T>
void adjoint_cfg(const Problem& P, const Coef<T>& K, const T* u, const T* rr, double* corr, int nth) {
    const int nx = P.nx, ny = P.ny, N = P.N, nt = P.nt, nch = P.nch;
    std::vector<T> zb((size_t)3 * N, T(0));
    std::vector<T> inj(N, T(0));
    std::vector<T> d(P.damp.begin(), P.damp.end());
    const T* c = K.c.data();
#pragma omp parallel num_threads(nth)
    for (int m = nt - 1; m >= 2; --m) {
        T* zm = zb.data() + (size_t)(m % 3) * N;
        const T* z1 = zb.data() + (size_t)((m + 1) % 3) * N;
        const T* z2 = zb.data() + (size_t)((m + 2) % 3) * N;
        const T* um = u + (size_t)(m - 1) * N;
#pragma omp single
        {
            const T* rm = rr + (size_t)m * nch;
            for (int ch = 0; ch < nch; ++ch) inj[P.rcv[ch]] += rm[ch];
        }
#pragma omp for schedule(static)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                const int q = j * nx + i;
                const T e = i + 1 < nx ? c[q + 1] * z1[q + 1] : T(0);
                const T w = i > 0 ? c[q - 1] * z1[q - 1] : T(0);
                const T s = j > 0 ? c[q - nx] * z1[q - nx] : T(0);
                const T n = j + 1 < ny ? c[q + nx] * z1[q + nx] : T(0);
                const T lz = (e + w + s + n) - T(4) * c[q] * z1[q];
                zm[q] = d[q] * ((T(2) * z1[q] - z2[q]) + lz + inj[q]);
                const T ue = i + 1 < nx ? um[q + 1] : T(0);
                const T uw = i > 0 ? um[q - 1] : T(0);
                const T us = j > 0 ? um[q - nx] : T(0);
                const T un = j + 1 < ny ? um[q + nx] : T(0);
                const T lu = (ue + uw + us + un) - T(4) * um[q];
                corr[q] += (double)zm[q] * (double)lu;
            }
#pragma omp single
        {
            for (int ch = 0; ch < nch; ++ch) inj[P.rcv[ch]] = T(0);
        }
    }
}

// One group's raw correlation C_g (added into corr) and residual.
template <typename T>
void group_sweep(const Problem& P, const Coef<T>& K, int g, std::vector<T>& hist, const float* meas,
                 float* rec_out, double* corr, double* resid2, int nth) {
    std::fill(hist.begin(), hist.end(), T(0));
    if (P.ref) forward_ref<T>(P, K, g, hist.data(), nth);
    else forward_cfg<T>(P, K, g, hist.data(), nth);
    const size_t rs = (size_t)P.nt * P.nch;
    if (!meas) {
        record<T>(P, hist.data(), rec_out ? rec_out + (size_t)g * rs : nullptr, nullptr, nullptr, nullptr);
        return;
    }
    std::vector<T> rr(rs);
    record<T>(P, hist.data(), rec_out ? rec_out + (size_t)g * rs : nullptr, meas + (size_t)g * rs, rr.data(),
              resid2);
    if (corr) {
        if (P.ref) adjoint_ref<T>(P, K, hist.data(), rr.data(), corr, nth);
        else adjoint_cfg<T>(P, K, hist.data(), rr.data(), corr, nth);
    }
}

template <typename T>
void gradient_all(const Problem& P, const double* f, const float* meas, double* dfg, double* resid2, int nth) {
    Coef<T> K;
    make_coef<T>(P, f, K);
    std::vector<T> hist((size_t)P.nt * P.N);
    std::vector<double> corr(P.N);
    double r2 = 0.0;
    for (int g = 0; g < P.G; ++g) {
        std::fill(corr.begin(), corr.end(), 0.0);
        group_sweep<T>(P, K, g, hist, meas, nullptr, corr.data(), &r2, nth);
        if (dfg)
            for (int q = 0; q < P.N; ++q) dfg[(size_t)g * P.N + q] = corr[q] * P.corr_scale / (1.0 + f[q]);
    }
    if (resid2) *resid2 = r2;
}

double sched_scale(const tomo_schedule* s, int it) {
    switch (s->kind) {
    case TOMO_SCHED_CONST: return s->omega;
    case TOMO_SCHED_POWER: return (double)s->omega * (s->alpha + s->beta / std::pow((double)(it + 1), (double)s->gamma));
    case TOMO_SCHED_LINEAR: return (double)s->omega * (s->alpha + s->beta * (double)(it + 1));
    default: return std::numeric_limits<double>::quiet_NaN();
    }
}

void normalize_dir(const Problem& P, std::vector<double>& dir) {
    double m = 0.0;
    for (int q = 0; q < P.N; ++q)
        if (P.mask[q]) m = std::max(m, std::fabs(dir[q]));
    if (m > 0.0)
        for (double& x : dir) x /= m;
}

double epsilon_of(const Problem& P, const double* f, const double* fo) {
    double a = 0.0, b = 0.0;
    for (int q = 0; q < P.N; ++q) {
        const double e = f[q] - fo[q];
        a += e * e;
        b += fo[q] * fo[q];
    }
    return 100.0 * std::sqrt(a) / std::sqrt(b);
}

template <typename T>
int iterate_t(const Problem& P, int method, const tomo_schedule* sch, int it, double* f, const float* meas,
              const double* fo, double* stats, int nth) {
    const int N = P.N, G = P.G;
    const double s = sched_scale(sch, it);
    double r2 = 0.0;
    if (method == TOMO_ART) {
        // art-mimo.cu:688-736: every group updates f before the next one runs.
        std::vector<T> hist((size_t)P.nt * N);
        std::vector<double> corr(N), dir(N);
        for (int g = 0; g < G; ++g) {
            Coef<T> K;
            make_coef<T>(P, f, K);
            std::fill(corr.begin(), corr.end(), 0.0);
            group_sweep<T>(P, K, g, hist, meas, nullptr, corr.data(), &r2, nth);
            for (int q = 0; q < N; ++q) dir[q] = corr[q] * P.corr_scale / (1.0 + f[q]);
            if (sch->normalize) normalize_dir(P, dir);
            for (int q = 0; q < N; ++q)
                if (P.mask[q]) f[q] += s * dir[q];
        }
    } else {
        std::vector<double> dfg((size_t)G * N);
        gradient_all<T>(P, f, meas, dfg.data(), &r2, nth);
        std::vector<double> sum(N, 0.0), dir(N, 0.0);
        for (int g = 0; g < G; ++g)
            for (int q = 0; q < N; ++q) sum[q] += dfg[(size_t)g * N + q];
        switch (method) {
        case TOMO_SIRT_CLASSIC:   // sirt-mimo.cu:858-877
            dir = sum;
            break;
        case TOMO_SIRT_SCALED:    // sirt-mimo-io.cu:774-795
        case TOMO_SIRT_WEIGHT:    // sirt-mimo-weight.cu:786-839 (mean of f + s*mask*df_g)
        case TOMO_SIRT_AVG:       // sirt-mimo-avg.cu (same, fixed scale)
            for (int q = 0; q < N; ++q) dir[q] = sum[q] / G;
            break;
        case TOMO_SIRT_NORM: {    // sirt-mimo-norm.cu:56-118,440-448
            std::vector<double> w(G);
            double W = 0.0;
            for (int g = 0; g < G; ++g) {
                double a = 0.0;
                for (int q = 0; q < N; ++q) {
                    const double e = dfg[(size_t)g * N + q] - sum[q] / G;
                    a += e * e;
                }
                w[g] = 1.0 / std::sqrt(a);
                W += w[g];
            }
            for (int g = 0; g < G; ++g)
                for (int q = 0; q < N; ++q) dir[q] += dfg[(size_t)g * N + q] * (w[g] / W);
            break;
        }
        case TOMO_SIRT_AVG_WEIGHT: { // sirt-mimo-avg-weight.cu:130-203 (unnormalised sum kept)
            std::vector<double> fbar(N, 0.0), w(G);
            for (int g = 0; g < G; ++g)
                for (int q = 0; q < N; ++q)
                    fbar[q] += (f[q] + (P.mask[q] ? s : 0.0) * dfg[(size_t)g * N + q]) / G;
            for (int g = 0; g < G; ++g) {
                double a = 0.0;
                for (int q = 0; q < N; ++q) {
                    const double e = f[q] + (P.mask[q] ? s : 0.0) * dfg[(size_t)g * N + q] - fbar[q];
                    a += e * e;
                }
                w[g] = std::sqrt(a);
            }
            std::vector<double> add(N, 0.0);
            for (int g = 0; g < G; ++g)
                for (int q = 0; q < N; ++q)
                    add[q] += (f[q] + (P.mask[q] ? s : 0.0) * dfg[(size_t)g * N + q]) / w[g];
            for (int q = 0; q < N; ++q) f[q] += add[q];
            break;
        }
        default:
            return TOMO_ERR_ARG;
        }
        if (method != TOMO_SIRT_AVG_WEIGHT) {
            if (sch->normalize) normalize_dir(P, dir);
            for (int q = 0; q < N; ++q)
                if (P.mask[q]) f[q] += s * dir[q];
        }
    }
    if (stats) {
        stats[0] = fo ? epsilon_of(P, f, fo) : std::numeric_limits<double>::quiet_NaN();
        stats[1] = r2;
        stats[2] = s;
    }
    return TOMO_OK;
}

}  // namespace

extern "C" {

int orc_info_get(const tomo_config* cfg, orc_info* out) {
    Problem P;
    const int st = setup(cfg, P);
    if (st) return st;
    out->n_groups = P.G;
    out->n_channels = P.nch;
    out->n_transducers = P.NS;
    return TOMO_OK;
}

int orc_transducers(const tomo_config* cfg, int32_t* ii, int32_t* jj) {
    Problem P;
    const int st = setup(cfg, P);
    if (st) return st;
    for (int p = 0; p < P.NS; ++p) { ii[p] = P.ii[p]; jj[p] = P.jj[p]; }
    return TOMO_OK;
}

int orc_mask(const tomo_config* cfg, uint8_t* mask) {
    Problem P;
    const int st = setup(cfg, P);
    if (st) return st;
    std::memcpy(mask, P.mask.data(), P.N);
    return TOMO_OK;
}

int orc_phantom_ref(int32_t nx, int32_t ny, float* fo) {
    // field_setup (generate-field.cu:117-172) with x(i) = -0.1 + i*h (generate-field.cu:83-87)
    if (nx < 1 || ny < 1 || !fo) return TOMO_ERR_ARG;
    const float rc = 0.015f, rp = 0.005f, sc = 0.03f, sp = 0.05f;
    const float ang = 30.f * (3.14159265f / 180.f);
    const float cx = rc * std::cos(-ang), sy = rc * std::sin(ang);
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            const float x = -0.1f + (float)i * RH, y = -0.1f + (float)j * RH;
            float value = 0.f;
            if (x * x + y * y <= rc * rc) value = sc;
            if ((x - cx) * (x - cx) + (y - sy) * (y - sy) <= rp * rp) value = sp;
            if ((x + cx) * (x + cx) + (y - sy) * (y - sy) <= rp * rp) value = sp;
            if (x * x + (y + rc) * (y + rc) <= rp * rp) value = sp;
            fo[j * nx + i] = value;
        }
    return TOMO_OK;
}

int orc_forward(const tomo_config* cfg, int prec, int threads, const double* f, float* records, double* u_last) {
    Problem P;
    const int st = setup(cfg, P);
    if (st) return st;
    const int nth = nthreads(threads);
    auto run = [&](auto tag) {
        using T = decltype(tag);
        Coef<T> K;
        make_coef<T>(P, f, K);
        std::vector<T> hist((size_t)P.nt * P.N);
        for (int g = 0; g < P.G; ++g) {
            group_sweep<T>(P, K, g, hist, nullptr, records, nullptr, nullptr, nth);
            if (u_last)
                for (int q = 0; q < P.N; ++q)
                    u_last[(size_t)g * P.N + q] = (double)hist[(size_t)(P.nt - 1) * P.N + q];
        }
    };
    if (prec == 32) run(float{});
    else run(double{});
    return TOMO_OK;
}

int orc_gradient(const tomo_config* cfg, int prec, int threads, const double* f, const float* meas, double* dfg,
                 double* resid2) {
    Problem P;
    const int st = setup(cfg, P);
    if (st) return st;
    if (!f || !meas) return TOMO_ERR_ARG;
    const int nth = nthreads(threads);
    if (prec == 32) gradient_all<float>(P, f, meas, dfg, resid2, nth);
    else gradient_all<double>(P, f, meas, dfg, resid2, nth);
    return TOMO_OK;
}

int orc_gradient_groups(const tomo_config* cfg, int prec, int threads, const double* f, const float* meas, int g0,
                        int ng, double* dfg, double* resid2) {
    Problem P;
    const int st = setup(cfg, P);
    if (st) return st;
    if (!f || !meas || g0 < 0 || ng < 1 || g0 + ng > P.G) return TOMO_ERR_ARG;
    const int nth = nthreads(threads);
    auto run = [&](auto tag) {
        using T = decltype(tag);
        Coef<T> K;
        make_coef<T>(P, f, K);
        std::vector<T> hist((size_t)P.nt * P.N);
        std::vector<double> corr(P.N);
        double r2 = 0.0;
        for (int g = g0; g < g0 + ng; ++g) {
            std::fill(corr.begin(), corr.end(), 0.0);
            group_sweep<T>(P, K, g, hist, meas, nullptr, corr.data(), &r2, nth);
            if (dfg)
                for (int q = 0; q < P.N; ++q)
                    dfg[(size_t)(g - g0) * P.N + q] = corr[q] * P.corr_scale / (1.0 + f[q]);
        }
        if (resid2) *resid2 = r2;
    };
    if (prec == 32) run(float{});
    else run(double{});
    return TOMO_OK;
}

int orc_iterate(const tomo_config* cfg, int prec, int threads, int method, const tomo_schedule* sched, int iter,
                double* f_inout, const float* meas, const double* f_true, double* stats) {
    Problem P;
    const int st = setup(cfg, P);
    if (st) return st;
    if (!sched || !f_inout || !meas || method < 0 || method >= TOMO_METHOD_COUNT) return TOMO_ERR_ARG;
    const int nth = nthreads(threads);
    if (prec == 32) return iterate_t<float>(P, method, sched, iter, f_inout, meas, f_true, stats, nth);
    return iterate_t<double>(P, method, sched, iter, f_inout, meas, f_true, stats, nth);
}

int orc_sweep(const tomo_config* cfg, int prec, int threads, const double* f, const float* meas, int g0, int ng,
              double* cell_updates) {
    Problem P;
    const int st = setup(cfg, P);
    if (st) return st;
    if (g0 < 0 || ng < 1 || g0 + ng > P.G || !f || !meas) return TOMO_ERR_ARG;
    const int nth = nthreads(threads);
    auto run = [&](auto tag) {
        using T = decltype(tag);
        Coef<T> K;
        make_coef<T>(P, f, K);
        std::vector<T> hist((size_t)P.nt * P.N);
        std::vector<double> corr(P.N, 0.0);
        double r2 = 0.0;
        for (int g = g0; g < g0 + ng; ++g) group_sweep<T>(P, K, g, hist, meas, nullptr, corr.data(), &r2, nth);
    };
    if (prec == 32) run(float{});
    else run(double{});
    if (cell_updates) *cell_updates = 2.0 * (double)ng * (double)(P.nt - 2) * (double)P.N;
    return TOMO_OK;
}

}  // extern "C"
