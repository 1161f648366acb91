// kernels.cu -- sm_103a kernels of the reconstruction hot path.
//
// One forward step, one adjoint step with the fused residual injection and
// gradient correlation, the sensor gather, and the deterministic reductions and
// update rules.  The per-step kernels are launched once per time step inside a
// CUDA graph (engine.cu); every group of a pass advances in the same launch.
//
// Reference correspondence (paths inside the reference project):
//   k_fwd<REF>  propagation + source + one-way edges + corner fix-up
//               (sirt-mimo.cu:511-615)
//   k_gather    initial_signal / difference_signal (sirt-mimo.cu:617-684)
//   k_adj<REF>  backpropagation1 + backpropagation2 + laplace + laplace_corners
//               + update_differential, fused (sirt-mimo.cu:686-856)
//   k_combine / k_apply / norms   update_field family and the normalised
//               weights (sirt-mimo.cu:858-877, sirt-mimo-norm.cu:56-118)
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <cstdlib>

#include "internal.h"

namespace tomo {
namespace {

#include "cell.cuh"

constexpr int BX = 32;
constexpr int BY = 8;
constexpr int RED_BLOCKS = 304;   // 2 x 152 SMs
constexpr int RED_THREADS = 256;

__device__ __forceinline__ float ldg(const float* p) { return __ldg(p); }

// ---------------------------------------------------------------------------
// Explicitly rounded FP32 operations: the reference-profile kernels evaluate the reference's
// formulas in its operation order with every operation rounded to nearest and nothing
// contracted into a fused multiply-add, so they give the bits of the oracle's FP32 transcription
// of the reference (compiled without contraction) on every GPU and host.
__device__ __forceinline__ float rm(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float ra(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float rs(float a, float b) { return __fsub_rn(a, b); }

// Coefficients of one field.  REF (sirt-mimo.cu:525-526): v = 1500 sqrt(1+f),
// r = v dt / h in FP32, coef = r*r, rcoef = v (r is recomputed from v where needed, with the
// same operations).  CFG: c = C^2 (1+f) evaluated in FP64 and rounded once.
__global__ void k_coef(int profile, const float* __restrict__ f, float* __restrict__ coef,
                       float* __restrict__ rcoef, int64_t N, float courant) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < N; q += (int64_t)gridDim.x * blockDim.x) {
        if (profile == TOMO_PROFILE_REF) {
            const float v = rm(1500.f, __fsqrt_rn(ra(1.f, f[q])));
            const float r = __fdiv_rn(rm(v, kRefDT), kRefH);
            coef[q] = rm(r, r);
            rcoef[q] = v;
        } else {
            const double c2 = (double)courant * (double)courant;
            coef[q] = (float)(c2 * (1.0 + (double)f[q]));
        }
    }
}

// One-way absorbing edge update of the reference at edge cell (i, j) (sirt-mimo.cu:565-587),
// in its operation order: ((((2 - 2r - r r) u + 2r (1+r) ua) - r r ub) + (2r - 1) up) - 2r upa.
__device__ __forceinline__ float ref_abc(const float* __restrict__ uc, const float* __restrict__ up,
                                         const float* __restrict__ rcoef, int i, int j, int nx, int ny) {
    const bool top = (j == 0), bottom = (j == ny - 1);
    const bool left = (i == 0), right = (i == nx - 1);
    const int ja = top ? j + 1 : bottom ? j - 1 : j;
    const int jb = top ? j + 2 : bottom ? j - 2 : j;
    const int ia = left ? i + 1 : right ? i - 1 : i;
    const int ib = left ? i + 2 : right ? i - 2 : i;
    const int64_t q = (int64_t)j * nx + i, qa = (int64_t)ja * nx + ia, qb = (int64_t)jb * nx + ib;
    const float r = __fdiv_rn(rm(ldg(rcoef + q), kRefDT), kRefH);
    const float r2 = rm(r, r), tr = rm(2.f, r);
    const float a1 = rm(rs(rs(2.f, tr), r2), uc[q]);
    const float a2 = rm(rm(tr, ra(1.f, r)), uc[qa]);
    const float a3 = rm(r2, uc[qb]);
    const float a4 = rm(rs(tr, 1.f), up[q]);
    const float a5 = rm(tr, up[qa]);
    return rs(ra(rs(ra(a1, a2), a3), a4), a5);
}

// ---------------------------------------------------------------------------
// Forward step: slice k+1 of every group of the pass from slices k and k-1.
template <int PROF>
__global__ void __launch_bounds__(BX * BY) k_fwd(DevGeo g, const float* __restrict__ coef,
                                                 const float* __restrict__ rcoef, FwdStep s) {
    const int i = blockIdx.x * BX + threadIdx.x;
    const int j = blockIdx.y * BY + threadIdx.y;
    const int gl = blockIdx.z;
    const int nx = g.nx, ny = g.ny;
    if (i >= nx || j >= ny) return;
    const int64_t q = (int64_t)j * nx + i;
    const float* uc = s.uc + gl * s.gstride;
    const float* up = s.up + gl * s.gstride;
    float val;
    if (PROF == TOMO_PROFILE_REF) {
        if (i > 0 && i < nx - 1 && j > 0 && j < ny - 1) {
            // r r (((E + W) + S) + N) + (2 - 4 r r) u - up (sirt-mimo.cu:532-541); 4 r r is exact
            const float r2 = ldg(coef + q);
            const float nb = ra(ra(ra(uc[q + 1], uc[q - 1]), uc[q - nx]), uc[q + nx]);
            val = rs(ra(rm(r2, nb), rm(rs(2.f, rm(4.f, r2)), uc[q])), up[q]);
            if (s.k < g.n_src_steps) {                       // k + 1 <= 24 (sirt-mimo.cu:554)
                const int32_t* b = g.box + 4 * (s.g0 + gl);
                if (i >= b[0] && i <= b[1] && j >= b[2] && j <= b[3]) {
                    // v v DT DT cos(wc t) exp(-t^2 / 2 tau^2) (sirt-mimo.cu:555-560); the two FP32
                    // factors come from the host's table (src[k], src[n_src_steps + k])
                    const float v = ldg(rcoef + q);
                    const float a = rm(rm(rm(rm(v, v), kRefDT), kRefDT), ldg(g.src + s.k));
                    val = ra(val, rm(a, ldg(g.src + g.n_src_steps + s.k)));
                }
            }
        } else if ((i == 0 || i == nx - 1) && (j == 0 || j == ny - 1)) {
            // corner: the mean of its two edge neighbours, which propagation_at_corners
            // applies after the sweep (sirt-mimo.cu:595-615); corners feed no other cell.
            const int i1 = i == 0 ? 1 : nx - 2, j1 = j == 0 ? 1 : ny - 2;
            val = 0.5f * (ref_abc(uc, up, rcoef, i, j1, nx, ny) + ref_abc(uc, up, rcoef, i1, j, nx, ny));
        } else {
            val = ref_abc(uc, up, rcoef, i, j, nx, ny);
        }
    } else {
        // the strip kernels' cell arithmetic (cell.cuh), so every CFG path gives the same bits
        const float e = i + 1 < nx ? uc[q + 1] : 0.f;
        const float w = i > 0 ? uc[q - 1] : 0.f;
        const float so = j > 0 ? uc[q - nx] : 0.f;
        const float no = j + 1 < ny ? uc[q + nx] : 0.f;
        const float a = s.k < g.n_src_steps ? emit_at(g.emit + (int64_t)(s.g0 + gl) * g.gs, g.gs, q, ldg(g.src + s.k))
                                            : 0.f;
        val = fwd_cell(e, w, so, no, uc[q], up[q], ldg(coef + q), sponge(g, i, j), a);
    }
    s.un[gl * s.gstride + q] = val;
    if (s.ck) s.ck[gl * s.ckstride + q] = val;
}

// ---------------------------------------------------------------------------
// Adjoint step with fused residual injection and correlation.
//
// REF: z(k) = r2-weighted Laplacian of z(k+1) + 2 z(k+1) - z(k+2) on interior
// cells (backpropagation1); sensor lines take the inner neighbour's value plus
// the residual, edges the inner neighbour's, corners the mean of their edges
// (backpropagation2).  Every cell is a pure function of z(k+1), z(k+2), so each
// thread evaluates backpropagation1 at its "source" cell.  The correlation
// adds z(k) * Lu(k), Lu the clamped-edge Laplacian of u(k) with corner means
// (laplace, laplace_corners); the 1/h^2 factor is applied by the update.
// backpropagation1 at interior cell q (sirt-mimo.cu:697-707) in its operation order:
// ((A ((((of_s z_s + of_n z_n) + of_w z_w) + of_e z_e) - 4 of z)) / h^2 + 2 z) - z2, with
// A = (1500 1500)(DT DT) and of = 1 + f.
__device__ __forceinline__ float ref_bp1(const float* __restrict__ f, const float* __restrict__ z1,
                                         const float* __restrict__ z2, int64_t q, int nx) {
    constexpr float A = (1500.f * 1500.f) * (kRefDT * kRefDT);
    constexpr float HH = kRefH * kRefH;
    const float s = ra(ra(ra(rm(ra(1.f, ldg(f + q - nx)), z1[q - nx]), rm(ra(1.f, ldg(f + q + nx)), z1[q + nx])),
                          rm(ra(1.f, ldg(f + q - 1)), z1[q - 1])),
                       rm(ra(1.f, ldg(f + q + 1)), z1[q + 1]));
    const float l = rs(s, rm(rm(4.f, ra(1.f, ldg(f + q))), z1[q]));
    return rs(ra(__fdiv_rn(rm(A, l), HH), rm(2.f, z1[q])), z2[q]);
}

// (((u_ja + u_jb) + u_ia) + u_ib) - 4 u with clamped edges (sirt-mimo.cu:786-803), unscaled
__device__ __forceinline__ float clamped_lap(const float* __restrict__ u, int i, int j, int nx, int ny) {
    const int ja = j > 0 ? j - 1 : j, jb = j < ny - 1 ? j + 1 : j;
    const int ia = i > 0 ? i - 1 : i, ib = i < nx - 1 ? i + 1 : i;
    return rs(ra(ra(ra(u[(int64_t)ja * nx + i], u[(int64_t)jb * nx + i]), u[(int64_t)j * nx + ia]),
                 u[(int64_t)j * nx + ib]),
              rm(4.f, u[(int64_t)j * nx + i]));
}

template <int PROF>
__global__ void __launch_bounds__(BX * BY) k_adj(DevGeo g, const float* __restrict__ coef,
                                                 const float* __restrict__ fref, AdjStep s) {
    const int i = blockIdx.x * BX + threadIdx.x;
    const int j = blockIdx.y * BY + threadIdx.y;
    const int gl = blockIdx.z;
    const int nx = g.nx, ny = g.ny;
    if (i >= nx || j >= ny) return;
    const int64_t q = (int64_t)j * nx + i;
    const float* z1 = s.z1 + gl * s.zstride;
    const float* z2 = s.z2 + gl * s.zstride;
    const float* u = s.uq + gl * s.ustride;
    const float* rr = s.rr + gl * s.rrstride;
    float val, lu;
    if (PROF == TOMO_PROFILE_REF) {
        int si = i, sj = j, ch = -1;
        const int lo = g.lo, hi = g.hi;
        if (i == 0 || i == nx - 1 || j == 0 || j == ny - 1) {
            si = min(max(i, 1), nx - 2);
            sj = min(max(j, 1), ny - 2);
        } else if (j == hi && i > lo && i < hi) {
            sj = hi - 1; ch = i;                 // bottom
        } else if (j == lo && i > lo && i < hi) {
            sj = lo + 1; ch = 2 * nx + i;        // top
        } else if (i == hi && j > lo && j < hi) {
            si = hi - 1; ch = nx + j;            // right
        } else if (i == lo && j > lo && j < hi) {
            si = lo + 1; ch = 3 * nx + j;        // left
        }
        val = ref_bp1(fref, z1, z2, (int64_t)sj * nx + si, nx);
        if (ch >= 0) val = ra(val, rm(rm(rr[ch], kRefH), 1000.f));   // z + rr H 1000 (sirt-mimo.cu:725-739)
        if ((i == 0 || i == nx - 1) && (j == 0 || j == ny - 1)) {
            const int i1 = i == 0 ? 1 : nx - 2, j1 = j == 0 ? 1 : ny - 2;
            lu = rm(0.5f, ra(clamped_lap(u, i, j1, nx, ny), clamped_lap(u, i1, j, nx, ny)));
        } else {
            lu = clamped_lap(u, i, j, nx, ny);
        }
    } else {
        // CFG: exact discrete adjoint z(m) = d((2 z1 - z2) + Lap(c z1) + inj),
        // correlation with the zero-padded Laplacian of u(m-1).
        const float e = i + 1 < nx ? mul(ldg(coef + q + 1), z1[q + 1]) : 0.f;
        const float w = i > 0 ? mul(ldg(coef + q - 1), z1[q - 1]) : 0.f;
        const float so = j > 0 ? mul(ldg(coef + q - nx), z1[q - nx]) : 0.f;
        const float no = j + 1 < ny ? mul(ldg(coef + q + nx), z1[q + nx]) : 0.f;
        const int r = g.rid[q];
        const float inj = r >= 0 ? rr[r] : 0.f;
        val = adj_cell(e, w, so, no, mul(ldg(coef + q), z1[q]), z1[q], z2[q], inj, sponge(g, i, j));
        const float ue = i + 1 < nx ? u[q + 1] : 0.f;
        const float uw = i > 0 ? u[q - 1] : 0.f;
        const float us = j > 0 ? u[q - nx] : 0.f;
        const float un = j + 1 < ny ? u[q + nx] : 0.f;
        lu = lap5(ue, uw, us, un, u[q]);
    }
    s.zk[gl * s.zstride + q] = val;
    float* cr = s.corr + gl * s.cstride + q;
    *cr = __fmaf_rn(val, lu, *cr);
}

// ---------------------------------------------------------------------------
// Sensor gather of slice k: simulated records, or residual meas - u with a
// per-(group, k) FP64 sum of squares (fixed-order block reduction).
__global__ void __launch_bounds__(256) k_gather(DevGeo g, GatherStep s) {
    const int gl = blockIdx.x;
    const float* u = s.u + gl * s.gstride;
    const int64_t base = ((int64_t)gl * g.nt + s.k) * g.nch;
    const bool noisy = s.meas && g.noise_key;
    const uint64_t key = noisy ? *g.noise_key : 0;
    double acc = 0.0;
    for (int c = threadIdx.x; c < g.nch; c += blockDim.x) {
        const int cell = g.rcv[c];
        float v = cell >= 0 ? u[cell] : 0.f;
        if (noisy) v *= noise_factor(key, g.noise_level, s.g0 + gl, s.k, c);
        if (s.meas) {
            const float e = cell >= 0 ? s.meas[base + c] - v : 0.f;
            s.out[base + c] = e;
            acc += (double)e * (double)e;
        } else {
            s.out[base + c] = v;
        }
    }
    if (!s.part) return;
    __shared__ double red[256];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) s.part[(int64_t)gl * g.nt + s.k] = red[0];
}

__global__ void k_zero_slots(float* base, int64_t gstride, int64_t off0, int64_t off1, int64_t N) {
    float* g = base + blockIdx.y * gstride;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < N; q += (int64_t)gridDim.x * blockDim.x) {
        g[off0 + q] = 0.f;
        g[off1 + q] = 0.f;
    }
}

__global__ void k_copy_groups(float* dst, int64_t dstride, const float* src, int64_t sstride, int64_t N) {
    const float* s = src + blockIdx.y * sstride;
    float* d = dst + blockIdx.y * dstride;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < N; q += (int64_t)gridDim.x * blockDim.x)
        d[q] = s[q];
}

__global__ void k_fill(float* p, int64_t n, float v) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
        p[q] = v;
}

// ---------------------------------------------------------------------------
// Update-rule helpers.  All sums over groups run in group order per cell; all
// FP64 reductions write one partial per block and are summed in block order.
__global__ void k_combine(const float* __restrict__ corr, int G, int64_t N, const float* __restrict__ f,
                          double scale, const double* __restrict__ w, double post, float* __restrict__ dir) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < N; q += (int64_t)gridDim.x * blockDim.x) {
        const double inv = scale / (1.0 + (double)f[q]);
        double acc = 0.0;
        for (int gg = 0; gg < G; ++gg) {
            const double d = (double)corr[(int64_t)gg * N + q] * inv;
            acc += w ? w[gg] * d : d;
        }
        dir[q] = (float)(acc * post);
    }
}

__device__ __forceinline__ void block_store_sum(double v, double* out) {
    __shared__ double red[RED_THREADS];
    red[threadIdx.x] = v;
    __syncthreads();
    for (int w = RED_THREADS / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = red[0];
}

__global__ void __launch_bounds__(RED_THREADS) k_group_dev_norm(const float* __restrict__ corr, int64_t N,
                                                              const float* __restrict__ f, double scale,
                                                              const float* __restrict__ mean, double* part) {
    const int gg = blockIdx.y;
    double acc = 0.0;
    for (int64_t q = blockIdx.x * (int64_t)RED_THREADS + threadIdx.x; q < N; q += (int64_t)gridDim.x * RED_THREADS) {
        const double d = (double)corr[(int64_t)gg * N + q] * scale / (1.0 + (double)f[q]) - (double)mean[q];
        acc += d * d;
    }
    block_store_sum(acc, part + (int64_t)gg * gridDim.x + blockIdx.x);
}

__device__ __forceinline__ double avgw_fg(const float* corr, int gg, int64_t N, int64_t q, const float* f,
                                          const uint8_t* mask, double scale, double s) {
    const double d = (double)corr[(int64_t)gg * N + q] * scale / (1.0 + (double)f[q]);
    return (double)f[q] + (mask[q] ? s : 0.0) * d;
}

__global__ void k_avgw_fbar(const float* __restrict__ corr, int G, int64_t N, const float* __restrict__ f,
                            const uint8_t* __restrict__ mask, double scale, double s, float* __restrict__ fbar) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < N; q += (int64_t)gridDim.x * blockDim.x) {
        double acc = 0.0;
        for (int gg = 0; gg < G; ++gg) acc += avgw_fg(corr, gg, N, q, f, mask, scale, s);
        fbar[q] = (float)(acc / G);
    }
}

__global__ void __launch_bounds__(RED_THREADS) k_avgw_norm(const float* __restrict__ corr, int64_t N,
                                                         const float* __restrict__ f, const uint8_t* __restrict__ mask,
                                                         double scale, double s, const float* __restrict__ fbar,
                                                         double* part) {
    const int gg = blockIdx.y;
    double acc = 0.0;
    for (int64_t q = blockIdx.x * (int64_t)RED_THREADS + threadIdx.x; q < N; q += (int64_t)gridDim.x * RED_THREADS) {
        const double d = avgw_fg(corr, gg, N, q, f, mask, scale, s) - (double)fbar[q];
        acc += d * d;
    }
    block_store_sum(acc, part + (int64_t)gg * gridDim.x + blockIdx.x);
}

// f += sum_g fg / ||fg - fbar||  -- the unnormalised sum of sirt-mimo-avg-weight.cu:167-203
__global__ void k_avgw_apply(const float* __restrict__ corr, int G, int64_t N, float* __restrict__ f,
                             const uint8_t* __restrict__ mask, double scale, double s, const double* __restrict__ wn) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < N; q += (int64_t)gridDim.x * blockDim.x) {
        double acc = 0.0;
        for (int gg = 0; gg < G; ++gg) acc += avgw_fg(corr, gg, N, q, f, mask, scale, s) / sqrt(wn[gg]);
        f[q] = (float)((double)f[q] + acc);
    }
}

// One block per row: strided per-thread sums, then a fixed-shape tree, so the
// order of the additions depends only on (nb, SUM_THREADS).
constexpr int SUM_THREADS = 256;
__global__ void __launch_bounds__(SUM_THREADS) k_sum_parts(const double* __restrict__ part, int nb,
                                                          double* __restrict__ out) {
    __shared__ double sh[SUM_THREADS];
    const double* p = part + (int64_t)blockIdx.x * nb;
    double acc = 0.0;
    for (int b = threadIdx.x; b < nb; b += SUM_THREADS) acc += p[b];
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int o = SUM_THREADS / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[blockIdx.x] = sh[0];
}

// Normalised-SIRT group weights in place (sirt-mimo-norm.cu:56-118): d2[g] (squared deviation
// norms) -> w[g] = (1 / sqrt(d2[g])) / sum_h 1 / sqrt(d2[h]), FP64, the sum in group order.
__global__ void k_norm_weights(double* __restrict__ d2w, int G) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    double W = 0.0;
    for (int g = 0; g < G; ++g) {
        const double w = 1.0 / sqrt(d2w[g]);
        d2w[g] = w;
        W += w;
    }
    for (int g = 0; g < G; ++g) d2w[g] /= W;
}

__global__ void k_maxabs(const float* __restrict__ dir, const uint8_t* __restrict__ mask, int64_t N,
                         unsigned int* out) {
    float m = 0.f;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < N; q += (int64_t)gridDim.x * blockDim.x)
        if (mask[q]) m = fmaxf(m, fabsf(dir[q]));
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, __float_as_uint(m));   // order-free for m >= 0
}

__global__ void k_apply(float* __restrict__ f, const float* __restrict__ dir, const uint8_t* __restrict__ mask,
                        int64_t N, double s, const unsigned int* __restrict__ maxabs) {
    double sc = s;
    if (maxabs) {
        const float m = __uint_as_float(*maxabs);
        if (m > 0.f) sc = s / (double)m;
    }
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < N; q += (int64_t)gridDim.x * blockDim.x)
        if (mask[q]) f[q] = (float)((double)f[q] + sc * (double)dir[q]);
}

__global__ void __launch_bounds__(RED_THREADS) k_eps_parts(const float* __restrict__ f, const float* __restrict__ fo,
                                                          int64_t N, double* part) {
    double a = 0.0, b = 0.0;
    for (int64_t q = blockIdx.x * (int64_t)RED_THREADS + threadIdx.x; q < N; q += (int64_t)gridDim.x * RED_THREADS) {
        const double e = (double)f[q] - (double)fo[q];
        a += e * e;
        b += (double)fo[q] * (double)fo[q];
    }
    block_store_sum(a, part + blockIdx.x);
    __syncthreads();
    block_store_sum(b, part + gridDim.x + blockIdx.x);
}

// Illumination: I[q] += sum over the pass's groups of u[q]^2 (group order fixed).
__global__ void k_illum_add(const float* __restrict__ u, int ng, int64_t gstride, int64_t N, float* __restrict__ I) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < N; q += (int64_t)gridDim.x * blockDim.x) {
        float acc = I[q];
        for (int gl = 0; gl < ng; ++gl) {
            const float v = u[gl * gstride + q];
            acc = fmaf(v, v, acc);
        }
        I[q] = acc;
    }
}

// Network features, planar [3][N]: f, dir / max|dir|, I / max I (maxima over the mask).
__global__ void k_features(const float* __restrict__ f, const float* __restrict__ dir, const unsigned int* dmax,
                           const float* __restrict__ I, const unsigned int* imax, int64_t N, float* __restrict__ feat) {
    const float dm = __uint_as_float(*dmax), im = __uint_as_float(*imax);
    const float ds = dm > 0.f ? 1.f / dm : 0.f, is = im > 0.f ? 1.f / im : 0.f;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < N; q += (int64_t)gridDim.x * blockDim.x) {
        feat[q] = f[q];
        feat[N + q] = dir[q] * ds;
        feat[2 * N + q] = I[q] * is;
    }
}

inline cudaStream_t S(void* s) { return (cudaStream_t)s; }
inline int grid1(int64_t n, int t) {
    const int64_t b = (n + t - 1) / t;
    return (int)(b < 4 * RED_BLOCKS ? (b < 1 ? 1 : b) : 4 * RED_BLOCKS);
}

}  // namespace

int reduce_blocks() { return RED_BLOCKS; }

void launch_coef(int profile, const float* f, float* coef, float* rcoef, int64_t N, float courant, void* st) {
    k_coef<<<grid1(N, 256), 256, 0, S(st)>>>(profile, f, coef, rcoef, N, courant);
}

void launch_fwd_step(int profile, const DevGeo& g, const float* coef, const float* rcoef, const FwdStep& s,
                     void* st) {
    dim3 grid((g.nx + BX - 1) / BX, (g.ny + BY - 1) / BY, s.ng);
    if (profile == TOMO_PROFILE_REF) k_fwd<TOMO_PROFILE_REF><<<grid, dim3(BX, BY), 0, S(st)>>>(g, coef, rcoef, s);
    else k_fwd<TOMO_PROFILE_CFG><<<grid, dim3(BX, BY), 0, S(st)>>>(g, coef, rcoef, s);
}

void launch_adj_step(int profile, const DevGeo& g, const float* coef, const float* f, const AdjStep& s, void* st) {
    dim3 grid((g.nx + BX - 1) / BX, (g.ny + BY - 1) / BY, s.ng);
    if (profile == TOMO_PROFILE_REF) k_adj<TOMO_PROFILE_REF><<<grid, dim3(BX, BY), 0, S(st)>>>(g, coef, f, s);
    else k_adj<TOMO_PROFILE_CFG><<<grid, dim3(BX, BY), 0, S(st)>>>(g, coef, f, s);
}

void launch_gather(const DevGeo& g, const GatherStep& s, void* st) {
    k_gather<<<s.ng, 256, 0, S(st)>>>(g, s);
}

void launch_fill(float* p, int64_t n, float v, void* st) { k_fill<<<grid1(n, 256), 256, 0, S(st)>>>(p, n, v); }

void launch_illum_add(const float* u, int ng, int64_t gstride, int64_t N, float* I, void* st) {
    k_illum_add<<<grid1(N, 256), 256, 0, S(st)>>>(u, ng, gstride, N, I);
}

void launch_features(const float* f, const float* dir, const unsigned int* dmax, const float* I, const unsigned int* imax,
                     int64_t N, float* feat, void* st) {
    k_features<<<grid1(N, 256), 256, 0, S(st)>>>(f, dir, dmax, I, imax, N, feat);
}

void launch_zero_slots(float* base, int ng, int64_t gstride, int64_t off0, int64_t off1, int64_t N, void* st) {
    const int bx = (int)((N + 255) / 256 < 64 ? (N + 255) / 256 : 64);
    k_zero_slots<<<dim3(bx, ng), 256, 0, S(st)>>>(base, gstride, off0, off1, N);
}

void launch_copy_groups(float* dst, int64_t dstride, const float* src, int64_t sstride, int ng, int64_t N,
                        void* st) {
    const int bx = (int)((N + 255) / 256 < 64 ? (N + 255) / 256 : 64);
    k_copy_groups<<<dim3(bx, ng), 256, 0, S(st)>>>(dst, dstride, src, sstride, N);
}

void launch_combine(const float* corr, int G, int64_t N, const float* f, double scale, const double* w, double post,
                    float* dir, void* st) {
    k_combine<<<grid1(N, 256), 256, 0, S(st)>>>(corr, G, N, f, scale, w, post, dir);
}

void launch_group_dev_norm(const float* corr, int G, int64_t N, const float* f, double scale, const float* mean,
                           double* part, int nb, void* st) {
    k_group_dev_norm<<<dim3(nb, G), RED_THREADS, 0, S(st)>>>(corr, N, f, scale, mean, part);
}

void launch_avgw_fbar(const float* corr, int G, int64_t N, const float* f, const uint8_t* mask, double scale,
                      double s, float* fbar, void* st) {
    k_avgw_fbar<<<grid1(N, 256), 256, 0, S(st)>>>(corr, G, N, f, mask, scale, s, fbar);
}

void launch_avgw_norm(const float* corr, int G, int64_t N, const float* f, const uint8_t* mask, double scale,
                      double s, const float* fbar, double* part, int nb, void* st) {
    k_avgw_norm<<<dim3(nb, G), RED_THREADS, 0, S(st)>>>(corr, N, f, mask, scale, s, fbar, part);
}

void launch_avgw_apply(const float* corr, int G, int64_t N, float* f, const uint8_t* mask, double scale, double s,
                       const double* w, void* st) {
    k_avgw_apply<<<grid1(N, 256), 256, 0, S(st)>>>(corr, G, N, f, mask, scale, s, w);
}

void launch_sum_parts(const double* part, int rows, int nb, double* out, void* st) {
    if (rows > 0) k_sum_parts<<<rows, SUM_THREADS, 0, S(st)>>>(part, nb, out);
}

void launch_norm_weights(double* d2w, int G, void* st) { k_norm_weights<<<1, 32, 0, S(st)>>>(d2w, G); }

void launch_maxabs(const float* dir, const uint8_t* mask, int64_t N, unsigned int* out, void* st) {
    cudaMemsetAsync(out, 0, sizeof(unsigned int), S(st));
    k_maxabs<<<grid1(N, 256), 256, 0, S(st)>>>(dir, mask, N, out);
}

void launch_apply(float* f, const float* dir, const uint8_t* mask, int64_t N, double s, const unsigned int* maxabs,
                  void* st) {
    k_apply<<<grid1(N, 256), 256, 0, S(st)>>>(f, dir, mask, N, s, maxabs);
}

void launch_eps_parts(const float* f, const float* fo, int64_t N, double* part, int nb, void* st) {
    k_eps_parts<<<nb, RED_THREADS, 0, S(st)>>>(f, fo, N, part);
}

}  // namespace tomo
