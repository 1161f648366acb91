// tile.cu -- multi-step tile kernels of the benchmark-profile (CFG) physics.
//
// The warp-strip kernels (strip.cu) advance every group of a pass by one or two time steps per
// launch.  On small grids (128 x 128, or one group of 512 x 512 in an ART pass) a step is too
// little work to fill the GPU, and the time goes into the launches themselves.  These kernels
// advance a 2-D tile by up to TMAX steps per launch: a block stages its 32 x 32 tile plus a halo
// of 8 cells (48 x 48) of the two input slices, the coefficient, the sponge factor and the
// receiver map in shared memory, then runs the steps there -- the computed region shrinks by
// one cell per step, so the halo cells are computed redundantly and no block waits for another
// inside a launch -- and writes every step's owned cells (the forward history, records,
// checkpoints; the adjoint's last two slices and the correlation).
//
// Cells are evaluated with the helpers of cell.cuh in the strip kernels' operation order, so a
// sweep gives the strip kernels' bits (tested).  Adjoint launches advance T in {1, 2, 6} steps:
// the adjoint ring has four slots and these are the step counts whose two output slices never
// fall on the two input slices' slots.
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

#include "internal.h"

namespace tomo {
namespace {

#include "cell.cuh"

constexpr int TW = 32;               // owned tile width and height
constexpr int HALO = 8;              // staged halo (TMAX steps)
constexpr int RW = TW + 2 * HALO;    // staged region: 48 x 48
constexpr int RC = RW * RW;
constexpr int BXT = 32, BYT = 32;    // block: 32 x 32 threads (one block per SM on small grids: many warps)
constexpr int TPB = BXT * BYT;
constexpr int OWN = TW / BYT;        // owned rows per thread (one column, rows ty + 32 j)
constexpr int UW = TW + 2;           // correlation's forward slice: owned tile plus one cell
constexpr int UC = UW * UW;

struct TileSmem {
    float a[RC];       // forward: u(k0) / adjoint: z(kz0+1), then rotating
    float b[RC];       // forward: u(k0-1) / adjoint: z(kz0+2)
    float c[RC];       // coefficient C^2 (1+f)
    float d[RC];       // sponge factor
    int rid[RC];       // receiver channel of the cell, -1 none
    unsigned char em[RC];  // forward only: 1 where the cell emits for the block's group
    float u[3][UC];    // adjoint only: forward slices for the correlation (step t uses u[t % 3])
};
constexpr size_t FWD_SMEM = sizeof(TileSmem);
constexpr size_t ADJ_SMEM = sizeof(TileSmem);

// Stages the region whose cell (rx, ry) is grid cell (gx0 + rx, gy0 + ry): values outside the
// grid are 0 (the zero-padded field), the sponge factor 1, no receiver.
__device__ __forceinline__ void stage_region(const DevGeo& g, const float* __restrict__ pa,
                                             const float* __restrict__ pb, const float* __restrict__ coef,
                                             int gx0, int gy0, int group, TileSmem& sm) {
    for (int ry = threadIdx.y; ry < RW; ry += BYT) {
        const int y = gy0 + ry;
        for (int rx = threadIdx.x; rx < RW; rx += BXT) {
            const int x = gx0 + rx;
            const int idx = ry * RW + rx;
            float va = 0.f, vb = 0.f, vc = 0.f, vd = 1.f;
            int r = -1;
            if (x >= 0 && x < g.nx && y >= 0 && y < g.ny) {
                const int64_t q = (int64_t)y * g.nx + x;
                va = pa[q];
                vb = pb[q];
                vc = coef[q];
                vd = damp_at(g, edge_dist(x, g.nx), edge_dist(y, g.ny));
                r = g.rid[q];
            }
            sm.a[idx] = va;
            sm.b[idx] = vb;
            sm.c[idx] = vc;
            sm.d[idx] = vd;
            sm.rid[idx] = r;
            sm.em[idx] = r >= 0 && r / g.gs == group;   // channel = transducer; group = transducer / gs
        }
    }
}

__global__ void __launch_bounds__(TPB) k_fwd_tile(DevGeo g, const float* __restrict__ coef, TileFwd a,
                                                  int tiles_x) {
    extern __shared__ __align__(16) unsigned char smraw[];
    TileSmem& sm = *reinterpret_cast<TileSmem*>(smraw);
    const int gl = blockIdx.y;
    const int tx = blockIdx.x % tiles_x, ty = blockIdx.x / tiles_x;
    const int gx0 = tx * TW - HALO, gy0 = ty * TW - HALO;
    const int64_t N = (int64_t)g.nx * g.ny;
    float* base = a.hist + gl * a.gstride;
    const int ggl = a.g0 + gl;                     // global group index
    stage_region(g, base + (int64_t)(a.k0 % a.S) * N, base + (int64_t)((a.k0 - 1) % a.S) * N, coef, gx0, gy0, ggl,
                 sm);
    __syncthreads();
    const bool noisy = a.gmeas && g.noise_key;
    const uint64_t key = noisy ? *g.noise_key : 0;
    float* cur = sm.a;   // u(m-1)
    float* prv = sm.b;   // u(m-2), overwritten in place by u(m)
    for (int t = 1; t <= a.T; ++t) {
        const int m = a.k0 + t;                    // slice computed
        const int k = m - 1;                       // step index of the source
        const float src = k < g.n_src_steps ? g.src[k] : 0.f;
        const int lo = HALO - (a.T - t);           // computed region [lo, RW - lo)^2
        float* outslice = base + (int64_t)(m % a.S) * N;
        float* ck = nullptr;
        if (a.ckpt) {
            int ch = -1, which = 0;
            if (m % a.K == 0) { ch = m / a.K; which = 0; }
            else if ((m - 1) % a.K == 0) { ch = (m - 1) / a.K; which = 1; }
            if (ch >= 1 && ch < a.nchunk) ck = a.ckpt + gl * a.ckstride + ((int64_t)ch * 2 + which) * N;
        }
        const int64_t gbase = ((int64_t)gl * g.nt + m) * g.nch;
        for (int ry = lo + threadIdx.y; ry < RW - lo; ry += BYT) {
            const int y = gy0 + ry;
            if (y < 0 || y >= g.ny) continue;
            const bool own_row = ry >= HALO && ry < HALO + TW;
            for (int rx = lo + threadIdx.x; rx < RW - lo; rx += BXT) {
                const int x = gx0 + rx;
                if (x < 0 || x >= g.nx) continue;
                const int s = ry * RW + rx;
                const int r = sm.rid[s];
                const float am = sm.em[s] ? src : 0.f;
                const float v = fwd_cell(cur[s + 1], cur[s - 1], cur[s - RW], cur[s + RW], cur[s], prv[s], sm.c[s],
                                         sm.d[s], am);
                prv[s] = v;
                if (own_row && rx >= HALO && rx < HALO + TW) {
                    const int64_t q = (int64_t)y * g.nx + x;
                    outslice[q] = v;
                    if (ck) ck[q] = v;
                    if (r >= 0 && a.gout) {
                        float vv = v;
                        if (noisy) vv *= noise_factor(key, g.noise_level, ggl, m, r);
                        a.gout[gbase + r] = a.gmeas ? a.gmeas[gbase + r] - vv : vv;
                    }
                }
            }
        }
        __syncthreads();
        float* tmp = cur;
        cur = prv;
        prv = tmp;
    }
}

// Stages the correlation's forward slice (owned tile plus one cell, zero outside the grid).
__device__ __forceinline__ void stage_u(const DevGeo& g, const float* __restrict__ u, int gx0, int gy0,
                                        float* __restrict__ dst) {
    for (int uy = threadIdx.y; uy < UW; uy += BYT) {
        const int y = gy0 + HALO - 1 + uy;
        for (int ux = threadIdx.x; ux < UW; ux += BXT) {
            const int x = gx0 + HALO - 1 + ux;
            dst[uy * UW + ux] = (x >= 0 && x < g.nx && y >= 0 && y < g.ny) ? u[(int64_t)y * g.nx + x] : 0.f;
        }
    }
}

__global__ void __launch_bounds__(TPB) k_adj_tile(DevGeo g, const float* __restrict__ coef, TileAdj a,
                                                  int tiles_x) {
    extern __shared__ __align__(16) unsigned char smraw[];
    TileSmem& sm = *reinterpret_cast<TileSmem*>(smraw);
    const int gl = blockIdx.y;
    const int tx = blockIdx.x % tiles_x, ty = blockIdx.x / tiles_x;
    const int gx0 = tx * TW - HALO, gy0 = ty * TW - HALO;
    const int64_t N = (int64_t)g.nx * g.ny;
    float* zb = a.z + gl * a.zstride;
    const float* ub = a.hist + gl * a.ustride;
    const float* rr = a.rr + gl * a.rrstride;
    stage_region(g, zb + (int64_t)((a.kz0 + 1) & 3) * N, zb + (int64_t)((a.kz0 + 2) & 3) * N, coef, gx0, gy0, -1, sm);
    stage_u(g, ub + (int64_t)((a.kz0 - 1) % a.S) * N, gx0, gy0, sm.u[1]);
    // owned cells of this thread: column threadIdx.x, rows threadIdx.y + 32 j of the tile; the
    // correlation stays in registers for the launch
    const int ox = threadIdx.x;
    const int x_own = gx0 + HALO + ox;
    float cr[OWN];
#pragma unroll
    for (int j = 0; j < OWN; ++j) {
        const int y = gy0 + HALO + threadIdx.y + BYT * j;
        cr[j] = (x_own < g.nx && y < g.ny) ? a.corr[gl * a.cstride + (int64_t)y * g.nx + x_own] : 0.f;
    }
    __syncthreads();
    float* z1 = sm.a;    // z(m+1)
    float* z2 = sm.b;    // z(m+2), overwritten in place by z(m)
    for (int t = 1; t <= a.T; ++t) {
        const int m = a.kz0 - t + 1;
        const float* rrm = rr + (int64_t)m * g.nch;
        const int lo = HALO - (a.T - t);
        for (int ry = lo + threadIdx.y; ry < RW - lo; ry += BYT) {
            const int y = gy0 + ry;
            if (y < 0 || y >= g.ny) continue;
            for (int rx = lo + threadIdx.x; rx < RW - lo; rx += BXT) {
                const int x = gx0 + rx;
                if (x < 0 || x >= g.nx) continue;
                const int s = ry * RW + rx;
                const int r = sm.rid[s];
                const float inj = r >= 0 ? rrm[r] : 0.f;
                const float* c = sm.c;
                z2[s] = adj_cell(mul(c[s + 1], z1[s + 1]), mul(c[s - 1], z1[s - 1]), mul(c[s - RW], z1[s - RW]),
                                 mul(c[s + RW], z1[s + RW]), mul(c[s], z1[s]), z1[s], z2[s], inj, sm.d[s]);
            }
        }
        // the next step's forward slice goes to the next of three buffers: the buffer written here
        // was last read by step t-2's correlation, which every thread finished before the barrier
        // of step t-1
        if (t < a.T) stage_u(g, ub + (int64_t)((m - 2) % a.S) * N, gx0, gy0, sm.u[(t + 1) % 3]);
        __syncthreads();
        // correlation of the owned cells with the Laplacian of u(m-1)
        const float* us = sm.u[t % 3];
#pragma unroll
        for (int j = 0; j < OWN; ++j) {
            const int oy = threadIdx.y + BYT * j;
            const int su = (oy + 1) * UW + ox + 1;
            const float lu = lap5(us[su + 1], us[su - 1], us[su - UW], us[su + UW], us[su]);
            cr[j] = __fmaf_rn(z2[(oy + HALO) * RW + ox + HALO], lu, cr[j]);
        }
        float* tmp = z1;
        z1 = z2;
        z2 = tmp;
    }
    // z(kz0-T+1) is in z1, z(kz0-T+2) in z2; both go to the ring (T = 1: only the first)
    const int mlast = a.kz0 - a.T + 1;
    if (x_own < g.nx) {
#pragma unroll
        for (int j = 0; j < OWN; ++j) {
            const int oy = threadIdx.y + BYT * j;
            const int y = gy0 + HALO + oy;
            if (y >= g.ny) continue;
            const int64_t q = (int64_t)y * g.nx + x_own;
            const int s = (oy + HALO) * RW + ox + HALO;
            zb[(int64_t)(mlast & 3) * N + q] = z1[s];
            if (a.T > 1) zb[(int64_t)((mlast + 1) & 3) * N + q] = z2[s];
            a.corr[gl * a.cstride + q] = cr[j];
        }
    }
}

}  // namespace

bool tile_supported(const DevGeo& g, int profile) { return profile == TOMO_PROFILE_CFG && g.rid != nullptr; }

void launch_fwd_tile(const DevGeo& g, const float* coef, const TileFwd& a, void* stream) {
    const int tiles_x = (g.nx + TW - 1) / TW, tiles_y = (g.ny + TW - 1) / TW;
    cudaFuncSetAttribute(k_fwd_tile, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)FWD_SMEM);
    k_fwd_tile<<<dim3(tiles_x * tiles_y, a.ng), dim3(BXT, BYT), FWD_SMEM, (cudaStream_t)stream>>>(g, coef, a, tiles_x);
}

void launch_adj_tile(const DevGeo& g, const float* coef, const TileAdj& a, void* stream) {
    const int tiles_x = (g.nx + TW - 1) / TW, tiles_y = (g.ny + TW - 1) / TW;
    cudaFuncSetAttribute(k_adj_tile, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ADJ_SMEM);
    k_adj_tile<<<dim3(tiles_x * tiles_y, a.ng), dim3(BXT, BYT), ADJ_SMEM, (cudaStream_t)stream>>>(g, coef, a, tiles_x);
}

}  // namespace tomo
