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
// Work layout: a block of 32 warps; each warp computes whole rows of the region, a lane two
// neighbouring cells (64-bit shared-memory accesses, west / east neighbours by shuffles).  Warp w
// always computes the tile's row w (owned rows 8 .. 39 of the region), so a lane's owned cells
// stay in its registers from step to step (the adjoint's correlation accumulates there); warps
// 0 .. 13 also compute the 14 halo rows.  Each step computes rows 1 .. 46 and columns 0 .. 47 of
// the region: cells outside the shrinking valid region produce values that only cells outside
// it read, so no cell needs a branch.
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
constexpr int TPB = 1024;            // 32 warps
constexpr int UR = TW + 2;           // correlation's forward slice: rows 7 .. 40 of the region, pitch RW
constexpr int UC = UR * RW;

__device__ __forceinline__ float2 lds2(const float* p) { return *reinterpret_cast<const float2*>(p); }
__device__ __forceinline__ void sts2(float* p, float2 v) { *reinterpret_cast<float2*>(p) = v; }

// Rows a warp computes each step: its owned row 8 + w, and for warps 0 .. 13 one halo row
// (1 .. 7, then 40 .. 46).
__device__ __forceinline__ int halo_row(int w) { return w < 7 ? 1 + w : 33 + w; }

struct FwdSmem {
    float a[RC], b[RC];   // u(m-1) and u(m-2), rotating (u(m) overwrites u(m-2) in place)
    float c[RC];          // coefficient C^2 (1+f)
    float d[RC];          // sponge factor
    int rid[RC];          // receiver channel of the cell, -1 none
    float em[RC];         // 1 where the cell emits for the block's group, else 0
};
struct AdjSmem {
    float za[RC], zb[RC]; // z(m+1) and z(m+2), rotating (z(m) overwrites z(m+2) in place)
    float pa[RC], pb[RC]; // products c z of the current z(m+1) and of the z(m) being computed
    float c[RC];
    float d[RC];
    int rid[RC];
    float u[3][UC];       // forward slices for the correlation (step t uses u[t % 3])
};

// Region cell (rx, ry) is grid cell (gx0 + rx, gy0 + ry).  The five arrays arrive by 16-byte
// cp.async copies (a row of the region is 12 four-cell chunks; nx % 4 == 0, so a chunk is wholly
// inside or outside the grid), zero-filled outside the grid: field 0 and coefficient 0 (cells
// outside stay 0, or never reach an inside cell), sponge 0, receiver entry fixed to -1 after.
constexpr int CHUNKS = RW / 4;      // 12
__device__ __forceinline__ void stage_async(const DevGeo& g, const float* pa, const float* pb, const float* coef,
                                            int gx0, int gy0, float* sa, float* sb, float* sc, float* sd, int* srid) {
#pragma unroll
    for (int arr = 0; arr < 5; ++arr) {
        const float* src = arr == 0 ? pa : arr == 1 ? pb : arr == 2 ? coef : arr == 3 ? g.dmap
                                                                       : reinterpret_cast<const float*>(g.rid);
        float* dst = arr == 0 ? sa : arr == 1 ? sb : arr == 2 ? sc : arr == 3 ? sd : reinterpret_cast<float*>(srid);
        for (int c = threadIdx.x; c < RW * CHUNKS; c += TPB) {
            const int ry = c / CHUNKS, rx = 4 * (c % CHUNKS);
            const int x = gx0 + rx, y = gy0 + ry;
            const bool ok = x >= 0 && x < g.nx && y >= 0 && y < g.ny;
            cp_async16((unsigned)__cvta_generic_to_shared(dst + ry * RW + rx), ok ? src + (int64_t)y * g.nx + x : src,
                       ok);
        }
    }
}

__device__ __forceinline__ bool region_in_grid(const DevGeo& g, int gx0, int gy0, int idx) {
    const int x = gx0 + idx % RW, y = gy0 + idx / RW;
    return x >= 0 && x < g.nx && y >= 0 && y < g.ny;
}

// One forward row: cells (2 lane, 2 lane + 1) of region row ry from u(m-1) (cur) and u(m-2)
// (prv, overwritten).  Lanes 24 .. 31 hold no cells but join the shuffles.
__device__ __forceinline__ float2 fwd_row(const FwdSmem& sm, const float* cur, float* prv, int ry, int lane, float src) {
    const bool act = lane < RW / 2;
    const int s = ry * RW + 2 * lane;
    const float2 zero = make_float2(0.f, 0.f);
    const float2 uc = act ? lds2(cur + s) : zero;
    const float w = __shfl_up_sync(FULL, uc.y, 1), e = __shfl_down_sync(FULL, uc.x, 1);
    float2 v = zero;
    if (act) {
        const float2 us = lds2(cur + s - RW), un = lds2(cur + s + RW), up = lds2(prv + s);
        const float2 c = lds2(sm.c + s), d = lds2(sm.d + s), em = lds2(sm.em + s);
        v.x = fwd_cell(uc.y, w, us.x, un.x, uc.x, up.x, c.x, d.x, em.x != 0.f ? src : 0.f);
        v.y = fwd_cell(e, uc.x, us.y, un.y, uc.y, up.y, c.y, d.y, em.y != 0.f ? src : 0.f);
        sts2(prv + s, v);
    }
    return v;
}

constexpr int TMAXF = 8;   // forward steps per launch at most

__global__ void __launch_bounds__(TPB) k_fwd_tile(DevGeo g, const float* __restrict__ coef, TileFwd a,
                                                  int tiles_x) {
    extern __shared__ __align__(16) unsigned char smraw[];
    FwdSmem& sm = *reinterpret_cast<FwdSmem*>(smraw);
    const int gl = blockIdx.y;
    const int tx = blockIdx.x % tiles_x, ty = blockIdx.x / tiles_x;
    const int gx0 = tx * TW - HALO, gy0 = ty * TW - HALO;
    const int64_t N = (int64_t)g.nx * g.ny;
    float* base = a.hist + gl * a.gstride;
    const int ggl = a.g0 + gl;                     // global group index
    stage_async(g, base + (int64_t)(a.k0 % a.S) * N, base + (int64_t)((a.k0 - 1) % a.S) * N, coef, gx0, gy0, sm.a,
                sm.b, sm.c, sm.d, sm.rid);
    cp_async_commit();
    // the source amplitude of each step, read while the copies fly
    float srcv[TMAXF];
#pragma unroll
    for (int t = 0; t < TMAXF; ++t) {
        const int k = a.k0 + t;                    // step t+1 computes slice k+1
        srcv[t] = (t < a.T && k < g.n_src_steps) ? g.src[k] : 0.f;
    }
    cp_async_wait<0>();
    __syncthreads();
    // receiver entries outside the grid, and the emitter flags (channel = transducer; its group =
    // transducer / group size)
    for (int idx = threadIdx.x; idx < RC; idx += TPB) {
        int r = sm.rid[idx];
        if (!region_in_grid(g, gx0, gy0, idx)) sm.rid[idx] = r = -1;
        sm.em[idx] = (r >= 0 && r / g.gs == ggl) ? 1.f : 0.f;
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const bool noisy = a.gmeas && g.noise_key;
    const uint64_t key = noisy ? *g.noise_key : 0;
    // owned cells of this lane: row 8 + warp, columns 2 lane, 2 lane + 1 for lanes 4 .. 19
    const int orow = HALO + warp;
    const int ox = gx0 + 2 * lane, oy = gy0 + orow;
    const bool own = lane >= HALO / 2 && lane < (HALO + TW) / 2 && ox < g.nx && oy < g.ny;
    const int64_t oq = (int64_t)oy * g.nx + ox;
    const int2 orid = own ? *reinterpret_cast<const int2*>(sm.rid + orow * RW + 2 * lane) : make_int2(-1, -1);
    const int hrow = warp < 14 ? halo_row(warp) : -1;
    float* cur = sm.a;   // u(m-1)
    float* prv = sm.b;   // u(m-2), overwritten in place by u(m)
    int slot = (a.k0 + 1) % a.S;                   // slot of slice m
    int mk = a.ckpt ? (a.k0 + 1) % a.K : -1;       // m mod K
#pragma unroll 1
    for (int t = 1; t <= a.T; ++t) {
        const int m = a.k0 + t;                    // slice computed
        float src = 0.f;
#pragma unroll
        for (int j = 0; j < TMAXF; ++j) src = j == t - 1 ? srcv[j] : src;
        const float2 v = fwd_row(sm, cur, prv, orow, lane, src);
        if (hrow >= 0) fwd_row(sm, cur, prv, hrow, lane, src);
        if (own) {
            *reinterpret_cast<float2*>(base + (int64_t)slot * N + oq) = v;
            if (mk == 0 || mk == 1) {
                // checkpoint: chunk ch >= 1 keeps slices ch K - 1 (which 1 ... ) as engine.cu ck_of
                const int ch = mk == 0 ? m / a.K : (m - 1) / a.K, which = mk == 0 ? 0 : 1;
                if (ch >= 1 && ch < a.nchunk)
                    *reinterpret_cast<float2*>(a.ckpt + gl * a.ckstride + ((int64_t)ch * 2 + which) * N + oq) = v;
            }
            if ((orid.x >= 0 || orid.y >= 0) && a.gout) {
                const int64_t gbase = ((int64_t)gl * g.nt + m) * g.nch;
                if (orid.x >= 0) {
                    const float vv = noisy ? v.x * noise_factor(key, g.noise_level, ggl, m, orid.x) : v.x;
                    a.gout[gbase + orid.x] = a.gmeas ? a.gmeas[gbase + orid.x] - vv : vv;
                }
                if (orid.y >= 0) {
                    const float vv = noisy ? v.y * noise_factor(key, g.noise_level, ggl, m, orid.y) : v.y;
                    a.gout[gbase + orid.y] = a.gmeas ? a.gmeas[gbase + orid.y] - vv : vv;
                }
            }
        }
        slot = slot + 1 == a.S ? 0 : slot + 1;
        if (mk >= 0) mk = mk + 1 == a.K ? 0 : mk + 1;
        __syncthreads();
        float* tmp = cur;
        cur = prv;
        prv = tmp;
    }
}

// Issues the correlation's forward slice as cp.async copies: rows 7 .. 40 (owned rows plus one)
// and the chunks of columns 4 .. 43 of the region, pitch RW, zero-filled outside the grid.
constexpr int UCH = 10;             // four-cell chunks of a staged row (columns 4 .. 43)
__device__ __forceinline__ void stage_u_async(const DevGeo& g, const float* __restrict__ u, int gx0, int gy0,
                                              float* __restrict__ dst) {
    const int c = threadIdx.x;
    if (c < UR * UCH) {
        const int cy = c / UCH, cx = 4 + 4 * (c % UCH);
        const int x = gx0 + cx, y = gy0 + HALO - 1 + cy;
        const bool ok = x >= 0 && x < g.nx && y >= 0 && y < g.ny;
        cp_async16((unsigned)__cvta_generic_to_shared(dst + cy * RW + cx), ok ? u + (int64_t)y * g.nx + x : u, ok);
    }
}

// One adjoint row: z(m) at cells (2 lane, 2 lane + 1) of region row ry from z(m+1) (z1, with its
// products p1) and z(m+2) (z2, overwritten); writes the products c z(m) to p2.
__device__ __forceinline__ float2 adj_row(const AdjSmem& sm, const float* z1, float* z2, const float* p1, float* p2,
                                          int ry, int lane, const float* __restrict__ rrm) {
    const bool act = lane < RW / 2;
    const int s = ry * RW + 2 * lane;
    const float2 zero = make_float2(0.f, 0.f);
    const float2 p0 = act ? lds2(p1 + s) : zero;
    const float pw = __shfl_up_sync(FULL, p0.y, 1), pe = __shfl_down_sync(FULL, p0.x, 1);
    float2 v = zero;
    if (act) {
        const float2 ps = lds2(p1 + s - RW), pn = lds2(p1 + s + RW);
        const float2 z = lds2(z1 + s), zz = lds2(z2 + s), c = lds2(sm.c + s), d = lds2(sm.d + s);
        const int2 r = *reinterpret_cast<const int2*>(sm.rid + s);
        const float ix = r.x >= 0 ? rrm[r.x] : 0.f, iy = r.y >= 0 ? rrm[r.y] : 0.f;
        v.x = adj_cell(p0.y, pw, ps.x, pn.x, p0.x, z.x, zz.x, ix, d.x);
        v.y = adj_cell(pe, p0.x, ps.y, pn.y, p0.y, z.y, zz.y, iy, d.y);
        sts2(z2 + s, v);
        sts2(p2 + s, make_float2(mul(c.x, v.x), mul(c.y, v.y)));
    }
    return v;
}

__global__ void __launch_bounds__(TPB) k_adj_tile(DevGeo g, const float* __restrict__ coef, TileAdj a,
                                                  int tiles_x) {
    extern __shared__ __align__(16) unsigned char smraw[];
    AdjSmem& sm = *reinterpret_cast<AdjSmem*>(smraw);
    const int gl = blockIdx.y;
    const int tx = blockIdx.x % tiles_x, ty = blockIdx.x / tiles_x;
    const int gx0 = tx * TW - HALO, gy0 = ty * TW - HALO;
    const int64_t N = (int64_t)g.nx * g.ny;
    float* zbase = a.z + gl * a.zstride;
    const float* ub = a.hist + gl * a.ustride;
    const float* rr = a.rr + gl * a.rrstride;
    // copy groups: the region, then the forward slices of steps 1 and 2 (step t reads slice kz0 - t,
    // u[t % 3]); every step then issues step t+2's slice and waits for its own, one group behind
    stage_async(g, zbase + (int64_t)((a.kz0 + 1) & 3) * N, zbase + (int64_t)((a.kz0 + 2) & 3) * N, coef, gx0, gy0,
                sm.za, sm.zb, sm.c, sm.d, sm.rid);
    cp_async_commit();
    int us = (a.kz0 - 1) % a.S;                    // slot of the slice step 1 reads
    stage_u_async(g, ub + (int64_t)us * N, gx0, gy0, sm.u[1]);
    cp_async_commit();
    int un = us == 0 ? a.S - 1 : us - 1;           // slot of the next slice to issue (step 2's)
    if (a.T >= 2) stage_u_async(g, ub + (int64_t)un * N, gx0, gy0, sm.u[2]);
    cp_async_commit();
    un = un == 0 ? a.S - 1 : un - 1;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int orow = HALO + warp;
    const int ox = gx0 + 2 * lane, oy = gy0 + orow;
    const bool own = lane >= HALO / 2 && lane < (HALO + TW) / 2 && ox < g.nx && oy < g.ny;
    const int64_t oq = (int64_t)oy * g.nx + ox;
    float2 cr = own ? *reinterpret_cast<const float2*>(a.corr + gl * a.cstride + oq) : make_float2(0.f, 0.f);
    const int hrow = warp < 14 ? halo_row(warp) : -1;
    cp_async_wait<2>();                            // the region
    __syncthreads();
    // receiver entries outside the grid, and the products c z(kz0+1)
    for (int idx = threadIdx.x; idx < RC; idx += TPB) {
        if (!region_in_grid(g, gx0, gy0, idx)) sm.rid[idx] = -1;
        sm.pa[idx] = mul(sm.c[idx], sm.za[idx]);
    }
    float* z1 = sm.za;   // z(m+1)
    float* z2 = sm.zb;   // z(m+2), overwritten in place by z(m)
    float* p1 = sm.pa;   // c z(m+1)
    float* p2 = sm.pb;   // c z(m)
    float2 zl = make_float2(0.f, 0.f), zp = zl;   // this lane's owned z(m) and z(m+1)
#pragma unroll 1
    for (int t = 1; t <= a.T; ++t) {
        const int m = a.kz0 - t + 1;
        const float* rrm = rr + (int64_t)m * g.nch;
        cp_async_wait<1>();                        // this thread's copies of u[t % 3] are done ...
        __syncthreads();                           // ... and every thread's; step t-1 is complete
        const float2 v = adj_row(sm, z1, z2, p1, p2, orow, lane, rrm);
        if (hrow >= 0) adj_row(sm, z1, z2, p1, p2, hrow, lane, rrm);
        // the correlation of the owned cells with the Laplacian of u(m-1), in registers
        const float* usl = sm.u[t % 3] + (orow - (HALO - 1)) * RW + 2 * lane;
        const bool act = lane < RW / 2;
        const float2 u0 = act ? lds2(usl) : make_float2(0.f, 0.f);
        const float uw = __shfl_up_sync(FULL, u0.y, 1), ue = __shfl_down_sync(FULL, u0.x, 1);
        if (own) {
            const float2 usn = lds2(usl - RW), unn = lds2(usl + RW);
            cr.x = __fmaf_rn(v.x, lap5(u0.y, uw, usn.x, unn.x, u0.x), cr.x);
            cr.y = __fmaf_rn(v.y, lap5(ue, u0.x, usn.y, unn.y, u0.y), cr.y);
        }
        zp = zl;
        zl = v;
        // step t+2's slice into u[(t+2) % 3], last read by step t-1 (complete at the barrier above)
        if (t + 2 <= a.T) {
            stage_u_async(g, ub + (int64_t)un * N, gx0, gy0, sm.u[(t + 2) % 3]);
            un = un == 0 ? a.S - 1 : un - 1;
        }
        cp_async_commit();
        float* tmp = z1; z1 = z2; z2 = tmp;
        tmp = p1; p1 = p2; p2 = tmp;
    }
    cp_async_wait<0>();
    // z(kz0-T+1) and z(kz0-T+2) go to the ring (T = 1: only the first), with the correlation
    if (own) {
        const int mlast = a.kz0 - a.T + 1;
        *reinterpret_cast<float2*>(zbase + (int64_t)(mlast & 3) * N + oq) = zl;
        if (a.T > 1) *reinterpret_cast<float2*>(zbase + (int64_t)((mlast + 1) & 3) * N + oq) = zp;
        *reinterpret_cast<float2*>(a.corr + gl * a.cstride + oq) = cr;
    }
}

}  // namespace

bool tile_supported(const DevGeo& g, int profile) {
    return profile == TOMO_PROFILE_CFG && g.rid != nullptr && g.dmap != nullptr && g.nx % 4 == 0;
}

void launch_fwd_tile(const DevGeo& g, const float* coef, const TileFwd& a, void* stream) {
    const int tiles_x = (g.nx + TW - 1) / TW, tiles_y = (g.ny + TW - 1) / TW;
    cudaFuncSetAttribute(k_fwd_tile, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(FwdSmem));
    k_fwd_tile<<<dim3(tiles_x * tiles_y, a.ng), TPB, sizeof(FwdSmem), (cudaStream_t)stream>>>(g, coef, a, tiles_x);
}

void launch_adj_tile(const DevGeo& g, const float* coef, const TileAdj& a, void* stream) {
    const int tiles_x = (g.nx + TW - 1) / TW, tiles_y = (g.ny + TW - 1) / TW;
    cudaFuncSetAttribute(k_adj_tile, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(AdjSmem));
    k_adj_tile<<<dim3(tiles_x * tiles_y, a.ng), TPB, sizeof(AdjSmem), (cudaStream_t)stream>>>(g, coef, a, tiles_x);
}

}  // namespace tomo
