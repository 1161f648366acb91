// tile.cu -- multi-step tile kernels of the benchmark-profile (CFG) physics.
//
// The warp-strip kernels (strip.cu) advance every group of a pass by one or two time steps per
// launch.  On small grids (128 x 128, or one group of 512 x 512 in an ART pass) a step is too
// little work to fill the GPU, and the time goes into the launches themselves.  These kernels
// advance a 2-D tile by up to 8 steps per launch.  A block owns a 48 x 48 tile; the tile plus a
// halo of 8 cells (a 64 x 64 region) of the two input slices, the coefficient, the sponge factor
// and the receiver map arrive in shared memory as five TMA tile copies (cp.async.bulk.tensor,
// zero-filled outside the grid) completing on one mbarrier.  The block then runs the steps with
// the region's cells in registers: the computed region shrinks by one cell per step, so the halo
// is computed redundantly and no block waits for another inside a launch.  Every step writes
// the owned cells (the forward history, records and checkpoints; for the adjoint only the last
// two slices and the correlation at the end).
//
// Work layout: 16 warps; warp w holds region rows 4w .. 4w+3, lane l the columns 2l, 2l+1 of
// each, so a thread keeps 8 cells (both input slices, coefficient and sponge factor) in
// registers from step to step.  East / west neighbours come by warp shuffles, north / south
// neighbours from the thread's own rows, and at the edges of a warp's band from the first and
// last rows each warp publishes per step in a double-buffered exchange array (one barrier per
// step).  A lane's two cells are evaluated in packed FP32x2 arithmetic with the operation order
// and rounding of the cell.cuh helpers, so a sweep gives the strip kernels' bits (tested).  The
// adjoint's correlation needs u(m-1) around the owned cells each step: one TMA copy per step
// (rows 7 .. 56 of the region) into a three-slot ring, issued two steps ahead.
//
// Adjoint launches advance T in {1, 2, 6} steps: the adjoint ring has four slots and these are
// the step counts whose two output slices never fall on the two input slices' slots.  Forward
// launches take T <= S - 2 so the slices they write never land on the slots they read.
//
// Waits: every mbarrier wait is bounded by TileWait::wait_ns of %globaltimer; a block whose copy
// has not arrived by then records the failure in the host-visible error word, waits (again
// bounded) for its other copies and returns; the host turns the word into TOMO_ERR_TIMEOUT.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "internal.h"

namespace tomo {
namespace {

#include "cell.cuh"

constexpr int TW = TILE_OWNED;       // owned tile width: 48 columns
constexpr int HALO = 8;              // halo (steps per forward launch at most)
constexpr int RX = TW + 2 * HALO;    // region width: 64 columns (32 lanes x 2 cells)
constexpr int UOFF = HALO - 1;       // correlation slice: owned rows plus one above and below
constexpr int TMAXF = TILE_MAX_FWD;
constexpr size_t MAX_NCH = 2048;     // record channels at most (a launch's rows stay in shared memory)
static_assert(TMAXF <= HALO, "forward steps per launch exceed the halo");

// Tile shapes: WARPS warps of 4 region rows, region RX x 4 WARPS, owned TW x (4 WARPS - 16).
template <int WARPS>
struct Shape {
    static constexpr int TPB = 32 * WARPS;
    static constexpr int RH = 4 * WARPS;                  // region rows
    static constexpr int TH = RH - 2 * HALO;              // owned rows
    static constexpr int RCH = RX * RH;
    static constexpr int UROWS = TH + 2;
    static constexpr uint32_t REGION_BYTES = 5u * RCH * 4u;
    static constexpr uint32_t USLICE_BYTES = (uint32_t)UROWS * RX * 4u;
    static constexpr int SET = WARPS == 16 ? 0 : 1;       // map set of encode_tile_maps
    static constexpr int MINB = WARPS <= 10 ? 2 : 1;      // blocks per SM the launch bounds ask for
};

// Kernel-parameter copy of one shape's maps: slot tensor (region boxes), slot tensor
// (correlation-slice boxes), adjoint ring, coefficient, sponge map, receiver map.
struct TileTma {
    CUtensorMap hist, histu, z, coef, dmap, rid;
};
static_assert(sizeof(TileTma) == sizeof(TileMaps::raw[0]), "tensor map size");

__device__ __forceinline__ float2 lds2(const float* p) { return *reinterpret_cast<const float2*>(p); }
__device__ __forceinline__ void sts2(float* p, float2 v) { *reinterpret_cast<float2*>(p) = v; }

// Record rows (T steps x nch channels) into shared memory by asynchronous 4-byte copies: a
// thread's copies are all in flight at once, where a load-then-store loop through generic
// pointers waits out one memory latency per element it copies.  The caller completes them with
// cp_async_wait_all() before the barrier that publishes the region.
__device__ __forceinline__ void copy_rows_async(float* dst, const float* src, int n, int tid, int nthreads) {
    for (int i = tid; i < n; i += nthreads)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"((uint32_t)__cvta_generic_to_shared(dst + i)),
                     "l"(__cvta_generic_to_global(src + i))
                     : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }
#include "async.cuh"

// Forward cell update of a lane's two cells (fwd_cell of cell.cuh, packed).
__device__ __forceinline__ float2 fwd_cell2(float2 e, float2 w, float2 s, float2 n, float2 u, float2 up, float2 c,
                                            float2 d, float2 a) {
    return pk_fma(d, pk_fma(c, lap5_2(e, w, s, n, u), pk_fma(make_float2(2.f, 2.f), u, make_float2(-up.x, -up.y))),
                  a);
}

// Whether some row of warp w's band is still inside the valid region at step t (rows t .. RH-1-t).
template <int RH>
__device__ __forceinline__ bool band_live(int w, int t) {
    return 4 * w + 3 >= t && 4 * w <= RH - 1 - t;
}

template <int WARPS>
struct FwdSmem {
    using S = Shape<WARPS>;
    float u1[S::RCH], u2[S::RCH], c[S::RCH], d[S::RCH];   // region: u(k0), u(k0-1), coefficient, sponge
    int rid[S::RCH];                                      // receiver channel (0 outside the grid: masked)
    float xch[2][WARPS][2][RX];                           // per step: each warp's first and last row
    uint64_t bar;
};
template <int WARPS>
struct AdjSmem {
    using S = Shape<WARPS>;
    float z1[S::RCH], z2[S::RCH], c[S::RCH], d[S::RCH];   // region: z(kz0+1), z(kz0+2), coefficient, sponge
    int rid[S::RCH];
    float u[3][S::UROWS * RX];                            // correlation slices, step t in u[t % 3]
    float xch[2][WARPS][2][RX];                           // per step: products c z of each warp's edge rows
    uint64_t bar[4];                                      // region; u[0], u[1], u[2]
};

// Receiver / emitter bits of a thread's 8 cells (bit 2r + i: row r, column i of the pair) from
// the staged receiver map, cells outside the grid excluded.
__device__ __forceinline__ void cell_masks(const DevGeo& g, const int* rid, int gx0, int gy0, int ry0, int lane,
                                           int ggl, unsigned& rmask, unsigned& emask) {
    rmask = emask = 0u;
    const int x = gx0 + 2 * lane;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const int y = gy0 + ry0 + r;
        const int2 rv = *reinterpret_cast<const int2*>(rid + (ry0 + r) * RX + 2 * lane);
        const bool iny = y >= 0 && y < g.ny;
        if (iny && x >= 0 && x < g.nx && rv.x >= 0) {
            rmask |= 1u << (2 * r);
            if (rv.x / g.gs == ggl) emask |= 1u << (2 * r);
        }
        if (iny && x + 1 >= 0 && x + 1 < g.nx && rv.y >= 0) {
            rmask |= 2u << (2 * r);
            if (rv.y / g.gs == ggl) emask |= 2u << (2 * r);
        }
    }
}

// Grid barrier between the chunks of a persistent launch: every block has issued its chunk's
// global writes before any block copies its next region (the halo is other blocks' cells).
// Bounded by wait_ns; false (bit 0 of the error word set) when the arrivals did not all come.
__device__ __forceinline__ bool grid_sync(const TileWait& w, unsigned int chunk) {
    __syncthreads();
    bool ok = true;
    if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(w.gbar, 1u);
        const unsigned int target = gridDim.x * gridDim.y * chunk + w.gbar_extra;
        if (ld_acquire(w.gbar) < target) {
            const uint64_t t0 = gtimer();
            while (ld_acquire(w.gbar) < target)
                if (gtimer() - t0 >= w.wait_ns) {
                    ok = false;
                    atomicOr(w.err, 1u);
                    break;
                }
        }
        fence_proxy_async_global();   // this thread's next TMA copies see the other blocks' writes
    }
    return __syncthreads_and(ok);
}

// One forward chunk of a block: slices k0+1 .. k0+T of its tile (the body of a launch); the
// region barrier completes its phase `parity`.  False when a copy wait timed out.  NOISY: the
// launch applies in-loop record noise.  A separate instantiation keeps the noise draw out of
// the noise-free kernel entirely: as a run-time select inside the receiver branch, the draw (a
// 64-bit hash) was evaluated for every receiver cell every step and held up the warps on the
// transducer circle (0.36 ms of a 6.7 ms one-group pass on 512x512 with 256 receivers).
template <int WARPS, bool NOISY>
__device__ __forceinline__ bool fwd_chunk(const DevGeo& g, const TileTma& tm, const TileFwd& a, int tiles_x,
                                          unsigned char* smraw, uint32_t parity) {
    using S = Shape<WARPS>;
    constexpr int RH = S::RH, TH = S::TH;
    FwdSmem<WARPS>& sm = *reinterpret_cast<FwdSmem<WARPS>*>(smraw);
    const int gl = blockIdx.y;
    const int tx = blockIdx.x % tiles_x, ty = blockIdx.x / tiles_x;
    const int gx0 = tx * TW - HALO, gy0 = ty * TH - HALO;
    const int64_t N = (int64_t)g.nx * g.ny;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int ggl = a.g0 + gl;
    // source amplitudes and measured record rows of the launch's steps, loaded while the copies fly
    // (no global load stays on a step's critical path)
    float* const ssrc = reinterpret_cast<float*>(smraw + sizeof(FwdSmem<WARPS>));   // [TMAXF]
    float* const smeas = ssrc + TMAXF;                                              // [T][nch]
    if (threadIdx.x < TMAXF) {
        const int k = a.k0 + threadIdx.x;          // step threadIdx.x + 1 computes slice k + 1
        ssrc[threadIdx.x] = (int)threadIdx.x < a.T && k < g.n_src_steps ? g.src[k] : 0.f;
    }
    if (a.gmeas)     // measured records: set before the passes, written by no kernel
        copy_rows_async(smeas, a.gmeas + ((int64_t)gl * g.nt + a.k0 + 1) * g.nch, a.T * g.nch, threadIdx.x, S::TPB);
    grid_dep_wait();
    grid_dep_trigger();
    if (threadIdx.x == 0) {
        mbar_expect_tx(&sm.bar, S::REGION_BYTES + a.w.extra_tx);
        tma_load_3d(sm.u1, &tm.hist, gx0, gy0, gl * a.S + a.k0 % a.S, &sm.bar);
        tma_load_3d(sm.u2, &tm.hist, gx0, gy0, gl * a.S + (a.k0 - 1) % a.S, &sm.bar);
        tma_load_2d(sm.c, &tm.coef, gx0, gy0, &sm.bar);
        tma_load_2d(sm.d, &tm.dmap, gx0, gy0, &sm.bar);
        tma_load_2d(sm.rid, &tm.rid, gx0, gy0, &sm.bar);
    }
    cp_async_wait_all();                           // this thread's record-row copies
    if (!__syncthreads_and(mbar_wait(&sm.bar, parity, a.w.wait_ns))) {
        if (threadIdx.x == 0) atomicOr(a.w.err, 1u);
        mbar_wait(&sm.bar, parity, a.w.wait_ns);
        return false;
    }
    const int ry0 = 4 * w;
    float2 ua[4], ub[4], cc[4], dd[4];   // ua = u(k0), ub = u(k0-1); then alternately overwritten
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const int s = (ry0 + r) * RX + 2 * lane;
        ua[r] = lds2(sm.u1 + s);
        ub[r] = lds2(sm.u2 + s);
        cc[r] = lds2(sm.c + s);
        dd[r] = lds2(sm.d + s);
    }
    unsigned rmask, emask;
    cell_masks(g, sm.rid, gx0, gy0, ry0, lane, ggl, rmask, emask);
    // owned cells: rows 8 .. RH-9 (warps 2 .. WARPS-3), columns 8 .. 55 (lanes 4 .. 27), inside the grid
    const int ox = gx0 + 2 * lane;
    const bool own = w >= HALO / 4 && w < WARPS - HALO / 4 && lane >= HALO / 2 && lane < (HALO + TW) / 2 && ox < g.nx;
    if (!own) rmask = 0u;
    const bool noisy = NOISY && a.gmeas && g.noise_key;
    const uint64_t key = noisy ? *g.noise_key : 0;
    float* const obase = a.hist + gl * a.gstride + (int64_t)(gy0 + ry0) * g.nx + ox;   // owned row 0 of slot 0
    float* const cbase = a.ckpt ? a.ckpt + gl * a.ckstride + (int64_t)(gy0 + ry0) * g.nx + ox : nullptr;
    const int orows = own ? min(4, g.ny - (gy0 + ry0)) : 0;   // owned rows of this thread inside the grid
    int slot = (a.k0 + 1) % a.S;                   // slot of slice m
    int mk = a.ckpt ? (a.k0 + 1) % a.K : -1;       // m mod K
    const float2 zero = make_float2(0.f, 0.f);
    // one step: u(m) from cur = u(m-1) and prv = u(m-2), written over prv
    auto step = [&](float2 (&cur)[4], float2 (&prv)[4], int t) {
        const int m = a.k0 + t;                    // slice computed
        const float src = ssrc[t - 1];
        // the rows below and above the band, u(m-1)
        float2 sb, nb;
        if (t == 1) {
            sb = w > 0 ? lds2(sm.u1 + (ry0 - 1) * RX + 2 * lane) : zero;
            nb = w < WARPS - 1 ? lds2(sm.u1 + (ry0 + 4) * RX + 2 * lane) : zero;
        } else {
            const float* xb = &sm.xch[(t - 1) & 1][0][0][0];
            sb = w > 0 ? lds2(xb + ((w - 1) * 2 + 1) * RX + 2 * lane) : zero;
            nb = w < WARPS - 1 ? lds2(xb + ((w + 1) * 2) * RX + 2 * lane) : zero;
        }
        if (band_live<RH>(w, t)) {
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                const float2 u = cur[r];
                const float wv = __shfl_up_sync(FULL, u.y, 1), ev = __shfl_down_sync(FULL, u.x, 1);
                const float2 s = r == 0 ? sb : cur[r - 1], n = r == 3 ? nb : cur[r + 1];
                const float2 am = make_float2((emask >> (2 * r)) & 1u ? src : 0.f, (emask >> (2 * r)) & 2u ? src : 0.f);
                prv[r] = fwd_cell2(make_float2(u.y, ev), make_float2(wv, u.x), s, n, u, prv[r], cc[r], dd[r], am);
            }
            sts2(&sm.xch[t & 1][w][0][2 * lane], prv[0]);
            sts2(&sm.xch[t & 1][w][1][2 * lane], prv[3]);
            if (orows > 0) {
                float* const os = obase + (int64_t)slot * N;
                // checkpoint: chunk ch >= 1 keeps slices ch K - 1 (which 1) and ch K (which 0)
                const int ch = mk == 0 ? m / a.K : mk == 1 ? (m - 1) / a.K : -1, which = mk == 0 ? 0 : 1;
                float* const ck = (ch >= 1 && ch < a.nchunk) ? cbase + ((int64_t)ch * 2 + which) * N : nullptr;
#pragma unroll
                for (int r = 0; r < 4; ++r) {
                    if (r >= orows) break;
                    *reinterpret_cast<float2*>(os + (int64_t)r * g.nx) = prv[r];
                    if (ck) *reinterpret_cast<float2*>(ck + (int64_t)r * g.nx) = prv[r];
                    const unsigned rb = (rmask >> (2 * r)) & 3u;
                    if (rb && a.gout) {
                        const int2 rv = *reinterpret_cast<const int2*>(sm.rid + (ry0 + r) * RX + 2 * lane);
                        const int64_t gbase = ((int64_t)gl * g.nt + m) * g.nch;
                        const float* sme = smeas + (t - 1) * g.nch;
                        if (rb & 1u) {
                            const float vv = noisy ? prv[r].x * noise_factor(key, g.noise_level, ggl, m, rv.x) : prv[r].x;
                            a.gout[gbase + rv.x] = a.gmeas ? sme[rv.x] - vv : vv;
                        }
                        if (rb & 2u) {
                            const float vv = noisy ? prv[r].y * noise_factor(key, g.noise_level, ggl, m, rv.y) : prv[r].y;
                            a.gout[gbase + rv.y] = a.gmeas ? sme[rv.y] - vv : vv;
                        }
                    }
                }
            }
        }
        slot = slot + 1 == a.S ? 0 : slot + 1;
        if (mk >= 0) mk = mk + 1 == a.K ? 0 : mk + 1;
        __syncthreads();
    };
#pragma unroll 1
    for (int t = 1; t <= a.T; t += 2) {
        step(ua, ub, t);                           // u(k0+t) into ub
        if (t + 1 <= a.T) step(ub, ua, t + 1);     // u(k0+t+1) into ua
    }
    return true;
}

// A launch computes one chunk (k_last = 0) or, persistent, the chunks k0+1 .. k_last one after
// another with a grid barrier between them (every block resident: cooperative launch).
template <int WARPS, bool NOISY>
__global__ void __launch_bounds__(Shape<WARPS>::TPB, Shape<WARPS>::MINB)
    k_fwd_tile(DevGeo g, const __grid_constant__ TileTma tm, TileFwd a0, int tiles_x) {
    extern __shared__ __align__(1024) unsigned char smraw[];
    FwdSmem<WARPS>& sm = *reinterpret_cast<FwdSmem<WARPS>*>(smraw);
    if (threadIdx.x == 0) {
        mbar_init(&sm.bar, 1);
        mbar_fence_init();
    }
    __syncthreads();
    TileFwd a = a0;
    for (unsigned int chunk = 0;; ++chunk) {
        if (a0.k_last > 0) a.T = min(min(a0.k_last - a.k0, TMAXF), a0.S - 2);
        if (!fwd_chunk<WARPS, NOISY>(g, tm, a, tiles_x, smraw, chunk & 1u)) return;
        a.k0 += a.T;
        if (a0.k_last <= 0 || a.k0 >= a0.k_last) return;
        if (!grid_sync(a0.w, chunk + 1)) return;
    }
}

// Issues the correlation slice of step t (u(kz0 - t), region rows 7 .. 8+TH) into u[q % 3], q
// the step's number since the launch began (its barrier is bar[1 + q % 3]).
template <int WARPS>
__device__ __forceinline__ void issue_u(AdjSmem<WARPS>& sm, const TileTma& tm, const TileAdj& a, int gl, int gx0,
                                        int gy0, int t, int q) {
    uint64_t* bar = &sm.bar[1 + q % 3];
    mbar_expect_tx(bar, Shape<WARPS>::USLICE_BYTES);
    tma_load_3d(sm.u[q % 3], &tm.histu, gx0, gy0 + UOFF, gl * a.S + (a.kz0 - t) % a.S, bar);
}
// Parity of the u[q % 3] barrier phase that launch step q waits for (its (q-1)/3-th use).
__device__ __forceinline__ uint32_t u_parity(int q) { return (uint32_t)((q - 1) / 3) & 1u; }

// One adjoint chunk of a block: z(kz0) .. z(kz0-T+1) with the correlation (the body of a
// launch); the region barrier completes its phase `parity`, the launch's steps before this
// chunk number q0.  False when a copy wait timed out.
template <int WARPS>
__device__ __forceinline__ bool adj_chunk(const DevGeo& g, const TileTma& tm, const TileAdj& a, int tiles_x,
                                          unsigned char* smraw, uint32_t parity, int q0) {
    using S = Shape<WARPS>;
    constexpr int RH = S::RH, TH = S::TH;
    AdjSmem<WARPS>& sm = *reinterpret_cast<AdjSmem<WARPS>*>(smraw);
    const int gl = blockIdx.y;
    const int tx = blockIdx.x % tiles_x, ty = blockIdx.x / tiles_x;
    const int gx0 = tx * TW - HALO, gy0 = ty * TH - HALO;
    const int64_t N = (int64_t)g.nx * g.ny;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    // residual rows of the launch's steps (z(m) injects rr[m]; row j holds m = kz0-T+1+j), loaded
    // while the copies fly
    float* const srr = reinterpret_cast<float*>(smraw + sizeof(AdjSmem<WARPS>));   // [T][nch]
    grid_dep_wait();
    grid_dep_trigger();
    copy_rows_async(srr, a.rr + gl * a.rrstride + (int64_t)(a.kz0 - a.T + 1) * g.nch, a.T * g.nch, threadIdx.x, S::TPB);
    if (threadIdx.x == 0) {
        mbar_expect_tx(&sm.bar[0], S::REGION_BYTES + a.w.extra_tx);
        tma_load_3d(sm.z1, &tm.z, gx0, gy0, gl * 4 + ((a.kz0 + 1) & 3), &sm.bar[0]);
        tma_load_3d(sm.z2, &tm.z, gx0, gy0, gl * 4 + ((a.kz0 + 2) & 3), &sm.bar[0]);
        tma_load_2d(sm.c, &tm.coef, gx0, gy0, &sm.bar[0]);
        tma_load_2d(sm.d, &tm.dmap, gx0, gy0, &sm.bar[0]);
        tma_load_2d(sm.rid, &tm.rid, gx0, gy0, &sm.bar[0]);
        issue_u(sm, tm, a, gl, gx0, gy0, 1, q0 + 1);
        if (a.T >= 2) issue_u(sm, tm, a, gl, gx0, gy0, 2, q0 + 2);
    }
    const int ry0 = 4 * w;
    const int ox = gx0 + 2 * lane;
    const bool own_rows = w >= HALO / 4 && w < WARPS - HALO / 4;
    const bool own = own_rows && lane >= HALO / 2 && lane < (HALO + TW) / 2 && ox < g.nx;
    const int orows = own ? min(4, g.ny - (gy0 + ry0)) : 0;
    float* const cbase = a.corr + gl * a.cstride + (int64_t)(gy0 + ry0) * g.nx + ox;
    float2 cr[4];
    const float2 zero = make_float2(0.f, 0.f);
#pragma unroll
    for (int r = 0; r < 4; ++r) cr[r] = r < orows ? *reinterpret_cast<const float2*>(cbase + (int64_t)r * g.nx) : zero;
    cp_async_wait_all();                           // this thread's residual-row copies
    if (!__syncthreads_and(mbar_wait(&sm.bar[0], parity, a.w.wait_ns))) {
        if (threadIdx.x == 0) atomicOr(a.w.err, 1u);
        for (int s = 1; s <= a.T && s <= 2; ++s)
            mbar_wait(&sm.bar[1 + (q0 + s) % 3], u_parity(q0 + s), a.w.wait_ns);
        return false;
    }
    // za = z(kz0+1), zb = z(kz0+2), pa = c z(kz0+1); then alternately overwritten
    float2 za[4], zb[4], cc[4], dd[4], pa[4], pb[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const int s = (ry0 + r) * RX + 2 * lane;
        za[r] = lds2(sm.z1 + s);
        zb[r] = lds2(sm.z2 + s);
        cc[r] = lds2(sm.c + s);
        dd[r] = lds2(sm.d + s);
        pa[r] = pk_mul(cc[r], za[r]);
    }
    unsigned rmask, emask;
    cell_masks(g, sm.rid, gx0, gy0, ry0, lane, 0, rmask, emask);
    // one step: z(m) from zc = z(m+1) (products pc) and zp = z(m+2), written over zp, its
    // products over pn; false when a copy wait timed out (the launch is abandoned)
    auto step = [&](float2 (&zc)[4], float2 (&zp)[4], float2 (&pc)[4], float2 (&pn)[4], int t) -> bool {
        const float* rrm = srr + (a.T - t) * g.nch;   // rr[m] of the slice computed, z(m), m = kz0-t+1
        // warp-uniform, so the shuffles below run with every lane of the warp
        const bool ok = __all_sync(FULL, mbar_wait(&sm.bar[1 + (q0 + t) % 3], u_parity(q0 + t), a.w.wait_ns));
        // products c z(m+1) of the rows below and above the band
        float2 sb, nb;
        if (t == 1) {
            sb = w > 0 ? pk_mul(lds2(sm.c + (ry0 - 1) * RX + 2 * lane), lds2(sm.z1 + (ry0 - 1) * RX + 2 * lane)) : zero;
            nb = w < WARPS - 1 ? pk_mul(lds2(sm.c + (ry0 + 4) * RX + 2 * lane), lds2(sm.z1 + (ry0 + 4) * RX + 2 * lane))
                               : zero;
        } else {
            const float* xb = &sm.xch[(t - 1) & 1][0][0][0];
            sb = w > 0 ? lds2(xb + ((w - 1) * 2 + 1) * RX + 2 * lane) : zero;
            nb = w < WARPS - 1 ? lds2(xb + ((w + 1) * 2) * RX + 2 * lane) : zero;
        }
        if (ok && band_live<RH>(w, t)) {
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                const float2 p = pc[r];
                const float pw = __shfl_up_sync(FULL, p.y, 1), pe = __shfl_down_sync(FULL, p.x, 1);
                const float2 ps = r == 0 ? sb : pc[r - 1], pnb = r == 3 ? nb : pc[r + 1];
                float2 inj = zero;
                const unsigned rb = (rmask >> (2 * r)) & 3u;
                if (rb) {
                    const int2 rv = *reinterpret_cast<const int2*>(sm.rid + (ry0 + r) * RX + 2 * lane);
                    if (rb & 1u) inj.x = rrm[rv.x];
                    if (rb & 2u) inj.y = rrm[rv.y];
                }
                zp[r] = adj_cell2(make_float2(p.y, pe), make_float2(pw, p.x), ps, pnb, p, zc[r], zp[r], inj, dd[r]);
                pn[r] = pk_mul(cc[r], zp[r]);
            }
            if (own_rows) {
                // correlation with the Laplacian of u(m-1) (rows ry0-1 .. ry0+4 of the region)
                const float* ub = sm.u[(q0 + t) % 3] + (ry0 - UOFF) * RX + 2 * lane;
                float2 ur[6];
#pragma unroll
                for (int i = 0; i < 6; ++i) ur[i] = lds2(ub + (i - 1) * RX);
#pragma unroll
                for (int r = 0; r < 4; ++r) {
                    const float2 u = ur[r + 1];
                    const float uw = __shfl_up_sync(FULL, u.y, 1), ue = __shfl_down_sync(FULL, u.x, 1);
                    cr[r] = pk_fma(zp[r], lap5_2(make_float2(u.y, ue), make_float2(uw, u.x), ur[r], ur[r + 2], u), cr[r]);
                }
            }
            sts2(&sm.xch[t & 1][w][0][2 * lane], pn[0]);
            sts2(&sm.xch[t & 1][w][1][2 * lane], pn[3]);
        }
        if (!__syncthreads_and(ok)) {
            if (threadIdx.x == 0) atomicOr(a.w.err, 1u);
            for (int s = t; s <= a.T && s <= t + 1; ++s)
                mbar_wait(&sm.bar[1 + (q0 + s) % 3], u_parity(q0 + s), a.w.wait_ns);
            return false;
        }
        // step t+2's slice into the ring slot last read by step t-1 (complete at the barrier above)
        if (threadIdx.x == 0 && t + 2 <= a.T) issue_u(sm, tm, a, gl, gx0, gy0, t + 2, q0 + t + 2);
        return true;
    };
#pragma unroll 1
    for (int t = 1; t <= a.T; t += 2) {
        if (!step(za, zb, pa, pb, t)) return false;                        // z(kz0-t+1) into zb
        if (t + 1 <= a.T && !step(zb, za, pb, pa, t + 1)) return false;    // z(kz0-t) into za
    }
    // z(kz0-T+1) and z(kz0-T+2) go to the ring (T = 1: only the first), with the correlation
    if (orows > 0) {
        const bool odd = a.T & 1;                  // odd T: the last slice is in zb
        float* zbase = a.z + gl * a.zstride + (int64_t)(gy0 + ry0) * g.nx + ox;
        const int mlast = a.kz0 - a.T + 1;
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            if (r >= orows) break;
            const int64_t o = (int64_t)r * g.nx;
            *reinterpret_cast<float2*>(zbase + (int64_t)(mlast & 3) * N + o) = odd ? zb[r] : za[r];
            if (a.T > 1) *reinterpret_cast<float2*>(zbase + (int64_t)((mlast + 1) & 3) * N + o) = odd ? za[r] : zb[r];
            *reinterpret_cast<float2*>(cbase + o) = cr[r];
        }
    }
    return true;
}

// Adjoint steps of the next chunk when L steps remain: 6, 2 or 1 (the step counts whose output
// slices miss the input slices' slots of the four-slot ring).
__device__ __forceinline__ int adj_chunk_steps(int L) { return L >= 6 ? 6 : L >= 2 ? 2 : 1; }

// A launch computes one chunk (kz_last = 0) or, persistent, z(kz0) .. z(kz_last) in chunks with
// a grid barrier between them (every block resident: cooperative launch).
template <int WARPS>
__global__ void __launch_bounds__(Shape<WARPS>::TPB, Shape<WARPS>::MINB)
    k_adj_tile(DevGeo g, const __grid_constant__ TileTma tm, TileAdj a0, int tiles_x) {
    extern __shared__ __align__(1024) unsigned char smraw[];
    AdjSmem<WARPS>& sm = *reinterpret_cast<AdjSmem<WARPS>*>(smraw);
    if (threadIdx.x < 4) mbar_init(&sm.bar[threadIdx.x], 1);
    if (threadIdx.x == 0) mbar_fence_init();
    __syncthreads();
    TileAdj a = a0;
    int q0 = 0;
    for (unsigned int chunk = 0;; ++chunk) {
        if (a0.kz_last > 0) a.T = adj_chunk_steps(a.kz0 - a0.kz_last + 1);
        if (!adj_chunk<WARPS>(g, tm, a, tiles_x, smraw, chunk & 1u, q0)) return;
        q0 += a.T;
        a.kz0 -= a.T;
        if (a0.kz_last <= 0 || a.kz0 < a0.kz_last) return;
        if (!grid_sync(a0.w, chunk + 1)) return;
    }
}

// ---- host: tensor-map encoding (driver entry point, no link against libcuda)
using EncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                 const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encoder() {
    static const EncodeTiled fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess) {
            cudaGetLastError();
            p = nullptr;
        }
        return reinterpret_cast<EncodeTiled>(p);
    }();
    return fn;
}

// One map over nx x ny (x planes) cells of 4 bytes, boxes of bx x by (x 1) cells, zero fill
// outside the tensor.
bool encode(EncodeTiled fn, unsigned char* out, CUtensorMapDataType type, const void* base, const DevGeo& g,
            int64_t planes, int bx, int by, std::string* why, const char* what) {
    CUtensorMap m;
    const cuuint64_t dims[3] = {(cuuint64_t)g.nx, (cuuint64_t)g.ny, (cuuint64_t)(planes > 0 ? planes : 1)};
    const cuuint64_t strides[2] = {(cuuint64_t)g.nx * 4u, (cuuint64_t)g.nx * (cuuint64_t)g.ny * 4u};
    const cuuint32_t box[3] = {(cuuint32_t)bx, (cuuint32_t)by, 1u};
    const cuuint32_t estr[3] = {1u, 1u, 1u};
    const CUresult r = fn(&m, type, planes > 0 ? 3u : 2u, const_cast<void*>(base), dims, strides, box, estr,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        if (why) *why = std::string("cuTensorMapEncodeTiled refused the ") + what + " map (" + std::to_string((int)r) + ")";
        return false;
    }
    std::memcpy(out, &m, sizeof m);
    return true;
}

}  // namespace

void* tensor_map_encoder() { return reinterpret_cast<void*>(encoder()); }

bool tile_supported(const DevGeo& g, int profile) {
    // nx % 4 == 0: 16-byte row strides and tile origins (multiples of 4 cells) for the TMA copies;
    // nch <= 2048: a launch's record rows (8 x nch floats) fit in shared memory next to the region
    return profile == TOMO_PROFILE_CFG && g.rid != nullptr && g.dmap != nullptr && g.nx % 4 == 0 &&
           g.nch <= (int)MAX_NCH;
}

bool encode_tile_maps(TileMaps* m, const DevGeo& g, const float* hist, int64_t hist_planes, const float* z,
                      int64_t z_planes, const float* coef, std::string* why) {
    m->ok = false;
    if (!tile_supported(g, TOMO_PROFILE_CFG)) return false;
    const EncodeTiled fn = encoder();
    if (!fn) {
        if (why) *why = "no cuTensorMapEncodeTiled entry point";
        return false;
    }
    bool ok = true;
    for (int set = 0; set < 2 && ok; ++set) {
        const int rh = set == 0 ? Shape<16>::RH : Shape<10>::RH, ur = set == 0 ? Shape<16>::UROWS : Shape<10>::UROWS;
        unsigned char(*r)[128] = m->raw[set];
        ok = encode(fn, r[0], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, hist, g, hist_planes, RX, rh, why, "slot") &&
             encode(fn, r[1], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, hist, g, hist_planes, RX, ur, why, "correlation slice") &&
             encode(fn, r[2], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, z, g, z_planes, RX, rh, why, "adjoint ring") &&
             encode(fn, r[3], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, coef, g, 0, RX, rh, why, "coefficient") &&
             encode(fn, r[4], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, g.dmap, g, 0, RX, rh, why, "sponge") &&
             encode(fn, r[5], CU_TENSOR_MAP_DATA_TYPE_INT32, g.rid, g, 0, RX, rh, why, "receiver");
    }
    m->ok = ok;
    return ok;
}

namespace {
// Dynamic shared memory of a launch at most: the region and exchange rows, plus 8 source values
// and the record rows of up to 8 (forward) or 6 (adjoint) steps of up to MAX_NCH channels.
template <int WARPS>
constexpr size_t fwd_smem_cap() { return sizeof(FwdSmem<WARPS>) + 4 * (TMAXF + TMAXF * MAX_NCH); }
template <int WARPS>
constexpr size_t adj_smem_cap() { return sizeof(AdjSmem<WARPS>) + 4 * 6 * MAX_NCH; }

template <int WARPS>
void fwd_tile(const DevGeo& g, const TileMaps& m, const TileFwd& a, void* stream) {
    using S = Shape<WARPS>;
    const int tiles_x = (g.nx + TW - 1) / TW, tiles_y = (g.ny + S::TH - 1) / S::TH;
    TileTma tm;
    std::memcpy(&tm, m.raw[S::SET], sizeof tm);
    const size_t smem = sizeof(FwdSmem<WARPS>) + 4 * (TMAXF + (a.gmeas ? (size_t)a.T * g.nch : 0));
    // one fixed cap (the largest any launch asks for) rather than this launch's size: contexts on
    // other host threads launch the same kernel with other sizes
    const auto kern = a.gmeas && g.noise_key ? k_fwd_tile<WARPS, true> : k_fwd_tile<WARPS, false>;
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fwd_smem_cap<WARPS>());
    if (a.k_last > 0) launch_coop(kern, dim3(tiles_x * tiles_y, a.ng), S::TPB, smem, stream, g, tm, a, tiles_x);
    else launch_pdl(kern, dim3(tiles_x * tiles_y, a.ng), S::TPB, smem, stream, g, tm, a, tiles_x);
}
template <int WARPS>
void adj_tile(const DevGeo& g, const TileMaps& m, const TileAdj& a, void* stream) {
    using S = Shape<WARPS>;
    const int tiles_x = (g.nx + TW - 1) / TW, tiles_y = (g.ny + S::TH - 1) / S::TH;
    TileTma tm;
    std::memcpy(&tm, m.raw[S::SET], sizeof tm);
    const size_t smem = sizeof(AdjSmem<WARPS>) + 4 * (size_t)a.T * g.nch;
    cudaFuncSetAttribute(k_adj_tile<WARPS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)adj_smem_cap<WARPS>());
    if (a.kz_last > 0) launch_coop(k_adj_tile<WARPS>, dim3(tiles_x * tiles_y, a.ng), S::TPB, smem, stream, g, tm, a, tiles_x);
    else launch_pdl(k_adj_tile<WARPS>, dim3(tiles_x * tiles_y, a.ng), S::TPB, smem, stream, g, tm, a, tiles_x);
}

// Blocks of a launch of `ng` groups against the blocks every SM can hold at once (at the fixed
// shared-memory cap), for a persistent launch's grid barrier.
template <int WARPS, bool FWD>
bool persistent_fits(const DevGeo& g, int ng) {
    using S = Shape<WARPS>;
    const int tiles = ((g.nx + TW - 1) / TW) * ((g.ny + S::TH - 1) / S::TH) * ng;
    const size_t cap = FWD ? fwd_smem_cap<WARPS>() : adj_smem_cap<WARPS>();
    // every instantiation a launch may use (the forward's noise-free and noisy forms)
    const void* kerns[2] = {
        FWD ? reinterpret_cast<const void*>(k_fwd_tile<WARPS, false>) : reinterpret_cast<const void*>(k_adj_tile<WARPS>),
        FWD ? reinterpret_cast<const void*>(k_fwd_tile<WARPS, true>) : reinterpret_cast<const void*>(k_adj_tile<WARPS>)};
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    for (const void* kern : kerns) {
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cap);
        int per_sm = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, S::TPB, cap) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        if (tiles > per_sm * sms) return false;
    }
    return true;
}
}  // namespace

void launch_fwd_tile(const DevGeo& g, const TileMaps& m, const TileFwd& a, void* stream) {
    if (a.warps == 10) fwd_tile<10>(g, m, a, stream);
    else fwd_tile<16>(g, m, a, stream);
}

void launch_adj_tile(const DevGeo& g, const TileMaps& m, const TileAdj& a, void* stream) {
    if (a.warps == 10) adj_tile<10>(g, m, a, stream);
    else adj_tile<16>(g, m, a, stream);
}

bool tile_persistent_fits(const DevGeo& g, int warps, bool fwd, int ng) {
    if (warps == 10) return fwd ? persistent_fits<10, true>(g, ng) : persistent_fits<10, false>(g, ng);
    return fwd ? persistent_fits<16, true>(g, ng) : persistent_fits<16, false>(g, ng);
}

}  // namespace tomo
