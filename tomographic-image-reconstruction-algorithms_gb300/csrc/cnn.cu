// cnn.cu -- kernels of the learned update network: a 5-layer 3x3 CNN with
// 32 channels, ReLU, BF16 weights and activations, FP32 accumulation.
//
//   layer 1: 16 -> 32 (3 input features f, SIRT direction, illumination,
//            zero-padded to 16 channels), bias, ReLU
//   layers 2-4: 32 -> 32, bias, ReLU
//   layer 5: 32 -> 1, bias, FP32 output (the proposed field update)
//
// Activations are BF16 in a channel-blocked layout, [image][y][channel / 8][x][8]: each
// 8-channel chunk of an image row is contiguous, so one TMA box brings a whole input row (all
// chunks, 130 pixels) into shared memory already in the tensor cores' K-major core-matrix
// layout (8 pixels x 16 bytes).  Every convolution and every weight gradient runs on the
// fifth-generation tensor cores (tcgen05.mma, kind::f16, BF16 operands, FP32 accumulators in
// tensor memory), in warp-specialised blocks: one thread issues the TMA copies, one the MMAs,
// four warps drain the accumulators; barriers are mbarriers whose waits are bounded.
//
// Convolution (k_conv_tc): an implicit GEMM per output row of 128 pixels (the MMA's M), all
// output channels (N = 32, or 16 for the output layer), K = 9 taps x input channels.  A block
// streams a strip of rows of one 128-pixel column: each input row is loaded once into a ring of
// row slots, and the A operand of tap (dy, dx) is row slot y + dy - 1 with the descriptor's
// start moved by dx pixels, so no im2col copy exists.  Output rows rotate through four TMEM
// accumulators, so the epilogue of one row overlaps the MMAs of the next.  The data gradient of
// a layer is the same kernel on the output gradient with rotated, transposed weights and a
// ReLU-mask epilogue.
//
// Output layer (one channel): its FP32 weights are split into BF16 high and low
// parts (w = hi + lo to 16 bits), placed in two output columns whose sum is the
// result; its data gradient reads the loss gradient packed the same way
// (dout = dh + dl) as a 16-channel input.  Both keep the FP32 layer's accuracy.
//
// Weight gradient (k_wgrad_tc): dW[tap][ci][co] = sum_p x[p + off(tap)][ci] dz[p][co]
// with K = pixels, both operands MN-major.  Each input row arrives as three copies shifted by
// one pixel, plus a constant plane of ones whose products give the bias gradient; accumulators
// stay in TMEM over all the block's rows; each block writes one partial sum, reduced later in
// fixed order, so training steps are deterministic.
//
// Waits: every mbarrier wait is bounded by wait_ns of %globaltimer.  A block
// whose copy or MMA has not completed by then sets bit 1 of the host-visible
// error word, waits (bounded) for what it issued, frees its TMEM and returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>

#include "cnn.h"
#include "internal.h"

namespace tomo {
namespace cnn {
namespace {

#include "async.cuh"

constexpr int COUT = 32;
constexpr int TX = 128;                     // pixels per tile (the convolution MMA's M)
constexpr int PX = TX + 2;                  // staged pixels per row: one halo pixel each side
constexpr int PLANE = TX * 16;              // weight gradient: bytes per 128-pixel 8-channel plane
constexpr unsigned int ERR_BIT = 2u;        // bit of the error word set by a timed-out wait here

enum { EPI_RELU = 0, EPI_MASK = 1, EPI_OUT = 2 };

struct ConvArgs {
    const __nv_bfloat16* w;      // B operand, [tap][chunk][N][8] BF16 (K-major core matrices)
    const float* bias;           // EPI_RELU: [N]; EPI_OUT: [1]
    const __nv_bfloat16* mask;   // EPI_MASK: blocked [B][H][N / 8][W][8] (output zero where mask <= 0)
    void* out;                   // EPI_RELU / EPI_MASK: blocked BF16 [B][H][N / 8][W][8]; EPI_OUT: FP32 [B][H][W]
    int B, H, W;
    unsigned int* err;
    uint64_t wait_ns;
};

// Row-streaming convolution.  A work item is a strip of up to RC output rows of one 128-pixel
// column tile of one image; each of its RC + 2 input rows arrives as one TMA box (every
// 8-channel chunk, 130 pixels: one halo pixel each side) into a ring of R row slots.
template <int CIN, int N>
struct ConvShape {
    static constexpr int NCH = CIN / 8;                        // input chunks
    static constexpr int CP = PX * 16;                         // bytes per chunk row: 130 pixels x 16 B
    static constexpr int R = 8;                                // input row slots
    static constexpr int NA = 4;                               // TMEM accumulators (output rows in flight)
    static constexpr int SLOT = (NCH * CP + 127) / 128 * 128;  // one input row, all chunks (one TMA box)
    static constexpr int WBYTES = 9 * NCH * N * 16;            // weights
    static constexpr uint32_t ROW_BYTES = (uint32_t)NCH * PX * 16;
    static constexpr uint32_t NCOL = NA * N < 32 ? 32 : NA * N;
    static constexpr size_t SMEM = (size_t)R * SLOT + WBYTES + (2 * R + 2 * NA + 1) * 8 + 16 + 4 * N;
    static_assert(CP % 16 == 0, "chunk row pitch");
};

// Warp roles (192 threads): warp 0 lane 0 issues the TMA row loads, warp 1 lane 0 issues the
// MMAs (9 taps x CIN / 16 per output row into one of NA accumulators; the A operand of tap
// (dy, dx) is row slot (k + dy) moved by dx pixels), warps 2-5 drain the accumulators (their
// TMEM lane quarters are warp % 4) and store.  Barriers: full / empty per row slot (TMA
// transaction bytes / MMA commit once the slot's last reader has run), full / empty per
// accumulator (MMA commit / one arrival per epilogue warp).
template <int CIN, int N, int EPI>
__global__ void __launch_bounds__(192, 2) k_conv_tc(const __grid_constant__ CUtensorMap in_map, ConvArgs a, int RC) {
    using S = ConvShape<CIN, N>;
    constexpr int NCH = S::NCH, KS = CIN / 16, R = S::R, NA = S::NA;
    constexpr uint32_t IDESC = idesc_bf16(128, N, 0, 0);
    extern __shared__ __align__(1024) unsigned char sm[];
    unsigned char* const rows = sm;                                          // [R][NCH][CP]
    unsigned char* const wsm = sm + R * S::SLOT;                             // [9][NCH][N][16 B]
    uint64_t* const full = reinterpret_cast<uint64_t*>(wsm + S::WBYTES);     // [R]
    uint64_t* const empty = full + R;                                        // [R]
    uint64_t* const accf = empty + R;                                        // [NA]
    uint64_t* const acce = accf + NA;                                        // [NA]
    uint64_t* const done = acce + NA;
    uint32_t* const tslot = reinterpret_cast<uint32_t*>(done + 1);
    volatile int* const abort = reinterpret_cast<volatile int*>(tslot + 1);
    float* const sbias = reinterpret_cast<float*>(tslot + 4);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nxt = (a.W + TX - 1) / TX, nyc = (a.H + RC - 1) / RC;
    const int items = a.B * nxt * nyc;

    if (tid == 0) {
        for (int i = 0; i < R; ++i) {
            mbar_init(&full[i], 1);
            mbar_init(&empty[i], 1);
        }
        for (int i = 0; i < NA; ++i) {
            mbar_init(&accf[i], 1);
            mbar_init(&acce[i], 4);
        }
        mbar_init(done, 1);
        *abort = 0;
        mbar_fence_init();
    }
    __syncwarp();
    if (warp == 0) tmem_alloc(tslot, S::NCOL);
    for (int i = tid; i < S::WBYTES / 16; i += blockDim.x)
        reinterpret_cast<uint4*>(wsm)[i] = reinterpret_cast<const uint4*>(a.w)[i];
    if (EPI == EPI_RELU && tid < N) sbias[tid] = a.bias[tid];
    if (EPI == EPI_OUT && tid == 0) sbias[0] = a.bias[0];
    fence_proxy_async();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;

    // item -> image b, column tile x0, first output row y0, output rows n
    auto item_at = [&](int it, int& b, int& x0, int& y0, int& n) {
        const int yc = it % nyc, r = it / nyc;
        x0 = (r % nxt) * TX;
        b = r / nxt;
        y0 = yc * RC;
        n = min(RC, a.H - y0);
    };

    if (warp == 0) {
        if (lane == 0) {   // producer: input rows y0 - 1 .. y0 + n of every item, in order
            int q = 0;
            bool ok = true;
            for (int it = blockIdx.x; it < items && ok; it += gridDim.x) {
                int b, x0, y0, n;
                item_at(it, b, x0, y0, n);
                for (int j = 0; j < n + 2; ++j, ++q) {
                    const int s = q % R;
                    if (q >= R && !role_wait(&empty[s], (uint32_t)(q / R - 1) & 1u, a.wait_ns, abort)) {
                        ok = false;
                        break;
                    }
                    mbar_expect_tx(&full[s], S::ROW_BYTES);
                    tma_load_5d(rows + s * S::SLOT, &in_map, 0, x0 - 1, 0, y0 - 1 + j, b, &full[s]);
                }
            }
            // no copy may land after the block has left: wait (bounded) for the last use of each slot
            for (int k = q - 1; k >= 0 && k >= q - R; --k) mbar_wait(&full[k % R], (uint32_t)(k / R) & 1u, a.wait_ns);
        }
    } else if (warp == 1) {
        if (lane == 0) {   // MMA issuer
            int qb = 0, t = 0;
            bool ok = true;
            const uint64_t adesc0 = smem_desc(sm_addr(rows), S::CP, 128);   // row slot 0, chunk 0, pixel 0
            const uint64_t bdesc0 = smem_desc(sm_addr(wsm), N * 16, 128);   // tap 0, chunk 0
            for (int it = blockIdx.x; it < items && ok; it += gridDim.x) {
                int b, x0, y0, n;
                item_at(it, b, x0, y0, n);
                for (int k = 0; k < n; ++k, ++t) {
                    for (int r = k == 0 ? 0 : 2; r < 3 && ok; ++r) {
                        const int qq = qb + k + r;
                        ok = role_wait(&full[qq % R], (uint32_t)(qq / R) & 1u, a.wait_ns, abort);
                    }
                    const int acc = t % NA;
                    if (ok && t >= NA) ok = role_wait(&acce[acc], (uint32_t)(t / NA - 1) & 1u, a.wait_ns, abort);
                    if (!ok) break;
                    tc_fence_after();
                    // descriptors: the start-address field is the low 14 bits (address / 16), so a
                    // byte offset o below 256 KB is added as o / 16
                    uint64_t arow[3];
#pragma unroll
                    for (int dy = 0; dy < 3; ++dy) arow[dy] = adesc0 + (uint64_t)(((qb + k + dy) % R) * (S::SLOT / 16));
#pragma unroll
                    for (int tap = 0; tap < 9; ++tap) {
#pragma unroll
                        for (int ks = 0; ks < KS; ++ks) {
                            const uint64_t ad = arow[tap / 3] + (uint64_t)(((tap % 3) * 16 + 2 * ks * S::CP) / 16);
                            const uint64_t bd = bdesc0 + (uint64_t)((tap * NCH + 2 * ks) * N);
                            umma_bf16(tmem + acc * N, ad, bd, IDESC, (tap | ks) != 0);
                        }
                    }
                    umma_commit(&accf[acc]);
                    umma_commit(&empty[(qb + k) % R]);   // input row k has had its last reader
                }
                if (!ok) break;
                umma_commit(&empty[(qb + n) % R]);
                umma_commit(&empty[(qb + n + 1) % R]);
                qb += n + 2;
            }
            // every MMA this thread issued has completed once `done` flips
            umma_commit(done);
            mbar_wait(done, 0u, a.wait_ns);
        }
    } else {   // epilogue warps: TMEM lane quarter warp % 4 = 32 pixels of the tile
        const int quarter = warp & 3;
        int t = 0;
        bool ok = true;
        for (int it = blockIdx.x; it < items && ok; it += gridDim.x) {
            int b, x0, y0, n;
            item_at(it, b, x0, y0, n);
            for (int k = 0; k < n; ++k, ++t) {
                const int acc = t % NA;
                ok = __all_sync(0xffffffffu, role_wait(&accf[acc], (uint32_t)(t / NA) & 1u, a.wait_ns, abort));
                if (!ok) break;
                tc_fence_after();
                float v[N];
                const uint32_t taddr = tmem + ((uint32_t)(32 * quarter) << 16) + (uint32_t)(acc * N);
                if constexpr (N == 32) tmem_ld32(taddr, v);
                else tmem_ld16(taddr, v);
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(&acce[acc]);   // the accumulator may take the next row
                const int x = x0 + 32 * quarter + lane;
                if (x < a.W) {
                    const int64_t row = (int64_t)b * a.H + y0 + k;
                    const int64_t p = row * a.W + x;
                    // element offset of channel chunk q of this pixel in the blocked layout
                    auto chunk_at = [&](int q) { return ((row * (N / 8) + q) * a.W + x) * 8; };
                    if constexpr (EPI == EPI_OUT) {
                        reinterpret_cast<float*>(a.out)[p] = (v[0] + v[1]) + sbias[0];
                    } else {
                        uint4 o[N / 8];
                        uint32_t* ow = reinterpret_cast<uint32_t*>(o);
                        if constexpr (EPI == EPI_MASK) {
                            uint4 m[N / 8];
#pragma unroll
                            for (int q = 0; q < N / 8; ++q) m[q] = *reinterpret_cast<const uint4*>(a.mask + chunk_at(q));
                            const __nv_bfloat16* mh = reinterpret_cast<const __nv_bfloat16*>(m);
#pragma unroll
                            for (int c = 0; c < N; ++c)
                                if (!(__bfloat162float(mh[c]) > 0.f)) v[c] = 0.f;
                        } else {
#pragma unroll
                            for (int c = 0; c < N; ++c) v[c] = fmaxf(v[c] + sbias[c], 0.f);
                        }
#pragma unroll
                        for (int c = 0; c < N / 2; ++c) {
                            const __nv_bfloat162 h = __floats2bfloat162_rn(v[2 * c], v[2 * c + 1]);
                            ow[c] = *reinterpret_cast<const uint32_t*>(&h);
                        }
                        __nv_bfloat16* const ob = reinterpret_cast<__nv_bfloat16*>(a.out);
#pragma unroll
                        for (int q = 0; q < N / 8; ++q) *reinterpret_cast<uint4*>(ob + chunk_at(q)) = o[q];
                    }
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (tid == 0 && *abort) atomicOr(a.err, ERR_BIT);
    __syncwarp();
    if (warp == 0) tmem_dealloc(tmem, S::NCOL);
}

struct WgradArgs {
    float* part;   // [gridDim.x][nout] partial sums of this launch's blocks
    int B, H, W;
    unsigned int* err;
    uint64_t wait_ns;
};

// Row-streaming weight gradient.  Input row j of a strip lands in a ring slot as three copies
// shifted by dx = 0, 1, 2 pixels (3 x CIN / 8 planes of 128 pixels x 16 B) plus a plane of
// ones; slots 0 and 1 are mirrored after the last slot, so for any output row the three input
// rows y - 1, y, y + 1 are consecutive slots and the planes (dy, dx, chunk) sit one plane apart:
// the MMA's A operand rows are (tap, ci) at a uniform stride, with no im2col copy.
template <int CIN, int NB>
struct WgradShape {
    static constexpr int NCHX = CIN / 8;
    static constexpr int NPL = 3 * NCHX + 1;                  // planes per input-row slot (ones last)
    static constexpr int MG = (3 * NPL * 8 + 127) / 128;      // M groups of 128 rows (16 planes)
    static constexpr int R = CIN == 32 ? 5 : 8;               // input row slots
    static constexpr int XSLOTS = ((R - 1) * NPL + MG * 16 - 1) / NPL + 1;   // + mirrors and read slack
    static constexpr int RD = CIN == 32 ? 2 : 4;              // output-gradient row slots
    static constexpr int XBYTES = XSLOTS * NPL * PLANE;
    static constexpr int DSLOT = NB / 8 * PLANE;
    static constexpr uint32_t NCOL = MG * NB <= 32 ? 32 : MG * NB <= 64 ? 64 : MG * NB <= 128 ? 128 : 256;
    static constexpr size_t SMEM = (size_t)XBYTES + (size_t)RD * DSLOT + (2 * R + 2 * RD + 1) * 8 + 16;
    static constexpr int NOUT = NB == 16 ? 9 * CIN + 1 : 9 * CIN * NB + NB;
    static_assert(XSLOTS >= R + 2, "mirror slots");
    static_assert(SMEM <= 232448, "shared memory");
};

// NB = 32: part row = dW[tap][ci][co] (9 CIN 32 values) then db[co];
// NB = 16 (output layer, dz = the packed loss gradient dh, dl): dW5[tap][ci] then db5, each the
// sum of the dh and dl columns.  Roles as in k_conv_tc: warp 0 lane 0 loads, warp 1 lane 0 issues
// the MMAs (3 M groups x 8 K steps per output row, accumulated over all the block's rows), warps
// 2-5 read the accumulators at the end.
template <int CIN, int NB>
__global__ void __launch_bounds__(192, 1) k_wgrad_tc(const __grid_constant__ CUtensorMap x_map,
                                                    const __grid_constant__ CUtensorMap d_map, WgradArgs a, int RC) {
    using S = WgradShape<CIN, NB>;
    constexpr int NCHX = S::NCHX, NPL = S::NPL, MG = S::MG, R = S::R, RD = S::RD;
    constexpr uint32_t IDESC = idesc_bf16(128, NB, 1, 1);
    extern __shared__ __align__(1024) unsigned char sm[];
    unsigned char* const xs = sm;                                            // [XSLOTS][NPL][PLANE]
    unsigned char* const ds = sm + S::XBYTES;                                // [RD][NB / 8][PLANE]
    uint64_t* const xfull = reinterpret_cast<uint64_t*>(ds + RD * S::DSLOT); // [R]
    uint64_t* const xempty = xfull + R;
    uint64_t* const dfull = xempty + R;                                      // [RD]
    uint64_t* const dempty = dfull + RD;
    uint64_t* const done = dempty + RD;
    uint32_t* const tslot = reinterpret_cast<uint32_t*>(done + 1);
    volatile int* const abort = reinterpret_cast<volatile int*>(tslot + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nxt = (a.W + TX - 1) / TX, nyc = (a.H + RC - 1) / RC;
    const int items = a.B * nxt * nyc;

    if (tid == 0) {
        for (int i = 0; i < R; ++i) {
            mbar_init(&xfull[i], 1);
            mbar_init(&xempty[i], 1);
        }
        for (int i = 0; i < RD; ++i) {
            mbar_init(&dfull[i], 1);
            mbar_init(&dempty[i], 1);
        }
        mbar_init(done, 1);
        *abort = 0;
        mbar_fence_init();
    }
    __syncwarp();
    if (warp == 0) tmem_alloc(tslot, S::NCOL);
    // the ones plane of every slot (bias rows); TMA never writes it
    for (int sl = 0; sl < S::XSLOTS; ++sl) {
        uint4* p = reinterpret_cast<uint4*>(xs + (sl * NPL + 3 * NCHX) * PLANE);
        for (int i = tid; i < PLANE / 16; i += blockDim.x) p[i] = make_uint4(0x3F803F80u, 0x3F803F80u, 0x3F803F80u, 0x3F803F80u);
    }
    fence_proxy_async();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;
    auto item_at = [&](int it, int& b, int& x0, int& y0, int& n) {
        const int yc = it % nyc, r = it / nyc;
        x0 = (r % nxt) * TX;
        b = r / nxt;
        y0 = yc * RC;
        n = min(RC, a.H - y0);
    };
    const bool any = (int)blockIdx.x < items;

    if (warp == 0) {
        if (lane == 0) {   // producer: per item input rows 0, 1, then (input row k + 2, output row k)
            int q = 0, qd = 0;
            bool ok = true;
            auto load_x = [&](int b, int x0, int yy) {
                const int s = q % R;
                if (q >= R && !role_wait(&xempty[s], (uint32_t)(q / R - 1) & 1u, a.wait_ns, abort)) return false;
                const int copies = s < 2 ? 2 : 1;   // slots 0 and 1 are mirrored at R and R + 1
                mbar_expect_tx(&xfull[s], (uint32_t)(copies * 3 * NCHX * PLANE));
                for (int m = 0; m < copies; ++m) {
                    unsigned char* dst = xs + (m == 0 ? s : R + s) * NPL * PLANE;
                    for (int dx = 0; dx < 3; ++dx)   // one box: every chunk of the row, shifted by dx
                        tma_load_5d(dst + dx * NCHX * PLANE, &x_map, 0, x0 + dx - 1, 0, yy, b, &xfull[s]);
                }
                ++q;
                return true;
            };
            auto load_d = [&](int b, int x0, int yy) {
                const int s = qd % RD;
                if (qd >= RD && !role_wait(&dempty[s], (uint32_t)(qd / RD - 1) & 1u, a.wait_ns, abort)) return false;
                mbar_expect_tx(&dfull[s], (uint32_t)S::DSLOT);
                tma_load_5d(ds + s * S::DSLOT, &d_map, 0, x0, 0, yy, b, &dfull[s]);
                ++qd;
                return true;
            };
            for (int it = blockIdx.x; it < items && ok; it += gridDim.x) {
                int b, x0, y0, n;
                item_at(it, b, x0, y0, n);
                ok = load_x(b, x0, y0 - 1) && load_x(b, x0, y0);
                for (int k = 0; k < n && ok; ++k) ok = load_x(b, x0, y0 + k + 1) && load_d(b, x0, y0 + k);
            }
            for (int k = q - 1; k >= 0 && k >= q - R; --k) mbar_wait(&xfull[k % R], (uint32_t)(k / R) & 1u, a.wait_ns);
            for (int k = qd - 1; k >= 0 && k >= qd - RD; --k)
                mbar_wait(&dfull[k % RD], (uint32_t)(k / RD) & 1u, a.wait_ns);
        }
    } else if (warp == 1) {
        if (lane == 0) {   // MMA issuer
            int qb = 0, t = 0;
            bool ok = true;
            // MN-major: 8-channel groups along M one plane apart, 8-pixel groups along K 128 B apart
            const uint64_t xdesc0 = smem_desc(sm_addr(xs), 128, PLANE);
            const uint64_t ddesc0 = smem_desc(sm_addr(ds), 128, PLANE);
            for (int it = blockIdx.x; it < items && ok; it += gridDim.x) {
                int b, x0, y0, n;
                item_at(it, b, x0, y0, n);
                for (int k = 0; k < n; ++k, ++t) {
                    for (int r = k == 0 ? 0 : 2; r < 3 && ok; ++r) {
                        const int qq = qb + k + r;
                        ok = role_wait(&xfull[qq % R], (uint32_t)(qq / R) & 1u, a.wait_ns, abort);
                    }
                    if (ok) ok = role_wait(&dfull[t % RD], (uint32_t)(t / RD) & 1u, a.wait_ns, abort);
                    if (!ok) break;
                    tc_fence_after();
                    // window: slots (qb + k) % R .. + 2, consecutive thanks to the mirrors; byte
                    // offsets enter the descriptors' start-address field as offset / 16
                    const uint64_t xd = xdesc0 + (uint64_t)(((qb + k) % R) * (NPL * PLANE / 16));
                    const uint64_t dd = ddesc0 + (uint64_t)((t % RD) * (S::DSLOT / 16));
#pragma unroll
                    for (int g = 0; g < MG; ++g) {
#pragma unroll
                        for (int kk = 0; kk < TX / 16; ++kk)
                            umma_bf16(tmem + g * NB, xd + (uint64_t)((g * 16 * PLANE + kk * 256) / 16),
                                      dd + (uint64_t)(kk * 256 / 16), IDESC, (t | kk) != 0);
                    }
                    umma_commit(&dempty[t % RD]);
                    umma_commit(&xempty[(qb + k) % R]);
                }
                if (!ok) break;
                umma_commit(&xempty[(qb + n) % R]);
                umma_commit(&xempty[(qb + n + 1) % R]);
                qb += n + 2;
            }
            umma_commit(done);
        }
    }
    // epilogue (warps 2-5): the accumulators once every MMA has completed
    bool ok = true;
    if (warp >= 2) ok = __all_sync(0xffffffffu, role_wait(done, 0u, a.wait_ns, abort)) && !*abort;
    tc_fence_before();
    ok = !__syncthreads_or(!ok || *abort);
    tc_fence_after();
    if (ok && warp >= 2) {
        const int quarter = warp & 3;
        float* const out = a.part + (int64_t)blockIdx.x * S::NOUT;
#pragma unroll
        for (int g = 0; g < MG; ++g) {
            float v[NB];
            const uint32_t taddr = tmem + ((uint32_t)(32 * quarter) << 16) + (uint32_t)(g * NB);
            if constexpr (NB == 32) tmem_ld32(taddr, v);
            else tmem_ld16(taddr, v);
            if (!any) {
#pragma unroll
                for (int n = 0; n < NB; ++n) v[n] = 0.f;
            }
            const int m = g * 128 + 32 * quarter + lane;   // window row: plane m / 8, channel m % 8
            const int p = m / 8, i = m % 8, dy = p / NPL, rem = p % NPL;
            int row = -1;                                   // output row: tap * CIN + ci, or 9 CIN = bias
            if (dy < 3 && rem < 3 * NCHX) row = (dy * 3 + rem / NCHX) * CIN + (rem % NCHX) * 8 + i;
            else if (dy == 0 && rem == 3 * NCHX && i == 0) row = 9 * CIN;
            if (row < 0) continue;
            if constexpr (NB == 16) {
                out[row] = v[0] + v[1];
            } else {
                float4* o = reinterpret_cast<float4*>(out + (int64_t)row * NB);
#pragma unroll
                for (int q = 0; q < NB / 4; ++q) o[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (tid == 0 && *abort) atomicOr(a.err, ERR_BIT);
    __syncwarp();
    if (warp == 0) tmem_dealloc(tmem, S::NCOL);
}

// Input features: planar FP32 [b][3][H][W] -> blocked BF16 [b][y][2][x][8] with 16 channels (3
// used): chunk 0 of a pixel holds f, the direction and the illumination, chunk 1 is zero.
__global__ void k_pack_input(const float* __restrict__ feat, __nv_bfloat16* __restrict__ x, int B, int H, int W) {
    const int64_t HW = (int64_t)H * W, n = (int64_t)B * HW;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
        const int64_t b = p / HW, q = p - b * HW, row = p / W, xx = p - row * W;
        const float* f = feat + b * 3 * HW + q;
        const __nv_bfloat162 c01 = __floats2bfloat162_rn(f[0], f[HW]);
        const __nv_bfloat162 c2 = __floats2bfloat162_rn(f[2 * HW], 0.f);
        __nv_bfloat16* o = x + (row * 2 * W + xx) * 8;
        *reinterpret_cast<uint4*>(o) =
            make_uint4(*reinterpret_cast<const uint32_t*>(&c01), *reinterpret_cast<const uint32_t*>(&c2), 0u, 0u);
        *reinterpret_cast<uint4*>(o + (int64_t)W * 8) = make_uint4(0u, 0u, 0u, 0u);
    }
}

// Masked MSE: loss partial per block; dout = 2 mask (out - tgt) / msum, also packed as BF16
// channels (dh, dl, dh, 0 ...) with dh + dl = dout to 16 bits, the output layer's gradient input.
__global__ void __launch_bounds__(256) k_loss(const float* __restrict__ out, const float* __restrict__ tgt,
                                             const float* __restrict__ msk, int64_t n, int W, float inv_msum,
                                             float* __restrict__ dout, __nv_bfloat16* __restrict__ dpk,
                                             double* __restrict__ part) {
    double acc = 0.0;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
        const float e = (out[p] - tgt[p]) * msk[p];
        acc += (double)e * e;
        const float d = 2.f * e * inv_msum;
        dout[p] = d;
        const __nv_bfloat16 dh = __float2bfloat16(d);
        const __nv_bfloat16 dl = __float2bfloat16(d - __bfloat162float(dh));
        const __nv_bfloat162 h01 = __halves2bfloat162(dh, dl), h2 = __halves2bfloat162(dh, __float2bfloat16(0.f));
        uint4 q0 = make_uint4(*reinterpret_cast<const uint32_t*>(&h01), *reinterpret_cast<const uint32_t*>(&h2), 0u, 0u);
        const int64_t row = p / W, xx = p - row * W;   // blocked layout [row][2][x][8]
        __nv_bfloat16* o = dpk + (row * 2 * W + xx) * 8;
        *reinterpret_cast<uint4*>(o) = q0;
        *reinterpret_cast<uint4*>(o + (int64_t)W * 8) = make_uint4(0u, 0u, 0u, 0u);
    }
    __shared__ double red[256];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// dst[j] = sum over blocks of part[blk][j], fixed order.
__global__ void k_reduce_parts(const float* __restrict__ part, int nblk, int nout, float* __restrict__ dst) {
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < nout; j += gridDim.x * blockDim.x) {
        float acc = 0.f;
        for (int b = 0; b < nblk; ++b) acc += part[(int64_t)b * nout + j];
        dst[j] = acc;
    }
}

__global__ void k_sum_double(const double* __restrict__ part, int n, double* __restrict__ out) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        double acc = 0.0;
        for (int i = 0; i < n; ++i) acc += part[i];
        *out = acc;
    }
}

// Adam (bias-corrected) on the FP32 master parameters.
__global__ void k_adam(float* __restrict__ w, float* __restrict__ m, float* __restrict__ v, const float* __restrict__ grad,
                       int n, float lr, float b1, float b2, float eps, float c1, float c2) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float gi = grad[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        w[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + eps);
    }
}

// Master W[tap][ci][co] -> the convolution's B operand [tap][ci / 8][co][ci % 8] and the data
// gradient's [tap'][co / 8][ci][co % 8] with tap' = 8 - tap (input channels co, outputs ci).
__global__ void k_pack_weights(const float* __restrict__ wm, int cin, __nv_bfloat16* __restrict__ wf,
                               __nv_bfloat16* __restrict__ wd) {
    const int n = 9 * cin * COUT;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
        const int co = e % COUT, ci = (e / COUT) % cin, tap = e / COUT / cin;
        const __nv_bfloat16 v = __float2bfloat16(wm[e]);
        wf[((tap * (cin / 8) + ci / 8) * COUT + co) * 8 + ci % 8] = v;
        if (wd) wd[(((8 - tap) * (COUT / 8) + co / 8) * cin + ci) * 8 + co % 8] = v;
    }
}

// Output layer W5[tap][ci] (FP32) -> forward B operand [tap][ci / 8][16][ci % 8] with column 0 =
// hi, 1 = lo, and data-gradient B operand [tap'][k / 8][32][k % 8] over the packed gradient's
// channels k = (dh, dl, dh): (hi, hi, lo) of W5[8 - tap'][ci].
__global__ void k_pack_out_weights(const float* __restrict__ w5, __nv_bfloat16* __restrict__ wo,
                                   __nv_bfloat16* __restrict__ wod) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= 9 * 16 * COUT) return;
    // forward: e = ((tap * 4 + chunk) * 16 + n) * 8 + i
    {
        const int i = e % 8, nn = (e / 8) % 16, ch = (e / 128) % 4, tap = e / 512;
        const float w = w5[tap * COUT + ch * 8 + i];
        const __nv_bfloat16 hi = __float2bfloat16(w), lo = __float2bfloat16(w - __bfloat162float(hi));
        wo[e] = nn == 0 ? hi : nn == 1 ? lo : __float2bfloat16(0.f);
    }
    // data gradient: e = ((tap' * 2 + k / 8) * 32 + ci) * 8 + k % 8
    {
        const int k = (e / 256) % 2 * 8 + e % 8, ci = (e / 8) % 32, tp = e / 512;
        const float w = w5[(8 - tp) * COUT + ci];
        const __nv_bfloat16 hi = __float2bfloat16(w), lo = __float2bfloat16(w - __bfloat162float(hi));
        wod[e] = k == 0 || k == 1 ? hi : k == 2 ? lo : __float2bfloat16(0.f);
    }
}

inline int blocks_for(int64_t n, int t) {
    const int64_t b = (n + t - 1) / t;
    return (int)(b < 2048 ? (b < 1 ? 1 : b) : 2048);
}

int sm_count() {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 1;
}

template <int CIN, int N, int EPI>
void conv_launch(const void* map, const ConvArgs& a, cudaStream_t st) {
    using S = ConvShape<CIN, N>;
    auto kern = k_conv_tc<CIN, N, EPI>;
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S::SMEM);
    // two blocks per SM (their TMEM: 2 x NCOL <= 512 columns); each 128-pixel column is cut into
    // as many strips as there are blocks for it, so a block takes about one strip and every input
    // row but a strip's two halo rows is loaded once
    const int64_t columns = (int64_t)a.B * ((a.W + TX - 1) / TX);
    const int64_t slots = 2 * (int64_t)sm_count();
    const int64_t strips = std::max<int64_t>(1, slots / columns);
    const int RC = (int)std::max<int64_t>(2, (a.H + strips - 1) / strips);
    const int64_t items = columns * ((a.H + RC - 1) / RC);
    const int grid = (int)std::max<int64_t>(1, std::min(items, slots));
    CUtensorMap m;
    std::memcpy(&m, map, sizeof m);
    kern<<<grid, 192, S::SMEM, st>>>(m, a, RC);
}

template <int CIN, int NB>
int wgrad_launch(const void* xmap, const void* dmap, const WgradArgs& a, int max_blocks, cudaStream_t st) {
    using S = WgradShape<CIN, NB>;
    auto kern = k_wgrad_tc<CIN, NB>;
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S::SMEM);
    // one block per SM (one wave: every block's partial is summed afterwards); each 128-pixel
    // column cut into about SMs / columns strips
    const int64_t columns = (int64_t)a.B * ((a.W + TX - 1) / TX);
    const int64_t slots = std::min<int64_t>(sm_count(), max_blocks);
    const int64_t strips = std::max<int64_t>(1, slots / columns);
    const int RC = (int)std::max<int64_t>(2, (a.H + strips - 1) / strips);
    const int64_t items = columns * ((a.H + RC - 1) / RC);
    const int grid = (int)std::max<int64_t>(1, std::min(items, slots));
    CUtensorMap xm, dm;
    std::memcpy(&xm, xmap, sizeof xm);
    std::memcpy(&dm, dmap, sizeof dm);
    kern<<<grid, 192, S::SMEM, st>>>(xm, dm, a, RC);
    return grid;
}

using EncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                 const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

}  // namespace

// ---- tensor maps ------------------------------------------------------------------
bool encode_act_map(unsigned char out[128], const __nv_bfloat16* base, int C, int B, int H, int W, bool conv_box) {
    const EncodeTiled fn = reinterpret_cast<EncodeTiled>(tensor_map_encoder());
    if (!fn || C % 8 != 0) return false;
    CUtensorMap m;
    // blocked layout [b][y][C / 8][x][8]: dimensions (channel in chunk, x, chunk, y, image)
    const cuuint64_t nch = (cuuint64_t)C / 8;
    const cuuint64_t dims[5] = {8u, (cuuint64_t)W, nch, (cuuint64_t)H, (cuuint64_t)B};
    const cuuint64_t strides[4] = {16u, (cuuint64_t)W * 16u, nch * W * 16u, (cuuint64_t)H * nch * W * 16u};
    const cuuint32_t box[5] = {8u, (cuuint32_t)(conv_box ? PX : TX), (cuuint32_t)nch, 1u, 1u};
    const cuuint32_t estr[5] = {1u, 1u, 1u, 1u, 1u};
    const CUresult r = fn(&m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5u, const_cast<__nv_bfloat16*>(base), dims, strides,
                          box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return false;
    std::memcpy(out, &m, sizeof m);
    return true;
}

// ---- launchers -------------------------------------------------------------------
void pack_input(const float* feat, __nv_bfloat16* x, int B, int H, int W, cudaStream_t st) {
    k_pack_input<<<blocks_for((int64_t)B * H * W, 256), 256, 0, st>>>(feat, x, B, H, W);
}

void conv(ConvKind kind, const void* in_map, const __nv_bfloat16* w, const float* bias, const __nv_bfloat16* mask,
          void* out, int B, int H, int W, unsigned int* err, uint64_t wait_ns, cudaStream_t st) {
    const ConvArgs a{w, bias, mask, out, B, H, W, err, wait_ns};
    switch (kind) {
    case CONV_IN: conv_launch<16, 32, EPI_RELU>(in_map, a, st); break;
    case CONV_MID: conv_launch<32, 32, EPI_RELU>(in_map, a, st); break;
    case CONV_DGRAD: conv_launch<32, 32, EPI_MASK>(in_map, a, st); break;
    case CONV_OUT: conv_launch<32, 16, EPI_OUT>(in_map, a, st); break;
    case CONV_OUT_DGRAD: conv_launch<16, 32, EPI_MASK>(in_map, a, st); break;
    }
}

void wgrad(WgradKind kind, const void* x_map, const void* d_map, float* part, int max_blocks, float* grad, int B, int H,
           int W, unsigned int* err, uint64_t wait_ns, cudaStream_t st) {
    const WgradArgs a{part, B, H, W, err, wait_ns};
    int nblk = 1, nout = 1;
    switch (kind) {
    case WGRAD_IN:
        nblk = wgrad_launch<16, 32>(x_map, d_map, a, max_blocks, st);
        nout = WgradShape<16, 32>::NOUT;
        break;
    case WGRAD_MID:
        nblk = wgrad_launch<32, 32>(x_map, d_map, a, max_blocks, st);
        nout = WgradShape<32, 32>::NOUT;
        break;
    case WGRAD_OUT:
        nblk = wgrad_launch<32, 16>(x_map, d_map, a, max_blocks, st);
        nout = WgradShape<32, 16>::NOUT;
        break;
    }
    k_reduce_parts<<<blocks_for(nout, 256), 256, 0, st>>>(part, nblk, nout, grad);
}

void loss(const float* out, const float* tgt, const float* msk, int64_t n, int W, float inv_msum, float* dout,
          __nv_bfloat16* dpk, double* part, int nblk, double* total, cudaStream_t st) {
    k_loss<<<nblk, 256, 0, st>>>(out, tgt, msk, n, W, inv_msum, dout, dpk, part);
    k_sum_double<<<1, 32, 0, st>>>(part, nblk, total);
}

void adam(float* w, float* m, float* v, const float* g, int n, float lr, float b1, float b2, float eps, float c1, float c2,
          cudaStream_t st) {
    k_adam<<<blocks_for(n, 256), 256, 0, st>>>(w, m, v, g, n, lr, b1, b2, eps, c1, c2);
}

void pack_weights(const float* wm, int cin, __nv_bfloat16* wf, __nv_bfloat16* wd, cudaStream_t st) {
    k_pack_weights<<<blocks_for(9 * cin * COUT, 256), 256, 0, st>>>(wm, cin, wf, wd);
}

void pack_out_weights(const float* w5, __nv_bfloat16* wo, __nv_bfloat16* wod, cudaStream_t st) {
    k_pack_out_weights<<<(9 * 16 * COUT + 255) / 256, 256, 0, st>>>(w5, wo, wod);
}

}  // namespace cnn
}  // namespace tomo
