// cnn.cu -- kernels of the learned update network: a 5-layer 3x3 CNN with
// 32 channels, ReLU, BF16 weights and activations, FP32 accumulation.
//
//   layer 1: 16 -> 32 (3 input features f, SIRT direction, illumination,
//            zero-padded to 16 channels), bias, ReLU
//   layers 2-4: 32 -> 32, bias, ReLU
//   layer 5: 32 -> 1, bias, FP32 output (the proposed field update)
//
// Activations are NHWC BF16 ([image][y][x][channel]).  Every convolution and
// every weight gradient runs on the fifth-generation tensor cores (tcgen05.mma,
// kind::f16, BF16 operands, FP32 accumulators in tensor memory), with operands
// staged in shared memory by TMA tile copies (cp.async.bulk.tensor) and
// completion tracked by mbarriers whose waits are bounded.
//
// Convolution (k_conv_tc): an implicit GEMM per tile of 128 pixels of one
// image row (the MMA's M), all output channels (N = 32, or 16 for the output
// layer), K = 9 taps x input channels.  The tile's 3 rows x 130 pixels of
// input arrive as one TMA box per 8-channel chunk; because a chunk is stored as
// pixels x 16 bytes, the A operand of tap (dy, dx) is the same buffer with the
// descriptor's start moved by dy rows and dx pixels, so no im2col copy exists.
// A persistent block keeps the weights in shared memory, double-buffers the
// input patch and the TMEM accumulator, and stores tile i - 1 while the tensor
// cores run tile i.  The data gradient of a layer is the same kernel on the
// output gradient with rotated, transposed weights and a ReLU-mask epilogue.
//
// Output layer (one channel): its FP32 weights are split into BF16 high and low
// parts (w = hi + lo to 16 bits), placed in two output columns whose sum is the
// result; its data gradient reads the loss gradient packed the same way
// (dout = dh + dl) as a 16-channel input.  Both keep the FP32 layer's accuracy.
//
// Weight gradient (k_wgrad_tc): dW[tap][ci][co] = sum_p x[p + off(tap)][ci] dz[p][co]
// with K = pixels.  Per tile of 128 pixels the block stages, by TMA, one
// 128-pixel box per (tap, chunk) of x (the tap shift applied by the copy's
// coordinates) plus a constant all-ones plane whose products give the bias
// gradient, and the tile's dz; both operands are MN-major.  Accumulators stay in
// TMEM over all the block's tiles; each block writes one partial sum, reduced
// later in fixed order, so training steps are deterministic.
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
constexpr int CPITCH = 6272;                // bytes per staged 8-channel chunk: 3 x 130 x 16 B, 128-B aligned
constexpr int PLANE = TX * 16;              // weight gradient: bytes per 128-pixel 8-channel plane
constexpr unsigned int ERR_BIT = 2u;        // bit of the error word set by a timed-out wait here
static_assert(3 * PX * 16 <= CPITCH && CPITCH % 128 == 0, "chunk pitch");

enum { EPI_RELU = 0, EPI_MASK = 1, EPI_OUT = 2 };

struct ConvArgs {
    const __nv_bfloat16* w;      // B operand, [tap][chunk][N][8] BF16 (K-major core matrices)
    const float* bias;           // EPI_RELU: [N]; EPI_OUT: [1]
    const __nv_bfloat16* mask;   // EPI_MASK: [B][H][W][N] (output zero where mask <= 0)
    void* out;                   // EPI_RELU / EPI_MASK: BF16 [B][H][W][N]; EPI_OUT: FP32 [B][H][W]
    int B, H, W;
    unsigned int* err;
    uint64_t wait_ns;
};

template <int CIN, int N>
struct ConvShape {
    static constexpr int NCH = CIN / 8;                       // input chunks
    static constexpr int PBYTES = NCH * CPITCH;               // one patch buffer
    static constexpr int WBYTES = 9 * NCH * N * 16;           // weights
    static constexpr uint32_t LOAD_BYTES = (uint32_t)NCH * 3 * PX * 16;
    static constexpr uint32_t NCOL = 2 * N < 32 ? 32 : 2 * N; // TMEM columns: two accumulators
    static constexpr size_t SMEM = 2 * PBYTES + WBYTES + 4 * 8 + 16 + 4 * N;
};

template <int CIN, int N, int EPI>
__global__ void __launch_bounds__(128) k_conv_tc(const __grid_constant__ CUtensorMap in_map, ConvArgs a) {
    using S = ConvShape<CIN, N>;
    constexpr int NCH = S::NCH, KS = CIN / 16;
    constexpr uint32_t IDESC = idesc_bf16(128, N, 0, 0);
    extern __shared__ __align__(1024) unsigned char sm[];
    unsigned char* const patch = sm;                                     // [2][NCH][3][PX][16 B]
    unsigned char* const wsm = sm + 2 * S::PBYTES;                       // [9][NCH][N][16 B]
    uint64_t* const bars = reinterpret_cast<uint64_t*>(wsm + S::WBYTES); // loaded[2], computed[2]
    uint32_t* const tslot = reinterpret_cast<uint32_t*>(bars + 4);
    float* const sbias = reinterpret_cast<float*>(tslot + 4);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nxt = (a.W + TX - 1) / TX;
    const int ntiles = a.B * a.H * nxt;
    const int mine = ntiles > (int)blockIdx.x ? (ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;

    if (tid == 0) {
        for (int i = 0; i < 4; ++i) mbar_init(&bars[i], 1);
        mbar_fence_init();
    }
    __syncwarp();
    if (warp == 0) tmem_alloc(tslot, S::NCOL);
    for (int i = tid; i < S::WBYTES / 16; i += 128)
        reinterpret_cast<uint4*>(wsm)[i] = reinterpret_cast<const uint4*>(a.w)[i];
    if (EPI == EPI_RELU && tid < N) sbias[tid] = a.bias[tid];
    if (EPI == EPI_OUT && tid == 0) sbias[0] = a.bias[0];
    fence_proxy_async();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;

    auto tile_at = [&](int i, int& b, int& y, int& x0) {
        const int t = (int)blockIdx.x + i * (int)gridDim.x;
        const int r = t / nxt;
        x0 = (t - r * nxt) * TX;
        y = r % a.H;
        b = r / a.H;
    };
    int issued = 0, landed = 0, computed = 0, drained = 0;   // thread 0's counts of loads and MMA batches
    auto issue_load = [&](int i) {
        int b, y, x0;
        tile_at(i, b, y, x0);
        uint64_t* bar = &bars[i & 1];
        unsigned char* dst = patch + (i & 1) * S::PBYTES;
        mbar_expect_tx(bar, S::LOAD_BYTES);
        for (int c = 0; c < NCH; ++c) tma_load_4d(dst + c * CPITCH, &in_map, 8 * c, x0 - 1, y - 1, b, bar);
        ++issued;
    };
    if (tid == 0) {
        if (mine > 0) issue_load(0);
        if (mine > 1) issue_load(1);
    }

    bool ok = true;
    for (int i = 0; i <= mine; ++i) {
        // tensor-core work of tile i: one thread issues 9 x KS MMAs into accumulator i % 2
        if (i < mine && tid == 0) {
            const int s = i & 1;
            if (mbar_wait(&bars[s], (uint32_t)(i >> 1) & 1u, a.wait_ns)) {
                ++landed;
                tc_fence_after();
                const uint32_t pb = sm_addr(patch + s * S::PBYTES), wb = sm_addr(wsm);
#pragma unroll
                for (int tap = 0; tap < 9; ++tap) {
#pragma unroll
                    for (int ks = 0; ks < KS; ++ks) {
                        const uint64_t ad =
                            smem_desc(pb + 2 * ks * CPITCH + ((tap / 3) * PX + tap % 3) * 16, CPITCH, 128);
                        const uint64_t bd = smem_desc(wb + (tap * NCH + 2 * ks) * N * 16, N * 16, 128);
                        umma_bf16(tmem + s * N, ad, bd, IDESC, (tap | ks) != 0);
                    }
                }
                umma_commit(&bars[2 + s]);
                ++computed;
            } else {
                ok = false;
            }
        }
        // epilogue of tile i - 1 (every thread: its TMEM lane is one pixel), overlapping tile i
        if (i >= 1) {
            const int j = i - 1, s = j & 1;
            // warp-uniform outcome: the TMEM load below is warp-collective
            const bool got = __all_sync(0xffffffffu, mbar_wait(&bars[2 + s], (uint32_t)(j >> 1) & 1u, a.wait_ns));
            if (!got) {
                ok = false;
            } else {
                tc_fence_after();
                if (tid == 0) {
                    ++drained;
                    if (ok && j + 2 < mine) issue_load(j + 2);   // tile j's MMAs have read buffer s
                }
                float v[N];
                const uint32_t taddr = tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)(s * N);
                if constexpr (N == 32) tmem_ld32(taddr, v);
                else tmem_ld16(taddr, v);
                int b, y, x0;
                tile_at(j, b, y, x0);
                const int x = x0 + 32 * warp + lane;
                if (x < a.W) {
                    const int64_t p = ((int64_t)b * a.H + y) * a.W + x;
                    if constexpr (EPI == EPI_OUT) {
                        reinterpret_cast<float*>(a.out)[p] = (v[0] + v[1]) + sbias[0];
                    } else {
                        uint4 o[N / 8];
                        uint32_t* ow = reinterpret_cast<uint32_t*>(o);
                        if constexpr (EPI == EPI_MASK) {
                            const uint4* mp = reinterpret_cast<const uint4*>(a.mask + p * N);
                            uint4 m[N / 8];
#pragma unroll
                            for (int q = 0; q < N / 8; ++q) m[q] = mp[q];
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
                        uint4* op = reinterpret_cast<uint4*>(reinterpret_cast<__nv_bfloat16*>(a.out) + p * N);
#pragma unroll
                        for (int q = 0; q < N / 8; ++q) op[q] = o[q];
                    }
                }
            }
        }
        // accumulator i - 1 is read: the MMAs of tile i + 1 may overwrite it
        tc_fence_before();
        if (__syncthreads_or(!ok)) {
            ok = false;
            break;
        }
        tc_fence_after();
    }
    if (tid == 0 && !ok) {
        atomicOr(a.err, ERR_BIT);
        for (int k = landed; k < issued; ++k) mbar_wait(&bars[k & 1], (uint32_t)(k >> 1) & 1u, a.wait_ns);
        for (int k = drained; k < computed; ++k) mbar_wait(&bars[2 + (k & 1)], (uint32_t)(k >> 1) & 1u, a.wait_ns);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    __syncwarp();
    if (warp == 0) tmem_dealloc(tmem, S::NCOL);
}

struct WgradArgs {
    float* part;   // [gridDim.x][nout] partial sums of this launch's blocks
    int B, H, W;
    unsigned int* err;
    uint64_t wait_ns;
};

template <int CIN, int NB>
struct WgradShape {
    static constexpr int NXP = 9 * CIN / 8;                   // x planes per tile: (tap, chunk)
    static constexpr int ONES = NXP;                          // plane of ones (bias gradient)
    static constexpr int MG = (8 * (NXP + 1) + 127) / 128;    // M groups of 128 rows (16 planes)
    static constexpr int XBYTES = MG * 16 * PLANE;            // one x buffer
    static constexpr int DBYTES = NB / 8 * PLANE;             // one dz buffer
    static constexpr uint32_t LOAD_BYTES = (uint32_t)(NXP + NB / 8) * PLANE;
    static constexpr uint32_t NCOL = MG * NB <= 32 ? 32 : MG * NB <= 64 ? 64 : MG * NB <= 128 ? 128 : 256;
    static constexpr size_t SMEM = 2 * (size_t)XBYTES + 2 * (size_t)DBYTES + 4 * 8 + 16;
    static constexpr int NOUT = NB == 16 ? 9 * CIN + 1 : 9 * CIN * NB + NB;
};

// NB = 32: part row = dW[tap][ci][co] (9 CIN 32 values) then db[co];
// NB = 16 (output layer, dz = the packed loss gradient dh, dl): dW5[tap][ci] then db5, each the
// sum of the dh and dl columns.
template <int CIN, int NB>
__global__ void __launch_bounds__(128) k_wgrad_tc(const __grid_constant__ CUtensorMap x_map,
                                                 const __grid_constant__ CUtensorMap d_map, WgradArgs a) {
    using S = WgradShape<CIN, NB>;
    constexpr uint32_t IDESC = idesc_bf16(128, NB, 1, 1);
    extern __shared__ __align__(1024) unsigned char sm[];
    unsigned char* const xs = sm;                                   // [2][MG * 16][128 px][16 B]
    unsigned char* const ds = sm + 2 * S::XBYTES;                   // [2][NB / 8][128 px][16 B]
    uint64_t* const bars = reinterpret_cast<uint64_t*>(ds + 2 * S::DBYTES);   // loaded[2], computed[2]
    uint32_t* const tslot = reinterpret_cast<uint32_t*>(bars + 4);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nxt = (a.W + TX - 1) / TX;
    const int ntiles = a.B * a.H * nxt;
    const int mine = ntiles > (int)blockIdx.x ? (ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;

    if (tid == 0) {
        for (int i = 0; i < 4; ++i) mbar_init(&bars[i], 1);
        mbar_fence_init();
    }
    __syncwarp();
    if (warp == 0) tmem_alloc(tslot, S::NCOL);
    // constant planes of both buffers: ones (bias rows), then zeros up to the last M group
    for (int buf = 0; buf < 2; ++buf) {
        uint4* p = reinterpret_cast<uint4*>(xs + buf * S::XBYTES + S::ONES * PLANE);
        const int n16 = (S::MG * 16 - S::ONES) * PLANE / 16;
        for (int i = tid; i < n16; i += 128)
            p[i] = i < PLANE / 16 ? make_uint4(0x3F803F80u, 0x3F803F80u, 0x3F803F80u, 0x3F803F80u)
                                  : make_uint4(0u, 0u, 0u, 0u);
    }
    fence_proxy_async();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;

    bool ok = true;
    if (tid == 0 && mine > 0) {
        int issued = 0, landed = 0, computed = 0, drained = 0;
        auto issue_load = [&](int i) {
            const int t = (int)blockIdx.x + i * (int)gridDim.x;
            const int r = t / nxt, x0 = (t - r * nxt) * TX, y = r % a.H, b = r / a.H;
            uint64_t* bar = &bars[i & 1];
            unsigned char* xd = xs + (i & 1) * S::XBYTES;
            unsigned char* dd = ds + (i & 1) * S::DBYTES;
            mbar_expect_tx(bar, S::LOAD_BYTES);
            for (int tap = 0; tap < 9; ++tap)
                for (int c = 0; c < CIN / 8; ++c)
                    tma_load_4d(xd + (tap * (CIN / 8) + c) * PLANE, &x_map, 8 * c, x0 + tap % 3 - 1, y + tap / 3 - 1,
                                b, bar);
            for (int c = 0; c < NB / 8; ++c) tma_load_4d(dd + c * PLANE, &d_map, 8 * c, x0, y, b, bar);
            ++issued;
        };
        issue_load(0);
        if (mine > 1) issue_load(1);
        for (int i = 0; i < mine && ok; ++i) {
            const int s = i & 1;
            if (!mbar_wait(&bars[s], (uint32_t)(i >> 1) & 1u, a.wait_ns)) {
                ok = false;
                break;
            }
            ++landed;
            tc_fence_after();
            const uint32_t xb = sm_addr(xs + s * S::XBYTES), db = sm_addr(ds + s * S::DBYTES);
#pragma unroll
            for (int g = 0; g < S::MG; ++g) {
#pragma unroll
                for (int k = 0; k < TX / 16; ++k) {
                    // MN-major: 8-element groups along M (channels) one plane apart, along K
                    // (pixels) 128 bytes apart
                    const uint64_t ad = smem_desc(xb + g * 16 * PLANE + k * 256, 128, PLANE);
                    const uint64_t bd = smem_desc(db + k * 256, 128, PLANE);
                    umma_bf16(tmem + g * NB, ad, bd, IDESC, (i | k) != 0);
                }
            }
            umma_commit(&bars[2 + s]);
            ++computed;
            // buffer (i - 1) % 2 is free once tile i - 1's MMAs are done: tile i + 1 lands there
            if (i >= 1) {
                if (!mbar_wait(&bars[2 + ((i - 1) & 1)], (uint32_t)((i - 1) >> 1) & 1u, a.wait_ns)) {
                    ok = false;
                    break;
                }
                ++drained;
                if (i + 1 < mine) issue_load(i + 1);
            }
        }
        // the last batch of MMAs (every earlier one completed before it in issue order)
        if (ok) {
            if (mbar_wait(&bars[2 + ((mine - 1) & 1)], (uint32_t)((mine - 1) >> 1) & 1u, a.wait_ns)) drained = computed;
            else ok = false;
        }
        if (!ok) {
            atomicOr(a.err, ERR_BIT);
            for (int k = landed; k < issued; ++k) mbar_wait(&bars[k & 1], (uint32_t)(k >> 1) & 1u, a.wait_ns);
            for (int k = drained; k < computed; ++k)
                mbar_wait(&bars[2 + (k & 1)], (uint32_t)(k >> 1) & 1u, a.wait_ns);
        }
    }
    tc_fence_before();
    ok = !__syncthreads_or(!ok);
    tc_fence_after();
    float* const out = a.part + (int64_t)blockIdx.x * S::NOUT;
    __syncwarp();
    if (ok) {
#pragma unroll
        for (int g = 0; g < S::MG; ++g) {
            float v[NB];
            const uint32_t taddr = tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)(g * NB);
            if constexpr (NB == 32) tmem_ld32(taddr, v);
            else tmem_ld16(taddr, v);
            const int r = g * 128 + 32 * warp + lane;   // row = tap * CIN + ci, or the first ones row
            if (mine == 0) {
#pragma unroll
                for (int n = 0; n < NB; ++n) v[n] = 0.f;
            }
            if constexpr (NB == 16) {
                if (r <= 9 * CIN) out[r] = v[0] + v[1];
            } else if (r <= 9 * CIN) {
                float4* o = reinterpret_cast<float4*>(out + (int64_t)r * NB);
#pragma unroll
                for (int q = 0; q < NB / 4; ++q) o[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    __syncwarp();
    if (warp == 0) tmem_dealloc(tmem, S::NCOL);
}

// Input features: planar FP32 [b][3][H][W] -> NHWC BF16 with 16 channels (3 used).
__global__ void k_pack_input(const float* __restrict__ feat, __nv_bfloat16* __restrict__ x, int B, int H, int W) {
    const int64_t HW = (int64_t)H * W, n = (int64_t)B * HW;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
        const int64_t b = p / HW, q = p % HW;
        __nv_bfloat16* o = x + p * 16;
        for (int c = 0; c < 16; ++c)
            o[c] = __float2bfloat16(c < 3 ? feat[(b * 3 + c) * HW + q] : 0.f);
    }
}

// Masked MSE: loss partial per block; dout = 2 mask (out - tgt) / msum, also packed as BF16
// channels (dh, dl, dh, 0 ...) with dh + dl = dout to 16 bits, the output layer's gradient input.
__global__ void __launch_bounds__(256) k_loss(const float* __restrict__ out, const float* __restrict__ tgt,
                                             const float* __restrict__ msk, int64_t n, float inv_msum,
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
        uint4* o = reinterpret_cast<uint4*>(dpk + p * 16);
        o[0] = q0;
        o[1] = make_uint4(0u, 0u, 0u, 0u);
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
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 128, S::SMEM);
    const int64_t tiles = (int64_t)a.B * a.H * ((a.W + TX - 1) / TX);
    const int grid = (int)std::min<int64_t>(tiles, (int64_t)sm_count() * (per_sm > 0 ? per_sm : 1));
    CUtensorMap m;
    std::memcpy(&m, map, sizeof m);
    kern<<<grid, 128, S::SMEM, st>>>(m, a);
}

template <int CIN, int NB>
int wgrad_launch(const void* xmap, const void* dmap, const WgradArgs& a, int max_blocks, cudaStream_t st) {
    using S = WgradShape<CIN, NB>;
    auto kern = k_wgrad_tc<CIN, NB>;
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S::SMEM);
    const int64_t tiles = (int64_t)a.B * a.H * ((a.W + TX - 1) / TX);
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(std::min<int64_t>(tiles, sm_count()), max_blocks));
    CUtensorMap xm, dm;
    std::memcpy(&xm, xmap, sizeof xm);
    std::memcpy(&dm, dmap, sizeof dm);
    kern<<<grid, 128, S::SMEM, st>>>(xm, dm, a);
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
    const cuuint64_t dims[4] = {(cuuint64_t)C, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)B};
    const cuuint64_t strides[3] = {(cuuint64_t)C * 2u, (cuuint64_t)W * C * 2u, (cuuint64_t)H * W * C * 2u};
    const cuuint32_t box[4] = {8u, (cuuint32_t)(conv_box ? PX : TX), conv_box ? 3u : 1u, 1u};
    const cuuint32_t estr[4] = {1u, 1u, 1u, 1u};
    const CUresult r = fn(&m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4u, const_cast<__nv_bfloat16*>(base), dims, strides,
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

void loss(const float* out, const float* tgt, const float* msk, int64_t n, float inv_msum, float* dout,
          __nv_bfloat16* dpk, double* part, int nblk, double* total, cudaStream_t st) {
    k_loss<<<nblk, 256, 0, st>>>(out, tgt, msk, n, inv_msum, dout, dpk, part);
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
