// cnn.cu -- kernels of the learned update network: a 5-layer 3x3 CNN with
// 32 channels, ReLU, BF16 weights and activations, FP32 accumulation.
//
//   layer 1: 16 -> 32 (3 input features f, SIRT direction, illumination,
//            zero-padded to 16 channels), bias, ReLU
//   layers 2-4: 32 -> 32, bias, ReLU
//   layer 5: 32 -> 1, bias, FP32 output (the proposed field update)
//
// Activations are NHWC BF16 ([image][y][x][channel]); images are W % 64 == 0
// wide.  The 32-output-channel convolutions are implicit GEMMs on the tensor
// cores (mma.sync m16n8k16 BF16, FP32 accumulators): a block takes 64 pixels of
// one row and all 32 output channels, stages the 3 x 66 pixel input patch and
// the layer's weights in shared memory, and each warp runs the 9 taps x (Cin/16)
// K-steps for its 16 pixels.  The same kernel computes the data gradient of a
// layer (input: the output gradient, weights rotated by 180 degrees with input
// and output channels swapped; epilogue: the next layer's ReLU mask).  The
// weight gradient is a GEMM over pixels with per-block partial sums reduced in
// fixed order, so training steps are deterministic.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "internal.h"

namespace tomo {
namespace cnn {
namespace {

constexpr int TILE_X = 64;     // pixels per block
constexpr int PATCH = TILE_X + 2;
constexpr int COUT = 32;

__device__ __forceinline__ uint32_t pack2(__nv_bfloat16 a, __nv_bfloat16 b) {
    return (uint32_t)__bfloat16_as_ushort(a) | ((uint32_t)__bfloat16_as_ushort(b) << 16);
}

__device__ __forceinline__ void mma16816(float c[4], const uint32_t a[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Epilogue modes of the convolution kernel.
enum { EPI_RELU = 0, EPI_MASK = 1 };

// out[b][y][x][co] = epi( sum_{tap, ci} in[b][y+dy-1][x+dx-1][ci] * w[tap][co][ci] (+ bias[co]) )
// EPI_RELU: + bias, max(0, .);  EPI_MASK: * (mask[b][y][x][co] > 0)  (no bias)
// CIN in {16, 32}; w is [9][32][CIN] BF16 (ci fastest).
template <int CIN, int EPI>
__global__ void __launch_bounds__(128) k_conv32(const __nv_bfloat16* __restrict__ in, const __nv_bfloat16* __restrict__ w,
                                               const float* __restrict__ bias, const __nv_bfloat16* __restrict__ mask,
                                               __nv_bfloat16* __restrict__ out, int H, int W) {
    constexpr int CS = CIN + 8;   // padded channel stride in shared memory (halves)
    __shared__ __align__(16) __nv_bfloat16 patch[3][PATCH][CS];
    __shared__ __align__(16) __nv_bfloat16 ws[9][COUT][CS];
    const int x0 = blockIdx.x * TILE_X, y = blockIdx.y, b = blockIdx.z;
    const int tid = threadIdx.x;
    // stage the input patch (zero outside the image) and the weights
    for (int e = tid; e < 3 * PATCH * (CIN / 2); e += 128) {
        const int c2 = e % (CIN / 2), px = (e / (CIN / 2)) % PATCH, r = e / (CIN / 2) / PATCH;
        const int yy = y + r - 1, xx = x0 + px - 1;
        uint32_t v = 0;
        if (yy >= 0 && yy < H && xx >= 0 && xx < W)
            v = *reinterpret_cast<const uint32_t*>(in + (((int64_t)b * H + yy) * W + xx) * CIN + 2 * c2);
        *reinterpret_cast<uint32_t*>(&patch[r][px][2 * c2]) = v;
    }
    for (int e = tid; e < 9 * COUT * (CIN / 2); e += 128) {
        const int c2 = e % (CIN / 2), co = (e / (CIN / 2)) % COUT, tap = e / (CIN / 2) / COUT;
        *reinterpret_cast<uint32_t*>(&ws[tap][co][2 * c2]) =
            *reinterpret_cast<const uint32_t*>(w + ((int64_t)tap * COUT + co) * CIN + 2 * c2);
    }
    __syncthreads();
    const int lane = tid & 31, warp = tid >> 5, g = lane >> 2, t = lane & 3;
    float acc[4][4] = {};
    const int p0 = warp * 16;   // first pixel of this warp within the tile
#pragma unroll
    for (int tap = 0; tap < 9; ++tap) {
        const int dy = tap / 3, dx = tap % 3;
#pragma unroll
        for (int kc = 0; kc < CIN / 16; ++kc) {
            const int k0 = kc * 16 + 2 * t;
            uint32_t a[4];
            a[0] = *reinterpret_cast<const uint32_t*>(&patch[dy][p0 + g + dx][k0]);
            a[1] = *reinterpret_cast<const uint32_t*>(&patch[dy][p0 + g + 8 + dx][k0]);
            a[2] = *reinterpret_cast<const uint32_t*>(&patch[dy][p0 + g + dx][k0 + 8]);
            a[3] = *reinterpret_cast<const uint32_t*>(&patch[dy][p0 + g + 8 + dx][k0 + 8]);
#pragma unroll
            for (int nt = 0; nt < 4; ++nt) {
                const uint32_t b0 = *reinterpret_cast<const uint32_t*>(&ws[tap][nt * 8 + g][k0]);
                const uint32_t b1 = *reinterpret_cast<const uint32_t*>(&ws[tap][nt * 8 + g][k0 + 8]);
                mma16816(acc[nt], a, b0, b1);
            }
        }
    }
    // epilogue: rows g and g+8 of the warp's 16 pixels, columns nt*8 + 2t, +1
#pragma unroll
    for (int half = 0; half < 2; ++half) {
        const int x = x0 + p0 + g + 8 * half;
        const int64_t base = (((int64_t)b * H + y) * W + x) * COUT;
#pragma unroll
        for (int nt = 0; nt < 4; ++nt) {
            const int co = nt * 8 + 2 * t;
            float v0 = acc[nt][2 * half], v1 = acc[nt][2 * half + 1];
            if (EPI == EPI_RELU) {
                v0 = fmaxf(v0 + bias[co], 0.f);
                v1 = fmaxf(v1 + bias[co + 1], 0.f);
            } else {
                const __nv_bfloat162 m = *reinterpret_cast<const __nv_bfloat162*>(mask + base + co);
                if (!(__bfloat162float(m.x) > 0.f)) v0 = 0.f;
                if (!(__bfloat162float(m.y) > 0.f)) v1 = 0.f;
            }
            *reinterpret_cast<uint32_t*>(out + base + co) = pack2(__float2bfloat16(v0), __float2bfloat16(v1));
        }
    }
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

// Layer 5 forward: out[p] = b5 + sum_{tap, ci} y4[p + off(tap)][ci] * w5[tap][ci] (FP32, taps
// then channels in order).  One block row per image row (blockIdx.y = b*H + y), one thread per
// pixel, 16-byte loads of 8 channels, the 288 weights in shared memory.
__global__ void __launch_bounds__(128) k_conv_out(const __nv_bfloat16* __restrict__ y4, const float* __restrict__ w5,
                                                  const float* __restrict__ b5, float* __restrict__ out, int B, int H,
                                                  int W) {
    __shared__ float ws[9 * COUT];
    for (int j = threadIdx.x; j < 9 * COUT; j += blockDim.x) ws[j] = w5[j];
    __syncthreads();
    const int row = blockIdx.y, b = row / H, y = row - b * H;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= W) return;
    float acc = b5[0];
    for (int tap = 0; tap < 9; ++tap) {
        const int yy = y + tap / 3 - 1, xx = x + tap % 3 - 1;
        if (yy < 0 || yy >= H || xx < 0 || xx >= W) continue;
        const uint4* v = reinterpret_cast<const uint4*>(y4 + ((int64_t)(b * H + yy) * W + xx) * COUT);
#pragma unroll
        for (int q = 0; q < COUT / 8; ++q) {
            const uint4 u = v[q];
            const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&u);
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const float2 f = __bfloat1622float2(h[k]);
                acc = fmaf(f.x, ws[tap * COUT + q * 8 + 2 * k], acc);
                acc = fmaf(f.y, ws[tap * COUT + q * 8 + 2 * k + 1], acc);
            }
        }
    }
    out[(int64_t)row * W + x] = acc;
}

// Masked MSE: loss partial per block, dout = 2 mask (out - tgt) / msum.
__global__ void __launch_bounds__(256) k_loss(const float* __restrict__ out, const float* __restrict__ tgt,
                                             const float* __restrict__ msk, int64_t n, float inv_msum,
                                             float* __restrict__ dout, double* __restrict__ part) {
    double acc = 0.0;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
        const float e = (out[p] - tgt[p]) * msk[p];
        acc += (double)e * e;
        dout[p] = 2.f * e * inv_msum;
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

// Layer 5 backward: dz4[p][ci] = (y4 > 0) * sum_tap dout[p - off(tap)] * w5[tap][ci]
__global__ void k_conv_out_dgrad(const float* __restrict__ dout, const float* __restrict__ w5,
                                 const __nv_bfloat16* __restrict__ y4, __nv_bfloat16* __restrict__ dz4, int B, int H,
                                 int W) {
    const int64_t HW = (int64_t)H * W, n = (int64_t)B * HW * COUT;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
        const int ci = (int)(e % COUT);
        const int64_t p = e / COUT, b = p / HW;
        const int y = (int)((p % HW) / W), x = (int)(p % W);
        float acc = 0.f;
        for (int tap = 0; tap < 9; ++tap) {
            const int yy = y - (tap / 3 - 1), xx = x - (tap % 3 - 1);
            if (yy < 0 || yy >= H || xx < 0 || xx >= W) continue;
            acc = fmaf(dout[(b * H + yy) * W + xx], w5[tap * COUT + ci], acc);
        }
        dz4[e] = __float2bfloat16(__bfloat162float(y4[e]) > 0.f ? acc : 0.f);
    }
}

// Layer 5 weight gradient partials: part[blk][tap*32+ci] and part[blk][288] (bias), each
// block a grid-stride share of the image rows, pixels in order within a row; thread j =
// tap*32 + ci reads one channel of the shifted row (a warp reads 64 contiguous bytes).
__global__ void __launch_bounds__(COUT * 9) k_conv_out_wgrad(const float* __restrict__ dout,
                                                           const __nv_bfloat16* __restrict__ y4, int B, int H, int W,
                                                           float* __restrict__ part) {
    const int j = threadIdx.x;   // tap*32 + ci
    const int tap = j / COUT, ci = j % COUT;
    const int dy = tap / 3 - 1, dx = tap % 3 - 1;
    const bool centre = tap == 4;               // covers every pixel: it also sums the bias gradient
    const int xa = dx < 0 ? 1 : 0, xb = dx > 0 ? W - 1 : W;
    float acc = 0.f, accb = 0.f;
    for (int row = blockIdx.x; row < B * H; row += gridDim.x) {
        const int b = row / H, yy = row - b * H + dy;
        if (yy < 0 || yy >= H) continue;
        const float* d = dout + (int64_t)row * W;
        const __nv_bfloat16* src = y4 + (int64_t)(b * H + yy) * W * COUT + ci;
        for (int x = xa; x < xb; ++x) {
            const float dv = d[x];
            acc = fmaf(dv, __bfloat162float(src[(int64_t)(x + dx) * COUT]), acc);
            if (centre) accb += dv;
        }
    }
    part[(int64_t)blockIdx.x * (9 * COUT + 1) + j] = acc;
    if (tap == 4 && ci == 0) part[(int64_t)blockIdx.x * (9 * COUT + 1) + 9 * COUT] = accb;
}

// Weight gradient of a 32-output-channel layer as a GEMM over pixels:
// dW[tap][ci][co] = sum_p x[p + off(tap)][ci] * dz[p][co],  db[co] = sum_p dz[p][co].
// Each block takes a grid-stride share of the 64-pixel row segments; the warps
// split the 9 x (CIN/16) x 4 (tap, ci-tile, co-tile) output tiles and keep them in
// registers; the block writes one partial per output, reduced later in fixed order.
template <int CIN>
__global__ void __launch_bounds__(128) k_conv_wgrad(const __nv_bfloat16* __restrict__ x, const __nv_bfloat16* __restrict__ dz,
                                                   int B, int H, int W, float* __restrict__ part) {
    constexpr int CS = CIN + 8, DS = COUT + 8;
    constexpr int TILES = 9 * (CIN / 16) * 4, PER_WARP = TILES / 4;
    constexpr int NOUT = 9 * CIN * COUT + COUT;
    __shared__ __align__(16) __nv_bfloat16 patch[3][PATCH][CS];
    __shared__ __align__(16) __nv_bfloat16 dzs[TILE_X][DS];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, g = lane >> 2, t = lane & 3;
    float acc[PER_WARP][4] = {};
    float accb = 0.f;
    const int segs_x = W / TILE_X;
    const int64_t nseg = (int64_t)B * H * segs_x;
    for (int64_t sgi = blockIdx.x; sgi < nseg; sgi += gridDim.x) {
        const int xs = (int)(sgi % segs_x), y = (int)((sgi / segs_x) % H);
        const int64_t b = sgi / segs_x / H;
        const int x0 = xs * TILE_X;
        __syncthreads();
        for (int e = tid; e < 3 * PATCH * (CIN / 2); e += 128) {
            const int c2 = e % (CIN / 2), px = (e / (CIN / 2)) % PATCH, r = e / (CIN / 2) / PATCH;
            const int yy = y + r - 1, xx = x0 + px - 1;
            uint32_t v = 0;
            if (yy >= 0 && yy < H && xx >= 0 && xx < W)
                v = *reinterpret_cast<const uint32_t*>(x + ((b * H + yy) * W + xx) * CIN + 2 * c2);
            *reinterpret_cast<uint32_t*>(&patch[r][px][2 * c2]) = v;
        }
        for (int e = tid; e < TILE_X * (COUT / 2); e += 128) {
            const int c2 = e % (COUT / 2), px = e / (COUT / 2);
            *reinterpret_cast<uint32_t*>(&dzs[px][2 * c2]) =
                *reinterpret_cast<const uint32_t*>(dz + ((b * H + y) * W + x0 + px) * COUT + 2 * c2);
        }
        __syncthreads();
        if (tid < COUT)
            for (int px = 0; px < TILE_X; ++px) accb += __bfloat162float(dzs[px][tid]);
#pragma unroll
        for (int ks = 0; ks < TILE_X / 16; ++ks) {
            const int pk = ks * 16 + 2 * t;   // pixels pk, pk+1 (and +8, +9)
#pragma unroll
            for (int j = 0; j < PER_WARP; ++j) {
                const int tile = warp + 4 * j;
                const int nt = tile % 4, mt = (tile / 4) % (CIN / 16), tap = tile / 4 / (CIN / 16);
                const int dy = tap / 3, dx = tap % 3, c0 = mt * 16 + g;
                uint32_t a[4];
                a[0] = pack2(patch[dy][pk + dx][c0], patch[dy][pk + 1 + dx][c0]);
                a[1] = pack2(patch[dy][pk + dx][c0 + 8], patch[dy][pk + 1 + dx][c0 + 8]);
                a[2] = pack2(patch[dy][pk + 8 + dx][c0], patch[dy][pk + 9 + dx][c0]);
                a[3] = pack2(patch[dy][pk + 8 + dx][c0 + 8], patch[dy][pk + 9 + dx][c0 + 8]);
                const int n = nt * 8 + g;
                const uint32_t b0 = pack2(dzs[pk][n], dzs[pk + 1][n]);
                const uint32_t b1 = pack2(dzs[pk + 8][n], dzs[pk + 9][n]);
                mma16816(acc[j], a, b0, b1);
            }
        }
    }
    float* out = part + (int64_t)blockIdx.x * NOUT;
#pragma unroll
    for (int j = 0; j < PER_WARP; ++j) {
        const int tile = warp + 4 * j;
        const int nt = tile % 4, mt = (tile / 4) % (CIN / 16), tap = tile / 4 / (CIN / 16);
        const int ci = mt * 16 + g, co = nt * 8 + 2 * t;
        out[(tap * CIN + ci) * COUT + co] = acc[j][0];
        out[(tap * CIN + ci) * COUT + co + 1] = acc[j][1];
        out[(tap * CIN + ci + 8) * COUT + co] = acc[j][2];
        out[(tap * CIN + ci + 8) * COUT + co + 1] = acc[j][3];
    }
    if (tid < COUT) out[9 * CIN * COUT + tid] = accb;
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

// Master W[tap][ci][co] -> forward layout [tap][co][ci] and data-gradient layout
// [8 - tap][ci][co] (rotated taps; the data-gradient kernel reads co as its input
// channel and writes ci), both BF16.
__global__ void k_pack_weights(const float* __restrict__ wm, int cin, __nv_bfloat16* __restrict__ wf,
                               __nv_bfloat16* __restrict__ wd) {
    const int n = 9 * cin * COUT;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
        const int co = e % COUT, ci = (e / COUT) % cin, tap = e / COUT / cin;
        const __nv_bfloat16 v = __float2bfloat16(wm[e]);
        wf[(tap * COUT + co) * cin + ci] = v;
        if (wd) wd[((8 - tap) * cin + ci) * COUT + co] = v;
    }
}

inline int blocks_for(int64_t n, int t) {
    const int64_t b = (n + t - 1) / t;
    return (int)(b < 2048 ? (b < 1 ? 1 : b) : 2048);
}

}  // namespace

// ---- launchers -------------------------------------------------------------------
void pack_input(const float* feat, __nv_bfloat16* x, int B, int H, int W, cudaStream_t st) {
    k_pack_input<<<blocks_for((int64_t)B * H * W, 256), 256, 0, st>>>(feat, x, B, H, W);
}

void conv32_relu(int cin, const __nv_bfloat16* in, const __nv_bfloat16* w, const float* bias, __nv_bfloat16* out, int B,
                 int H, int W, cudaStream_t st) {
    const dim3 grid(W / TILE_X, H, B);
    if (cin == 16) k_conv32<16, EPI_RELU><<<grid, 128, 0, st>>>(in, w, bias, nullptr, out, H, W);
    else k_conv32<32, EPI_RELU><<<grid, 128, 0, st>>>(in, w, bias, nullptr, out, H, W);
}

void conv32_dgrad(const __nv_bfloat16* dz, const __nv_bfloat16* wd, const __nv_bfloat16* mask, __nv_bfloat16* out, int B,
                  int H, int W, cudaStream_t st) {
    k_conv32<32, EPI_MASK><<<dim3(W / TILE_X, H, B), 128, 0, st>>>(dz, wd, nullptr, mask, out, H, W);
}

void conv_out(const __nv_bfloat16* y4, const float* w5, const float* b5, float* out, int B, int H, int W, cudaStream_t st) {
    k_conv_out<<<dim3((W + 127) / 128, B * H), 128, 0, st>>>(y4, w5, b5, out, B, H, W);
}

void loss(const float* out, const float* tgt, const float* msk, int64_t n, float inv_msum, float* dout, double* part,
          int nblk, double* total, cudaStream_t st) {
    k_loss<<<nblk, 256, 0, st>>>(out, tgt, msk, n, inv_msum, dout, part);
    k_sum_double<<<1, 32, 0, st>>>(part, nblk, total);
}

void conv_out_backward(const float* dout, const float* w5, const __nv_bfloat16* y4, __nv_bfloat16* dz4, float* part, int nblk,
                       float* grad_w5b5, int B, int H, int W, cudaStream_t st) {
    k_conv_out_dgrad<<<blocks_for((int64_t)B * H * W * COUT, 256), 256, 0, st>>>(dout, w5, y4, dz4, B, H, W);
    k_conv_out_wgrad<<<nblk, 9 * COUT, 0, st>>>(dout, y4, B, H, W, part);
    k_reduce_parts<<<2, 160, 0, st>>>(part, nblk, 9 * COUT + 1, grad_w5b5);
}

void conv32_wgrad(int cin, const __nv_bfloat16* x, const __nv_bfloat16* dz, float* part, int nblk, float* grad_wb, int B,
                  int H, int W, cudaStream_t st) {
    const int nout = 9 * cin * COUT + COUT;
    if (cin == 16) k_conv_wgrad<16><<<nblk, 128, 0, st>>>(x, dz, B, H, W, part);
    else k_conv_wgrad<32><<<nblk, 128, 0, st>>>(x, dz, B, H, W, part);
    k_reduce_parts<<<blocks_for(nout, 256), 256, 0, st>>>(part, nblk, nout, grad_wb);
}

void adam(float* w, float* m, float* v, const float* g, int n, float lr, float b1, float b2, float eps, float c1, float c2,
          cudaStream_t st) {
    k_adam<<<blocks_for(n, 256), 256, 0, st>>>(w, m, v, g, n, lr, b1, b2, eps, c1, c2);
}

void pack_weights(const float* wm, int cin, __nv_bfloat16* wf, __nv_bfloat16* wd, cudaStream_t st) {
    k_pack_weights<<<blocks_for(9 * cin * COUT, 256), 256, 0, st>>>(wm, cin, wf, wd);
}

}  // namespace cnn
}  // namespace tomo
