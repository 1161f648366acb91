// cnn.h -- launchers of the learned update network's kernels (cnn.cu), used by net.cu.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace tomo {
namespace cnn {

// Convolutions on the tensor cores: the layer they compute and their epilogue.
enum ConvKind {
    CONV_IN,          // 16 -> 32 channels, bias, ReLU (layer 1)
    CONV_MID,         // 32 -> 32 channels, bias, ReLU (layers 2-4)
    CONV_DGRAD,       // data gradient of a 32 -> 32 layer, masked by the layer input's ReLU
    CONV_OUT,         // 32 -> 1 channel, bias, FP32 output (layer 5)
    CONV_OUT_DGRAD,   // data gradient of layer 5 from the packed loss gradient, ReLU mask
};
// Weight gradients on the tensor cores: layer 1 (16 input channels), layers 2-4, layer 5.
enum WgradKind { WGRAD_IN, WGRAD_MID, WGRAD_OUT };

// Activations are BF16 in a channel-blocked layout [B][H][C / 8][W][8]: each 8-channel chunk of
// an image row is W x 16 contiguous bytes.
// TMA map of an activation (C % 8 == 0): boxes of one row, every chunk, 130 pixels (convolution
// input: one halo pixel each side) or 128 pixels (weight-gradient operand); false when the
// driver has no encoder or refuses the map.
bool encode_act_map(unsigned char out[128], const __nv_bfloat16* base, int C, int B, int H, int W, bool conv_box);

void pack_input(const float* feat, __nv_bfloat16* x, int B, int H, int W, cudaStream_t st);
// out = conv(in) with the packed weights w (pack_weights / pack_out_weights layouts); a timed-out
// wait sets bit 1 of *err (host-visible).
void conv(ConvKind kind, const void* in_map, const __nv_bfloat16* w, const float* bias, const __nv_bfloat16* mask,
          void* out, int B, int H, int W, unsigned int* err, uint64_t wait_ns, cudaStream_t st);
// grad = weight and bias gradient of a layer from its input (x_map) and output gradient (d_map),
// through per-block partials in part (at most max_blocks rows) reduced in fixed order.
void wgrad(WgradKind kind, const void* x_map, const void* d_map, float* part, int max_blocks, float* grad, int B, int H,
           int W, unsigned int* err, uint64_t wait_ns, cudaStream_t st);
// masked MSE: dout (FP32) and its packed BF16 form dpk (16 channels, blocked) = (dh, dl, dh, 0 ...);
// the loss sum in *total
void loss(const float* out, const float* tgt, const float* msk, int64_t n, int W, float inv_msum, float* dout,
          __nv_bfloat16* dpk, double* part, int nblk, double* total, cudaStream_t st);
void adam(float* w, float* m, float* v, const float* g, int n, float lr, float b1, float b2, float eps, float c1, float c2,
          cudaStream_t st);
// master W[9][cin][32] -> convolution operand wf and (cin == 32) data-gradient operand wd
void pack_weights(const float* wm, int cin, __nv_bfloat16* wf, __nv_bfloat16* wd, cudaStream_t st);
// master W5[9][32] -> output-layer operands (BF16 high and low parts): forward wo, data gradient wod
void pack_out_weights(const float* w5, __nv_bfloat16* wo, __nv_bfloat16* wod, cudaStream_t st);

}  // namespace cnn
}  // namespace tomo
