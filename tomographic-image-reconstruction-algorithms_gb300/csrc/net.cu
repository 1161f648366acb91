// net.cu -- the learned update network (tomo_net): parameters, forward pass,
// backward pass and Adam training step on the GPU, all with the kernels in
// cnn.cu.  Parameters are kept in FP32 (master copy) and repacked to BF16 after
// every update.
//
// Flat parameter layout (TOMO_NET_PARAMS floats):
//   W1 [9][16][32] b1 [32]   (input channels 3..15 are zero padding)
//   W2 [9][32][32] b2 [32]   W3, b3   W4, b4
//   W5 [9][32]     b5 [1]
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "internal.h"

namespace tomo {
namespace cnn {
void pack_input(const float* feat, __nv_bfloat16* x, int B, int H, int W, cudaStream_t st);
void conv32_relu(int cin, const __nv_bfloat16* in, const __nv_bfloat16* w, const float* bias, __nv_bfloat16* out, int B,
                 int H, int W, cudaStream_t st);
void conv32_dgrad(const __nv_bfloat16* dz, const __nv_bfloat16* wd, const __nv_bfloat16* mask, __nv_bfloat16* out, int B,
                  int H, int W, cudaStream_t st);
void conv_out(const __nv_bfloat16* y4, const float* w5, const float* b5, float* out, int B, int H, int W, cudaStream_t st);
void loss(const float* out, const float* tgt, const float* msk, int64_t n, float inv_msum, float* dout, double* part,
          int nblk, double* total, cudaStream_t st);
void conv_out_backward(const float* dout, const float* w5, const __nv_bfloat16* y4, __nv_bfloat16* dz4, float* part,
                       int nblk, float* grad_w5b5, int B, int H, int W, cudaStream_t st);
void conv32_wgrad(int cin, const __nv_bfloat16* x, const __nv_bfloat16* dz, float* part, int nblk, float* grad_wb, int B,
                  int H, int W, cudaStream_t st);
void adam(float* w, float* m, float* v, const float* g, int n, float lr, float b1, float b2, float eps, float c1, float c2,
          cudaStream_t st);
void pack_weights(const float* wm, int cin, __nv_bfloat16* wf, __nv_bfloat16* wd, cudaStream_t st);
}  // namespace cnn
}  // namespace tomo

using namespace tomo;

namespace {
constexpr int C = 32;
constexpr int64_t kW1 = 9 * 16 * C, kWmid = 9 * C * C, kW5 = 9 * C;
// offsets into the flat parameter vector
constexpr int64_t oW1 = 0, ob1 = oW1 + kW1;
constexpr int64_t oW2 = ob1 + C, ob2 = oW2 + kWmid;
constexpr int64_t oW3 = ob2 + C, ob3 = oW3 + kWmid;
constexpr int64_t oW4 = ob3 + C, ob4 = oW4 + kWmid;
constexpr int64_t oW5 = ob4 + C, ob5 = oW5 + kW5;
constexpr int64_t kParams = ob5 + 1;
constexpr int kPartBlocks = 304;   // 2 x 152 SMs
}  // namespace

struct tomo_net {
    int dev = 0;
    cudaStream_t st = nullptr;
    std::string err;
    float *w = nullptr, *g = nullptr, *m = nullptr, *v = nullptr;   // FP32 master, grad, Adam moments
    __nv_bfloat16 *wf1 = nullptr, *wf[3] = {}, *wd[3] = {};          // BF16 forward / data-gradient weights
    float* part = nullptr;                                            // weight-gradient partials
    double *lpart = nullptr, *ltot = nullptr;
    // activations for the current capacity (pixels)
    int64_t cap = 0;
    __nv_bfloat16 *x0 = nullptr, *y[4] = {}, *dz[2] = {};
    float *out = nullptr, *dout = nullptr, *msk_sum = nullptr;
    int64_t step = 0;
    std::vector<void*> allocs;
    ~tomo_net() {
        cudaSetDevice(dev);
        for (void* p : allocs) cudaFree(p);
        if (st) cudaStreamDestroy(st);
    }
    template <typename T>
    bool alloc(T** p, int64_t n) {
        allocs.push_back(nullptr);   // the slot first: a push_back that throws leaks no device memory
        if (cudaMalloc(&allocs.back(), sizeof(T) * (size_t)std::max<int64_t>(n, 1)) != cudaSuccess) {
            allocs.pop_back();
            cudaGetLastError();
            return false;
        }
        *p = (T*)allocs.back();
        return true;
    }
    tomo_status fail(tomo_status s, const std::string& why) {
        err = why;
        return s;
    }
    void release(void* p) {
        for (auto& a : allocs)
            if (a == p) { cudaFree(a); a = nullptr; }
    }
};

namespace {

tomo_status cuerr(tomo_net* n, cudaError_t e, const char* what) {
    if (e == cudaSuccess) return TOMO_OK;
    return n->fail(e == cudaErrorMemoryAllocation ? TOMO_ERR_OOM : TOMO_ERR_CUDA,
                   std::string(what) + ": " + cudaGetErrorString(e));
}
#define NCU(n, x)                                          \
    do {                                                   \
        const tomo_status _s = cuerr((n), (x), #x);        \
        if (_s != TOMO_OK) return _s;                      \
    } while (0)

void repack(tomo_net* n, cudaStream_t st) {
    cnn::pack_weights(n->w + oW1, 16, n->wf1, nullptr, st);
    const int64_t ow[3] = {oW2, oW3, oW4};
    for (int l = 0; l < 3; ++l) cnn::pack_weights(n->w + ow[l], C, n->wf[l], n->wd[l], st);
}

tomo_status ensure_capacity(tomo_net* n, int64_t pixels) {
    if (pixels <= n->cap) return TOMO_OK;
    for (void* p : {(void*)n->x0, (void*)n->y[0], (void*)n->y[1], (void*)n->y[2], (void*)n->y[3], (void*)n->dz[0],
                    (void*)n->dz[1], (void*)n->out, (void*)n->dout})
        if (p) n->release(p);
    bool ok = n->alloc(&n->x0, pixels * 16);
    for (int l = 0; l < 4; ++l) ok = ok && n->alloc(&n->y[l], pixels * C);
    ok = ok && n->alloc(&n->dz[0], pixels * C) && n->alloc(&n->dz[1], pixels * C);
    ok = ok && n->alloc(&n->out, pixels) && n->alloc(&n->dout, pixels);
    if (!ok) return n->fail(TOMO_ERR_OOM, "network activations do not fit");
    n->cap = pixels;
    return TOMO_OK;
}

tomo_status check_shape(tomo_net* n, int B, int H, int W) {
    if (B < 1 || H < 1 || W < 64 || W % 64 != 0) return n->fail(TOMO_ERR_ARG, "images must be W % 64 == 0 wide");
    return ensure_capacity(n, (int64_t)B * H * W);
}

void forward(tomo_net* n, const float* feat, int B, int H, int W, float* out, cudaStream_t st) {
    cnn::pack_input(feat, n->x0, B, H, W, st);
    cnn::conv32_relu(16, n->x0, n->wf1, n->w + ob1, n->y[0], B, H, W, st);
    cnn::conv32_relu(C, n->y[0], n->wf[0], n->w + ob2, n->y[1], B, H, W, st);
    cnn::conv32_relu(C, n->y[1], n->wf[1], n->w + ob3, n->y[2], B, H, W, st);
    cnn::conv32_relu(C, n->y[2], n->wf[2], n->w + ob4, n->y[3], B, H, W, st);
    cnn::conv_out(n->y[3], n->w + oW5, n->w + ob5, out, B, H, W, st);
}

// loss and gradient into n->g
tomo_status backward(tomo_net* n, const float* feat, const float* tgt, const float* msk, int B, int H, int W,
                     double* loss_out) {
    cudaStream_t st = n->st;
    const int64_t P = (int64_t)B * H * W;
    // mask sum on the host (the mask is a small input)
    std::vector<float> hm(P);
    NCU(n, cudaMemcpyAsync(hm.data(), msk, sizeof(float) * P, cudaMemcpyDeviceToHost, st));
    NCU(n, cudaStreamSynchronize(st));
    double ms = 0.0;
    for (float x : hm) ms += x;
    if (!(ms > 0.0)) return n->fail(TOMO_ERR_ARG, "mask is empty");
    forward(n, feat, B, H, W, n->out, st);
    cnn::loss(n->out, tgt, msk, P, (float)(1.0 / ms), n->dout, n->lpart, kPartBlocks, n->ltot, st);
    cnn::conv_out_backward(n->dout, n->w + oW5, n->y[3], n->dz[0], n->part, kPartBlocks, n->g + oW5, B, H, W, st);
    // layers 4, 3, 2: weight gradient, then data gradient masked by the layer input's ReLU
    const int64_t ow[3] = {oW2, oW3, oW4};
    int cur = 0;
    for (int l = 2; l >= 0; --l) {   // l = index of layers 2..4 in wf/wd; input activation y[l]
        cnn::conv32_wgrad(C, n->y[l], n->dz[cur], n->part, kPartBlocks, n->g + ow[l], B, H, W, st);
        cnn::conv32_dgrad(n->dz[cur], n->wd[l], n->y[l], n->dz[1 - cur], B, H, W, st);
        cur = 1 - cur;
    }
    cnn::conv32_wgrad(16, n->x0, n->dz[cur], n->part, kPartBlocks, n->g + oW1, B, H, W, st);
    double l = 0.0;
    NCU(n, cudaMemcpyAsync(&l, n->ltot, sizeof(double), cudaMemcpyDeviceToHost, st));
    NCU(n, cudaStreamSynchronize(st));
    NCU(n, cudaGetLastError());
    if (loss_out) *loss_out = l / ms;
    return TOMO_OK;
}

}  // namespace

// ---- internal use by the engine (learned iteration) ------------------------------------
namespace tomo {
tomo_status net_infer(tomo_net* n, const float* feat, int H, int W, float* out, void* stream) {
    tomo_status s = check_shape(n, 1, H, W);
    if (s != TOMO_OK) return s;
    forward(n, feat, 1, H, W, out, (cudaStream_t)stream);
    return TOMO_OK;
}
}  // namespace tomo

// ---- C ABI -----------------------------------------------------------------------------
// Entry points that can allocate on the host are function-try-blocks: a C++ exception below
// them becomes a status (abi_exception) and never crosses the C ABI.
extern "C" {

int64_t tomo_net_num_params(void) { return kParams; }

tomo_status tomo_net_create(int32_t device, uint64_t seed, tomo_net** out) try {
    if (!out) return TOMO_ERR_ARG;
    *out = nullptr;
    std::unique_ptr<tomo_net> n(new (std::nothrow) tomo_net());   // freed on every early return
    if (!n) return TOMO_ERR_OOM;
    n->dev = device;
    if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&n->st, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        return TOMO_ERR_CUDA;
    }
    bool ok = n->alloc(&n->w, kParams) && n->alloc(&n->g, kParams) && n->alloc(&n->m, kParams) &&
              n->alloc(&n->v, kParams) && n->alloc(&n->wf1, kW1);
    for (int l = 0; l < 3; ++l) ok = ok && n->alloc(&n->wf[l], kWmid) && n->alloc(&n->wd[l], kWmid);
    ok = ok && n->alloc(&n->part, (int64_t)kPartBlocks * (kWmid + C)) && n->alloc(&n->lpart, kPartBlocks) &&
         n->alloc(&n->ltot, 1);
    if (!ok) return TOMO_ERR_OOM;
    // He-normal initialisation for the ReLU layers, small output layer, zero biases
    std::vector<float> h(kParams, 0.f);
    Rng rng(seed);
    auto fill = [&](int64_t off, int64_t cnt, double fan_in, double gain, int cin_used, int cin) {
        const double sd = gain * std::sqrt(2.0 / fan_in);
        for (int64_t e = 0; e < cnt; ++e) {
            const int ci = (int)((e / C) % cin);
            h[off + e] = ci < cin_used ? (float)(sd * rng.normal()) : 0.f;
        }
    };
    fill(oW1, kW1, 9.0 * 3, 1.0, 3, 16);
    fill(oW2, kWmid, 9.0 * C, 1.0, C, C);
    fill(oW3, kWmid, 9.0 * C, 1.0, C, C);
    fill(oW4, kWmid, 9.0 * C, 1.0, C, C);
    for (int64_t e = 0; e < kW5; ++e) h[oW5 + e] = (float)(0.01 * std::sqrt(1.0 / (9.0 * C)) * rng.normal());
    if (cudaMemcpy(n->w, h.data(), sizeof(float) * kParams, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemset(n->m, 0, sizeof(float) * kParams) != cudaSuccess ||
        cudaMemset(n->v, 0, sizeof(float) * kParams) != cudaSuccess) {
        cudaGetLastError();
        return TOMO_ERR_CUDA;
    }
    repack(n.get(), n->st);
    if (cudaStreamSynchronize(n->st) != cudaSuccess) { cudaGetLastError(); return TOMO_ERR_CUDA; }
    *out = n.release();
    return TOMO_OK;
} catch (...) {
    return abi_exception(nullptr);
}

void tomo_net_destroy(tomo_net* n) { delete n; }

const char* tomo_net_last_error(const tomo_net* n) { return n ? n->err.c_str() : ""; }

tomo_status tomo_net_get_params(tomo_net* n, float* host) try {
    if (!n || !host) return TOMO_ERR_ARG;
    cudaSetDevice(n->dev);
    NCU(n, cudaMemcpy(host, n->w, sizeof(float) * kParams, cudaMemcpyDeviceToHost));
    return TOMO_OK;
} catch (...) {
    return abi_exception(n ? &n->err : nullptr);
}

tomo_status tomo_net_set_params(tomo_net* n, const float* host) try {
    if (!n || !host) return TOMO_ERR_ARG;
    cudaSetDevice(n->dev);
    NCU(n, cudaMemcpy(n->w, host, sizeof(float) * kParams, cudaMemcpyHostToDevice));
    NCU(n, cudaMemset(n->m, 0, sizeof(float) * kParams));
    NCU(n, cudaMemset(n->v, 0, sizeof(float) * kParams));
    n->step = 0;
    repack(n, n->st);
    NCU(n, cudaStreamSynchronize(n->st));
    return TOMO_OK;
} catch (...) {
    return abi_exception(n ? &n->err : nullptr);
}

tomo_status tomo_net_forward_device(tomo_net* n, const float* d_feat, int32_t B, int32_t H, int32_t W, float* d_out) try {
    if (!n || !d_feat || !d_out) return TOMO_ERR_ARG;
    cudaSetDevice(n->dev);
    tomo_status s = check_shape(n, B, H, W);
    if (s != TOMO_OK) return s;
    forward(n, d_feat, B, H, W, d_out, n->st);
    NCU(n, cudaStreamSynchronize(n->st));
    NCU(n, cudaGetLastError());
    return TOMO_OK;
} catch (...) {
    return abi_exception(n ? &n->err : nullptr);
}

tomo_status tomo_net_grad_device(tomo_net* n, const float* d_feat, const float* d_target, const float* d_mask, int32_t B,
                                 int32_t H, int32_t W, float* host_grad, double* loss) try {
    if (!n || !d_feat || !d_target || !d_mask) return TOMO_ERR_ARG;
    cudaSetDevice(n->dev);
    tomo_status s = check_shape(n, B, H, W);
    if (s != TOMO_OK) return s;
    if ((s = backward(n, d_feat, d_target, d_mask, B, H, W, loss)) != TOMO_OK) return s;
    if (host_grad) NCU(n, cudaMemcpy(host_grad, n->g, sizeof(float) * kParams, cudaMemcpyDeviceToHost));
    return TOMO_OK;
} catch (...) {
    return abi_exception(n ? &n->err : nullptr);
}

tomo_status tomo_net_train_step_device(tomo_net* n, const float* d_feat, const float* d_target, const float* d_mask,
                                       int32_t B, int32_t H, int32_t W, float lr, double* loss) try {
    if (!n || !d_feat || !d_target || !d_mask || !(lr > 0.f)) return TOMO_ERR_ARG;
    cudaSetDevice(n->dev);
    tomo_status s = check_shape(n, B, H, W);
    if (s != TOMO_OK) return s;
    if ((s = backward(n, d_feat, d_target, d_mask, B, H, W, loss)) != TOMO_OK) return s;
    ++n->step;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = (float)(1.0 / (1.0 - std::pow((double)b1, (double)n->step)));
    const float c2 = (float)(1.0 / (1.0 - std::pow((double)b2, (double)n->step)));
    cnn::adam(n->w, n->m, n->v, n->g, (int)kParams, lr, b1, b2, 1e-8f, c1, c2, n->st);
    repack(n, n->st);
    NCU(n, cudaStreamSynchronize(n->st));
    NCU(n, cudaGetLastError());
    return TOMO_OK;
} catch (...) {
    return abi_exception(n ? &n->err : nullptr);
}

tomo_status tomo_net_save(tomo_net* n, const char* path) try {
    if (!n || !path) return TOMO_ERR_ARG;
    std::vector<float> h(kParams);
    tomo_status s = tomo_net_get_params(n, h.data());
    if (s != TOMO_OK) return s;
    FILE* f = std::fopen(path, "wb");
    if (!f) return n->fail(TOMO_ERR_IO, std::string("cannot write ") + path);
    const char magic[8] = {'T', 'O', 'M', 'O', 'N', 'E', 'T', '1'};
    const int64_t cnt = kParams;
    bool ok = std::fwrite(magic, 1, 8, f) == 8 && std::fwrite(&cnt, sizeof cnt, 1, f) == 1 &&
              std::fwrite(h.data(), sizeof(float), h.size(), f) == h.size();
    ok = (std::fclose(f) == 0) && ok;
    return ok ? TOMO_OK : n->fail(TOMO_ERR_IO, "short write");
} catch (...) {
    return abi_exception(n ? &n->err : nullptr);
}

tomo_status tomo_net_load(tomo_net* n, const char* path) try {
    if (!n || !path) return TOMO_ERR_ARG;
    std::vector<float> h(kParams);   // before the file is opened: a throwing allocation leaks no FILE
    FILE* f = std::fopen(path, "rb");
    if (!f) return n->fail(TOMO_ERR_IO, std::string("cannot read ") + path);
    char magic[8];
    int64_t cnt = 0;
    const bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, "TOMONET1", 8) == 0 &&
                    std::fread(&cnt, sizeof cnt, 1, f) == 1 && cnt == kParams &&
                    std::fread(h.data(), sizeof(float), h.size(), f) == h.size();
    std::fclose(f);
    if (!ok) return n->fail(TOMO_ERR_IO, "not a network parameter file");
    return tomo_net_set_params(n, h.data());
} catch (...) {
    return abi_exception(n ? &n->err : nullptr);
}

}  // extern "C"
