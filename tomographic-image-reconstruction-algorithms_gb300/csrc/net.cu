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

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "cnn.h"
#include "internal.h"

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
    // BF16 tensor-core operands: forward and data-gradient weights of layers 1-4, output layer
    __nv_bfloat16 *wf1 = nullptr, *wf[3] = {}, *wd[3] = {}, *wo = nullptr, *wod = nullptr;
    float* part = nullptr;                                            // weight-gradient partials
    double *lpart = nullptr, *ltot = nullptr;
    // error word of the kernels' bounded waits (mapped host memory: host and device addresses)
    unsigned int *errh = nullptr, *errd = nullptr;
    uint64_t wait_ns = 1000000000ull;                                 // TOMO_WAIT_LIMIT_NS
    // activations for the current capacity (pixels); dpk = packed loss gradient [P][16]
    int64_t cap = 0;
    __nv_bfloat16 *x0 = nullptr, *y[4] = {}, *dz[2] = {}, *dpk = nullptr;
    float *out = nullptr, *dout = nullptr, *msk_sum = nullptr;
    // TMA maps of the activations for shape (mB, mH, mW): convolution-input boxes and
    // weight-gradient boxes
    enum { M_X0, M_Y0, M_Y1, M_Y2, M_Y3, M_DZ0, M_DZ1, M_DPK, NMAPS };
    alignas(64) unsigned char cmap[NMAPS][128];
    alignas(64) unsigned char wmap[NMAPS][128];
    int mB = 0, mH = 0, mW = 0;
    int64_t step = 0;
    std::vector<void*> allocs;
    ~tomo_net() {
        cudaSetDevice(dev);
        for (void* p : allocs) cudaFree(p);
        if (errh) cudaFreeHost(errh);
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
    // a timed-out wait of a network kernel since the last check (clears the word)
    bool timed_out() {
        if (!errh || *(volatile unsigned int*)errh == 0u) return false;
        *(volatile unsigned int*)errh = 0u;
        return true;
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
    cnn::pack_out_weights(n->w + oW5, n->wo, n->wod, st);
}

tomo_status ensure_capacity(tomo_net* n, int64_t pixels) {
    if (pixels <= n->cap) return TOMO_OK;
    for (void* p : {(void*)n->x0, (void*)n->y[0], (void*)n->y[1], (void*)n->y[2], (void*)n->y[3], (void*)n->dz[0],
                    (void*)n->dz[1], (void*)n->dpk, (void*)n->out, (void*)n->dout})
        if (p) n->release(p);
    n->mB = n->mH = n->mW = 0;   // the maps name the released buffers
    bool ok = n->alloc(&n->x0, pixels * 16);
    for (int l = 0; l < 4; ++l) ok = ok && n->alloc(&n->y[l], pixels * C);
    ok = ok && n->alloc(&n->dz[0], pixels * C) && n->alloc(&n->dz[1], pixels * C) && n->alloc(&n->dpk, pixels * 16);
    ok = ok && n->alloc(&n->out, pixels) && n->alloc(&n->dout, pixels);
    if (!ok) return n->fail(TOMO_ERR_OOM, "network activations do not fit");
    n->cap = pixels;
    return TOMO_OK;
}

// TMA maps of every activation for images B x H x W (re-encoded when the shape changes).
tomo_status ensure_maps(tomo_net* n, int B, int H, int W) {
    if (n->mB == B && n->mH == H && n->mW == W) return TOMO_OK;
    const __nv_bfloat16* base[tomo_net::NMAPS] = {n->x0, n->y[0], n->y[1], n->y[2], n->y[3], n->dz[0], n->dz[1], n->dpk};
    const int ch[tomo_net::NMAPS] = {16, C, C, C, C, C, C, 16};
    for (int i = 0; i < tomo_net::NMAPS; ++i)
        if (!cnn::encode_act_map(n->cmap[i], base[i], ch[i], B, H, W, true) ||
            !cnn::encode_act_map(n->wmap[i], base[i], ch[i], B, H, W, false)) {
            n->mB = n->mH = n->mW = 0;
            return n->fail(TOMO_ERR_CUDA, "cuTensorMapEncodeTiled refused an activation map");
        }
    n->mB = B;
    n->mH = H;
    n->mW = W;
    return TOMO_OK;
}

tomo_status check_shape(tomo_net* n, int B, int H, int W) {
    if (B < 1 || H < 1 || W < 64 || W % 64 != 0) return n->fail(TOMO_ERR_ARG, "images must be W % 64 == 0 wide");
    if ((int64_t)B * H > (int64_t)1 << 24 || W > 1 << 20) return n->fail(TOMO_ERR_ARG, "images too large");
    tomo_status s = ensure_capacity(n, (int64_t)B * H * W);
    return s != TOMO_OK ? s : ensure_maps(n, B, H, W);
}

tomo_status check_waits(tomo_net* n) {
    return n->timed_out() ? n->fail(TOMO_ERR_TIMEOUT, "network kernel: a TMA copy or MMA did not complete in time")
                          : TOMO_OK;
}

void forward(tomo_net* n, const float* feat, int B, int H, int W, float* out, cudaStream_t st) {
    cnn::pack_input(feat, n->x0, B, H, W, st);
    const float* bias[4] = {n->w + ob1, n->w + ob2, n->w + ob3, n->w + ob4};
    cnn::conv(cnn::CONV_IN, n->cmap[tomo_net::M_X0], n->wf1, bias[0], nullptr, n->y[0], B, H, W, n->errd, n->wait_ns, st);
    for (int l = 0; l < 3; ++l)
        cnn::conv(cnn::CONV_MID, n->cmap[tomo_net::M_Y0 + l], n->wf[l], bias[l + 1], nullptr, n->y[l + 1], B, H, W,
                  n->errd, n->wait_ns, st);
    cnn::conv(cnn::CONV_OUT, n->cmap[tomo_net::M_Y3], n->wo, n->w + ob5, nullptr, out, B, H, W, n->errd, n->wait_ns, st);
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
    cnn::loss(n->out, tgt, msk, P, W, (float)(1.0 / ms), n->dout, n->dpk, n->lpart, kPartBlocks, n->ltot, st);
    // layer 5: weight gradient from the packed loss gradient, then the data gradient into layer 4
    cnn::wgrad(cnn::WGRAD_OUT, n->wmap[tomo_net::M_Y3], n->wmap[tomo_net::M_DPK], n->part, kPartBlocks, n->g + oW5, B,
               H, W, n->errd, n->wait_ns, st);
    cnn::conv(cnn::CONV_OUT_DGRAD, n->cmap[tomo_net::M_DPK], n->wod, nullptr, n->y[3], n->dz[0], B, H, W, n->errd,
              n->wait_ns, st);
    // layers 4, 3, 2: weight gradient, then data gradient masked by the layer input's ReLU
    const int64_t ow[3] = {oW2, oW3, oW4};
    int cur = 0;
    for (int l = 2; l >= 0; --l) {   // l = index of layers 2..4 in wf/wd; input activation y[l]
        cnn::wgrad(cnn::WGRAD_MID, n->wmap[tomo_net::M_Y0 + l], n->wmap[tomo_net::M_DZ0 + cur], n->part, kPartBlocks,
                   n->g + ow[l], B, H, W, n->errd, n->wait_ns, st);
        cnn::conv(cnn::CONV_DGRAD, n->cmap[tomo_net::M_DZ0 + cur], n->wd[l], nullptr, n->y[l], n->dz[1 - cur], B, H, W,
                  n->errd, n->wait_ns, st);
        cur = 1 - cur;
    }
    cnn::wgrad(cnn::WGRAD_IN, n->wmap[tomo_net::M_X0], n->wmap[tomo_net::M_DZ0 + cur], n->part, kPartBlocks, n->g + oW1,
               B, H, W, n->errd, n->wait_ns, st);
    double l = 0.0;
    NCU(n, cudaMemcpyAsync(&l, n->ltot, sizeof(double), cudaMemcpyDeviceToHost, st));
    NCU(n, cudaStreamSynchronize(st));
    NCU(n, cudaGetLastError());
    if (tomo_status w = check_waits(n); w != TOMO_OK) return w;
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
tomo_status net_check(tomo_net* n) { return check_waits(n); }
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
    ok = ok && n->alloc(&n->wo, 9 * 16 * C) && n->alloc(&n->wod, 9 * 16 * C);
    ok = ok && n->alloc(&n->part, (int64_t)kPartBlocks * (kWmid + C)) && n->alloc(&n->lpart, kPartBlocks) &&
         n->alloc(&n->ltot, 1);
    if (!ok) return TOMO_ERR_OOM;
    if (cudaHostAlloc((void**)&n->errh, sizeof(unsigned int), cudaHostAllocMapped) != cudaSuccess) {
        n->errh = nullptr;
        cudaGetLastError();
        return TOMO_ERR_OOM;
    }
    *n->errh = 0u;
    if (cudaHostGetDevicePointer((void**)&n->errd, n->errh, 0) != cudaSuccess) {
        cudaGetLastError();
        return TOMO_ERR_CUDA;
    }
    if (const char* e = std::getenv("TOMO_WAIT_LIMIT_NS")) n->wait_ns = std::strtoull(e, nullptr, 10);
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
    return check_waits(n);
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
    return check_waits(n);
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
