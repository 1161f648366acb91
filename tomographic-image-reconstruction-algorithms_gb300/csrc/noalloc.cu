// noalloc.cu -- forward solve into caller-owned device buffers with no device
// allocation at all (tomo_forward_noalloc in include/tomo.h).
//
// Why it exists: tomo_create sizes and cudaMallocs a context.  Some callers
// cannot do that -- a host application that hands every byte of device memory
// to its own pool allocator and forbids raw cudaMalloc, or a latency-bound loop
// where cudaMalloc/cudaFree would synchronise the device and stall its other
// streams.  They pass their own input and output buffers; the wavefield
// scratch this solve needs lives in the file-scope array below instead.
//
// The scratch array g_scratch is a fixed kNoallocScratchBytes (about 5.1 MiB)
// that every GPU loading this library holds until the process exits.  It holds,
// for one emitter group at a time, the three forward time slots, the two
// coefficient fields and the geometry tables, so a call accepts grids of up to
// kNoallocMaxCells cells (512 x 512), kNoallocMaxChannels record channels and
// kNoallocMaxSteps time steps, plus kNoallocMaxEmitters emitters (benchmark
// profile) or kNoallocMaxGroups emission boxes (reference profile), and rejects
// anything larger with TOMO_ERR_ARG.
//
// In host code g_scratch names a host-side stand-in, not device memory.  Every
// call looks the array's device address up with cudaGetSymbolAddress on the
// current device and passes that pointer to the kernels, so the address is
// right for whatever context is current (also after a cudaDeviceReset, which
// reloads the module at a new address).  The first call on a device also loads
// the module's code there: make that first call before any stream capture.
//
// The geometry tables travel to the array as kernel arguments (k_put_words),
// not as copies from host memory, so nothing on the device side refers to the
// call's host-side tables after it returns.
//
// All calls share the one array and it keeps the last call's contents: each
// call zeroes the two initial time slots it starts from and the output records,
// and rewrites everything else before reading it.  Calls that overlap on the
// GPU (concurrent streams, or threads, on the same device) race on the array:
// serialise them on one stream.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <algorithm>
#include <string>

#include "internal.h"

namespace tomo {
namespace {

constexpr int64_t kNoallocMaxCells = 512 * 512;
constexpr int kNoallocMaxChannels = 2048;
constexpr int kNoallocMaxGroups = 2048;
constexpr int kNoallocMaxEmitters = 4096;
constexpr int kNoallocMaxSteps = 16384;

// float region: 3 time slots + coefficient + edge coefficient + source table
constexpr int64_t kFloats = 5 * kNoallocMaxCells + kNoallocMaxSteps;
// int region: receiver cells + emitter cells + emission boxes
constexpr int64_t kInts = kNoallocMaxChannels + kNoallocMaxEmitters + 4 * kNoallocMaxGroups;
constexpr int64_t kNoallocScratchBytes = 4 * (kFloats + kInts);

static __device__ __align__(256) unsigned char g_scratch[kNoallocScratchBytes];

// Words of table data carried by one k_put_words launch (the argument block stays under the
// 4 KB kernel-parameter limit of every CUDA version).
constexpr int kWordsPerLaunch = 1000;
struct Words {
    uint32_t v[kWordsPerLaunch];
};

__global__ void k_put_words(uint32_t* __restrict__ dst, int n, Words w) {
    for (int t = threadIdx.x; t < n; t += blockDim.x) dst[t] = w.v[t];
}

// Failures are returned as a status and explained in one line on stderr.
tomo_status fail(tomo_status s, const std::string& why) {
    std::fprintf(stderr, "tomo_forward_noalloc: %s\n", why.c_str());
    return s;
}

tomo_status cuda_fail(cudaError_t e, const char* what) {
    return fail(TOMO_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

// Device address of g_scratch in the current device's context, looked up on every call.
tomo_status scratch_address(unsigned char** out) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
    if (e != cudaSuccess || !p) return cuda_fail(e, "cudaGetSymbolAddress(g_scratch)");
    *out = (unsigned char*)p;
    return TOMO_OK;
}

// Writes n 32-bit words from host memory to dst on `st`, kWordsPerLaunch per launch, through
// kernel arguments: the words are captured at launch, so `src` may go out of scope on return.
tomo_status put_words(uint32_t* dst, const void* src, int64_t n, cudaStream_t st) {
    Words w;
    const uint32_t* s = (const uint32_t*)src;
    for (int64_t off = 0; off < n; off += kWordsPerLaunch) {
        const int m = (int)std::min<int64_t>(kWordsPerLaunch, n - off);
        std::memcpy(w.v, s + off, sizeof(uint32_t) * m);
        k_put_words<<<1, 256, 0, st>>>(dst + off, m, w);
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return cuda_fail(e, "k_put_words");
    }
    return TOMO_OK;
}

}  // namespace
}  // namespace tomo

using namespace tomo;

// A function-try-block: a C++ exception below it (host allocation failure) becomes a status.
extern "C" tomo_status tomo_forward_noalloc(const tomo_config* cfg, const float* d_f, float* d_records,
                                            void* stream) try {
    if (!cfg || !d_f || !d_records) return fail(TOMO_ERR_ARG, "NULL argument");
    Geometry geo;
    std::string why;
    tomo_status s = build_geometry(*cfg, geo, why);
    if (s != TOMO_OK) return fail(s, why);
    // the emitter table is read by the benchmark profile only, the emission boxes by the reference profile
    if (geo.N > kNoallocMaxCells || geo.nch > kNoallocMaxChannels || geo.nt > kNoallocMaxSteps ||
        (geo.ref && geo.G > kNoallocMaxGroups) || (!geo.ref && (int64_t)geo.G * geo.gs > kNoallocMaxEmitters))
        return fail(TOMO_ERR_ARG, "problem exceeds the allocation-free limits (cells <= 262144, channels <= 2048, "
                                  "steps <= 16384, emitters <= 4096, reference-profile groups <= 2048)");
    unsigned char* base = nullptr;
    if ((s = scratch_address(&base)) != TOMO_OK) return s;
    cudaStream_t st = (cudaStream_t)stream;
    const int64_t N = geo.N, nt = geo.nt, nch = geo.nch;
    float* slots = (float*)base;                       // 3 time slots
    float* coef = slots + 3 * kNoallocMaxCells;
    float* rcoef = coef + kNoallocMaxCells;
    float* src = rcoef + kNoallocMaxCells;
    int32_t* rcv = (int32_t*)(src + kNoallocMaxSteps);
    int32_t* emit = rcv + kNoallocMaxChannels;
    int32_t* box = emit + kNoallocMaxEmitters;
    cudaError_t e;
#define NA_CU(x)                                     \
    do {                                             \
        if ((e = (x)) != cudaSuccess) return cuda_fail(e, #x); \
    } while (0)
    if ((s = put_words((uint32_t*)src, geo.src.data(), (int64_t)geo.src.size(), st)) != TOMO_OK) return s;
    if ((s = put_words((uint32_t*)rcv, geo.rcv.data(), nch, st)) != TOMO_OK) return s;
    if (geo.ref) s = put_words((uint32_t*)box, geo.box.data(), 4 * (int64_t)geo.G, st);
    else s = put_words((uint32_t*)emit, geo.emit.data(), (int64_t)geo.G * geo.gs, st);
    if (s != TOMO_OK) return s;
    NA_CU(cudaMemsetAsync(d_records, 0, sizeof(float) * (size_t)geo.G * nt * nch, st));
    DevGeo dg{};
    dg.nx = geo.nx; dg.ny = geo.ny; dg.nt = geo.nt; dg.nch = geo.nch;
    dg.lo = geo.lo; dg.hi = geo.hi; dg.gs = geo.gs;
    dg.sponge_w = cfg->sponge_width; dg.sponge_max = cfg->sponge_max;
    fill_damp(dg);
    dg.box = box; dg.emit = emit; dg.rcv = rcv; dg.rid = nullptr; dg.rbits = nullptr; dg.rwords = 0; dg.src = src;
    dg.n_src_steps = geo.n_src_steps;
    const int prof = cfg->profile;
    launch_coef(prof, d_f, coef, rcoef, N, cfg->courant, st);
    auto slot = [&](int k) { return slots + (int64_t)(k % 3) * N; };
    for (int g = 0; g < geo.G; ++g) {
        launch_zero_slots(slots, 1, 3 * N, 0, N, N, st);   // u(0) = u(1) = 0
        for (int k = 1; k <= geo.nt - 2; ++k) {
            FwdStep fs{};
            fs.up = slot(k - 1);
            fs.uc = slot(k);
            fs.un = slot(k + 1);
            fs.gstride = 3 * N;
            fs.k = k;
            fs.g0 = g;
            fs.ng = 1;
            launch_fwd_step(prof, dg, coef, rcoef, fs, st);
            GatherStep gs{};
            gs.u = slot(k + 1);
            gs.gstride = 3 * N;
            gs.out = d_records + (int64_t)g * nt * nch;
            gs.k = k + 1;
            gs.ng = 1;
            launch_gather(dg, gs, st);
        }
    }
    NA_CU(cudaGetLastError());
#undef NA_CU
    return TOMO_OK;
} catch (...) {
    std::string why;
    const tomo_status s = abi_exception(&why);
    std::fprintf(stderr, "tomo_forward_noalloc: %s\n", why.c_str());
    return s;
}
