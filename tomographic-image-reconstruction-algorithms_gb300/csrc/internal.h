// internal.h -- shared declarations of the engine's host and device code.
#pragma once

#include <cstdint>
#include <exception>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include "tomo.h"

#ifdef __CUDACC__
#define TOMO_HD __host__ __device__
#else
#define TOMO_HD
#endif

namespace tomo {

// Counter-based uniform draw in [0, 1) for record sample (group g, step k, channel c) under
// `key` (a splitmix64 finaliser of the mixed indices; the same bits on host and device).
TOMO_HD inline float noise_uniform(uint64_t key, int g, int k, int c) {
    uint64_t z = key ^ ((uint64_t)(uint32_t)g << 42) ^ ((uint64_t)(uint32_t)k << 20) ^ (uint64_t)(uint32_t)c;
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (float)(z >> 40) * (1.0f / 16777216.0f);
}

// Multiplicative record noise factor 1 + level (2U - 1).
TOMO_HD inline float noise_factor(uint64_t key, float level, int g, int k, int c) {
    return 1.0f + level * (2.0f * noise_uniform(key, g, k, c) - 1.0f);
}

// Status for the C++ exception in flight (host allocation or thread creation failure), its
// message into *err.  The C entry points are function-try-blocks whose handler returns this, so
// no exception crosses the C ABI.  Call only from inside a catch handler.
inline tomo_status abi_exception(std::string* err) noexcept {
    tomo_status s = TOMO_ERR_STATE;
    const char* why = "unknown C++ exception";
    std::string what;
    try {
        throw;
    } catch (const std::bad_alloc&) {
        s = TOMO_ERR_OOM;
        why = "host memory allocation failed";
    } catch (const std::length_error&) {
        s = TOMO_ERR_OOM;
        why = "host allocation larger than the address space";
    } catch (const std::exception& e) {
        why = "C++ exception";
        try { what = e.what(); } catch (...) {}
    } catch (...) {
    }
    if (err) {
        try {
            *err = why;
            if (!what.empty()) *err += ": " + what;
        } catch (...) {
        }
    }
    return s;
}

// Reference constants (sirt-mimo.cu:26-35), the float values the reference uses.
constexpr float kRefH = 0.001f;
constexpr float kRefDT = 3.3333e-07f;
constexpr float kRefOmegaC = 7.8540e+05f;
constexpr float kRefTao = 4.0000e-06f;
constexpr float kRefTT = 8.1573e-06f;

// Host-side description of one problem: geometry, emitters, receivers.
struct Geometry {
    tomo_config cfg{};
    bool ref = true;
    int nx = 0, ny = 0, nt = 0;
    int64_t N = 0;       // nx*ny
    int G = 0;           // groups
    int gs = 0;          // group size
    int ns = 0;          // transducers
    int nch = 0;         // record channels
    int lo = 0, hi = 0;  // REF sensor lines
    std::vector<int32_t> ii, jj;       // transducers (REF 1-based, CFG 0-based cells)
    std::vector<int32_t> box;          // REF: per group {i0, i1, j0, j1} 0-based inclusive emission box
    std::vector<int32_t> emit;         // CFG: G*gs emitter cells
    std::vector<int32_t> rcv;          // receiver cell per channel, -1 none
    std::vector<int32_t> rid;          // CFG: per-cell channel index or -1
    std::vector<uint8_t> mask;         // update mask
    std::vector<float> src;            // CFG: per step C^2 ricker(n); REF: the FP32 factors cos(wc t_k) at
                                       // [k] and exp(-t_k^2 / 2 tau^2) at [n_src_steps + k]
    int n_src_steps = 0;               // steps k (computing u(k+1)) that add a source
    double corr_scale = 1.0;           // REF 1/h^2, CFG C^2
};

// Builds the geometry; returns TOMO_OK or TOMO_ERR_ARG with a reason.
tomo_status build_geometry(const tomo_config& cfg, Geometry& geo, std::string& why);
tomo_status phantom_ref(int nx, int ny, float* fo);
tomo_status phantom_cfg(int nx, int ny, int kind, int n, float rmin, float rmax, float vmax,
                        float noise_sigma, float support, uint64_t seed, float* fo);
// rec += level * std(trace) * N(0,1) per (group, channel) trace, seeded.
void add_record_noise(float* rec, int G, int nt, int nch, float level, uint64_t seed);
// rec *= noise_factor(seed, level, g, k, c) for every sample (multiplicative uniform noise).
void mul_record_noise(float* rec, int G, int nt, int nch, float level, uint64_t seed);

// splitmix64-based portable RNG (identical on x86 and Arm).
struct Rng {
    uint64_t s;
    explicit Rng(uint64_t seed) : s(seed ^ 0x9E3779B97F4A7C15ull) {}
    uint64_t next() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
    double normal();
};

// ---- device-side argument blocks -------------------------------------------------
struct DevGeo {
    int nx, ny, nt, nch;
    int lo, hi;            // REF sensor lines
    int gs;                // CFG emitters per group
    int sponge_w;          // CFG
    float sponge_max;      // CFG
    float damp[64];        // CFG sponge factor 1 - smax ((w - dd) / w)^2 at distance dd < w from the edge
    const int32_t* box;    // REF per-group emission box (4 ints), global group index
    const int32_t* emit;   // CFG emitter cells, global group index
    const int32_t* rcv;    // receiver cell per channel
    const int32_t* rid;    // CFG per-cell channel or -1
    const uint32_t* rbits; // CFG per row: bit b set when cells [32b, 32b+32) hold a receiver
    int rwords;            // words of rbits per row
    const float* dmap;     // CFG per-cell sponge factor (the damp table by edge distance), or null
    const float* src;      // source table (Geometry::src)
    int n_src_steps;
    // residual noise: simulated samples u become u * noise_factor(*noise_key, noise_level, ...)
    // in every residual gather while noise_key is non-null (its value can change between passes)
    const uint64_t* noise_key;
    float noise_level;
};

struct FwdStep {
    const float* up;   // slice k-1 of pass-group 0
    const float* uc;   // slice k
    float* un;         // slice k+1
    int64_t gstride;   // elements between consecutive groups of the pass
    float* ck;         // optional checkpoint copy of slice k+1 (pass-group 0), or null
    int64_t ckstride;
    int k;             // computing slice k+1
    int g0;            // global index of pass-group 0
    int ng;            // groups in the pass
    // fused sensor gather of slice k (strip kernels only; gk < 2: none)
    int gk = -1;
    const float* gmeas = nullptr;   // measured records of pass-group 0, or null (simulate)
    float* gout = nullptr;          // records / residual of pass-group 0
};

struct AdjStep {
    const float* z2;   // z(k+2)
    const float* z1;   // z(k+1)
    float* zk;         // z(k) output
    int64_t zstride;
    const float* uq;   // forward slice correlated with z(k): REF u(k), CFG u(k-1)
    int64_t ustride;
    const float* rr;   // residual records of pass-group 0 at step k: rr + k*nch
    int64_t rrstride;  // elements between groups in rr (nt*nch)
    float* corr;       // per-group correlation accumulators of pass-group 0
    int64_t cstride;
    int k;
    int ng;
};

struct GatherStep {
    const float* u;      // slice k of pass-group 0
    int64_t gstride;
    const float* meas;   // measured records of pass-group 0 (g*nt*nch layout) or null
    float* out;          // pass-group 0 records (simulated if meas null, residual otherwise)
    double* part;        // per (group, k) squared residual, pass-group 0, stride nt; or null
    int k;
    int ng;
    int g0 = 0;          // global index of pass-group 0
};

// ---- kernel launchers (kernels.cu) --------------------------------------------------
void launch_coef(int profile, const float* f, float* coef, float* rcoef, int64_t N, float courant,
                 void* stream);
void launch_fwd_step(int profile, const DevGeo& g, const float* coef, const float* rcoef,
                     const FwdStep& s, void* stream);
// f: the field the coefficients were made from (the reference-profile adjoint reads 1 + f)
void launch_adj_step(int profile, const DevGeo& g, const float* coef, const float* f, const AdjStep& s,
                     void* stream);
void launch_gather(const DevGeo& g, const GatherStep& s, void* stream);
void launch_fill(float* p, int64_t n, float v, void* stream);
// zero slots off0 and off1 (element offsets) of ng groups spaced gstride apart
void launch_zero_slots(float* base, int ng, int64_t gstride, int64_t off0, int64_t off1, int64_t N, void* stream);
// copy ng groups: dst[gl*dstride + q] = src[gl*sstride + q], q < N
void launch_copy_groups(float* dst, int64_t dstride, const float* src, int64_t sstride, int ng, int64_t N, void* stream);

// reductions and update rules (deterministic, FP64 where stated)
// dfg(g) = corr(g) * scale / (1 + f); dir = sum_g w_g dfg(g) (w may be null: all 1) times post
void launch_combine(const float* corr, int G, int64_t N, const float* f, double scale,
                    const double* w, double post, float* dir, void* stream);
// part[g*nb + b] = block partial of sum_q (corr(g)*scale/(1+f) - mean)^2, mean = dir/G-ish supplied
void launch_group_dev_norm(const float* corr, int G, int64_t N, const float* f, double scale,
                           const float* mean, double* part, int nb, void* stream);
// avg-weight: part[g*nb+b] partial of sum_q (f + s*mask*dfg - fbar)^2
void launch_avgw_norm(const float* corr, int G, int64_t N, const float* f, const uint8_t* mask,
                      double scale, double s, const float* fbar, double* part, int nb, void* stream);
void launch_avgw_fbar(const float* corr, int G, int64_t N, const float* f, const uint8_t* mask,
                      double scale, double s, float* fbar, void* stream);
void launch_avgw_apply(const float* corr, int G, int64_t N, float* f, const uint8_t* mask,
                       double scale, double s, const double* w, void* stream);
// Fills g.damp from g.sponge_w and g.sponge_max (evaluated in FP64, rounded once).
void fill_damp(DevGeo& g);

void launch_sum_parts(const double* part, int rows, int nb, double* out, void* stream);
// squared deviation norms d2[0..G) -> normalised inverse-norm weights, in place (FP64)
void launch_norm_weights(double* d2w, int G, void* stream);
void launch_maxabs(const float* dir, const uint8_t* mask, int64_t N, unsigned int* out, void* stream);
void launch_apply(float* f, const float* dir, const uint8_t* mask, int64_t N, double s,
                  const unsigned int* maxabs, void* stream);
void launch_eps_parts(const float* f, const float* fo, int64_t N, double* part, int nb, void* stream);

int reduce_blocks();  // number of partial blocks the reductions use
void launch_illum_add(const float* u, int ng, int64_t gstride, int64_t N, float* I, void* stream);
void launch_features(const float* f, const float* dir, const unsigned int* dmax, const float* I, const unsigned int* imax,
                     int64_t N, float* feat, void* stream);
// learned update network (net.cu): one image, features planar [3][H][W], output [H][W]
tomo_status net_infer(tomo_net* net, const float* feat, int H, int W, float* out, void* stream);
// TOMO_ERR_TIMEOUT when a network kernel's bounded wait ran out since the last check (call after
// the stream the network ran on has been synchronised), else TOMO_OK.
tomo_status net_check(tomo_net* net);

// warp-strip step kernels (strip.cu): CFG profile, nx % 4 == 0; rows per warp in {2,4,8,16,32}
bool strip_supported(const DevGeo& g, int profile);
void launch_fwd_strip(int rows, const DevGeo& g, const float* coef, const FwdStep& s, void* stream);
// variant: 0 default registers, unroll 2; 1 <= 64 registers, unroll 1; 2 default, unroll 1;
// 3 <= 80 registers, unroll 2
void launch_adj_strip(int rows, int variant, const DevGeo& g, const float* coef, const AdjStep& s, void* stream);
// two forward steps per launch: a computes slice k+1, b slice k+2 (a.un, b.un; four
// distinct slots); gather_prev / gather_cur record slices k-1 / k into a.gout.
// rows in {4,8,16,32}: two cells per lane; 100 + rows: four cells per lane
void launch_fwd2_strip(int rows, const DevGeo& g, const float* coef, const FwdStep& a, const FwdStep& b,
                       bool gather_prev, bool gather_cur, void* stream);
// two adjoint steps per launch: a = the step producing z(kz), b = the following
// step producing z(kz-1) (z slots must be four distinct slices)
void launch_adj2_strip(int rows, const DevGeo& g, const float* coef, const AdjStep& a, const AdjStep& b,
                       void* stream);
void launch_resid_parts(const float* rr, int ng, int nt, int nch, double* part, void* stream);

// multi-step tile kernels (tile.cu): CFG profile with a receiver map.  A forward launch computes
// slices k0+1 .. k0+T (T <= 8) of every group of the pass, writes each to its slot, its
// checkpoint copy and its records; an adjoint launch computes z(kz0) .. z(kz0-T+1) (T in
// {1, 2, 6}) with the correlation, writing the last two slices to the ring.
// Bounded waits of the tile kernels' TMA copies: a block that waits longer than wait_ns for a
// copy sets bit 0 of *err (host-visible) and leaves the launch.  extra_tx (0 in production)
// makes the region copy's barrier expect bytes that never arrive, so a test can run the wait
// out and check the status.  A persistent launch (k_last / kz_last set) runs a whole segment of
// chunks with a grid barrier between chunks on the counter *gbar (zeroed before the launch),
// bounded by the same wait_ns; gbar_extra (0 in production) makes it wait for arrivals that
// never come.
struct TileWait {
    unsigned int* err;
    uint64_t wait_ns;
    uint32_t extra_tx;
    unsigned int* gbar;
    uint32_t gbar_extra;
};
struct TileFwd {
    float* hist;         // forward slots of pass-group 0; slice m at slot m % S
    int64_t gstride;     // S * N: group gl's slot s is plane gl * S + s of the slot tensor
    int S;
    int k0, T;           // computes slices k0+1 .. k0+T; T <= 8 and T <= S - 2
    int g0, ng;
    float* ckpt;         // checkpoint copies (null: none): chunk ch >= 1 keeps slices ch K - 1 .. ch K
    int64_t ckstride;
    int K, nchunk;
    const float* gmeas;  // measured records of pass-group 0 (null: simulate)
    float* gout;         // records / residual of pass-group 0 (slices >= 2)
    int warps;           // tile shape: 16 (48 x 48 owned cells) or 10 (48 x 24)
    int k_last;          // persistent launch: slices k0+1 .. k_last in chunks of T <= 8 (0: one chunk of T)
    TileWait w;
};
struct TileAdj {
    float* z;            // adjoint ring of pass-group 0: z(m) at slot m % 4 (plane gl * 4 + slot)
    int64_t zstride;
    const float* hist;   // forward slots of pass-group 0: u(m-1) at slot (m-1) % S
    int64_t ustride;
    int S;
    const float* rr;     // residual records of pass-group 0: step m at rr + m * nch
    int64_t rrstride;
    float* corr;         // correlation of pass-group 0
    int64_t cstride;
    int kz0, T;
    int ng;
    int warps;           // tile shape: 16 (48 x 48 owned cells) or 10 (48 x 24)
    int kz_last;         // persistent launch: z(kz0) .. z(kz_last) in chunks of 6, 2, 1 (0: one chunk of T)
    TileWait w;
};
// TMA tensor maps of one context's buffers (forward slots, adjoint ring, coefficient, sponge
// map, receiver map) for each tile shape, encoded on the host by encode_tile_maps; opaque
// outside tile.cu.
struct TileMaps {
    alignas(64) unsigned char raw[2][6][128];
    bool ok = false;
};
bool tile_supported(const DevGeo& g, int profile);
// Encodes the maps for slot tensors of hist_planes (P * S) and z_planes (P * 4) planes of
// nx x ny cells; false (with the reason) when the driver has no tensor-map encoder or refuses.
bool encode_tile_maps(TileMaps* m, const DevGeo& g, const float* hist, int64_t hist_planes, const float* z,
                      int64_t z_planes, const float* coef, std::string* why);
void launch_fwd_tile(const DevGeo& g, const TileMaps& m, const TileFwd& a, void* stream);
void launch_adj_tile(const DevGeo& g, const TileMaps& m, const TileAdj& a, void* stream);
// Whether a persistent (cooperative) launch of ng groups keeps every block resident at once.
bool tile_persistent_fits(const DevGeo& g, int warps, bool fwd, int ng);
// cuTensorMapEncodeTiled, looked up from the driver once (no link against libcuda); null when
// the driver has none.
void* tensor_map_encoder();
constexpr int TILE_OWNED = 48;    // owned tile width and height of the tile kernels
constexpr int TILE_MAX_FWD = 8;   // forward steps per tile launch at most

}  // namespace tomo
