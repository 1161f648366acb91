// engine.cu -- the tomo_ctx: device buffers, memory plan, checkpoint/recompute
// schedule, CUDA-graph capture of the per-time-step launches, and the C ABI.
//
// The reference runs each iteration as a host loop of ~1200 launches over
// full-history buffers u(NX,NY,NT,Ng), z(NX,NY,NT+1,Ng) and Lu(NX,NY,NT,Ng)
// (sirt-mimo-norm.cu:259-297,407-489).  Here one iteration is:
//   coef(f) -> per pass of P groups: [forward sweep: one launch per step for all
//   P groups, sensor gather with residual, checkpoint stores] [adjoint sweep:
//   per chunk of K slices (last chunk first): restore checkpoint, recompute the
//   chunk's forward slices, adjoint steps with fused injection + correlation]
//   -> update rule (deterministic FP64 reductions).
// Each pass's launch sequence is captured once into a CUDA graph and replayed.
// Without checkpointing (K >= nt-2) the whole forward history stays resident
// and nothing is recomputed; with it, memory per group is (K+1 + 2*chunks)
// slices instead of nt (the on-device version of the reference's
// P-of-M-resident-groups strategy, sirt-mimo-norm-mem.cu:419-468).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <map>
#include <memory>
#include <string>
#include <tuple>
#include <thread>
#include <vector>

#include "internal.h"

using namespace tomo;

namespace {
thread_local std::string g_create_error;
}

struct tomo_ctx {
    Geometry geo;
    DevGeo dg{};
    int dev = 0;
    cudaStream_t st = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::string err;
    // plan
    int P = 1;       // groups per pass
    int S = 3;       // forward slots per group
    int K = 0;       // slices per chunk
    int nchunk = 1;
    bool full = true;
    // device buffers
    float *f = nullptr, *ftrue = nullptr, *coef = nullptr, *rcoef = nullptr, *dir = nullptr, *tmp = nullptr;
    float *hist = nullptr, *z = nullptr, *ckpt = nullptr, *corr = nullptr, *meas = nullptr, *rr = nullptr,
          *rec = nullptr, *dfg = nullptr;
    double *rpart = nullptr, *part = nullptr, *sums = nullptr;
    unsigned int* maxabs = nullptr;
    int32_t *box = nullptr, *emit = nullptr, *rcv = nullptr, *rid = nullptr;
    uint32_t* rbits = nullptr;
    int rwords = 0;
    float* src = nullptr;
    float* dmap = nullptr;       // CFG per-cell sponge factor
    uint8_t* mask = nullptr;
    int64_t bytes = 0;
    bool meas_set = false;
    std::map<std::tuple<int, int, int>, cudaGraphExec_t> graphs;
    std::map<std::tuple<int, int, int>, int64_t> graph_kernels;   // kernel nodes per graph
    int64_t launches = 0;                                          // kernels issued since reset
    bool strip = false;          // warp-strip kernels (CFG, nx % 4 == 0)
    int rows_fwd = 8, rows_adj = 8, adj_variant = 0;
    bool adj_pair = false;       // two adjoint steps per launch (strip kernels)
    int rows_adj2 = 8;
    bool fwd_pair = false;       // two forward steps per launch (needs S >= 4)
    int rows_fwd2 = 8;
    bool tile_fwd = false;       // multi-step tile kernels (tile.cu) for the forward sweeps
    bool tile_adj = false;       // ... and for the adjoint sweeps
    bool tile_fwd1 = false;      // the same choices for passes of one group (ART)
    bool tile_adj1 = false;
    int tile_warps_fwd = 16, tile_warps_adj = 16;     // tile shape: 16 warps (48 x 48) or 10 (48 x 24)
    int tile_warps_fwd1 = 16, tile_warps_adj1 = 16;   // ... for passes of one group
    // learned iteration (allocated on first use)
    float *illum = nullptr, *feat = nullptr, *fsave = nullptr, *dnet = nullptr, *dsave = nullptr;
    unsigned int *illum_max = nullptr, *maxsave = nullptr;
    bool illum_ready = false;
    double learned_scale = 1.0;  // the network's proposal is f + learned_scale * mask * net(features)
    int learned_backtrack = 0;   // retries of a rejected proposal at half the scale (tomo_run_learned)
    int learned_resume = 0;      // plain steps after which paused proposals resume (0: never)
    static constexpr int ZR = 4; // adjoint ring slots
    TileMaps tmaps;              // TMA maps of hist, z, coef, dmap, rid (tile kernels)
    TileMaps tmaps_ck;           // the same with the slice maps over the checkpoint buffer (pass_layout)
    unsigned int* err_host = nullptr;   // tile kernels' wait time-out word (mapped pinned memory)
    unsigned int* err_dev = nullptr;
    uint64_t wait_ns = 1000000000ull;   // bound of every tile-kernel copy wait (TOMO_WAIT_LIMIT_NS)
    uint32_t test_tx = 0;        // TOMO_TEST_UNDELIVERED_TX: bytes a region barrier expects in vain
    unsigned int* gbar = nullptr;  // grid barrier counter of the persistent tile launches
    uint32_t test_gbar = 0;      // TOMO_TEST_GRID_BARRIER_EXTRA: arrivals a grid barrier waits for in vain
    bool persist = false;        // tile sweeps as persistent launches where every block fits (TOMO_PERSIST=1)
    bool tuned = false;
    double plan_budget = 0;      // bytes the plan's per-group buffers may take (make_plan)
    std::vector<void*> allocs;
    std::vector<size_t> alloc_bytes;

    tomo_status fail(tomo_status s, const char* fmt, ...) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof buf, fmt, ap);
        va_end(ap);
        err = buf;
        return s;
    }
    tomo_status cuda(cudaError_t e, const char* what) {
        if (e == cudaSuccess) return TOMO_OK;
        if (e == cudaErrorMemoryAllocation) {
            cudaGetLastError();
            return fail(TOMO_ERR_OOM, "%s: %s", what, cudaGetErrorString(e));
        }
        return fail(TOMO_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
    }
    template <typename T>
    tomo_status alloc(T** p, int64_t n, const char* what) {
        const size_t b = (size_t)std::max<int64_t>(n, 1) * sizeof(T);
        alloc_bytes.push_back(0);
        allocs.push_back(nullptr);   // the slots first: a push_back that throws leaks no device memory
        const cudaError_t e = cudaMalloc(&allocs.back(), b);
        if (e != cudaSuccess) {
            allocs.pop_back();
            alloc_bytes.pop_back();
            cudaGetLastError();
            return fail(TOMO_ERR_OOM, "cudaMalloc(%s, %zu bytes): %s", what, b, cudaGetErrorString(e));
        }
        bytes += (int64_t)b;
        alloc_bytes.back() = b;
        *p = (T*)allocs.back();
        return TOMO_OK;
    }
    template <typename T>
    void release(T** p) {
        for (size_t i = 0; *p && i < allocs.size(); ++i)
            if (allocs[i] == (void*)*p) {
                cudaFree(allocs[i]);
                bytes -= (int64_t)alloc_bytes[i];
                allocs.erase(allocs.begin() + (std::ptrdiff_t)i);
                alloc_bytes.erase(alloc_bytes.begin() + (std::ptrdiff_t)i);
                break;
            }
        *p = nullptr;
    }
    // residual noise (tomo_set_residual_noise): kind 0 off, 2 a fresh draw per gradient sweep,
    // 3 one fixed draw; the key lives on the device so captured graphs see its updates
    int noise_kind = 0;
    uint64_t noise_seed = 0, noise_draws = 0, noise_key_host = 0;
    uint64_t* noise_key = nullptr;
    // batched iterations (tomo_iterate_batch): a serial number no later context reuses, a
    // generation that changes whenever captured launches go stale, the join event of the batch
    // capture, pinned results of an enqueued iteration (residual, image-error sums), and the
    // batch graph this context leads (with the key it was recorded for)
    uint64_t serial = 0, gen = 0;
    cudaEvent_t evj = nullptr;
    double* pin = nullptr;
    std::vector<uint64_t> batch_key;
    cudaGraphExec_t batch_exec = nullptr;
    std::vector<int64_t> batch_kernels;
    void drop_graphs() {
        for (auto& kv : graphs) cudaGraphExecDestroy(kv.second);
        graphs.clear();
        graph_kernels.clear();
        ++gen;
    }
    ~tomo_ctx() {
        if (dev >= 0) cudaSetDevice(dev);
        for (auto& kv : graphs) cudaGraphExecDestroy(kv.second);
        if (batch_exec) cudaGraphExecDestroy(batch_exec);
        for (void* p : allocs) cudaFree(p);
        if (err_host) cudaFreeHost(err_host);
        if (pin) cudaFreeHost(pin);
        if (evj) cudaEventDestroy(evj);
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
        if (st) cudaStreamDestroy(st);
    }

    int64_t N() const { return geo.N; }
    int64_t slot(int k) const { return (int64_t)(k % S) * geo.N; }
    int64_t recs_per_group() const { return (int64_t)geo.nt * geo.nch; }
};

#define TRY(x)                                   \
    do {                                         \
        const tomo_status _s = (x);              \
        if (_s != TOMO_OK) return _s;            \
    } while (0)
#define CU(ctx, x) TRY((ctx)->cuda((x), #x))

namespace {

// FWD: simulated records; GRAD: residual + checkpoints + adjoint; RESID: residual only;
// ILLUM: illumination sum of u^2 over all steps and groups
enum Mode { MODE_FWD = 0, MODE_GRAD = 1, MODE_RESID = 2, MODE_ILLUM = 3 };

void fwd_launch(tomo_ctx* c, const FwdStep& fs) {
    if (c->strip) launch_fwd_strip(c->rows_fwd, c->dg, c->coef, fs, c->st);
    else launch_fwd_step(c->geo.cfg.profile, c->dg, c->coef, c->rcoef, fs, c->st);
}

void adj_launch(tomo_ctx* c, const AdjStep& as) {
    if (c->strip) launch_adj_strip(c->rows_adj, c->adj_variant, c->dg, c->coef, as, c->st);
    else launch_adj_step(c->geo.cfg.profile, c->dg, c->coef, c->f, as, c->st);
}

FwdStep fwd_args(tomo_ctx* c, int k, int g0, int ng) {
    FwdStep fs{};
    fs.up = c->hist + c->slot(k - 1);
    fs.uc = c->hist + c->slot(k);
    fs.un = c->hist + c->slot(k + 1);
    fs.gstride = (int64_t)c->S * c->geo.N;
    fs.k = k;
    fs.g0 = g0;
    fs.ng = ng;
    return fs;
}

AdjStep adj_args(tomo_ctx* c, int q, int g0, int ng) {
    const int64_t N = c->geo.N;
    const int kz = (c->geo.cfg.profile == TOMO_PROFILE_REF) ? q : q + 1;
    const int zr = tomo_ctx::ZR;
    AdjStep as{};
    as.z2 = c->z + (int64_t)((kz + 2) % zr) * N;
    as.z1 = c->z + (int64_t)((kz + 1) % zr) * N;
    as.zk = c->z + (int64_t)(kz % zr) * N;
    as.zstride = zr * N;
    as.uq = c->hist + c->slot(q);
    as.ustride = (int64_t)c->S * N;
    as.rr = c->rr + (int64_t)kz * c->geo.nch;
    as.rrstride = c->recs_per_group();
    as.corr = c->corr + (int64_t)g0 * N;
    as.cstride = N;
    as.k = kz;
    as.ng = ng;
    return as;
}

// Multi-step tile forward launch: slices k0+1 .. k0+T of the pass.
TileFwd tile_fwd_args(tomo_ctx* c, int k0, int T, int g0, int ng) {
    TileFwd a{};
    a.hist = c->hist;
    a.gstride = (int64_t)c->S * c->geo.N;
    a.S = c->S;
    a.k0 = k0;
    a.T = T;
    a.g0 = g0;
    a.ng = ng;
    a.K = std::max(c->K, 1);
    a.nchunk = c->nchunk;
    a.warps = ng == 1 ? c->tile_warps_fwd1 : c->tile_warps_fwd;
    a.w = TileWait{c->err_dev, c->wait_ns, c->test_tx, c->gbar, c->test_gbar};
    return a;
}

// Multi-step tile adjoint launch: z(kz0) .. z(kz0-T+1) of the pass (CFG: kz = q + 1).
TileAdj tile_adj_args(tomo_ctx* c, int kz0, int T, int g0, int ng) {
    const int64_t N = c->geo.N;
    TileAdj a{};
    a.z = c->z;
    a.zstride = tomo_ctx::ZR * N;
    a.hist = c->hist;
    a.ustride = (int64_t)c->S * N;
    a.S = c->S;
    a.rr = c->rr;
    a.rrstride = c->recs_per_group();
    a.corr = c->corr + (int64_t)g0 * N;
    a.cstride = N;
    a.kz0 = kz0;
    a.T = T;
    a.ng = ng;
    a.warps = ng == 1 ? c->tile_warps_adj1 : c->tile_warps_adj;
    a.w = TileWait{c->err_dev, c->wait_ns, c->test_tx, c->gbar, c->test_gbar};
    return a;
}

// Forward steps of the next tile launch when L remain: at most 8, and at most S - 2 so the
// slices it writes never land on the two slots it reads.
int tile_fwd_steps(const tomo_ctx* c, int L) { return std::min(std::min(L, TILE_MAX_FWD), c->S - 2); }

bool tiles_ok(const tomo_ctx* c) { return tile_supported(c->dg, c->geo.cfg.profile) && c->tmaps.ok; }

// (Re)encodes the tile kernels' TMA maps for the current buffers; tiles stay off without them.
void encode_maps(tomo_ctx* c) {
    std::string why;
    if (!tile_supported(c->dg, c->geo.cfg.profile) ||
        !encode_tile_maps(&c->tmaps, c->dg, c->hist, (int64_t)c->P * c->S, c->z, (int64_t)c->P * tomo_ctx::ZR,
                          c->coef, &why)) {
        c->tmaps.ok = false;
        c->tile_fwd = c->tile_adj = c->tile_fwd1 = c->tile_adj1 = false;
        if (!why.empty() && std::getenv("TOMO_TUNE_LOG")) std::fprintf(stderr, "tomo: tile kernels off: %s\n", why.c_str());
    }
    // short passes that keep their history in the checkpoint buffer read it through these
    c->tmaps_ck.ok = false;
    if (c->tmaps.ok && !c->full && c->ckpt)
        encode_tile_maps(&c->tmaps_ck, c->dg, c->ckpt, (int64_t)c->P * c->nchunk * 2, c->z,
                         (int64_t)c->P * tomo_ctx::ZR, c->coef, nullptr);
}

// Stream synchronisation that also reports a tile kernel's timed-out copy wait.
tomo_status sync_check(tomo_ctx* c) {
    CU(c, cudaStreamSynchronize(c->st));
    if (c->err_host && *(volatile unsigned int*)c->err_host) {
        *(volatile unsigned int*)c->err_host = 0u;
        return c->fail(TOMO_ERR_TIMEOUT, "tile kernel: a TMA copy did not arrive within %llu ns",
                       (unsigned long long)c->wait_ns);
    }
    return TOMO_OK;
}

// Steps of the next tile adjoint launch when L steps remain: 6, 2 or 1 (the step counts whose
// output slices miss the input slices' slots of the four-slot ring).
int tile_adj_steps(int L) { return L >= 6 ? 6 : L >= 2 ? 2 : 1; }

// Tuning cache line: problem key, then the choices.
std::string tune_key(const tomo_ctx* c) {
    char b[160];
    std::snprintf(b, sizeof b, "tomo-tune-1 %d %d %d %d %d %d", c->geo.cfg.profile, c->geo.nx, c->geo.ny, c->geo.nt,
                  c->P, c->S);
    return b;
}

bool tune_cache_read(tomo_ctx* c, const char* path) {
    FILE* fp = std::fopen(path, "r");
    if (!fp) return false;
    const std::string key = tune_key(c);
    char line[512];
    bool hit = false;
    while (!hit && std::fgets(line, sizeof line, fp)) {
        if (std::strncmp(line, key.c_str(), key.size()) != 0 || line[key.size()] != ' ') continue;
        int v[15] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 16, 16, 16, 16};
        const int nv = std::sscanf(line + key.size(), "%d %d %d %d %d %d %d %d %d %d %d %d %d %d %d", &v[0], &v[1],
                                   &v[2], &v[3], &v[4], &v[5], &v[6], &v[7], &v[8], &v[9], &v[10], &v[11], &v[12],
                                   &v[13], &v[14]);
        if (nv == 7 || nv == 9 || nv == 11 || nv == 15) {
            c->rows_fwd = v[0]; c->rows_adj = v[1]; c->adj_variant = v[2]; c->adj_pair = v[3] != 0;
            c->rows_adj2 = v[4]; c->fwd_pair = v[5] != 0 && c->S >= 4; c->rows_fwd2 = v[6];
            c->tile_fwd = v[7] != 0 && tiles_ok(c);
            c->tile_adj = v[8] != 0 && tiles_ok(c);
            c->tile_fwd1 = v[9] != 0 && tiles_ok(c);
            c->tile_adj1 = v[10] != 0 && tiles_ok(c);
            c->tile_warps_fwd = v[11] == 10 ? 10 : 16;
            c->tile_warps_adj = v[12] == 10 ? 10 : 16;
            c->tile_warps_fwd1 = v[13] == 10 ? 10 : 16;
            c->tile_warps_adj1 = v[14] == 10 ? 10 : 16;
            hit = true;
        }
    }
    std::fclose(fp);
    return hit;
}

void tune_cache_append(const tomo_ctx* c, const char* path) {
    FILE* fp = std::fopen(path, "a");
    if (!fp) return;
    std::fprintf(fp, "%s %d %d %d %d %d %d %d %d %d %d %d %d %d %d %d\n", tune_key(c).c_str(), c->rows_fwd,
                 c->rows_adj, c->adj_variant, c->adj_pair ? 1 : 0, c->rows_adj2, c->fwd_pair ? 1 : 0, c->rows_fwd2,
                 c->tile_fwd ? 1 : 0, c->tile_adj ? 1 : 0, c->tile_fwd1 ? 1 : 0, c->tile_adj1 ? 1 : 0,
                 c->tile_warps_fwd, c->tile_warps_adj, c->tile_warps_fwd1, c->tile_warps_adj1);
    std::fclose(fp);
}

// TOMO_TILE=0 / 1 / f / a turns the multi-step tile kernels off, on for both sweeps, on for the
// forward or the adjoint sweeps only; TOMO_TILE_WARPS=16 / 10 fixes the tile shape (tests and
// profiling).
void tile_override(tomo_ctx* c) {
    const char* e = std::getenv("TOMO_TILE");
    if (!e || !*e) return;
    const bool ok = tiles_ok(c);
    c->tile_fwd = c->tile_fwd1 = ok && (e[0] == '1' || e[0] == 'f');
    c->tile_adj = c->tile_adj1 = ok && (e[0] == '1' || e[0] == 'a');
    if (const char* w = std::getenv("TOMO_TILE_WARPS")) {
        const int warps = std::atoi(w) == 10 ? 10 : 16;
        c->tile_warps_fwd = c->tile_warps_adj = c->tile_warps_fwd1 = c->tile_warps_adj1 = warps;
    }
}

// Picks the strip kernels (rows per warp, register variant, one or two steps
// per launch) by timing each candidate on this problem (mid-sweep steps of the
// first pass, best of three timed passes).  TOMO_STRIP_ROWS=<n> fixes the
// choice; TOMO_TUNE_CACHE=<file> reuses a choice recorded there for the same
// problem shape, or records the one made here; TOMO_TUNE_LOG prints each candidate's time.
tomo_status autotune(tomo_ctx* c) {
    if (c->tuned || !c->strip) { c->tuned = true; return TOMO_OK; }
    c->tuned = true;
    const char* cache = std::getenv("TOMO_TUNE_CACHE");
    if (cache && *cache && tune_cache_read(c, cache)) return TOMO_OK;
    if (const char* e = std::getenv("TOMO_STRIP_ROWS")) {
        c->rows_fwd = c->rows_adj = c->rows_adj2 = std::atoi(e);
        if (const char* v = std::getenv("TOMO_ADJ_VARIANT")) c->adj_variant = std::atoi(v);
        if (const char* v = std::getenv("TOMO_FWD_ROWS")) c->rows_fwd = std::atoi(v);
        if (const char* v = std::getenv("TOMO_ADJ_PAIR")) c->adj_pair = std::atoi(v) != 0;
        if (const char* v = std::getenv("TOMO_ADJ_PAIR_ROWS")) c->rows_adj2 = std::atoi(v);
        if (const char* v = std::getenv("TOMO_FWD_PAIR")) c->fwd_pair = std::atoi(v) != 0 && c->S >= 4;
        c->rows_fwd2 = c->rows_fwd;
        if (const char* v = std::getenv("TOMO_FWD_PAIR_ROWS")) c->rows_fwd2 = std::atoi(v);
        tile_override(c);
        return TOMO_OK;
    }
    const int cands[5] = {2, 4, 8, 16, 32};
    const int nt = c->geo.nt, ng = c->P, reps = 8, passes = 4;
    const bool tlog = std::getenv("TOMO_TUNE_LOG") != nullptr;   // print every candidate's time
    // trial steps k0 .. k0+reps stay inside [1, nt-2] (records are read at step q+1)
    if (nt < 4 * reps) return TOMO_OK;   // short sweeps keep the defaults
    const int k0 = nt / 2 - reps;
    float best_a = 1e30f;
    float best_f1 = 1e30f, best_f2 = 1e30f;    // best one-step and two-step forward
    int rows_f1 = c->rows_fwd, code_f2 = c->rows_fwd2;
    // forward: rows per warp; adjoint: rows per warp x register/unroll variant
    for (int rows : cands) {
        if (rows > 4 * c->geo.ny) continue;
        for (int which = 0; which < 5; ++which) {
            float ms = 1e30f;
            for (int pass = 0; pass < passes; ++pass) {   // first pass warms up
                CU(c, cudaEventRecord(c->ev0, c->st));
                for (int t = 0; t < reps; ++t) {
                    if (which == 0) launch_fwd_strip(rows, c->dg, c->coef, fwd_args(c, k0 + t, 0, ng), c->st);
                    else launch_adj_strip(rows, which - 1, c->dg, c->coef, adj_args(c, k0 + reps - t, 0, ng), c->st);
                }
                CU(c, cudaEventRecord(c->ev1, c->st));
                CU(c, cudaEventSynchronize(c->ev1));
                float t_ms = 0.f;
                CU(c, cudaEventElapsedTime(&t_ms, c->ev0, c->ev1));
                if (pass > 0) ms = std::min(ms, t_ms);
            }
            if (tlog) std::fprintf(stderr, "tomo tune: %s rows %d%s %.2f us/step\n", which ? "adjoint" : "forward", rows,
                                   which ? (" variant " + std::to_string(which - 1)).c_str() : "", 1e3 * ms / reps);
            if (which == 0 && ms < best_f1) { best_f1 = ms; rows_f1 = rows; }
            if (which > 0 && ms < best_a) {
                best_a = ms; c->rows_adj = rows; c->adj_variant = which - 1; c->adj_pair = false;
            }
        }
        // two forward steps per launch: 2 or 4 cells per lane, or inputs staged in shared memory
        for (int code : {rows, 100 + rows, 3200 + rows, 3300 + rows}) {
            if (rows < 4 || c->S < 4) break;
            float ms = 1e30f;
            for (int pass = 0; pass < passes; ++pass) {
                CU(c, cudaEventRecord(c->ev0, c->st));
                for (int t = 0; t < reps; t += 2)
                    launch_fwd2_strip(code, c->dg, c->coef, fwd_args(c, k0 + t, 0, ng), fwd_args(c, k0 + t + 1, 0, ng),
                                      false, false, c->st);
                CU(c, cudaEventRecord(c->ev1, c->st));
                CU(c, cudaEventSynchronize(c->ev1));
                float t_ms = 0.f;
                CU(c, cudaEventElapsedTime(&t_ms, c->ev0, c->ev1));
                if (pass > 0) ms = std::min(ms, t_ms);
            }
            if (tlog) std::fprintf(stderr, "tomo tune: forward pair code %d %.2f us/step\n", code, 1e3 * ms / reps);
            if (ms < best_f2) { best_f2 = ms; code_f2 = code; }
        }
        // two steps per launch (reps/2 launches cover the same steps); codes as launch_adj2_strip
        for (int code : {rows, 100 + rows, 200 + rows, 1000 + rows, 1100 + rows, 1200 + rows, 2000 + rows,
                         4000 + rows, 4100 + rows, 3200 + rows, 3300 + rows, 3400 + rows, 5200 + rows,
                         5300 + rows, 7000 + rows, 7100 + rows, 8200 + rows, 8300 + rows, 8400 + rows,
                         9200 + rows, 9300 + rows, 18200 + rows, 18300 + rows, 18400 + rows}) {
            if (code >= 18000 && rows != 8) continue;                 // packed unrolled staged: rows 8
            if (code >= 5000 && code < 7000 && rows < 16) continue;   // 8-block staged build: rows 16, 32
            if (code >= 7000 && code < 8000 && rows != 8 && rows != 16) continue;   // lean build: rows 8, 16
            if (code >= 8000 && code < 9000 && rows != 8 && code != 8316) continue;  // unrolled staged: rows 8 (16 at D 3)
            if (code >= 9000 && code < 10000 && rows != 8 && rows != 16) continue;   // four cells per lane, staged: rows 8, 16
            if (rows < 4) break;
            float ms = 1e30f;
            for (int pass = 0; pass < passes; ++pass) {
                CU(c, cudaEventRecord(c->ev0, c->st));
                for (int t = 0; t < reps; t += 2)
                    launch_adj2_strip(code, c->dg, c->coef, adj_args(c, k0 + reps - t, 0, ng),
                                      adj_args(c, k0 + reps - t - 1, 0, ng), c->st);
                CU(c, cudaEventRecord(c->ev1, c->st));
                CU(c, cudaEventSynchronize(c->ev1));
                float t_ms = 0.f;
                CU(c, cudaEventElapsedTime(&t_ms, c->ev0, c->ev1));
                if (pass > 0) ms = std::min(ms, t_ms);
            }
            if (tlog) std::fprintf(stderr, "tomo tune: adjoint pair code %d %.2f us/step\n", code, 1e3 * ms / reps);
            if (ms < best_a) { best_a = ms; c->rows_adj2 = code; c->adj_pair = true; }
        }
    }
    // one-step forward with its inputs staged in shared memory
    for (int code : {3204, 3208, 3216, 3304, 3308, 3316, 6004, 6008, 6016, 6104, 6108, 6116}) {
        if (code % 100 > 4 * c->geo.ny) continue;
        float ms = 1e30f;
        for (int pass = 0; pass < passes; ++pass) {
            CU(c, cudaEventRecord(c->ev0, c->st));
            for (int t = 0; t < reps; ++t) launch_fwd_strip(code, c->dg, c->coef, fwd_args(c, k0 + t, 0, ng), c->st);
            CU(c, cudaEventRecord(c->ev1, c->st));
            CU(c, cudaEventSynchronize(c->ev1));
            float t_ms = 0.f;
            CU(c, cudaEventElapsedTime(&t_ms, c->ev0, c->ev1));
            if (pass > 0) ms = std::min(ms, t_ms);
        }
        if (tlog) std::fprintf(stderr, "tomo tune: forward staged code %d %.2f us/step\n", code, 1e3 * ms / reps);
        if (ms < best_f1) { best_f1 = ms; rows_f1 = code; }
    }
    // A two-step forward must win clearly: inside a sweep it also carries the odd leftover step,
    // the sensor gather of two slices and the checkpoint copies, which the trial does not time.
    c->rows_fwd = rows_f1;
    c->rows_fwd2 = code_f2;
    c->fwd_pair = best_f2 < 0.97f * best_f1;
    // multi-step tile kernels against the chosen strip kernels, per step: forward launches of 8
    // steps and adjoint launches of 6 + 2 steps, for each tile shape (48 x 48 or 48 x 24 owned)
    if (tiles_ok(c)) {
        auto time_tiles = [&](int n, int warps, float& tf, float& ta) -> tomo_status {
            tf = ta = 1e30f;
            for (int pass = 0; pass < passes; ++pass) {
                float t_ms = 0.f;
                CU(c, cudaEventRecord(c->ev0, c->st));
                for (int t = 0; t < reps; t += tile_fwd_steps(c, reps - t)) {
                    TileFwd fa = tile_fwd_args(c, k0 + t, tile_fwd_steps(c, reps - t), 0, n);
                    fa.warps = warps;
                    launch_fwd_tile(c->dg, c->tmaps, fa, c->st);
                }
                CU(c, cudaEventRecord(c->ev1, c->st));
                CU(c, cudaEventSynchronize(c->ev1));
                CU(c, cudaEventElapsedTime(&t_ms, c->ev0, c->ev1));
                if (pass > 0) tf = std::min(tf, t_ms);
                CU(c, cudaEventRecord(c->ev0, c->st));
                for (const int kz : {k0 + reps + 1, k0 + reps - 5}) {
                    TileAdj aa = tile_adj_args(c, kz, kz == k0 + reps + 1 ? 6 : 2, 0, n);
                    aa.warps = warps;
                    launch_adj_tile(c->dg, c->tmaps, aa, c->st);
                }
                CU(c, cudaEventRecord(c->ev1, c->st));
                CU(c, cudaEventSynchronize(c->ev1));
                CU(c, cudaEventElapsedTime(&t_ms, c->ev0, c->ev1));
                if (pass > 0) ta = std::min(ta, t_ms);
            }
            if (tlog)
                std::fprintf(stderr, "tomo tune: %d-group tiles of %d warps: forward %.2f us/step, adjoint %.2f us/step\n",
                             n, warps, 1e3 * tf / reps, 1e3 * ta / reps);
            return TOMO_OK;
        };
        // the faster shape per sweep for passes of n groups
        auto best_tiles = [&](int n, float& tf, float& ta, int& wf, int& wa) -> tomo_status {
            tf = ta = 1e30f;
            for (const int warps : {16, 10}) {
                float f = 0.f, a = 0.f;
                TRY(time_tiles(n, warps, f, a));
                if (f < tf) { tf = f; wf = warps; }
                if (a < ta) { ta = a; wa = warps; }
            }
            return TOMO_OK;
        };
        float ms_tf = 1e30f, ms_ta = 1e30f;
        TRY(best_tiles(ng, ms_tf, ms_ta, c->tile_warps_fwd, c->tile_warps_adj));
        c->tile_fwd = ms_tf < 0.97f * std::min(best_f1, c->fwd_pair ? best_f2 : best_f1);
        c->tile_adj = ms_ta < 0.97f * best_a;
        c->tile_fwd1 = c->tile_fwd;
        c->tile_adj1 = c->tile_adj;
        c->tile_warps_fwd1 = c->tile_warps_fwd;
        c->tile_warps_adj1 = c->tile_warps_adj;
        if (c->geo.G > 1) {
            // passes of one group (ART): the chosen strip kernels against the tiles, 8 steps each
            float s_f = 1e30f, s_a = 1e30f, t_f = 1e30f, t_a = 1e30f;
            for (int pass = 0; pass < passes; ++pass) {
                float t_ms = 0.f;
                CU(c, cudaEventRecord(c->ev0, c->st));
                for (int t = 0; t < reps;) {
                    if (c->fwd_pair) {
                        launch_fwd2_strip(c->rows_fwd2, c->dg, c->coef, fwd_args(c, k0 + t, 0, 1),
                                          fwd_args(c, k0 + t + 1, 0, 1), false, false, c->st);
                        t += 2;
                    } else {
                        launch_fwd_strip(c->rows_fwd, c->dg, c->coef, fwd_args(c, k0 + t, 0, 1), c->st);
                        t += 1;
                    }
                }
                CU(c, cudaEventRecord(c->ev1, c->st));
                CU(c, cudaEventSynchronize(c->ev1));
                CU(c, cudaEventElapsedTime(&t_ms, c->ev0, c->ev1));
                if (pass > 0) s_f = std::min(s_f, t_ms);
                CU(c, cudaEventRecord(c->ev0, c->st));
                for (int t = 0; t < reps;) {
                    if (c->adj_pair) {
                        launch_adj2_strip(c->rows_adj2, c->dg, c->coef, adj_args(c, k0 + reps - t, 0, 1),
                                          adj_args(c, k0 + reps - t - 1, 0, 1), c->st);
                        t += 2;
                    } else {
                        launch_adj_strip(c->rows_adj, c->adj_variant, c->dg, c->coef, adj_args(c, k0 + reps - t, 0, 1),
                                         c->st);
                        t += 1;
                    }
                }
                CU(c, cudaEventRecord(c->ev1, c->st));
                CU(c, cudaEventSynchronize(c->ev1));
                CU(c, cudaEventElapsedTime(&t_ms, c->ev0, c->ev1));
                if (pass > 0) s_a = std::min(s_a, t_ms);
            }
            TRY(best_tiles(1, t_f, t_a, c->tile_warps_fwd1, c->tile_warps_adj1));
            if (tlog)
                std::fprintf(stderr, "tomo tune: one group: strip forward %.2f / tile %.2f us/step, strip adjoint "
                             "%.2f / tile %.2f us/step\n", 1e3 * s_f / reps, 1e3 * t_f / reps, 1e3 * s_a / reps,
                             1e3 * t_a / reps);
            c->tile_fwd1 = t_f < 0.97f * s_f;
            c->tile_adj1 = t_a < 0.97f * s_a;
        }
    }
    tile_override(c);
    CU(c, cudaGetLastError());
    if (cache && *cache) tune_cache_append(c, cache);
    return TOMO_OK;
}

// Memory plan: full forward history, or checkpoints every K slices with the chunk being swept
// recomputed; P groups resident per pass.
struct Plan {
    bool full;
    int K;    // slices per chunk (nt - 2 for full history)
    int P;    // groups per pass, 0: does not fit
};

// Device bytes one group of a pass holds under a plan: forward slots, adjoint ring, checkpoints
// and residual records.
double plan_bytes_per_group(const tomo_ctx* c, bool full, int K) {
    const Geometry& g = c->geo;
    const int64_t N = g.N, nt = g.nt;
    const int64_t slots = full ? nt : (int64_t)K + 1;
    const int64_t chunks = full ? 0 : (nt - 2 + K - 1) / K;
    return 4.0 * ((double)(slots + tomo_ctx::ZR + 2 * chunks) * N + (double)nt * g.nch);
}

// The plan with the most groups per pass that fits c->plan_budget (or the configured P).
Plan plan_of(const tomo_ctx* c, bool full, int K) {
    const Geometry& g = c->geo;
    Plan p{full, full ? g.nt - 2 : K, 0};
    const double per = plan_bytes_per_group(c, full, K);
    int P = g.cfg.groups_per_pass > 0 ? std::min(g.cfg.groups_per_pass, g.G) : g.G;
    if (g.cfg.groups_per_pass <= 0)
        while (P > 1 && per * P > c->plan_budget) --P;
    p.P = per * P <= c->plan_budget ? P : 0;
    return p;
}

void set_plan(tomo_ctx* c, const Plan& p) {
    const int nt = c->geo.nt;
    c->P = p.P;
    c->full = p.full;
    c->K = p.full ? nt - 2 : p.K;
    c->S = p.full ? nt : p.K + 1;
    c->nchunk = p.full ? 1 : (nt - 2 + p.K - 1) / p.K;
}

// Chosen memory plan.  ckpt_interval > 0 fixes K; 0 and -1 start from full history when it fits
// with all groups resident, else K = ceil(sqrt(2 (nt - 2))), the interval of least memory (-1
// then times the alternatives, tune_plan).
tomo_status make_plan(tomo_ctx* c) {
    const Geometry& g = c->geo;
    const int64_t N = g.N, nt = g.nt, G = g.G;
    size_t free_b = 0, total_b = 0;
    CU(c, cudaMemGetInfo(&free_b, &total_b));
    // fixed buffers (fields, coefficients, accumulators, records)
    const int64_t fixed = 4 * (7 * N) + 4 * (2 * G * N) + 4 * (2 * G * nt * g.nch) + 8 * (G * nt) +
                          8 * (int64_t)(G + 2) * reduce_blocks() + (int64_t)(64 << 20);
    double cap = 0.90 * (double)free_b;
    if (g.cfg.mem_limit_mb > 0) cap = std::min(cap, (double)g.cfg.mem_limit_mb * (1 << 20));
    c->plan_budget = cap - (double)fixed;
    const int K = g.cfg.ckpt_interval;
    Plan p{};
    if (K > 0) {
        if (K < nt - 2 && K < 2) return c->fail(TOMO_ERR_ARG, "ckpt_interval must be >= 2");
        p = plan_of(c, K >= nt - 2, K);
    } else {
        p = plan_of(c, true, 0);
        if (p.P < (g.cfg.groups_per_pass > 0 ? std::min<int64_t>(g.cfg.groups_per_pass, G) : G)) p = plan_of(c, false, std::max(2, (int)std::ceil(std::sqrt(2.0 * (double)(nt - 2)))));
    }
    if (p.P < 1)
        return c->fail(TOMO_ERR_OOM, "plan needs %.2f GB for one group per pass, %.2f GB available",
                       plan_bytes_per_group(c, p.full, p.K) / 1e9, c->plan_budget / 1e9);
    set_plan(c, p);
    return TOMO_OK;
}

// The buffers whose size the plan sets (forward slots, adjoint ring, checkpoints, residual
// records), zeroed.
tomo_status alloc_plan_buffers(tomo_ctx* c) {
    const Geometry& g = c->geo;
    const int64_t N = g.N, P = c->P;
    TRY(c->alloc(&c->hist, P * c->S * N, "forward slots"));
    TRY(c->alloc(&c->z, P * tomo_ctx::ZR * N, "adjoint slots"));
    if (!c->full) TRY(c->alloc(&c->ckpt, P * c->nchunk * 2 * N, "checkpoints"));
    TRY(c->alloc(&c->rr, P * g.nt * g.nch, "residual records"));
    CU(c, cudaMemsetAsync(c->hist, 0, sizeof(float) * (size_t)P * c->S * N, c->st));
    CU(c, cudaMemsetAsync(c->z, 0, sizeof(float) * (size_t)P * tomo_ctx::ZR * N, c->st));
    CU(c, cudaMemsetAsync(c->rr, 0, sizeof(float) * (size_t)(P * g.nt * g.nch), c->st));
    return TOMO_OK;
}

tomo_status create_buffers(tomo_ctx* c) {
    const Geometry& g = c->geo;
    const int64_t N = g.N, nt = g.nt, G = g.G, nch = g.nch;
    TRY(c->alloc(&c->f, N, "f"));
    TRY(c->alloc(&c->ftrue, N, "f_true"));
    TRY(c->alloc(&c->coef, N, "coef"));
    TRY(c->alloc(&c->rcoef, N, "rcoef"));
    TRY(c->alloc(&c->dir, N, "dir"));
    TRY(c->alloc(&c->tmp, N, "tmp"));
    TRY(alloc_plan_buffers(c));
    TRY(c->alloc(&c->corr, G * N, "correlation"));
    TRY(c->alloc(&c->meas, G * nt * nch, "measured records"));
    TRY(c->alloc(&c->rpart, G * nt, "residual partials"));
    TRY(c->alloc(&c->part, (G + 2) * (int64_t)reduce_blocks(), "reduction partials"));
    TRY(c->alloc(&c->sums, G + 8, "sums"));
    TRY(c->alloc(&c->maxabs, 1, "maxabs"));
    TRY(c->alloc(&c->mask, N, "mask"));
    TRY(c->alloc(&c->src, (int64_t)g.src.size(), "source"));
    TRY(c->alloc(&c->rcv, nch, "receivers"));
    if (g.ref) TRY(c->alloc(&c->box, 4 * G, "boxes"));
    else {
        TRY(c->alloc(&c->emit, G * g.gs, "emitters"));
        TRY(c->alloc(&c->rid, N, "receiver map"));
        c->rwords = ((g.nx + 31) / 32 + 31) / 32;
        TRY(c->alloc(&c->rbits, (int64_t)g.ny * c->rwords, "receiver row bitmap"));
        TRY(c->alloc(&c->dmap, N, "sponge map"));
    }
    CU(c, cudaMemsetAsync(c->meas, 0, sizeof(float) * G * nt * nch, c->st));
    CU(c, cudaMemsetAsync(c->rpart, 0, sizeof(double) * G * nt, c->st));
    CU(c, cudaMemsetAsync(c->f, 0, sizeof(float) * N, c->st));
    CU(c, cudaMemcpyAsync(c->mask, g.mask.data(), N, cudaMemcpyHostToDevice, c->st));
    CU(c, cudaMemcpyAsync(c->src, g.src.data(), sizeof(float) * g.src.size(), cudaMemcpyHostToDevice, c->st));
    CU(c, cudaMemcpyAsync(c->rcv, g.rcv.data(), sizeof(int32_t) * nch, cudaMemcpyHostToDevice, c->st));
    if (g.ref) CU(c, cudaMemcpyAsync(c->box, g.box.data(), sizeof(int32_t) * 4 * G, cudaMemcpyHostToDevice, c->st));
    else {
        CU(c, cudaMemcpyAsync(c->emit, g.emit.data(), sizeof(int32_t) * G * g.gs, cudaMemcpyHostToDevice, c->st));
        CU(c, cudaMemcpyAsync(c->rid, g.rid.data(), sizeof(int32_t) * N, cudaMemcpyHostToDevice, c->st));
        std::vector<uint32_t> bits((size_t)g.ny * c->rwords, 0u);
        for (int64_t q = 0; q < N; ++q)
            if (g.rid[q] >= 0) {
                const int b = (int)(q % g.nx) >> 5;
                bits[(size_t)(q / g.nx) * c->rwords + (b >> 5)] |= 1u << (b & 31);
            }
        CU(c, cudaMemcpyAsync(c->rbits, bits.data(), sizeof(uint32_t) * bits.size(), cudaMemcpyHostToDevice, c->st));
        TRY(sync_check(c));   // `bits` is local
    }
    TRY(sync_check(c));
    DevGeo& d = c->dg;
    d.nx = g.nx; d.ny = g.ny; d.nt = g.nt; d.nch = g.nch;
    d.lo = g.lo; d.hi = g.hi; d.gs = g.gs;
    d.sponge_w = g.cfg.sponge_width; d.sponge_max = g.cfg.sponge_max;
    fill_damp(d);
    d.box = c->box; d.emit = c->emit; d.rcv = c->rcv; d.rid = c->rid; d.rbits = c->rbits; d.rwords = c->rwords; d.src = c->src;
    d.n_src_steps = g.n_src_steps;
    if (!g.ref) {
        // per-cell sponge factor: the damp table by distance to the nearest edge
        std::vector<float> dm((size_t)N, 1.f);
        for (int j = 0; j < g.ny; ++j)
            for (int i = 0; i < g.nx; ++i) {
                const int dd = std::min(std::min(i, j), std::min(g.nx - 1 - i, g.ny - 1 - j));
                if (dd < d.sponge_w) dm[(size_t)j * g.nx + i] = d.damp[dd];
            }
        CU(c, cudaMemcpyAsync(c->dmap, dm.data(), sizeof(float) * N, cudaMemcpyHostToDevice, c->st));
        TRY(sync_check(c));   // `dm` is local
        d.dmap = c->dmap;
    }
    c->strip = strip_supported(d, g.cfg.profile) && !std::getenv("TOMO_NO_STRIP");
    // the tile kernels' wait time-out word, written by the device, read by sync_check
    CU(c, cudaHostAlloc((void**)&c->err_host, sizeof(unsigned int), cudaHostAllocMapped));
    *c->err_host = 0u;
    CU(c, cudaHostGetDevicePointer((void**)&c->err_dev, c->err_host, 0));
    if (const char* e = std::getenv("TOMO_WAIT_LIMIT_NS")) c->wait_ns = std::strtoull(e, nullptr, 10);
    if (const char* e = std::getenv("TOMO_TEST_UNDELIVERED_TX")) c->test_tx = (uint32_t)std::strtoul(e, nullptr, 10);
    if (const char* e = std::getenv("TOMO_TEST_GRID_BARRIER_EXTRA")) c->test_gbar = (uint32_t)std::strtoul(e, nullptr, 10);
    if (const char* e = std::getenv("TOMO_PERSIST")) c->persist = *e && *e != '0';
    TRY(c->alloc(&c->gbar, 1, "grid barrier"));
    encode_maps(c);
    CU(c, cudaMemsetAsync(c->corr, 0, sizeof(float) * (size_t)G * N, c->st));
    TRY(sync_check(c));
    return TOMO_OK;
}

// Records the launch sequence of one pass (groups g0 .. g0+ng-1) on the stream.
// Kernel nodes the recorded pass contains (each launch_* call below is one kernel).
int64_t record_pass(tomo_ctx* c, int mode, int g0, int ng) {
    int64_t n = 0;
    // multi-step tile kernels: the choice made for passes of one group when the pass has one
    const bool tile_fwd = ng == 1 ? c->tile_fwd1 : c->tile_fwd;
    const bool tile_adj = ng == 1 ? c->tile_adj1 : c->tile_adj;
    const Geometry& g = c->geo;
    const int nt = g.nt, S = c->S, K = c->K;
    const int64_t N = g.N, gstride = (int64_t)S * N, nch = g.nch, rpg = c->recs_per_group();
    void* st = c->st;
    // ---- forward sweep
    launch_zero_slots(c->hist, ng, gstride, c->slot(0), c->slot(1), N, st);
    ++n;
    const float* meas_g = c->meas + (int64_t)g0 * rpg;
    const bool resid = mode == MODE_GRAD || mode == MODE_RESID;
    float* out_g = resid ? c->rr : c->rec + (int64_t)g0 * rpg;
    if (mode == MODE_ILLUM) {
        for (int k = 1; k <= nt - 2; ++k) {
            fwd_launch(c, fwd_args(c, k, g0, ng));
            launch_illum_add(c->hist + c->slot(k + 1), ng, gstride, N, c->illum, st);
            n += 2;
        }
        return n;
    }
    // checkpoint copy of slice m: chunk ch >= 1 starts at qa = 1 + ch*K and keeps slices qa-1 and qa
    auto ck_of = [&](FwdStep& fs, int m) {
        if (mode != MODE_GRAD || c->full) return;
        int ch = -1, which = 0;
        if (m % K == 0) { ch = m / K; which = 0; }
        else if ((m - 1) % K == 0) { ch = (m - 1) / K; which = 1; }
        if (ch >= 1 && ch < c->nchunk) {
            fs.ck = c->ckpt + ((int64_t)ch * 2 + which) * N;
            fs.ckstride = (int64_t)c->nchunk * 2 * N;
        }
    };
    // persistent tile segments (opt-in): one cooperative launch per sweep segment where every block
    // fits, a grid barrier between its chunks.  Measured slower than one launch per chunk with
    // programmatic dependent launch (128x128: 1.57 against 1.45 ms per iteration; ART on 512x512:
    // 272 against 265 ms): the barrier and the region copy after it cost more than the launch gap
    // the overlapped launches already hide.
    const bool persist_fwd = tile_fwd && c->persist &&
                             tile_persistent_fits(c->dg, ng == 1 ? c->tile_warps_fwd1 : c->tile_warps_fwd, true, ng);
    const bool persist_adj = tile_adj && c->persist &&
                             tile_persistent_fits(c->dg, ng == 1 ? c->tile_warps_adj1 : c->tile_warps_adj, false, ng);
    if (tile_fwd) {
        // multi-step tile launches: every slice 2 .. nt-1 is recorded by the launch computing it
        for (int k = 1; k <= nt - 2;) {
            const int T = tile_fwd_steps(c, nt - 1 - k);
            TileFwd a = tile_fwd_args(c, k, T, g0, ng);
            if (mode == MODE_GRAD && !c->full) {
                a.ckpt = c->ckpt;
                a.ckstride = (int64_t)c->nchunk * 2 * N;
            }
            a.gmeas = resid ? meas_g : nullptr;
            a.gout = out_g;
            if (persist_fwd) {
                cudaMemsetAsync(c->gbar, 0, sizeof(unsigned int), (cudaStream_t)st);
                a.k_last = nt - 1;
                k = nt - 1;
            } else {
                k += T;
            }
            launch_fwd_tile(c->dg, c->tmaps, a, st);
            ++n;
        }
        if (resid) {
            launch_resid_parts(c->rr, ng, nt, (int)nch, c->rpart + (int64_t)g0 * nt, st);
            ++n;
        }
    }
    int gnext = 2;   // strip path: slices 2 .. gnext-1 are recorded, in order
    for (int k = 1; k <= nt - 2 && !tile_fwd;) {
        FwdStep fs = fwd_args(c, k, g0, ng);
        const int m = k + 1;
        ck_of(fs, m);
        if (c->strip) {
            fs.gmeas = resid ? meas_g : nullptr;
            fs.gout = out_g;
            if (c->fwd_pair && k + 1 <= nt - 2) {
                // slices k+1 and k+2; records slices k-1 and k from the launch's inputs
                FwdStep fb = fwd_args(c, k + 1, g0, ng);
                ck_of(fb, m + 1);
                const bool gp = (k - 1 == gnext);
                if (gp) ++gnext;
                const bool gc = (k == gnext);
                if (gc) ++gnext;
                launch_fwd2_strip(c->rows_fwd2, c->dg, c->coef, fs, fb, gp, gc, st);
                k += 2;
            } else {
                // slice k is gathered by the launch that computes slice k+1
                fs.gk = (k == gnext) ? k : -1;
                if (k == gnext) ++gnext;
                fwd_launch(c, fs);
                k += 1;
            }
            ++n;
            continue;
        }
        fwd_launch(c, fs);
        GatherStep gs{};
        gs.g0 = g0;
        gs.u = c->hist + c->slot(m);
        gs.gstride = gstride;
        gs.k = m;
        gs.ng = ng;
        gs.meas = resid ? meas_g : nullptr;
        gs.out = out_g;
        gs.part = resid ? c->rpart + (int64_t)g0 * nt : nullptr;
        launch_gather(c->dg, gs, st);
        n += 2;
        k += 1;
    }
    if (c->strip && !tile_fwd) {
        for (int m = std::max(gnext, 2); m < nt - 1; ++m) {   // slices left before the last
            GatherStep gs{};
            gs.g0 = g0;
            gs.u = c->hist + c->slot(m);
            gs.gstride = gstride;
            gs.k = m;
            gs.ng = ng;
            gs.meas = resid ? meas_g : nullptr;
            gs.out = out_g;
            launch_gather(c->dg, gs, st);
            ++n;
        }
    }
    if (c->strip && !tile_fwd) {
        GatherStep gs{};
        gs.g0 = g0;
        gs.u = c->hist + c->slot(nt - 1);
        gs.gstride = gstride;
        gs.k = nt - 1;
        gs.ng = ng;
        gs.meas = resid ? meas_g : nullptr;
        gs.out = out_g;
        launch_gather(c->dg, gs, st);
        ++n;
        if (resid) {
            launch_resid_parts(c->rr, ng, nt, (int)nch, c->rpart + (int64_t)g0 * nt, st);
            ++n;
        }
    }
    if (mode != MODE_GRAD) return n;
    // ---- adjoint sweep, chunks in reverse
    cudaMemsetAsync(c->z, 0, sizeof(float) * tomo_ctx::ZR * N * ng, (cudaStream_t)st);
    cudaMemsetAsync(c->corr + (int64_t)g0 * N, 0, sizeof(float) * N * ng, (cudaStream_t)st);
    for (int ch = c->nchunk - 1; ch >= 0; --ch) {
        const int qa = 1 + ch * K, qb = std::min(qa + K - 1, nt - 2);
        if (!c->full) {
            const bool in_ring = (ch == c->nchunk - 1) && (qa - 1 >= nt - S);
            if (!in_ring) {
                if (ch == 0) {
                    launch_zero_slots(c->hist, ng, gstride, c->slot(qa - 1), c->slot(qa), N, st);
                    ++n;
                } else {
                    n += 2;
                    const int64_t cks = (int64_t)c->nchunk * 2 * N;
                    launch_copy_groups(c->hist + c->slot(qa - 1), gstride, c->ckpt + ((int64_t)ch * 2 + 0) * N, cks,
                                       ng, N, st);
                    launch_copy_groups(c->hist + c->slot(qa), gstride, c->ckpt + ((int64_t)ch * 2 + 1) * N, cks, ng,
                                       N, st);
                }
                for (int m = qa + 1; m <= qb;) {
                    if (tile_fwd) {
                        const int T = tile_fwd_steps(c, qb - m + 1);
                        TileFwd a = tile_fwd_args(c, m - 1, T, g0, ng);
                        if (persist_fwd) {
                            cudaMemsetAsync(c->gbar, 0, sizeof(unsigned int), (cudaStream_t)st);
                            a.k_last = qb;
                            m = qb + 1;
                        } else {
                            m += T;
                        }
                        launch_fwd_tile(c->dg, c->tmaps, a, st);
                    } else if (c->strip && c->fwd_pair && m + 1 <= qb) {
                        launch_fwd2_strip(c->rows_fwd2, c->dg, c->coef, fwd_args(c, m - 1, g0, ng),
                                          fwd_args(c, m, g0, ng), false, false, st);
                        m += 2;
                    } else {
                        fwd_launch(c, fwd_args(c, m - 1, g0, ng));
                        m += 1;
                    }
                    ++n;
                }
            }
        }
        for (int q = qb; q >= qa;) {
            if (tile_adj) {
                const int T = tile_adj_steps(q - qa + 1);
                TileAdj a = tile_adj_args(c, q + 1, T, g0, ng);
                if (persist_adj) {
                    cudaMemsetAsync(c->gbar, 0, sizeof(unsigned int), (cudaStream_t)st);
                    a.kz_last = qa + 1;
                    q = qa - 1;
                } else {
                    q -= T;
                }
                launch_adj_tile(c->dg, c->tmaps, a, st);
            } else if (c->adj_pair && q - 1 >= qa) {
                launch_adj2_strip(c->rows_adj2, c->dg, c->coef, adj_args(c, q, g0, ng), adj_args(c, q - 1, g0, ng), st);
                q -= 2;
            } else {
                adj_launch(c, adj_args(c, q, g0, ng));
                q -= 1;
            }
            ++n;
        }
    }
    return n;
}

// Slice layout of one gradient pass.  A pass of fewer groups than the plan keeps resident (the
// one-group passes of ART, the last pass of a P-of-M plan) spreads its groups' slices over the
// whole slot buffer, L = P S / ng slots per group: it checkpoints less often and recomputes fewer
// steps (full history when nt slices fit) in the same memory.  With the fewest chunks L slots
// allow, K is the smallest interval that still leaves the last chunk in the ring after the
// forward sweep (nchunk K >= nt - 1), so only the other chunks are recomputed.  Checkpoints
// hold exact slices, so the pass gives the same bits either way.
struct PassLayout {
    int S, K, nchunk;
    bool full;
    bool in_ckpt;   // the pass's slices live in the checkpoint buffer (full history, no checkpoints)
};
PassLayout pass_layout(const tomo_ctx* c, int mode, int ng) {
    const PassLayout plan{c->S, c->K, c->nchunk, c->full, false};
    if (mode != MODE_GRAD || c->full || ng >= c->P || std::getenv("TOMO_FIXED_PASS_LAYOUT")) return plan;
    const int nt = c->geo.nt;
    const int64_t L = (int64_t)c->P * c->S / ng;
    if (L >= nt) return PassLayout{nt, nt - 2, 1, true, false};
    // a pass with full history needs no checkpoints: the checkpoint buffer (P nchunk 2 slices)
    // holds the history when the slot buffer does not (tile kernels need its maps)
    const bool ck_maps = !(ng == 1 ? c->tile_fwd1 || c->tile_adj1 : c->tile_fwd || c->tile_adj) || c->tmaps_ck.ok;
    if ((int64_t)c->P * c->nchunk * 2 / ng >= nt && ck_maps) return PassLayout{nt, nt - 2, 1, true, true};
    int nchunk = (int)((nt - 2 + L - 2) / (L - 1));
    int K = (nt - 1 + nchunk - 1) / nchunk;
    if (K + 1 > L) {
        ++nchunk;
        K = (nt - 1 + nchunk - 1) / nchunk;
    }
    if (K <= c->K) return plan;
    return PassLayout{K + 1, K, (nt - 2 + K - 1) / K, false, false};
}

// Applies a pass layout to the context while a pass is recorded, and restores the plan's.
struct LayoutScope {
    tomo_ctx* c;
    PassLayout keep;
    bool swapped;
    LayoutScope(tomo_ctx* ctx, const PassLayout& l)
        : c(ctx), keep{ctx->S, ctx->K, ctx->nchunk, ctx->full, false}, swapped(l.in_ckpt) {
        c->S = l.S;
        c->K = l.K;
        c->nchunk = l.nchunk;
        c->full = l.full;
        if (swapped) {
            std::swap(c->hist, c->ckpt);
            std::swap(c->tmaps, c->tmaps_ck);
        }
    }
    ~LayoutScope() {
        if (swapped) {
            std::swap(c->hist, c->ckpt);
            std::swap(c->tmaps, c->tmaps_ck);
        }
        c->S = keep.S;
        c->K = keep.K;
        c->nchunk = keep.nchunk;
        c->full = keep.full;
    }
};

tomo_status run_pass(tomo_ctx* c, int mode, int g0, int ng) {
    const auto key = std::make_tuple(mode, g0, ng);
    auto it = c->graphs.find(key);
    if (it == c->graphs.end()) {
        TRY(autotune(c));
        LayoutScope layout(c, pass_layout(c, mode, ng));
        cudaGraph_t graph = nullptr;
        CU(c, cudaStreamBeginCapture(c->st, cudaStreamCaptureModeThreadLocal));
        const int64_t nk = record_pass(c, mode, g0, ng);
        const cudaError_t e = cudaStreamEndCapture(c->st, &graph);
        if (e != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            return c->cuda(e, "cudaStreamEndCapture");
        }
        cudaGraphExec_t exec = nullptr;
        const cudaError_t e2 = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e2 != cudaSuccess) return c->cuda(e2, "cudaGraphInstantiate");
        it = c->graphs.emplace(key, exec).first;
        c->graph_kernels[key] = nk;
    }
    CU(c, cudaGraphLaunch(it->second, c->st));
    c->launches += c->graph_kernels[key];
    return TOMO_OK;
}

tomo_status ensure_rec(tomo_ctx* c) {
    if (!c->rec) TRY(c->alloc(&c->rec, (int64_t)c->geo.G * c->recs_per_group(), "simulated records"));
    return TOMO_OK;
}

// Forward sweep of every group into c->rec.
tomo_status forward_all(tomo_ctx* c, float* u_last_host) {
    TRY(ensure_rec(c));
    const Geometry& g = c->geo;
    CU(c, cudaMemsetAsync(c->rec, 0, sizeof(float) * (size_t)g.G * c->recs_per_group(), c->st));
    launch_coef(g.cfg.profile, c->f, c->coef, c->rcoef, g.N, g.cfg.courant, c->st);
    for (int g0 = 0; g0 < g.G; g0 += c->P) {
        const int ng = std::min(c->P, g.G - g0);
        TRY(run_pass(c, MODE_FWD, g0, ng));
        if (u_last_host)
            for (int gl = 0; gl < ng; ++gl)
                CU(c, cudaMemcpyAsync(u_last_host + (int64_t)(g0 + gl) * g.N,
                                      c->hist + (int64_t)gl * c->S * g.N + c->slot(g.nt - 1), sizeof(float) * g.N,
                                      cudaMemcpyDeviceToHost, c->st));
    }
    return TOMO_OK;
}

// Noise key of the next residual sweep (kind 2: a new draw each sweep).
tomo_status next_noise_draw(tomo_ctx* c) {
    if (c->noise_kind != 2) return TOMO_OK;
    uint64_t z = c->noise_seed + 0x9E3779B97F4A7C15ull * (++c->noise_draws);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    c->noise_key_host = z ^ (z >> 31);
    CU(c, cudaMemcpyAsync(c->noise_key, &c->noise_key_host, sizeof(uint64_t), cudaMemcpyHostToDevice, c->st));
    return TOMO_OK;
}

// Correlations of all groups for the current c->f (SIRT), residual partials.
tomo_status gradient_all(tomo_ctx* c) {
    TRY(next_noise_draw(c));
    const Geometry& g = c->geo;
    launch_coef(g.cfg.profile, c->f, c->coef, c->rcoef, g.N, g.cfg.courant, c->st);
    ++c->launches;
    for (int g0 = 0; g0 < g.G; g0 += c->P) TRY(run_pass(c, MODE_GRAD, g0, std::min(c->P, g.G - g0)));
    return TOMO_OK;
}

// Replaces the plan-sized buffers by those of plan p (contents zeroed); captured graphs and the
// kernel choice, both made for the old plan, are dropped.
tomo_status apply_plan(tomo_ctx* c, const Plan& p) {
    if (c->full == p.full && c->P == p.P && (p.full || c->K == p.K)) return TOMO_OK;
    TRY(sync_check(c));
    c->drop_graphs();
    c->release(&c->hist);
    c->release(&c->z);
    c->release(&c->ckpt);
    c->release(&c->rr);
    set_plan(c, p);
    c->tuned = false;
    ++c->gen;
    TRY(alloc_plan_buffers(c));
    encode_maps(c);
    return TOMO_OK;
}

// Cache line of a timed plan choice: the problem, then full history (0/1), K and P.
std::string plan_key(const tomo_ctx* c) {
    char b[160];
    std::snprintf(b, sizeof b, "tomo-plan-1 %d %d %d %d %d %d %d", c->geo.cfg.profile, c->geo.nx, c->geo.ny,
                  c->geo.nt, c->geo.G, c->geo.gs, c->geo.cfg.groups_per_pass);
    return b;
}

// ckpt_interval = -1: times one gradient pass (the first P groups: forward sweep, checkpoints,
// recompute, adjoint and correlation, as a captured graph, after one untimed pass that also
// picks the pass's kernels) under each candidate plan that fits the budget -- full history,
// two chunks (K = (nt - 2) / 2, half the recompute of the smallest interval), the interval of
// least memory K = ceil(sqrt(2 (nt - 2))), and an interval whose chunk of the pass fits in half
// the L2 (the adjoint then reads recomputed slices from L2) -- and keeps the plan of the least
// estimated iteration time, passes x pass time.  The plans give the same results bit for bit
// (checkpoints hold exact slices).  TOMO_TUNE_CACHE records and reuses the choice.
tomo_status tune_plan(tomo_ctx* c) {
    const Geometry& g = c->geo;
    const int nt = g.nt, G = g.G;
    std::vector<Plan> cands;
    auto add = [&](bool full, int K) {
        if (!full && (K < 4 || K >= nt - 2)) return;
        const Plan p = plan_of(c, full, K);
        if (p.P < 1) return;
        for (const Plan& q : cands)
            if (q.full == p.full && q.K == p.K) return;
        cands.push_back(p);
    };
    const int Ks = std::max(4, (int)std::ceil(std::sqrt(2.0 * (double)(nt - 2))));
    add(true, 0);
    add(false, (nt - 1) / 2);
    add(false, Ks);
    int l2 = 0;
    CU(c, cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, c->dev));
    const Plan ps = plan_of(c, false, Ks);
    if (ps.P >= 1) add(false, (int)(0.5 * (double)l2 / (4.0 * (double)g.N * ps.P)) - 1);
    if (cands.empty()) return TOMO_OK;   // make_plan's plan stands
    const char* cache = std::getenv("TOMO_TUNE_CACHE");
    const std::string key = plan_key(c);
    int chosen = -1;
    if (cache && *cache) {
        if (FILE* fp = std::fopen(cache, "r")) {
            char line[512];
            while (chosen < 0 && std::fgets(line, sizeof line, fp)) {
                int full = 0, K = 0, P = 0;
                if (std::strncmp(line, key.c_str(), key.size()) != 0 || line[key.size()] != ' ' ||
                    std::sscanf(line + key.size(), "%d %d %d", &full, &K, &P) != 3)
                    continue;
                for (size_t i = 0; i < cands.size(); ++i)
                    if (cands[i].full == (full != 0) && cands[i].K == K && cands[i].P == P) chosen = (int)i;
            }
            std::fclose(fp);
        }
    }
    const bool tlog = std::getenv("TOMO_TUNE_LOG") != nullptr;
    if (chosen < 0 && cands.size() == 1) chosen = 0;
    if (chosen < 0) {
        double best = 1e300;
        for (size_t i = 0; i < cands.size(); ++i) {
            const Plan& p = cands[i];
            TRY(apply_plan(c, p));
            launch_coef(g.cfg.profile, c->f, c->coef, c->rcoef, g.N, g.cfg.courant, c->st);
            TRY(run_pass(c, MODE_GRAD, 0, p.P));
            CU(c, cudaEventRecord(c->ev0, c->st));
            TRY(run_pass(c, MODE_GRAD, 0, p.P));
            CU(c, cudaEventRecord(c->ev1, c->st));
            CU(c, cudaEventSynchronize(c->ev1));
            float ms = 0.f;
            CU(c, cudaEventElapsedTime(&ms, c->ev0, c->ev1));
            const double est = (double)ms * ((G + p.P - 1) / p.P);
            if (tlog)
                std::fprintf(stderr, "tomo tune: plan %s K %d, %d groups per pass: pass %.3f ms, iteration %.3f ms\n",
                             p.full ? "full history" : "checkpoints", c->K, p.P, ms, est);
            if (est < best) { best = est; chosen = (int)i; }
        }
        if (cache && *cache)
            if (FILE* fp = std::fopen(cache, "a")) {
                std::fprintf(fp, "%s %d %d %d\n", key.c_str(), cands[chosen].full ? 1 : 0, cands[chosen].K,
                             cands[chosen].P);
                std::fclose(fp);
            }
    }
    TRY(apply_plan(c, cands[chosen]));
    // leave the state of a fresh context
    CU(c, cudaMemsetAsync(c->hist, 0, sizeof(float) * (size_t)c->P * c->S * g.N, c->st));
    CU(c, cudaMemsetAsync(c->z, 0, sizeof(float) * (size_t)c->P * tomo_ctx::ZR * g.N, c->st));
    CU(c, cudaMemsetAsync(c->rr, 0, sizeof(float) * (size_t)c->P * nt * g.nch, c->st));
    CU(c, cudaMemsetAsync(c->corr, 0, sizeof(float) * (size_t)G * g.N, c->st));
    CU(c, cudaMemsetAsync(c->rpart, 0, sizeof(double) * (size_t)G * nt, c->st));
    TRY(sync_check(c));
    c->launches = 0;
    return TOMO_OK;
}

double sched_scale(const tomo_schedule* s, int it) {
    switch (s->kind) {
    case TOMO_SCHED_CONST: return s->omega;
    case TOMO_SCHED_POWER: return (double)s->omega * ((double)s->alpha + (double)s->beta / std::pow((double)(it + 1), (double)s->gamma));
    case TOMO_SCHED_LINEAR: return (double)s->omega * ((double)s->alpha + (double)s->beta * (double)(it + 1));
    default: return std::numeric_limits<double>::quiet_NaN();
    }
}

tomo_status apply_dir(tomo_ctx* c, const tomo_schedule* s, double scale) {
    const unsigned int* mx = nullptr;
    if (s->normalize) {
        launch_maxabs(c->dir, c->mask, c->geo.N, c->maxabs, c->st);
        mx = c->maxabs;
        ++c->launches;
    }
    launch_apply(c->f, c->dir, c->mask, c->geo.N, scale, mx, c->st);
    ++c->launches;
    return TOMO_OK;
}

// Sum of the residual partials of all groups -> host.
tomo_status residual_norm(tomo_ctx* c, double* out) {
    const Geometry& g = c->geo;
    launch_sum_parts(c->rpart, 1, g.G * g.nt, c->sums, c->st);
    ++c->launches;
    CU(c, cudaMemcpyAsync(out, c->sums, sizeof(double), cudaMemcpyDeviceToHost, c->st));
    return TOMO_OK;
}

tomo_status epsilon(tomo_ctx* c, double* out) {
    const int nb = reduce_blocks();
    launch_eps_parts(c->f, c->ftrue, c->geo.N, c->part, nb, c->st);
    launch_sum_parts(c->part, 2, nb, c->sums + 2, c->st);
    c->launches += 2;
    double ab[2];
    CU(c, cudaMemcpyAsync(ab, c->sums + 2, sizeof ab, cudaMemcpyDeviceToHost, c->st));
    TRY(sync_check(c));
    *out = 100.0 * std::sqrt(ab[0]) / std::sqrt(ab[1]);
    return TOMO_OK;
}

// The update rule of a SIRT method from the correlations of all groups held in c->corr, applied
// to c->f (every method but ART, which updates after each group).
tomo_status update_core(tomo_ctx* c, int method, const tomo_schedule* sch, double s) {
    const Geometry& g = c->geo;
    const int64_t N = g.N;
    const int G = g.G;
    const double sc = g.corr_scale;
    const int nb = reduce_blocks();
    switch (method) {
    case TOMO_SIRT_CLASSIC:
        launch_combine(c->corr, G, N, c->f, sc, nullptr, 1.0, c->dir, c->st);
        ++c->launches;
        TRY(apply_dir(c, sch, s));
        break;
    case TOMO_SIRT_SCALED:
    case TOMO_SIRT_WEIGHT:
    case TOMO_SIRT_AVG:
        launch_combine(c->corr, G, N, c->f, sc, nullptr, 1.0 / G, c->dir, c->st);
        ++c->launches;
        TRY(apply_dir(c, sch, s));
        break;
    case TOMO_SIRT_NORM: {
        // mean, per-group deviation norms, inverse-norm weights (sirt-mimo-norm.cu:56-118)
        // weights on the device: no host round trip inside the iteration
        launch_combine(c->corr, G, N, c->f, sc, nullptr, 1.0 / G, c->tmp, c->st);
        launch_group_dev_norm(c->corr, G, N, c->f, sc, c->tmp, c->part, nb, c->st);
        launch_sum_parts(c->part, G, nb, c->sums, c->st);
        launch_norm_weights(c->sums, G, c->st);
        launch_combine(c->corr, G, N, c->f, sc, c->sums, 1.0, c->dir, c->st);
        c->launches += 5;
        TRY(apply_dir(c, sch, s));
        break;
    }
    case TOMO_SIRT_AVG_WEIGHT: {
        // fg = f + s*mask*df_g; f += sum_g fg/||fg - mean fg|| (sirt-mimo-avg-weight.cu:130-203)
        launch_avgw_fbar(c->corr, G, N, c->f, c->mask, sc, s, c->tmp, c->st);
        launch_avgw_norm(c->corr, G, N, c->f, c->mask, sc, s, c->tmp, c->part, nb, c->st);
        launch_sum_parts(c->part, G, nb, c->sums, c->st);
        launch_avgw_apply(c->corr, G, N, c->f, c->mask, sc, s, c->sums, c->st);
        c->launches += 4;
        break;
    }
    default:
        return c->fail(TOMO_ERR_ARG, "method %d has no update from held correlations", method);
    }
    return TOMO_OK;
}

// Fills the iteration statistics from the events ev0/ev1 around the iteration's device work.
void fill_stats(tomo_ctx* c, tomo_iter_stats* stats, double eps, double r2, double s, double groups,
                int64_t launches0) {
    if (!stats) return;
    const Geometry& g = c->geo;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, c->ev0, c->ev1);
    stats->epsilon = eps;
    stats->resid_norm2 = r2;
    stats->scale = s;
    stats->seconds = ms * 1e-3;
    stats->cell_updates = 2.0 * groups * (double)(g.nt - 2) * (double)g.N;
    stats->kernel_launches = (double)(c->launches - launches0);
}

// One iteration on c->f with c->meas; f_true in c->ftrue when have_true.
// One iteration of a SIRT method (not ART) on the context's stream with no host
// synchronisation, to be recorded into a batch graph: the passes are recorded in place rather
// than launched as their own graphs, the residual norm and the image-error sums land in pinned
// memory (pin[0], pin[1..2]).  The same launches, in the same order, as iterate_core.
tomo_status enqueue_iteration(tomo_ctx* c, int method, const tomo_schedule* sch, double s, float* d_f,
                              const float* d_ft, int64_t* kernels) {
    const Geometry& g = c->geo;
    const int64_t N = g.N, l0 = c->launches;
    CU(c, cudaMemcpyAsync(c->f, d_f, sizeof(float) * N, cudaMemcpyDeviceToDevice, c->st));
    if (d_ft) CU(c, cudaMemcpyAsync(c->ftrue, d_ft, sizeof(float) * N, cudaMemcpyDeviceToDevice, c->st));
    launch_coef(g.cfg.profile, c->f, c->coef, c->rcoef, N, g.cfg.courant, c->st);
    ++c->launches;
    for (int g0 = 0; g0 < g.G; g0 += c->P) {
        const int ng = std::min(c->P, g.G - g0);
        LayoutScope layout(c, pass_layout(c, MODE_GRAD, ng));
        c->launches += record_pass(c, MODE_GRAD, g0, ng);
    }
    launch_sum_parts(c->rpart, 1, g.G * g.nt, c->sums, c->st);
    ++c->launches;
    CU(c, cudaMemcpyAsync(c->pin, c->sums, sizeof(double), cudaMemcpyDeviceToHost, c->st));
    TRY(update_core(c, method, sch, s));
    if (d_ft) {
        const int nb = reduce_blocks();
        launch_eps_parts(c->f, c->ftrue, N, c->part, nb, c->st);
        launch_sum_parts(c->part, 2, nb, c->sums + 2, c->st);
        c->launches += 2;
        CU(c, cudaMemcpyAsync(c->pin + 1, c->sums + 2, 2 * sizeof(double), cudaMemcpyDeviceToHost, c->st));
    }
    CU(c, cudaMemcpyAsync(d_f, c->f, sizeof(float) * N, cudaMemcpyDeviceToDevice, c->st));
    *kernels = c->launches - l0;
    return TOMO_OK;
}

// Records one iteration of every context of a batch into one CUDA graph: a capture on the
// leading context's stream forks into every context's stream (an event each way), so the
// phantoms' launches are independent branches of one graph, replayed by one launch per
// iteration.  The graph stays with the leading context, keyed by the contexts (serial numbers
// and generations), the field pointers, the method and the step.
tomo_status record_batch_graph(tomo_ctx** ctxs, int n, int method, const tomo_schedule* sched, double s, float** d_f,
                               const float** d_ft, const std::vector<uint64_t>& key) {
    tomo_ctx* lead = ctxs[0];
    if (lead->batch_exec) {
        cudaGraphExecDestroy(lead->batch_exec);
        lead->batch_exec = nullptr;
        lead->batch_key.clear();
    }
    for (int i = 0; i < n; ++i) {
        tomo_ctx* c = ctxs[i];
        if (!c->evj) CU(c, cudaEventCreateWithFlags(&c->evj, cudaEventDisableTiming));
        if (!c->pin) CU(c, cudaHostAlloc((void**)&c->pin, 4 * sizeof(double), cudaHostAllocDefault));
    }
    cudaEvent_t fork = nullptr;
    CU(lead, cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
    std::vector<int64_t> kernels(n, 0);
    tomo_status st = TOMO_OK;
    cudaGraph_t graph = nullptr;
    // the capture runs on a stream of its own so that every context (the leading one included)
    // joins it the same way
    cudaStream_t cs = nullptr;
    cudaError_t e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        cudaEventRecord(fork, cs);
        for (int i = 0; i < n && st == TOMO_OK; ++i) {
            tomo_ctx* c = ctxs[i];
            cudaStreamWaitEvent(c->st, fork, 0);
            st = enqueue_iteration(c, method, sched, s, d_f[i], d_ft ? d_ft[i] : nullptr, &kernels[i]);
            cudaEventRecord(c->evj, c->st);
            cudaStreamWaitEvent(cs, c->evj, 0);
        }
        const cudaError_t e2 = cudaStreamEndCapture(cs, &graph);
        if (st == TOMO_OK && e2 != cudaSuccess) st = lead->cuda(e2, "cudaStreamEndCapture (batch)");
    } else {
        st = lead->cuda(e, "batch capture");
    }
    if (st == TOMO_OK) {
        cudaGraphExec_t exec = nullptr;
        e = cudaGraphInstantiate(&exec, graph, 0);
        if (e != cudaSuccess) st = lead->cuda(e, "cudaGraphInstantiate (batch)");
        else {
            lead->batch_exec = exec;
            lead->batch_key = key;
            lead->batch_kernels = kernels;
        }
    }
    if (graph) cudaGraphDestroy(graph);
    if (cs) cudaStreamDestroy(cs);
    cudaEventDestroy(fork);
    cudaGetLastError();
    return st;
}

// A batch runs as one graph when every iteration is device work only: a SIRT method (not ART),
// one device, one step size for all the call's iterations (it is recorded in the graph), no
// noise redrawn per sweep, measured records set.  TOMO_BATCH_THREADS=1 keeps the threaded path.
bool batch_graph_eligible(tomo_ctx** ctxs, int n, int method, const tomo_schedule* sched, int iter0, int iters) {
    if (method < TOMO_SIRT_CLASSIC || method > TOMO_SIRT_AVG_WEIGHT || iters < 1) return false;
    if (const char* e = std::getenv("TOMO_BATCH_THREADS"))
        if (*e && *e != '0') return false;
    const double s0 = sched_scale(sched, iter0);
    if (!std::isfinite(s0)) return false;
    for (int it = 1; it < iters; ++it)
        if (sched_scale(sched, iter0 + it) != s0) return false;
    for (int i = 0; i < n; ++i)
        if (ctxs[i]->dev != ctxs[0]->dev || ctxs[i]->noise_kind == 2 || !ctxs[i]->meas_set) return false;
    return true;
}

// Batch iterations as replays of one recorded graph (record_batch_graph), one launch and one
// host synchronisation per iteration for all the contexts together.
tomo_status iterate_batch_graph(tomo_ctx** ctxs, int n, int method, const tomo_schedule* sched, int iter0,
                                int iters, float** d_f, const float** d_ft, double* eps_log, double* seconds) {
    tomo_ctx* lead = ctxs[0];
    const auto t0 = std::chrono::steady_clock::now();
    CU(lead, cudaSetDevice(lead->dev));
    const double s = sched_scale(sched, iter0);
    // kernel choices first: the autotuner times trial passes, which a recording cannot hold
    for (int i = 0; i < n; ++i) {
        tomo_ctx* c = ctxs[i];
        if (!c->tuned) {
            launch_coef(c->geo.cfg.profile, c->f, c->coef, c->rcoef, c->geo.N, c->geo.cfg.courant, c->st);
            TRY(autotune(c));
        }
    }
    uint64_t sbits = 0;
    std::memcpy(&sbits, &s, sizeof sbits);
    std::vector<uint64_t> key = {(uint64_t)method, sbits, (uint64_t)sched->normalize, (uint64_t)n};
    for (int i = 0; i < n; ++i) {
        key.push_back(ctxs[i]->serial);
        key.push_back(ctxs[i]->gen);
        key.push_back((uint64_t)(uintptr_t)d_f[i]);
        key.push_back((uint64_t)(uintptr_t)(d_ft ? d_ft[i] : nullptr));
    }
    if (!lead->batch_exec || lead->batch_key != key)
        TRY(record_batch_graph(ctxs, n, method, sched, s, d_f, d_ft, key));
    // the graph starts after whatever each context's stream holds
    for (int i = 0; i < n; ++i) {
        CU(ctxs[i], cudaEventRecord(ctxs[i]->evj, ctxs[i]->st));
        CU(lead, cudaStreamWaitEvent(lead->st, ctxs[i]->evj, 0));
    }
    for (int it = 0; it < iters; ++it) {
        CU(lead, cudaGraphLaunch(lead->batch_exec, lead->st));
        CU(lead, cudaStreamSynchronize(lead->st));
        for (int i = 0; i < n; ++i) {
            tomo_ctx* c = ctxs[i];
            if (c->err_host && *(volatile unsigned int*)c->err_host) {
                *(volatile unsigned int*)c->err_host = 0u;
                return c->fail(TOMO_ERR_TIMEOUT, "tile kernel: a TMA copy did not arrive within %llu ns",
                               (unsigned long long)c->wait_ns);
            }
            c->launches += lead->batch_kernels[i];
            if (eps_log)
                eps_log[(int64_t)i * iters + it] = d_ft ? 100.0 * std::sqrt(c->pin[1]) / std::sqrt(c->pin[2])
                                                        : std::numeric_limits<double>::quiet_NaN();
        }
    }
    CU(lead, cudaGetLastError());
    if (seconds) *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return TOMO_OK;
}

tomo_status iterate_core(tomo_ctx* c, int method, const tomo_schedule* sch, int it, bool have_true,
                         tomo_iter_stats* stats) {
    const Geometry& g = c->geo;
    const int64_t N = g.N;
    const int G = g.G;
    if (method < 0 || method >= TOMO_METHOD_COUNT) return c->fail(TOMO_ERR_ARG, "unknown method %d", method);
    if (!sch) return c->fail(TOMO_ERR_ARG, "schedule is NULL");
    const double s = sched_scale(sch, it);
    if (!std::isfinite(s)) return c->fail(TOMO_ERR_ARG, "bad schedule");
    const double sc = g.corr_scale;
    const int64_t launches0 = c->launches;
    CU(c, cudaEventRecord(c->ev0, c->st));
    double r2 = 0.0;
    if (method == TOMO_ART) {
        // art-mimo.cu:688-736: each group sees the field updated by the previous one.
        double acc = 0.0;
        TRY(next_noise_draw(c));
        for (int gg = 0; gg < G; ++gg) {
            launch_coef(g.cfg.profile, c->f, c->coef, c->rcoef, N, g.cfg.courant, c->st);
            TRY(run_pass(c, MODE_GRAD, gg, 1));
            launch_combine(c->corr + (int64_t)gg * N, 1, N, c->f, sc, nullptr, 1.0, c->dir, c->st);
            c->launches += 2;
            TRY(apply_dir(c, sch, s));
        }
        TRY(residual_norm(c, &acc));
        TRY(sync_check(c));
        r2 = acc;
    } else {
        TRY(gradient_all(c));
        TRY(residual_norm(c, &r2));
        TRY(update_core(c, method, sch, s));
    }
    CU(c, cudaEventRecord(c->ev1, c->st));
    double eps = std::numeric_limits<double>::quiet_NaN();
    if (have_true) TRY(epsilon(c, &eps));
    TRY(sync_check(c));
    CU(c, cudaGetLastError());
    fill_stats(c, stats, eps, r2, s, (double)G, launches0);
    return TOMO_OK;
}

// Plain weighted (normalised) SIRT direction into c->dir from the correlations of
// c->f (sirt-mimo-norm.cu:56-118, the same rule as TOMO_SIRT_NORM).
tomo_status norm_direction(tomo_ctx* c) {
    const Geometry& g = c->geo;
    const int64_t N = g.N;
    const int G = g.G, nb = reduce_blocks();
    const double sc = g.corr_scale;
    launch_combine(c->corr, G, N, c->f, sc, nullptr, 1.0 / G, c->tmp, c->st);
    launch_group_dev_norm(c->corr, G, N, c->f, sc, c->tmp, c->part, nb, c->st);
    launch_sum_parts(c->part, G, nb, c->sums, c->st);
    launch_norm_weights(c->sums, G, c->st);
    launch_combine(c->corr, G, N, c->f, sc, c->sums, 1.0, c->dir, c->st);
    c->launches += 5;
    return TOMO_OK;
}

tomo_status ensure_learned_buffers(tomo_ctx* c) {
    if (c->feat) return TOMO_OK;
    const int64_t N = c->geo.N;
    TRY(c->alloc(&c->illum, N, "illumination"));
    TRY(c->alloc(&c->feat, 3 * N, "features"));
    TRY(c->alloc(&c->fsave, N, "saved field"));
    TRY(c->alloc(&c->dnet, N, "network update"));
    TRY(c->alloc(&c->illum_max, 1, "illumination max"));
    TRY(c->alloc(&c->dsave, N, "saved direction"));
    TRY(c->alloc(&c->maxsave, 1, "saved direction max"));
    return TOMO_OK;
}

// Illumination sum_g sum_k u_g(k)^2 of the field currently in c->f, once per context.
tomo_status compute_illumination(tomo_ctx* c) {
    if (c->illum_ready) return TOMO_OK;
    const Geometry& g = c->geo;
    CU(c, cudaMemsetAsync(c->illum, 0, sizeof(float) * g.N, c->st));
    launch_coef(g.cfg.profile, c->f, c->coef, c->rcoef, g.N, g.cfg.courant, c->st);
    for (int g0 = 0; g0 < g.G; g0 += c->P) TRY(run_pass(c, MODE_ILLUM, g0, std::min(c->P, g.G - g0)));
    launch_maxabs(c->illum, c->mask, g.N, c->illum_max, c->st);
    TRY(sync_check(c));
    c->illum_ready = true;
    return TOMO_OK;
}

// Features of c->f into c->feat; the direction stays in c->dir and its maximum in c->maxabs.
tomo_status features_core(tomo_ctx* c, double* r2) {
    TRY(ensure_learned_buffers(c));
    TRY(compute_illumination(c));
    TRY(gradient_all(c));
    TRY(residual_norm(c, r2));
    TRY(norm_direction(c));
    launch_maxabs(c->dir, c->mask, c->geo.N, c->maxabs, c->st);
    launch_features(c->f, c->dir, c->maxabs, c->illum, c->illum_max, c->geo.N, c->feat, c->st);
    c->launches += 2;
    return TOMO_OK;
}

}  // namespace

// ---------------------------------------------------------------------------
// C entry points.  Those that can allocate on the host are function-try-blocks: a C++
// exception below them becomes a status (abi_exception) and never crosses the C ABI.
extern "C" {

int32_t tomo_abi_version(void) { return TOMO_ABI_VERSION; }

const char* tomo_status_string(tomo_status s) {
    switch (s) {
    case TOMO_OK: return "ok";
    case TOMO_ERR_ARG: return "invalid argument";
    case TOMO_ERR_CUDA: return "CUDA error";
    case TOMO_ERR_OOM: return "out of device memory";
    case TOMO_ERR_TIMEOUT: return "device wait timed out";
    case TOMO_ERR_DIVERGED: return "diverged";
    case TOMO_ERR_IO: return "I/O error";
    case TOMO_ERR_STATE: return "invalid state";
    }
    return "unknown status";
}

tomo_status tomo_config_init(tomo_config* cfg, int32_t profile) {
    if (!cfg) return TOMO_ERR_ARG;
    std::memset(cfg, 0, sizeof *cfg);
    if (profile == TOMO_PROFILE_REF) {
        cfg->nx = 192; cfg->ny = 192; cfg->nt = 401;
        cfg->profile = TOMO_PROFILE_REF;
        cfg->group_size = 10;
        cfg->ring_lo = 20; cfg->ring_hi = 180;
    } else if (profile == TOMO_PROFILE_CFG) {
        cfg->nx = 128; cfg->ny = 128; cfg->nt = 600;
        cfg->profile = TOMO_PROFILE_CFG;
        cfg->group_size = 4;
        cfg->n_transducers = 32; cfg->radius = 50.f;
        cfg->courant = 0.5f; cfg->cells_per_wavelength = 12.f;
        cfg->sponge_width = 16; cfg->sponge_max = 0.05f;
    } else {
        return TOMO_ERR_ARG;
    }
    return TOMO_OK;
}

tomo_status tomo_create(const tomo_config* cfg, tomo_ctx** out) try {
    g_create_error.clear();
    if (!cfg || !out) { g_create_error = "NULL argument"; return TOMO_ERR_ARG; }
    *out = nullptr;
    std::unique_ptr<tomo_ctx> c(new (std::nothrow) tomo_ctx());   // freed on every early return
    if (!c) return TOMO_ERR_OOM;
    c->dev = -1;
    std::string why;
    tomo_status s = build_geometry(*cfg, c->geo, why);
    if (s != TOMO_OK) { g_create_error = why; return s; }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
        cudaGetLastError();
        g_create_error = "no CUDA device";
        return TOMO_ERR_CUDA;
    }
    if (cfg->device < 0 || cfg->device >= ndev) { g_create_error = "device ordinal out of range"; return TOMO_ERR_ARG; }
    c->dev = cfg->device;
    if ((s = c->cuda(cudaSetDevice(c->dev), "cudaSetDevice")) == TOMO_OK &&
        (s = c->cuda(cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking), "cudaStreamCreate")) == TOMO_OK &&
        (s = c->cuda(cudaEventCreate(&c->ev0), "cudaEventCreate")) == TOMO_OK &&
        (s = c->cuda(cudaEventCreate(&c->ev1), "cudaEventCreate")) == TOMO_OK && (s = make_plan(c.get())) == TOMO_OK &&
        (s = create_buffers(c.get())) == TOMO_OK && cfg->ckpt_interval < 0)
        s = tune_plan(c.get());
    if (s != TOMO_OK) {
        g_create_error = c->err;
        return s;
    }
    static std::atomic<uint64_t> serials{0};
    c->serial = ++serials;
    *out = c.release();
    return TOMO_OK;
} catch (...) {
    return abi_exception(&g_create_error);
}

void tomo_destroy(tomo_ctx* ctx) { delete ctx; }

const char* tomo_last_error(const tomo_ctx* ctx) { return ctx ? ctx->err.c_str() : g_create_error.c_str(); }

tomo_status tomo_get_info(const tomo_ctx* c, tomo_info* out) {
    if (!c || !out) return TOMO_ERR_ARG;
    out->n_groups = c->geo.G;
    out->n_channels = c->geo.nch;
    out->n_transducers = c->geo.ns;
    out->groups_per_pass = c->P;
    out->ckpt_interval = c->K;
    out->n_segments = c->nchunk;
    out->device_bytes = c->bytes;
    return TOMO_OK;
}

void* tomo_stream(const tomo_ctx* c) { return c ? (void*)c->st : nullptr; }

tomo_status tomo_transducers(const tomo_ctx* c, int32_t* ii, int32_t* jj) {
    if (!c || !ii || !jj) return TOMO_ERR_ARG;
    std::memcpy(ii, c->geo.ii.data(), sizeof(int32_t) * c->geo.ns);
    std::memcpy(jj, c->geo.jj.data(), sizeof(int32_t) * c->geo.ns);
    return TOMO_OK;
}

tomo_status tomo_phantom_ref(int32_t nx, int32_t ny, float* fo) try {
    return phantom_ref(nx, ny, fo);
} catch (...) {
    return abi_exception(nullptr);
}

tomo_status tomo_phantom_cfg(int32_t nx, int32_t ny, int32_t kind, int32_t n, float rmin, float rmax, float vmax,
                             float noise_sigma, float support, uint64_t seed, float* fo) try {
    return phantom_cfg(nx, ny, kind, n, rmin, rmax, vmax, noise_sigma, support, seed, fo);
} catch (...) {
    return abi_exception(nullptr);
}

tomo_status tomo_forward(tomo_ctx* c, const float* f, float* records, float* u_last) try {
    if (!c || !f || !records) return c ? c->fail(TOMO_ERR_ARG, "NULL argument") : TOMO_ERR_ARG;
    CU(c, cudaSetDevice(c->dev));
    const Geometry& g = c->geo;
    CU(c, cudaMemcpyAsync(c->f, f, sizeof(float) * g.N, cudaMemcpyHostToDevice, c->st));
    TRY(forward_all(c, u_last));
    CU(c, cudaMemcpyAsync(records, c->rec, sizeof(float) * (size_t)g.G * c->recs_per_group(),
                          cudaMemcpyDeviceToHost, c->st));
    TRY(sync_check(c));
    CU(c, cudaGetLastError());
    return TOMO_OK;
} catch (...) {
    return abi_exception(c ? &c->err : nullptr);
}

tomo_status tomo_generate_data(tomo_ctx* c, const float* f_true, float* records, const tomo_noise* noise) try {
    TRY(tomo_forward(c, f_true, records, nullptr));
    if (noise && noise->kind == 1 && noise->level > 0.f)
        add_record_noise(records, c->geo.G, c->geo.nt, c->geo.nch, noise->level, noise->seed);
    else if (noise && (noise->kind == 2 || noise->kind == 3) && noise->level > 0.f)
        mul_record_noise(records, c->geo.G, c->geo.nt, c->geo.nch, noise->level, noise->seed);
    else if (noise && (noise->kind < 0 || noise->kind > 3))
        return c->fail(TOMO_ERR_ARG, "unknown noise kind %d", noise->kind);
    return TOMO_OK;
} catch (...) {
    return abi_exception(c ? &c->err : nullptr);
}

tomo_status tomo_set_residual_noise(tomo_ctx* c, const tomo_noise* noise) try {
    if (!c) return TOMO_ERR_ARG;
    const int kind = noise ? noise->kind : 0;
    if (kind != 0 && kind != 2 && kind != 3) return c->fail(TOMO_ERR_ARG, "residual noise kind must be 0, 2 or 3");
    if (noise && kind != 0 && !(noise->level >= 0.f && noise->level < 1.f))
        return c->fail(TOMO_ERR_ARG, "residual noise level must be in [0, 1)");
    CU(c, cudaSetDevice(c->dev));
    if (kind != 0 && !c->noise_key) TRY(c->alloc(&c->noise_key, 1, "noise key"));
    TRY(sync_check(c));
    c->noise_kind = kind;
    c->noise_seed = noise ? noise->seed : 0;
    c->noise_draws = 0;
    c->noise_key_host = c->noise_seed;
    if (kind != 0)
        CU(c, cudaMemcpyAsync(c->noise_key, &c->noise_key_host, sizeof(uint64_t), cudaMemcpyHostToDevice, c->st));
    c->dg.noise_key = kind != 0 ? c->noise_key : nullptr;
    c->dg.noise_level = kind != 0 ? noise->level : 0.f;
    c->drop_graphs();                       // captured launches hold the old DevGeo
    TRY(sync_check(c));
    return TOMO_OK;
} catch (...) {
    return abi_exception(c ? &c->err : nullptr);
}

tomo_status tomo_set_records(tomo_ctx* c, const float* records) try {
    if (!c || !records) return c ? c->fail(TOMO_ERR_ARG, "NULL records") : TOMO_ERR_ARG;
    CU(c, cudaSetDevice(c->dev));
    CU(c, cudaMemcpyAsync(c->meas, records, sizeof(float) * (size_t)c->geo.G * c->recs_per_group(),
                          cudaMemcpyHostToDevice, c->st));
    TRY(sync_check(c));
    c->meas_set = true;
    return TOMO_OK;
} catch (...) {
    return abi_exception(c ? &c->err : nullptr);
}

tomo_status tomo_gradient(tomo_ctx* c, const float* f, const float* records, float* dfg, float* df,
                          double* resid_norm2) try {
    if (!c || !f) return c ? c->fail(TOMO_ERR_ARG, "NULL argument") : TOMO_ERR_ARG;
    if (records) TRY(tomo_set_records(c, records));
    if (!c->meas_set) return c->fail(TOMO_ERR_STATE, "no measured records");
    const Geometry& g = c->geo;
    CU(c, cudaSetDevice(c->dev));
    CU(c, cudaMemcpyAsync(c->f, f, sizeof(float) * g.N, cudaMemcpyHostToDevice, c->st));
    TRY(gradient_all(c));
    if (resid_norm2) TRY(residual_norm(c, resid_norm2));
    if (dfg) {
        if (!c->dfg) TRY(c->alloc(&c->dfg, (int64_t)g.G * g.N, "per-group gradients"));
        for (int gg = 0; gg < g.G; ++gg)
            launch_combine(c->corr + (int64_t)gg * g.N, 1, g.N, c->f, g.corr_scale, nullptr, 1.0,
                           c->dfg + (int64_t)gg * g.N, c->st);
        CU(c, cudaMemcpyAsync(dfg, c->dfg, sizeof(float) * (size_t)g.G * g.N, cudaMemcpyDeviceToHost, c->st));
    }
    if (df) {
        launch_combine(c->corr, g.G, g.N, c->f, g.corr_scale, nullptr, 1.0, c->dir, c->st);
        CU(c, cudaMemcpyAsync(df, c->dir, sizeof(float) * g.N, cudaMemcpyDeviceToHost, c->st));
    }
    TRY(sync_check(c));
    CU(c, cudaGetLastError());
    return TOMO_OK;
} catch (...) {
    return abi_exception(c ? &c->err : nullptr);
}

tomo_status tomo_iterate(tomo_ctx* c, int32_t method, const tomo_schedule* sched, int32_t iter, float* f_inout,
                         const float* records, const float* f_true, tomo_iter_stats* stats) try {
    if (!c || !f_inout) return c ? c->fail(TOMO_ERR_ARG, "NULL argument") : TOMO_ERR_ARG;
    CU(c, cudaSetDevice(c->dev));
    if (records) TRY(tomo_set_records(c, records));
    if (!c->meas_set) return c->fail(TOMO_ERR_STATE, "no measured records");
    const Geometry& g = c->geo;
    CU(c, cudaMemcpyAsync(c->f, f_inout, sizeof(float) * g.N, cudaMemcpyHostToDevice, c->st));
    if (f_true) CU(c, cudaMemcpyAsync(c->ftrue, f_true, sizeof(float) * g.N, cudaMemcpyHostToDevice, c->st));
    TRY(iterate_core(c, method, sched, iter, f_true != nullptr, stats));
    CU(c, cudaMemcpyAsync(f_inout, c->f, sizeof(float) * g.N, cudaMemcpyDeviceToHost, c->st));
    TRY(sync_check(c));
    return TOMO_OK;
} catch (...) {
    return abi_exception(c ? &c->err : nullptr);
}

tomo_status tomo_run(tomo_ctx* c, int32_t method, const tomo_schedule* sched, float* f_inout, const float* records,
                     const float* f_true, float target_epsilon, int32_t max_iters, double* eps_log,
                     int32_t* iters_done) try {
    if (!c || !f_inout || !f_true) return c ? c->fail(TOMO_ERR_ARG, "NULL argument") : TOMO_ERR_ARG;
    CU(c, cudaSetDevice(c->dev));
    if (records) TRY(tomo_set_records(c, records));
    if (!c->meas_set) return c->fail(TOMO_ERR_STATE, "no measured records");
    const Geometry& g = c->geo;
    CU(c, cudaMemcpyAsync(c->f, f_inout, sizeof(float) * g.N, cudaMemcpyHostToDevice, c->st));
    CU(c, cudaMemcpyAsync(c->ftrue, f_true, sizeof(float) * g.N, cudaMemcpyHostToDevice, c->st));
    const int64_t limit = max_iters < 0 ? std::numeric_limits<int32_t>::max() : max_iters;
    double prev = std::numeric_limits<double>::infinity();
    tomo_status result = TOMO_OK;
    int done = 0;
    for (int64_t it = 0; it < limit; ++it) {
        tomo_iter_stats st{};
        TRY(iterate_core(c, method, sched, (int)it, true, &st));
        if (eps_log && max_iters > 0) eps_log[it] = st.epsilon;
        done = (int)it + 1;
        if (st.epsilon <= target_epsilon) break;                         // sirt-mimo.cu:356
        if (st.epsilon > prev || std::isnan(st.epsilon)) { result = TOMO_ERR_DIVERGED; break; }   // :362
        prev = st.epsilon;
    }
    CU(c, cudaMemcpyAsync(f_inout, c->f, sizeof(float) * g.N, cudaMemcpyDeviceToHost, c->st));
    TRY(sync_check(c));
    if (iters_done) *iters_done = done;
    if (result == TOMO_ERR_DIVERGED) c->err = "epsilon rose or became NaN";
    return result;
} catch (...) {
    return abi_exception(c ? &c->err : nullptr);
}

tomo_status tomo_forward_device(tomo_ctx* c, const float* d_f, float* d_records) try {
    if (!c || !d_f || !d_records) return c ? c->fail(TOMO_ERR_ARG, "NULL argument") : TOMO_ERR_ARG;
    CU(c, cudaSetDevice(c->dev));
    const Geometry& g = c->geo;
    CU(c, cudaMemcpyAsync(c->f, d_f, sizeof(float) * g.N, cudaMemcpyDeviceToDevice, c->st));
    TRY(forward_all(c, nullptr));
    CU(c, cudaMemcpyAsync(d_records, c->rec, sizeof(float) * (size_t)g.G * c->recs_per_group(),
                          cudaMemcpyDeviceToDevice, c->st));
    return TOMO_OK;
} catch (...) {
    return abi_exception(c ? &c->err : nullptr);
}

tomo_status tomo_iterate_device(tomo_ctx* c, int32_t method, const tomo_schedule* sched, int32_t iter, float* d_f,
                                const float* d_records, const float* d_f_true, tomo_iter_stats* stats) try {
    if (!c || !d_f) return c ? c->fail(TOMO_ERR_ARG, "NULL argument") : TOMO_ERR_ARG;
    CU(c, cudaSetDevice(c->dev));
    const Geometry& g = c->geo;
    if (d_records) {
        CU(c, cudaMemcpyAsync(c->meas, d_records, sizeof(float) * (size_t)g.G * c->recs_per_group(),
                              cudaMemcpyDeviceToDevice, c->st));
        c->meas_set = true;
    }
    if (!c->meas_set) return c->fail(TOMO_ERR_STATE, "no measured records");
    CU(c, cudaMemcpyAsync(c->f, d_f, sizeof(float) * g.N, cudaMemcpyDeviceToDevice, c->st));
    if (d_f_true) CU(c, cudaMemcpyAsync(c->ftrue, d_f_true, sizeof(float) * g.N, cudaMemcpyDeviceToDevice, c->st));
    TRY(iterate_core(c, method, sched, iter, d_f_true != nullptr, stats));
    CU(c, cudaMemcpyAsync(d_f, c->f, sizeof(float) * g.N, cudaMemcpyDeviceToDevice, c->st));
    return TOMO_OK;
} catch (...) {
    return abi_exception(c ? &c->err : nullptr);
}

tomo_status tomo_gradient_groups_device(tomo_ctx* c, const float* d_f, int32_t g0, int32_t ng,
                                       double* resid_norm2) try {
    if (!c || !d_f) return c ? c->fail(TOMO_ERR_ARG, "NULL argument") : TOMO_ERR_ARG;
    const Geometry& g = c->geo;
    if (g0 < 0 || ng < 1 || g0 > g.G - ng) return c->fail(TOMO_ERR_ARG, "group range %d + %d outside 0..%d", g0, ng, g.G);
    if (!c->meas_set) return c->fail(TOMO_ERR_STATE, "no measured records");
    CU(c, cudaSetDevice(c->dev));
    CU(c, cudaMemcpyAsync(c->f, d_f, sizeof(float) * g.N, cudaMemcpyDeviceToDevice, c->st));
    TRY(next_noise_draw(c));
    launch_coef(g.cfg.profile, c->f, c->coef, c->rcoef, g.N, g.cfg.courant, c->st);
    ++c->launches;
    for (int a = g0; a < g0 + ng; a += c->P) TRY(run_pass(c, MODE_GRAD, a, std::min(c->P, g0 + ng - a)));
    if (resid_norm2) {
        launch_sum_parts(c->rpart + (int64_t)g0 * g.nt, 1, ng * g.nt, c->sums, c->st);
        ++c->launches;
        CU(c, cudaMemcpyAsync(resid_norm2, c->sums, sizeof(double), cudaMemcpyDeviceToHost, c->st));
    }
    TRY(sync_check(c));
    CU(c, cudaGetLastError());
    return TOMO_OK;
} catch (...) {
    return abi_exception(c ? &c->err : nullptr);
}

tomo_status tomo_get_correlations_device(tomo_ctx* c, int32_t g0, int32_t ng, float* d_out) try {
    if (!c || !d_out) return c ? c->fail(TOMO_ERR_ARG, "NULL argument") : TOMO_ERR_ARG;
    const Geometry& g = c->geo;
    if (g0 < 0 || ng < 1 || g0 > g.G - ng) return c->fail(TOMO_ERR_ARG, "group range %d + %d outside 0..%d", g0, ng, g.G);
    CU(c, cudaSetDevice(c->dev));
    CU(c, cudaMemcpyAsync(d_out, c->corr + (int64_t)g0 * g.N, sizeof(float) * (size_t)ng * g.N,
                          cudaMemcpyDeviceToDevice, c->st));
    return TOMO_OK;
} catch (...) {
    return abi_exception(c ? &c->err : nullptr);
}

tomo_status tomo_set_correlations_device(tomo_ctx* c, int32_t g0, int32_t ng, const float* d_in) try {
    if (!c || !d_in) return c ? c->fail(TOMO_ERR_ARG, "NULL argument") : TOMO_ERR_ARG;
    const Geometry& g = c->geo;
    if (g0 < 0 || ng < 1 || g0 > g.G - ng) return c->fail(TOMO_ERR_ARG, "group range %d + %d outside 0..%d", g0, ng, g.G);
    CU(c, cudaSetDevice(c->dev));
    CU(c, cudaMemcpyAsync(c->corr + (int64_t)g0 * g.N, d_in, sizeof(float) * (size_t)ng * g.N,
                          cudaMemcpyDeviceToDevice, c->st));
    return TOMO_OK;
} catch (...) {
    return abi_exception(c ? &c->err : nullptr);
}

tomo_status tomo_update_device(tomo_ctx* c, int32_t method, const tomo_schedule* sched, int32_t iter, float* d_f,
                               const float* d_f_true, tomo_iter_stats* stats) try {
    if (!c || !d_f || !sched) return c ? c->fail(TOMO_ERR_ARG, "NULL argument") : TOMO_ERR_ARG;
    if (method < 0 || method >= TOMO_METHOD_COUNT || method == TOMO_ART)
        return c->fail(TOMO_ERR_ARG, "tomo_update_device takes a SIRT method (not ART), got %d", method);
    const double s = sched_scale(sched, iter);
    if (!std::isfinite(s)) return c->fail(TOMO_ERR_ARG, "bad schedule");
    CU(c, cudaSetDevice(c->dev));
    const Geometry& g = c->geo;
    const int64_t launches0 = c->launches;
    CU(c, cudaMemcpyAsync(c->f, d_f, sizeof(float) * g.N, cudaMemcpyDeviceToDevice, c->st));
    if (d_f_true) CU(c, cudaMemcpyAsync(c->ftrue, d_f_true, sizeof(float) * g.N, cudaMemcpyDeviceToDevice, c->st));
    CU(c, cudaEventRecord(c->ev0, c->st));
    TRY(update_core(c, method, sched, s));
    CU(c, cudaEventRecord(c->ev1, c->st));
    double eps = std::numeric_limits<double>::quiet_NaN();
    if (d_f_true) TRY(epsilon(c, &eps));
    CU(c, cudaMemcpyAsync(d_f, c->f, sizeof(float) * g.N, cudaMemcpyDeviceToDevice, c->st));
    TRY(sync_check(c));
    CU(c, cudaGetLastError());
    fill_stats(c, stats, eps, std::numeric_limits<double>::quiet_NaN(), s, 0.0, launches0);
    return TOMO_OK;
} catch (...) {
    return abi_exception(c ? &c->err : nullptr);
}

tomo_status tomo_features_device(tomo_ctx* c, const float* d_f, float* d_feat, double* resid_norm2) try {
    if (!c || !d_f || !d_feat) return c ? c->fail(TOMO_ERR_ARG, "NULL argument") : TOMO_ERR_ARG;
    if (!c->meas_set) return c->fail(TOMO_ERR_STATE, "no measured records");
    CU(c, cudaSetDevice(c->dev));
    const int64_t N = c->geo.N;
    CU(c, cudaMemcpyAsync(c->f, d_f, sizeof(float) * N, cudaMemcpyDeviceToDevice, c->st));
    double r2 = 0.0;
    TRY(features_core(c, &r2));
    CU(c, cudaMemcpyAsync(d_feat, c->feat, sizeof(float) * 3 * N, cudaMemcpyDeviceToDevice, c->st));
    TRY(sync_check(c));
    if (resid_norm2) *resid_norm2 = r2;
    return TOMO_OK;
} catch (...) {
    return abi_exception(c ? &c->err : nullptr);
}

tomo_status tomo_iterate_learned(tomo_ctx* c, tomo_net* net, const tomo_schedule* fallback, int32_t iter, float* d_f,
                                 const float* d_f_true, tomo_iter_stats* stats, int32_t* accepted) try {
    if (!c || !net || !fallback || !d_f) return c ? c->fail(TOMO_ERR_ARG, "NULL argument") : TOMO_ERR_ARG;
    if (!c->meas_set) return c->fail(TOMO_ERR_STATE, "no measured records");
    CU(c, cudaSetDevice(c->dev));
    const Geometry& g = c->geo;
    const int64_t N = g.N;
    const double s = sched_scale(fallback, iter);
    if (!std::isfinite(s)) return c->fail(TOMO_ERR_ARG, "bad schedule");
    const int64_t launches0 = c->launches;
    CU(c, cudaMemcpyAsync(c->f, d_f, sizeof(float) * N, cudaMemcpyDeviceToDevice, c->st));
    if (d_f_true) CU(c, cudaMemcpyAsync(c->ftrue, d_f_true, sizeof(float) * N, cudaMemcpyDeviceToDevice, c->st));
    CU(c, cudaEventRecord(c->ev0, c->st));
    double r0 = 0.0, r1 = 0.0;
    TRY(features_core(c, &r0));
    // proposal f + mask * net(features)
    tomo_status ns = net_infer(net, c->feat, g.ny, g.nx, c->dnet, c->st);
    if (ns != TOMO_OK) return c->fail(ns, "network: %s", tomo_net_last_error(net));
    c->launches += 6;
    CU(c, cudaMemcpyAsync(c->fsave, c->f, sizeof(float) * N, cudaMemcpyDeviceToDevice, c->st));
    launch_apply(c->f, c->dnet, c->mask, N, c->learned_scale, nullptr, c->st);
    launch_coef(g.cfg.profile, c->f, c->coef, c->rcoef, N, g.cfg.courant, c->st);
    c->launches += 2;
    TRY(next_noise_draw(c));
    for (int g0 = 0; g0 < g.G; g0 += c->P) TRY(run_pass(c, MODE_RESID, g0, std::min(c->P, g.G - g0)));
    TRY(residual_norm(c, &r1));
    const bool ok = r1 < r0;
    if (!ok) {
        // plain weighted SIRT step from the saved field along its direction
        CU(c, cudaMemcpyAsync(c->f, c->fsave, sizeof(float) * N, cudaMemcpyDeviceToDevice, c->st));
        launch_apply(c->f, c->dir, c->mask, N, s, fallback->normalize ? c->maxabs : nullptr, c->st);
        ++c->launches;
    }
    CU(c, cudaEventRecord(c->ev1, c->st));
    double eps = std::numeric_limits<double>::quiet_NaN();
    if (d_f_true) TRY(epsilon(c, &eps));
    CU(c, cudaMemcpyAsync(d_f, c->f, sizeof(float) * N, cudaMemcpyDeviceToDevice, c->st));
    TRY(sync_check(c));
    CU(c, cudaGetLastError());
    if ((ns = net_check(net)) != TOMO_OK) return c->fail(ns, "network: %s", tomo_net_last_error(net));
    if (accepted) *accepted = ok ? 1 : 0;
    if (stats) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, c->ev0, c->ev1);
        stats->epsilon = eps;
        stats->resid_norm2 = r0;
        stats->scale = ok ? 1.0 : s;
        stats->seconds = ms * 1e-3;
        stats->cell_updates = 3.0 * (double)g.G * (double)(g.nt - 2) * (double)N;
        stats->kernel_launches = (double)(c->launches - launches0);
    }
    return TOMO_OK;
} catch (...) {
    return abi_exception(c ? &c->err : nullptr);
}

tomo_status tomo_run_learned(tomo_ctx* c, tomo_net* net, const tomo_schedule* fallback, float* d_f,
                             const float* d_f_true, double target_epsilon, int32_t max_iters, double min_decrease,
                             int32_t patience, double* eps_log, int32_t* step_log, int32_t* iters_done,
                             int32_t* sweeps, double* seconds) try {
    if (!c || !net || !fallback || !d_f || max_iters < 0 || !(min_decrease >= 0.0 && min_decrease < 1.0) ||
        patience < 0)
        return c ? c->fail(TOMO_ERR_ARG, "bad tomo_run_learned arguments") : TOMO_ERR_ARG;
    if (!c->meas_set) return c->fail(TOMO_ERR_STATE, "no measured records");
    CU(c, cudaSetDevice(c->dev));
    const Geometry& g = c->geo;
    const int64_t N = g.N;
    const size_t fb = sizeof(float) * N;
    TRY(ensure_learned_buffers(c));
    CU(c, cudaMemcpyAsync(c->f, d_f, fb, cudaMemcpyDeviceToDevice, c->st));
    if (d_f_true) CU(c, cudaMemcpyAsync(c->ftrue, d_f_true, fb, cudaMemcpyDeviceToDevice, c->st));
    TRY(compute_illumination(c));
    const auto t0 = std::chrono::steady_clock::now();
    double r0 = 0.0, r1 = 0.0;
    TRY(features_core(c, &r0));            // gradient, direction and features at the start field
    int done = 0, nsweep = 1, rejected = 0;
    bool learning = true;
    int paused = 0;                        // plain steps since the proposals paused
    for (int it = 0; it < max_iters; ++it) {
        const double s = sched_scale(fallback, it);
        if (!std::isfinite(s)) return c->fail(TOMO_ERR_ARG, "bad schedule");
        int kind = -1;                     // 1 accepted, 0 rejected (plain step), -1 plain step only
        if (learning) {
            tomo_status ns = net_infer(net, c->feat, g.ny, g.nx, c->dnet, c->st);
            if (ns != TOMO_OK) return c->fail(ns, "network: %s", tomo_net_last_error(net));
            CU(c, cudaMemcpyAsync(c->fsave, c->f, fb, cudaMemcpyDeviceToDevice, c->st));
            CU(c, cudaMemcpyAsync(c->dsave, c->dir, fb, cudaMemcpyDeviceToDevice, c->st));
            CU(c, cudaMemcpyAsync(c->maxsave, c->maxabs, sizeof(unsigned int), cudaMemcpyDeviceToDevice, c->st));
            c->launches += 6;
            double sc = c->learned_scale;
            for (int tries = 0;; ++tries) {
                if (tries > 0) CU(c, cudaMemcpyAsync(c->f, c->fsave, fb, cudaMemcpyDeviceToDevice, c->st));
                launch_apply(c->f, c->dnet, c->mask, N, sc, nullptr, c->st);
                ++c->launches;
                // the check is the gradient sweep of the proposal: accepted, it is the next step's gradient
                TRY(features_core(c, &r1));
                ++nsweep;
                if (r1 <= (1.0 - min_decrease) * r0) {
                    kind = tries == 0 ? 1 : 2;
                    break;
                }
                kind = 0;
                if (tries >= c->learned_backtrack) break;
                sc *= 0.5;   // the same network output at half the scale
            }
        }
        if (kind >= 1) {
            r0 = r1;
            rejected = 0;
        } else {
            // plain weighted-SIRT step: from the saved field after a rejected proposal, else from f
            if (kind == 0) CU(c, cudaMemcpyAsync(c->f, c->fsave, fb, cudaMemcpyDeviceToDevice, c->st));
            const float* dir = kind == 0 ? c->dsave : c->dir;
            const unsigned int* mx = kind == 0 ? c->maxsave : c->maxabs;
            launch_apply(c->f, dir, c->mask, N, s, fallback->normalize ? mx : nullptr, c->st);
            ++c->launches;
            TRY(features_core(c, &r0));
            ++nsweep;
            if (kind == 0 && patience > 0 && ++rejected >= patience) {
                learning = false;   // plain from here on, or for learned_resume plain steps
                paused = 0;
            } else if (kind == -1 && c->learned_resume > 0 && ++paused >= c->learned_resume) {
                learning = true;
                rejected = 0;
            }
        }
        double eps = std::numeric_limits<double>::quiet_NaN();
        if (d_f_true) TRY(epsilon(c, &eps));
        if (eps_log) eps_log[it] = eps;
        if (step_log) step_log[it] = kind;
        done = it + 1;
        if (d_f_true && eps <= target_epsilon) break;
    }
    CU(c, cudaMemcpyAsync(d_f, c->f, fb, cudaMemcpyDeviceToDevice, c->st));
    TRY(sync_check(c));
    CU(c, cudaGetLastError());
    if (tomo_status ns = net_check(net); ns != TOMO_OK) return c->fail(ns, "network: %s", tomo_net_last_error(net));
    if (iters_done) *iters_done = done;
    if (sweeps) *sweeps = nsweep;
    if (seconds) *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return TOMO_OK;
} catch (...) {
    return abi_exception(c ? &c->err : nullptr);
}

tomo_status tomo_time_kernel(tomo_ctx* c, int32_t which, int32_t steps, double* ms_per_launch,
                             double* bytes_per_launch) try {
    if (!c || (which != 0 && which != 1) || steps < 1 || !ms_per_launch)
        return c ? c->fail(TOMO_ERR_ARG, "bad tomo_time_kernel arguments") : TOMO_ERR_ARG;
    CU(c, cudaSetDevice(c->dev));
    const Geometry& g = c->geo;
    const int nt = g.nt, ng = c->P, prof = g.cfg.profile;
    const int64_t N = g.N;
    if (nt < 5) return c->fail(TOMO_ERR_ARG, "tomo_time_kernel needs nt >= 5");
    steps = std::min(steps, nt - 4);
    const int k0 = std::max(2, (nt - steps) / 2);
    launch_coef(prof, c->f, c->coef, c->rcoef, N, g.cfg.courant, c->st);
    TRY(autotune(c));
    // the steps are captured into a graph and replayed, as the iterations run them, so the time
    // per step carries the launch gaps of graph replay, not of stream launches
    cudaGraph_t graph = nullptr;
    CU(c, cudaStreamBeginCapture(c->st, cudaStreamCaptureModeThreadLocal));
    for (int t = 0; t < steps;) {
        if (which == 0 && c->tile_fwd) {
            const int T = tile_fwd_steps(c, steps - t);
            launch_fwd_tile(c->dg, c->tmaps, tile_fwd_args(c, k0 + t, T, 0, ng), c->st);
            t += T;
        } else if (which == 1 && c->tile_adj) {
            const int T = tile_adj_steps(steps - t);
            launch_adj_tile(c->dg, c->tmaps, tile_adj_args(c, k0 + steps - t, T, 0, ng), c->st);
            t += T;
        } else if (which == 0 && c->fwd_pair && t + 1 < steps) {
            launch_fwd2_strip(c->rows_fwd2, c->dg, c->coef, fwd_args(c, k0 + t, 0, ng), fwd_args(c, k0 + t + 1, 0, ng),
                              false, false, c->st);
            t += 2;
        } else if (which == 0) {
            fwd_launch(c, fwd_args(c, k0 + t, 0, ng));
            t += 1;
        } else if (c->adj_pair && t + 1 < steps) {
            const int q = k0 + steps - 1 - t;
            launch_adj2_strip(c->rows_adj2, c->dg, c->coef, adj_args(c, q, 0, ng), adj_args(c, q - 1, 0, ng), c->st);
            t += 2;
        } else {
            adj_launch(c, adj_args(c, k0 + steps - 1 - t, 0, ng));
            t += 1;
        }
    }
    const cudaError_t ec = cudaStreamEndCapture(c->st, &graph);
    if (ec != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        return c->cuda(ec, "cudaStreamEndCapture");
    }
    cudaGraphExec_t exec = nullptr;
    const cudaError_t ei = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ei != cudaSuccess) return c->cuda(ei, "cudaGraphInstantiate");
    float ms = 0.f;
    cudaError_t e = cudaGraphLaunch(exec, c->st);     // warm-up replay
    if (e == cudaSuccess) e = cudaEventRecord(c->ev0, c->st);
    if (e == cudaSuccess) e = cudaGraphLaunch(exec, c->st);
    if (e == cudaSuccess) e = cudaEventRecord(c->ev1, c->st);
    if (e == cudaSuccess) e = cudaEventSynchronize(c->ev1);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, c->ev0, c->ev1);
    cudaGraphExecDestroy(exec);
    CU(c, e);
    CU(c, cudaGetLastError());
    *ms_per_launch = (double)ms / steps;
    if (bytes_per_launch) *bytes_per_launch = (which == 0 ? 16.0 : 20.0) * (double)ng * (double)N;
    return TOMO_OK;
} catch (...) {
    return abi_exception(c ? &c->err : nullptr);
}

tomo_status tomo_iterate_batch(tomo_ctx** ctxs, int32_t n, int32_t method, const tomo_schedule* sched,
                               int32_t iter0, int32_t iters, float** d_f, const float** d_f_true, double* eps_log,
                               double* seconds) try {
    if (!ctxs || n < 1 || !sched || !d_f || iters < 0) return TOMO_ERR_ARG;
    for (int i = 0; i < n; ++i) {
        if (!ctxs[i] || !d_f[i]) return TOMO_ERR_ARG;
        for (int j = 0; j < i; ++j)
            if (ctxs[j] == ctxs[i]) return ctxs[i]->fail(TOMO_ERR_ARG, "a context appears twice in the batch");
    }
    if (batch_graph_eligible(ctxs, n, method, sched, iter0, iters))
        return iterate_batch_graph(ctxs, n, method, sched, iter0, iters, d_f, d_f_true, eps_log, seconds);
    std::vector<tomo_status> st(n, TOMO_OK);
    auto work = [&](int i) noexcept {   // the entry points it calls catch their own exceptions
        const float* ft = d_f_true ? d_f_true[i] : nullptr;
        for (int it = 0; it < iters && st[i] == TOMO_OK; ++it) {
            tomo_iter_stats s{};
            st[i] = tomo_iterate_device(ctxs[i], method, sched, iter0 + it, d_f[i], nullptr, ft, &s);
            if (eps_log) eps_log[(int64_t)i * iters + it] = s.epsilon;
        }
        if (st[i] == TOMO_OK) st[i] = tomo_synchronize(ctxs[i]);
    };
    const auto t0 = std::chrono::steady_clock::now();
    {
        std::vector<std::thread> pool;
        pool.reserve(n);
        for (int i = 0; i < n; ++i) {
            try {
                pool.emplace_back(work, i);
            } catch (...) {
                work(i);   // no thread to be had: this context runs on the calling thread
            }
        }
        for (auto& t : pool) t.join();
    }
    if (seconds) *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    for (int i = 0; i < n; ++i)
        if (st[i] != TOMO_OK) return st[i];
    return TOMO_OK;
} catch (...) {
    return abi_exception(nullptr);
}

tomo_status tomo_set_learned_resume(tomo_ctx* c, int32_t plain_steps) {
    if (!c) return TOMO_ERR_ARG;
    if (plain_steps < 0 || plain_steps > 1000) return c->fail(TOMO_ERR_ARG, "learned resume must be in 0..1000");
    c->learned_resume = plain_steps;
    return TOMO_OK;
}

tomo_status tomo_set_learned_backtrack(tomo_ctx* c, int32_t retries) {
    if (!c) return TOMO_ERR_ARG;
    if (retries < 0 || retries > 4) return c->fail(TOMO_ERR_ARG, "learned backtrack retries must be in 0..4");
    c->learned_backtrack = retries;
    return TOMO_OK;
}

tomo_status tomo_set_learned_scale(tomo_ctx* c, double scale) {
    if (!c) return TOMO_ERR_ARG;
    if (!(scale > 0.0 && scale <= 4.0)) return c->fail(TOMO_ERR_ARG, "learned scale must be in (0, 4]");
    c->learned_scale = scale;
    return TOMO_OK;
}

tomo_status tomo_synchronize(tomo_ctx* c) try {
    if (!c) return TOMO_ERR_ARG;
    CU(c, cudaSetDevice(c->dev));
    TRY(sync_check(c));
    CU(c, cudaGetLastError());
    return TOMO_OK;
} catch (...) {
    return abi_exception(c ? &c->err : nullptr);
}

}  // extern "C"
