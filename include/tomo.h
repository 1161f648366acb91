/*
 * tomo.h -- C ABI of the GB300 wave-tomography engine (libtomo.so).
 *
 * The reference (crogers719/Tomographic-Image-Reconstruction-Algorithms) has no
 * library boundary: each driver is a CUDA program whose hot path is a host loop
 * of kernel launches over compile-time sized buffers.  This header is the
 * boundary that replaces those loops.  Every entry point below names the
 * reference code it stands in for.
 *
 * Conventions
 *   - Every call returns a tomo_status; nothing throws across the ABI and
 *     nothing calls exit().  tomo_last_error() gives a one-line reason.
 *   - Host pointers are caller-owned and are copied in/out during the call.
 *     Device memory is owned by the context.  Entry points with the suffix
 *     _device take device pointers on the context's GPU and run on the
 *     context's stream (tomo_stream()).
 *   - One context per host thread; a context serialises on its own stream.
 *   - Layouts are FP32 with i (x) fastest, as in the reference
 *     (cuda_ptr.cuh:141, index i + nx*(j + ny*(k + nz*l))):
 *       field   f[j*nx + i]                                (nx*ny)
 *       records rec[(g*nt + k)*n_channels + c]             (G*nt*n_channels)
 *       per-group gradients dfg[(g*ny + j)*nx + i]         (G*nx*ny)
 *     For the reference profile the n_channels = 4*nx record channels are the
 *     four sensor lines side by side, c = side*nx + i with side order
 *     bottom, right, top, left (the order generate-data.cu:202-223 writes its
 *     four files); channels outside i in [lo+1, hi-1] are always zero.
 */
#ifndef TOMO_H
#define TOMO_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TOMO_ABI_VERSION 1

typedef enum tomo_status {
    TOMO_OK = 0,
    TOMO_ERR_ARG = 1,      /* invalid argument or configuration */
    TOMO_ERR_CUDA = 2,     /* a CUDA runtime call failed */
    TOMO_ERR_OOM = 3,      /* device allocation failed / plan does not fit */
    TOMO_ERR_TIMEOUT = 4,  /* a bounded device wait ran out */
    TOMO_ERR_DIVERGED = 5, /* epsilon rose or became NaN (tomo_run) */
    TOMO_ERR_IO = 6,       /* file missing or malformed (CLI helpers) */
    TOMO_ERR_STATE = 7     /* call not valid in the context's current state */
} tomo_status;

/* Physics profiles.
 * REF: the reference's discretisation in SI units (sirt-mimo.cu:17-35,511-877):
 *      h = 1 mm, dt = 3.3333e-7 s, c0 = 1500 m/s, one-way absorbing edges with a
 *      corner fix-up, square transducer ring, bounding-box Gaussian-cosine
 *      emission, four sensor lines, residual written onto the sensor lines.
 * CFG: the same method in nondimensional units on the synthetic benchmark
 *      workloads: h = 1, Courant number C, quadratic sponge, transducers on a
 *      circle, point Ricker emitters, point receivers, exact discrete adjoint. */
typedef enum tomo_profile { TOMO_PROFILE_REF = 0, TOMO_PROFILE_CFG = 1 } tomo_profile;

typedef struct tomo_config {
    int32_t nx, ny, nt;           /* grid and time steps (reference: 192, 192, 401) */
    int32_t profile;              /* tomo_profile */
    int32_t group_size;           /* transducers per MIMO emitter group */
    /* REF profile: sensor lines at rows/cols ring_lo and ring_hi (0-based);
     * transducers (1-based, as Position_Transducers) on the ring ring_lo+1 ..
     * ring_hi+1; n_transducers = 4*(ring_hi-ring_lo).  Reference: 20, 180. */
    int32_t ring_lo, ring_hi;
    /* CFG profile */
    int32_t n_transducers;        /* transducers evenly on a circle */
    float radius;                 /* circle radius in cells, centred at (nx/2, ny/2) */
    float courant;                /* C = c0 dt / h */
    float cells_per_wavelength;   /* Ricker peak wavelength in cells */
    int32_t sponge_width;         /* cells */
    float sponge_max;             /* sigma at the outer edge; sigma(d)=max*((W-d)/W)^2 */
    /* execution plan */
    int32_t ckpt_interval;        /* forward slices between checkpoints; 0 = plan picks
                                     (full history when it fits, else ~sqrt(2 nt));
                                     -1 = the fastest of full history and three intervals,
                                     timed at tomo_create */
    int32_t groups_per_pass;      /* P of G groups resident per sweep; 0 = plan picks */
    int32_t device;               /* CUDA device ordinal */
    int32_t mem_limit_mb;         /* device memory the plan may use, MiB; 0 = 90 % of free */
    int32_t reserved[3];
} tomo_config;

/* Update rules.  Each is the field update of one reference driver; all of them
 * consume the per-group correlation C_g = sum_k z_g(k) * Lu_g(k). */
typedef enum tomo_method {
    TOMO_SIRT_CLASSIC = 0,    /* sirt-mimo.cu:858-877       f += s*mask*sum_g df_g */
    TOMO_SIRT_SCALED = 1,     /* sirt-mimo-io.cu:774-795, sirt-iter.cu, sirt-test-weight.cu:
                                 f += s*mask*(sum_g df_g)/G */
    TOMO_SIRT_NORM = 2,       /* sirt-mimo-norm.cu:56-118,873-892  inverse-deviation weights */
    TOMO_SIRT_WEIGHT = 3,     /* sirt-mimo-weight.cu:786-839  mean of intermediate fields */
    TOMO_SIRT_AVG = 4,        /* sirt-mimo-avg.cu  same, fixed scale */
    TOMO_SIRT_AVG_WEIGHT = 5, /* sirt-mimo-avg-weight.cu:130-203  unnormalised weighted sum */
    TOMO_ART = 6,             /* art-mimo.cu:683-736  sequential (Kaczmarz) over groups */
    TOMO_METHOD_COUNT = 7
} tomo_method;

/* Step-size schedules, s(it) for 0-based iteration it. */
typedef enum tomo_sched_kind {
    TOMO_SCHED_CONST = 0,  /* s = omega                          (sirt-mimo.cu, art-mimo.cu) */
    TOMO_SCHED_POWER = 1,  /* s = omega*(alpha + beta/(it+1)^gamma)   (sirt-mimo-norm.cu:450) */
    TOMO_SCHED_LINEAR = 2  /* s = omega*(alpha + beta*(it+1))          (sirt-iter.cu:678) */
} tomo_sched_kind;

typedef struct tomo_schedule {
    int32_t kind;          /* tomo_sched_kind */
    float omega, alpha, beta, gamma;
    int32_t normalize;     /* 1: scale the update direction by 1/max|dir| over the mask */
    int32_t reserved[2];
} tomo_schedule;

typedef struct tomo_iter_stats {
    double epsilon;        /* 100*||f - f_true||/||f_true|| (NaN without f_true) */
    double resid_norm2;    /* sum of squared record residuals at the start of the iteration */
    double scale;          /* step size used */
    double seconds;        /* device time of the iteration */
    double cell_updates;   /* forward + adjoint cell-updates credited (no recompute) */
    double kernel_launches;/* kernels launched by the iteration (graph nodes included) */
} tomo_iter_stats;

typedef struct tomo_info {
    int32_t n_groups;        /* G */
    int32_t n_channels;      /* record channels per group and time step */
    int32_t n_transducers;
    int32_t groups_per_pass; /* P chosen by the plan */
    int32_t ckpt_interval;   /* K chosen by the plan (>= nt-2: full history) */
    int32_t n_segments;
    int64_t device_bytes;    /* device memory held by the context */
} tomo_info;

typedef struct tomo_noise {
    int32_t kind;            /* 0 none; 1 Gaussian rec += level*std(trace)*N(0,1);
                                2, 3 multiplicative uniform: every record sample times
                                1 + level*(2U - 1), U in [0,1) from a counter-based hash
                                of (seed, group, step, channel) (the reference's
                                0.9..1.1 factor of sirt-mimo-noise.cu:661-745 is level 0.1) */
    float level;
    uint64_t seed;
} tomo_noise;

typedef struct tomo_ctx tomo_ctx;

/* ---- library ---------------------------------------------------------- */
int32_t     tomo_abi_version(void);
const char* tomo_status_string(tomo_status s);
/* Fill *cfg with the reference problem (profile REF: 192^2, nt 401, ring 20/180,
 * group size 10; sirt-mimo.cu:17-35) or the 128^2 synthetic workload (CFG). */
tomo_status tomo_config_init(tomo_config* cfg, int32_t profile);

/* ---- context (replaces the device_ptr set-up in Ultrasonic_Tomography,
 *      e.g. sirt-mimo-norm.cu:161-303) ------------------------------------ */
tomo_status tomo_create(const tomo_config* cfg, tomo_ctx** out);
void        tomo_destroy(tomo_ctx* ctx);
const char* tomo_last_error(const tomo_ctx* ctx);
tomo_status tomo_get_info(const tomo_ctx* ctx, tomo_info* out);
void*       tomo_stream(const tomo_ctx* ctx); /* cudaStream_t of the context */

/* Transducer cells.  REF: 1-based (ii, jj) exactly as Position_Transducers
 * (sirt-mimo.cu:438-466).  CFG: 0-based cell coordinates on the circle. */
tomo_status tomo_transducers(const tomo_ctx* ctx, int32_t* ii, int32_t* jj);

/* generate-field (generate-field.cu:117-172): the reference phantom of a 30 mm
 * disc (0.03) with three 10 mm discs (0.05) on x = -0.1 + i*h. */
tomo_status tomo_phantom_ref(int32_t nx, int32_t ny, float* fo);
/* Seeded synthetic phantom: kind 0 = n discs (radius U[rmin,rmax], value
 * U[-vmax,vmax]); kind 1 = n ellipses (axes U[rmin,rmax], value U[-vmax,vmax])
 * plus Gaussian-smoothed N(0, noise_sigma^2) texture inside the circle of
 * radius `support`. */
tomo_status tomo_phantom_cfg(int32_t nx, int32_t ny, int32_t kind, int32_t n,
                             float rmin, float rmax, float vmax, float noise_sigma,
                             float support, uint64_t seed, float* fo);

/* ---- hot path ----------------------------------------------------------- */
/* Forward solve of every group and sensor recording.  Replaces the
 * propagation / propagation_at_corners / initial_signal launches
 * (generate-data.cu:157-185).  records: G*nt*n_channels.  u_last (optional):
 * G*nx*ny wavefields at the last time step nt-1. */
tomo_status tomo_forward(tomo_ctx* ctx, const float* f, float* records, float* u_last);
/* generate-data: forward solve plus optional seeded noise on the records. */
tomo_status tomo_generate_data(tomo_ctx* ctx, const float* f_true, float* records,
                               const tomo_noise* noise);
/* In-loop record noise for noise-robustness studies (sirt-mimo-noise.cu:661-745):
 * every residual the context forms afterwards uses simulated samples times the
 * multiplicative factor of `noise` (kind 2: a fresh draw for every gradient
 * sweep, keyed by seed and the sweep count; kind 3: the same draw every sweep,
 * equal to tomo_generate_data's kind-3 draw for the same seed, which is the
 * reference's case of one factor shared by data and residual).  NULL or kind 0
 * turns it off.  Captured graphs are rebuilt on the next call. */
tomo_status tomo_set_residual_noise(tomo_ctx* ctx, const tomo_noise* noise);
/* Store measured records on the device for later tomo_iterate calls. */
tomo_status tomo_set_records(tomo_ctx* ctx, const float* records);
/* Gradient of one SIRT sweep: forward, residual, time-reversed adjoint and
 * the correlation (sirt-mimo-norm.cu:418-439).  Outputs (each optional):
 * dfg = per-group df_g = C_g * scale / (1 + f) (G*nx*ny), df = sum_g df_g,
 * resid_norm2 = sum of squared record residuals. */
tomo_status tomo_gradient(tomo_ctx* ctx, const float* f, const float* records,
                          float* dfg, float* df, double* resid_norm2);
/* One iteration of `method` from 0-based iteration `iter` (the body of the
 * reference drivers' iteration loops, e.g. sirt-mimo.cu:305-370).
 * records may be NULL to use tomo_set_records data.  f_true may be NULL. */
tomo_status tomo_iterate(tomo_ctx* ctx, int32_t method, const tomo_schedule* sched,
                         int32_t iter, float* f_inout, const float* records,
                         const float* f_true, tomo_iter_stats* stats);
/* Iterate with the reference stopping rule (sirt-mimo.cu:355-366): stop when
 * epsilon <= target_epsilon, when epsilon rises above the previous iteration's
 * or is NaN, or after max_iters (-1: unbounded, sirt-mimo.cu:79-80).  Needs
 * f_true.  eps_log (optional, max_iters entries when max_iters > 0) receives
 * epsilon per iteration; *iters_done the number of iterations run.  Returns
 * TOMO_OK when the target was reached or the iteration budget ran out and
 * TOMO_ERR_DIVERGED when the divergence rule stopped the loop. */
tomo_status tomo_run(tomo_ctx* ctx, int32_t method, const tomo_schedule* sched,
                     float* f_inout, const float* records, const float* f_true,
                     float target_epsilon, int32_t max_iters, double* eps_log,
                     int32_t* iters_done);

/* Device-resident variants: pointers live on the context's GPU. */
tomo_status tomo_forward_device(tomo_ctx* ctx, const float* d_f, float* d_records);
tomo_status tomo_iterate_device(tomo_ctx* ctx, int32_t method, const tomo_schedule* sched,
                                int32_t iter, float* d_f, const float* d_records,
                                const float* d_f_true, tomo_iter_stats* stats);
tomo_status tomo_synchronize(tomo_ctx* ctx);

/* Group-sharded SIRT: the emitter groups of one iteration are independent, so
 * they can be split over several contexts (one per GPU or process), which
 * exchange their groups' correlations before the update.  The reference runs
 * P of the M groups per pass on one GPU (sirt-mimo-norm-mem.cu:429-458); here
 * a context runs the passes of its own group range and the caller moves the
 * correlations between contexts (the reduce_df step).
 *   tomo_gradient_groups_device  forward, residual, adjoint and correlation of
 *       groups g0 .. g0+ng-1 for the field d_f (the context's records must be
 *       set); their raw correlations C_g stay in the context, resid_norm2
 *       (optional) receives their squared record residual;
 *   tomo_get_correlations_device / tomo_set_correlations_device  copy the raw
 *       correlations of groups g0 .. g0+ng-1 (ng*nx*ny floats, group-major)
 *       out of / into the context, device to device on the context's stream;
 *   tomo_update_device  the update rule of a SIRT method (every method but
 *       TOMO_ART, which is sequential over groups) from the correlations the
 *       context holds for all groups, applied to d_f; stats->resid_norm2 is NaN
 *       (the caller sums the ranks' residuals).
 * With every group's correlation in place, tomo_update_device gives the field
 * tomo_iterate_device would, bit for bit. */
tomo_status tomo_gradient_groups_device(tomo_ctx* ctx, const float* d_f, int32_t g0, int32_t ng,
                                        double* resid_norm2);
tomo_status tomo_get_correlations_device(tomo_ctx* ctx, int32_t g0, int32_t ng, float* d_out);
tomo_status tomo_set_correlations_device(tomo_ctx* ctx, int32_t g0, int32_t ng, const float* d_in);
tomo_status tomo_update_device(tomo_ctx* ctx, int32_t method, const tomo_schedule* sched, int32_t iter,
                               float* d_f, const float* d_f_true, tomo_iter_stats* stats);

/* Profiling hook (no reference counterpart): runs `steps` consecutive time steps
 * of one hot kernel for the first pass's groups on the context stream, captured
 * into a CUDA graph and replayed (as the iterations replay theirs), bracketed by
 * CUDA events, after at least one tomo_iterate.  which: 0 forward step,
 * 1 adjoint step.  Returns the mean duration of one time step (kernels that
 * advance two steps per launch count as two) and the algorithmic bytes of one
 * step (16 B forward / 20 B adjoint per cell-update).
 * Clobbers the iteration's scratch state (the next tomo_iterate rebuilds it). */
tomo_status tomo_time_kernel(tomo_ctx* ctx, int32_t which, int32_t steps,
                             double* ms_per_launch, double* bytes_per_launch);

/* ---- learned update (no reference counterpart: the reference's updates are
 * hand-set step rules) --------------------------------------------------------
 * A 5-layer 3x3 CNN, 32 channels, ReLU, BF16 weights/activations with FP32
 * accumulation, reading per pixel (f, normalised SIRT direction, normalised
 * illumination) and proposing a field update.  Feature tensors are planar FP32
 * [B][3][H][W]; outputs [B][H][W]; W must be a multiple of 64. */
typedef struct tomo_net tomo_net;
int64_t     tomo_net_num_params(void);
tomo_status tomo_net_create(int32_t device, uint64_t seed, tomo_net** out);
void        tomo_net_destroy(tomo_net* net);
const char* tomo_net_last_error(const tomo_net* net);
tomo_status tomo_net_get_params(tomo_net* net, float* host);
tomo_status tomo_net_set_params(tomo_net* net, const float* host);
tomo_status tomo_net_save(tomo_net* net, const char* path);
tomo_status tomo_net_load(tomo_net* net, const char* path);
tomo_status tomo_net_forward_device(tomo_net* net, const float* d_feat, int32_t B, int32_t H, int32_t W,
                                    float* d_out);
/* Masked mean-squared-error gradient w.r.t. the parameters (binary mask). */
tomo_status tomo_net_grad_device(tomo_net* net, const float* d_feat, const float* d_target, const float* d_mask,
                                 int32_t B, int32_t H, int32_t W, float* host_grad, double* loss);
/* One Adam step (beta 0.9/0.999) on the masked MSE. */
tomo_status tomo_net_train_step_device(tomo_net* net, const float* d_feat, const float* d_target,
                                       const float* d_mask, int32_t B, int32_t H, int32_t W, float lr,
                                       double* loss);
/* Features of the field d_f (device): planar [3][ny][nx] = f, the plain
 * weighted-SIRT direction scaled to max 1 over the mask, the illumination
 * sum_g sum_k u^2 scaled to max 1 over the mask.  Also returns the squared
 * record residual at d_f.  The context's records must be set. */
tomo_status tomo_features_device(tomo_ctx* ctx, const float* d_f, float* d_feat, double* resid_norm2);
/* One learned iteration: the network proposes f + mask * net(features); the
 * proposal is accepted only if the squared record residual decreases,
 * otherwise the step falls back to plain weighted SIRT (TOMO_SIRT_NORM with
 * `fallback`).  *accepted (optional) receives 1 or 0. */
tomo_status tomo_iterate_learned(tomo_ctx* ctx, tomo_net* net, const tomo_schedule* fallback, int32_t iter,
                                 float* d_f, const float* d_f_true, tomo_iter_stats* stats, int32_t* accepted);
/* Learned iterations on the device field d_f until the image error against
 * d_f_true (optional) reaches target_epsilon (percent) or max_iters.  Each
 * iteration proposes f + mask * net(features); the gradient sweep of the
 * proposal is its residual check and, when it passes, also the next
 * iteration's gradient, so an accepted step costs one gradient sweep.  The
 * check passes when the squared record residual of the proposal is at most
 * (1 - min_decrease) times the current field's (0 <= min_decrease < 1).  A
 * rejected proposal falls back to the plain weighted-SIRT step from the saved
 * field (TOMO_SIRT_NORM with `fallback`); after `patience` consecutive
 * rejections (0: never) the run stops proposing and continues with plain
 * steps only (or, with tomo_set_learned_resume, proposes again after that
 * many plain steps).  With tomo_set_learned_backtrack(ctx, n), a rejected proposal is
 * first retried up to n times at half the previous scale (one gradient sweep
 * each, the same network output) before the plain fallback.  Per iteration
 * eps_log gets the image error (NaN without d_f_true) and step_log 1 (learned
 * step), 2 (learned step accepted after backtracking), 0 (rejected proposal,
 * plain step) or -1 (plain step, no proposal); both optional, at least
 * max_iters entries.
 * *sweeps counts the gradient sweeps (forward + adjoint of all groups) the run
 * made, *seconds its host wall time after the one-off illumination sweep.  The
 * counterpart of tomo_run for the learned update; the reference has none. */
tomo_status tomo_run_learned(tomo_ctx* ctx, tomo_net* net, const tomo_schedule* fallback, float* d_f,
                             const float* d_f_true, double target_epsilon, int32_t max_iters, double min_decrease,
                             int32_t patience, double* eps_log, int32_t* step_log, int32_t* iters_done,
                             int32_t* sweeps, double* seconds);

/* Scale of the learned proposal: tomo_iterate_learned and tomo_run_learned propose
 * f + scale * mask * net(features) (default 1; 0 < scale <= 4). */
tomo_status tomo_set_learned_scale(tomo_ctx* ctx, double scale);

/* Retries of a rejected learned proposal in tomo_run_learned, each at half the
 * previous scale, before the plain fallback (default 0; 0 <= retries <= 4).  No
 * counterpart in the reference. */
tomo_status tomo_set_learned_backtrack(tomo_ctx* ctx, int32_t retries);

/* Plain steps after which tomo_run_learned resumes proposing once `patience`
 * rejections in a row have paused it (default 0: never resume; 0..1000).  No
 * counterpart in the reference. */
tomo_status tomo_set_learned_resume(tomo_ctx* ctx, int32_t plain_steps);

/* Several independent reconstructions advanced together (the batched
 * many-phantom workload: phantoms of different grid sizes, each its own
 * context and stream).  Context i runs `iters` iterations of `method` from
 * iteration index iter0 on its device field d_f[i] (records set beforehand).
 * When every iteration is device work only (a SIRT method, one device, the
 * same step for all the call's iterations, no noise redrawn per sweep), one
 * iteration of every context is recorded into one CUDA graph, a branch per
 * context, kept with ctxs[0] and replayed once per iteration (recorded again
 * when the contexts, field pointers, method or step change); otherwise each
 * context runs on a host thread of its own.  Either way the contexts' kernels
 * overlap on the GPU and give the same bits as one context at a time.
 * d_f_true (optional, per context) fills eps_log[i * iters + it] (optional).
 * *seconds (optional) is the wall time of the whole batch.  Returns the first
 * failing context's status (its tomo_last_error has the reason).  Replaces
 * running the reference drivers one after another; the reference has no batch
 * entry point. */
tomo_status tomo_iterate_batch(tomo_ctx** ctxs, int32_t n, int32_t method, const tomo_schedule* sched,
                               int32_t iter0, int32_t iters, float** d_f, const float** d_f_true, double* eps_log,
                               double* seconds);

/* Forward solve without any device allocation (no counterpart in the
 * reference).  For callers that cannot call cudaMalloc: applications whose own
 * pool allocator owns all device memory, or latency-bound loops where
 * cudaMalloc/cudaFree would synchronise the device.  d_f (nx*ny) and d_records
 * (G*nt*n_channels, the tomo_forward layout) are caller-owned device buffers on
 * the current device; work is enqueued on `stream` (NULL: legacy default) and
 * the records are valid once it completes.  The wavefield scratch lives in a
 * fixed file-scope device array of about 5.1 MiB that each GPU loading the
 * library holds until exit, so problems are limited to 512*512 cells, 2048
 * record channels and 16384 time steps (and 4096 emitters in the benchmark
 * profile, 2048 groups in the reference profile); larger ones return
 * TOMO_ERR_ARG with a one-line reason on stderr.  Each call looks the array's
 * device address up in the current context (cudaGetSymbolAddress); the first
 * call on a device also loads the library's device code there, so make that
 * first call before any stream capture.  The geometry tables reach the array
 * as kernel arguments, so no device work refers to host memory after the call
 * returns.  All calls on a device share the one array: calls that overlap on
 * the GPU (concurrent streams or threads) race, so serialise them on one
 * stream. */
tomo_status tomo_forward_noalloc(const tomo_config* cfg, const float* d_f, float* d_records,
                                 void* stream);

#ifdef __cplusplus
}
#endif
#endif /* TOMO_H */
