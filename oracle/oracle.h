/*
 * oracle.h -- CPU restatement of the reference's reconstruction hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference arm of bench.py may load this library; the product
 * (libtomo.so, the CLI drivers) never links or calls it.
 *
 * Pinning: the oracle is checked against the reference's own recorded outputs,
 * the epsilon-per-iteration logs data_dynamic/sirt{,-norm}-dyn-<gs>-0.txt,
 * by replaying each log's recorded step sizes (tests/test_oracle_pins.py).
 *
 * prec selects the arithmetic: 64 (default oracle) or 32 (an FP32 transcription
 * used to separate rounding from bugs and as the timed CPU baseline).
 * threads <= 0 uses every OpenMP thread.
 */
#ifndef TOMO_ORACLE_H
#define TOMO_ORACLE_H

#include <stdint.h>
#include "tomo.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_info {
    int32_t n_groups;
    int32_t n_channels;
    int32_t n_transducers;
} orc_info;

int orc_info_get(const tomo_config* cfg, orc_info* out);

/* Transducer cells (REF: 1-based, as Position_Transducers; CFG: 0-based). */
int orc_transducers(const tomo_config* cfg, int32_t* ii, int32_t* jj);
/* Update mask (1 inside the reconstruction region). */
int orc_mask(const tomo_config* cfg, uint8_t* mask);
/* generate-field's phantom (generate-field.cu:117-172). */
int orc_phantom_ref(int32_t nx, int32_t ny, float* fo);

/* Forward solve of all groups; records G*nt*n_channels; u_last (optional)
 * G*nx*ny wavefield at step nt-1. */
int orc_forward(const tomo_config* cfg, int prec, int threads, const double* f,
                float* records, double* u_last);

/* Per-group gradients dfg (G*nx*ny, optional) = C_g*scale/(1+f), and the
 * squared record residual (optional). meas: G*nt*n_channels. */
int orc_gradient(const tomo_config* cfg, int prec, int threads, const double* f,
                 const float* meas, double* dfg, double* resid2);

/* The same for groups g0 .. g0+ng-1 only: dfg (ng*nx*ny, optional) and their
 * squared record residual (optional). */
int orc_gradient_groups(const tomo_config* cfg, int prec, int threads, const double* f,
                        const float* meas, int g0, int ng, double* dfg, double* resid2);

/* One iteration of `method`; stats[0]=epsilon (NaN without f_true),
 * stats[1]=resid2 at the start, stats[2]=scale. */
int orc_iterate(const tomo_config* cfg, int prec, int threads, int method,
                const tomo_schedule* sched, int iter, double* f_inout,
                const float* meas, const double* f_true, double* stats);

/* Forward+adjoint sweep of groups [g0, g0+ng) without the update, for timing
 * the CPU baseline: returns the credited cell-updates in *cell_updates. */
int orc_sweep(const tomo_config* cfg, int prec, int threads, const double* f,
              const float* meas, int g0, int ng, double* cell_updates);

#ifdef __cplusplus
}
#endif
#endif
