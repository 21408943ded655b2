/*
 * libibgb300 diagnostics: timing and introspection used by benchmarks and profilers.
 * These entry points have no counterpart in the reference (which has no instrumentation);
 * they observe the same step that ib_advance runs.
 */
#ifndef IBGB300_DIAG_H
#define IBGB300_DIAG_H

#include <stdint.h>

#include "ibgb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ib_info {
  int32_t kernels_per_step;  /* kernel nodes in the captured step graph */
  int32_t nx, ny, nlevels;
  int32_t nbodies, npoints;
  int64_t device_bytes;      /* device memory held by the handle */
  double setup_ms;           /* wall time of ib_create (tables, delta weights, Schur inverse) */
  int32_t vort2flux_order;   /* the order in effect: IB_V2F_LEVELS or IB_V2F_SEQUENTIAL */
  int32_t transform_form;    /* the sine-transform passes in effect: IB_FORM_* */
  int32_t scheme;            /* IB_SCHEME_* */
  int32_t rkc_stages;        /* stages of the Runge-Kutta-Chebyshev scheme (0 for CNAB) */
  int32_t sm_count;          /* streaming multiprocessors of the handle's device */
} ib_info;

#define IB_FORM_STOCKHAM 0   /* shared-memory Stockham FFT passes, 64 threads per line */
#define IB_FORM_WARP 1       /* warp-per-line FFT passes with a transposed intermediate */
#define IB_FORM_TENSOR 2     /* BF16x3 sine-matrix GEMMs on the tensor cores (tcgen05) */

int ib_get_info(ib_handle* h, ib_info* info);

/* The setup-time autotuner's measurements: ms[(form * 2 + levels) * 2 + y8] = device time of the
 * timed unit (the batched Crank-Nicolson solve of all levels, a projection solve, a full and a
 * level-1 Vort2Flux) for transform form IB_FORM_*, Vort2Flux order (levels = 1: all levels in
 * one batch) and warp y-pass occupancy (y8 = 1: the variant compiled for 8 resident blocks per
 * SM), -1 where the candidate was not tried; *chosen = the index in effect (-1 when the tuner
 * did not run: IBGB300_AUTOTUNE=0 or every choice pinned).  No counterpart in the reference,
 * whose FFTW plans are chosen by FFTW's own EXHAUSTIVE planner (fluid-ops.jl:25). */
int ib_get_autotune(ib_handle* h, double* ms /* [12] */, int32_t* chosen);

/* ib_advance_n bracketed by CUDA events on the handle's stream: *device_ms is the device time
 * of the n steps (graph replays plus their per-step base-flux uploads) */
int ib_advance_n_timed(ib_handle* h, int32_t n, const double* t, const double* uv, double* device_ms);

/* n steps issued eagerly (no graph) with CUDA events around every launch of one kernel class
 * (0: x-direction sine-transform pass, 1: y-direction pass, 2: nonlinear term); returns the
 * summed launch time and the launch count.  The steps advance the state like ib_advance_n. */
int ib_profile_steps(ib_handle* h, int32_t n, const double* t, const double* uv, int32_t kernel_class,
                     double* total_ms, int64_t* launches);

/* FMA throughput of the FP64 and FP32 pipes of a device (independent dependency chains, no
 * memory traffic), in TFLOP/s */
int ib_measure_fp_peaks(int32_t device, double* fp64_tflops, double* fp32_tflops);

/* cudaProfilerStart / cudaProfilerStop, so a profiler started with capture disabled records
 * only the region between them (e.g. the timed steps, not the setup) */
int ib_profiler_start(void);
int ib_profiler_stop(void);

#ifdef __cplusplus
}
#endif

#endif /* IBGB300_DIAG_H */
