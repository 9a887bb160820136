/*
 * ptgpu_prof.h -- measurement hooks of libptgpu (not part of the reference's interface; the
 * reference times its phases with omp_get_wtime accumulators, basics.f90:27-31, printed at
 * main.f90:305-346).  Used by the benchmark to time kernels with CUDA events on the library's
 * own stream and to count kernel launches.
 */
#ifndef PTGPU_PROF_H
#define PTGPU_PROF_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* kernel classes timed when profiling is on */
#define PT_KT_RKC_FP64_L1 0 /* one FP64 RKC1 smoother stage on the finest level */
#define PT_KT_RKC_FP32_L1 1 /* one FP32 RKC1 smoother stage on the finest level (mixed precision) */
#define PT_KT_RK_STAGE 2    /* one RK4 tracer stage (3 interpolations + update per tracer) */
#define PT_KT_PROJECT 3     /* one tracer->grid projection (sort, partial sums, node sums) */

/* Bracket every batch of launches of the timed kernel classes with CUDA events (adds one
 * event synchronisation per batch). */
int pt_prof_enable(int on);
/* Zero the per-class counters and the kernel launch counter. */
int pt_prof_reset(void);
/* Launches and summed event time (ms) of a kernel class since the last reset. */
int pt_prof_kernel(int id, int64_t* launches, double* total_ms);
/* Number of kernels this library launched since the last reset. */
int64_t pt_prof_launches(void);
/* Device-timed region on the library's stream: end=0 records the start event and opens the NVTX
 * range "pt_timed"; end=1 records the stop event, waits for it, closes the range and returns the
 * elapsed milliseconds in *ms. */
int pt_prof_region(int end, double* ms);
/* Mixed precision tracer order (internal: tracer fields are always exchanged in the caller's
 * order): re-sorts by cell since the last pt_upload_state, and the average number of cell runs per
 * projection thread (of 16 consecutive tracers) in the last projection. */
int pt_prof_tracer_order(int64_t* resorts, double* runs_per_thread);
/* Mixed precision: the RK stage's FP32 interpolation table `which` (0 u, 1 w, 2 the tracer-space
 * term) as last built, nodes i = 0..nx of rows k = -3..nz+3, row-major, four floats per node
 * (value and x-derivatives of order 1, 2, 3): (nz+7)(nx+1)*4 floats. */
int pt_prof_table(int which, float* host);
/* Relative residual mean|r| / mean|RHS| of the last psi solve at each convergence test, in order
 * (the reference logs the final one, iterative_solver.f90:338): the first min(count, cap) values
 * go to out, *count receives the number of tests.  Kept when the solve fails (cycle cap,
 * divergence), so a caller can read how far it got. */
int pt_prof_residuals(double* out, int cap, int* count);
/* Largest sub-record payload of the restart writer in bytes (0: gfortran's 2^31-9), so that tests
 * can exercise the sub-record form on small files. */
int pt_prof_record_limit(int64_t bytes);

#ifdef __cplusplus
}
#endif
#endif
