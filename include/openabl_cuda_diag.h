/* Diagnostics of the OpenABL CUDA runtime (no counterpart in the reference,
 * which has no GPU path of its own): instruction-rate probes used to state
 * the FP64 roofline of the neighbour kernels, and a device-side check of the
 * kernels' integer-divisor division. */
#ifndef OPENABL_CUDA_DIAG_H
#define OPENABL_CUDA_DIAG_H

#ifdef __cplusplus
extern "C" {
#endif

#define ABL_DIAG_E_ARG -2
#define ABL_DIAG_E_CUDA -3

/* Measured FP64 fused-multiply-add, add and multiply instructions per second
 * (per lane) on the current device; any pointer may be NULL. */
int abl_diag_fp64_rates(double *dfma_per_s, double *dadd_per_s, double *dmul_per_s);

/* Measured rate of FP64 additions issued as fma(x, 1.0, y) -- the same
 * correctly rounded sum as x + y -- in instructions per second (per lane). */
int abl_diag_fp64_add_as_fma_rate(double *per_s);

/* Checks the step kernels' division of a double by an int count (a two-term
 * reciprocal table, abl::div_int in the runtime) against IEEE division on
 * the device: per_n operands for every n from -3 to 1027 (both ends outside
 * the table), over the whole double range.  Reports how many quotients were
 * compared and how many differed in any bit (NaN equals NaN). */
int abl_diag_check_int_division(unsigned long long seed, long per_n,
                                unsigned long long *checked, unsigned long long *mismatches);

/* Failure injection for the persistent ensemble kernel's grid barriers
 * (abl_ensemble_set_persistent): every wait gives up after limit_seconds,
 * and each barrier waits for extra_arrivals arrivals beyond the launch's
 * blocks.  With extra_arrivals = 1 no barrier can complete, so the next run
 * returns ABL_E_TIMEOUT (-4) once the first wait has run out, with no kernel
 * left running.  (0.0, 0) restores the defaults.  The ensemble handle is an
 * abl_ensemble* of openabl_cuda.h. */
int abl_diag_ensemble_barrier(void *ensemble, double limit_seconds, int extra_arrivals);

#ifdef __cplusplus
}
#endif

#endif
