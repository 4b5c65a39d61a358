/* Diagnostics of the OpenABL CUDA runtime (no counterpart in the reference,
 * which has no GPU path of its own): instruction-rate probes used to state
 * the FP64 roofline of the neighbour kernels. */
#ifndef OPENABL_CUDA_DIAG_H
#define OPENABL_CUDA_DIAG_H

#ifdef __cplusplus
extern "C" {
#endif

#define ABL_DIAG_E_CUDA -3

/* Measured FP64 fused-multiply-add, add and multiply instructions per second
 * (per lane) on the current device; any pointer may be NULL. */
int abl_diag_fp64_rates(double *dfma_per_s, double *dadd_per_s, double *dmul_per_s);

#ifdef __cplusplus
}
#endif

#endif
