// Peak-rate probes used to state the FP64 roofline (the GPU's FP64 rate is
// not among the measured HBM / bf16 peaks).  Each thread runs 8 independent
// dependency chains of the instruction under test, long enough to hide
// latency; the grid covers every SM several times.
#include <cuda_runtime.h>

#include "openabl_cuda_diag.h"

namespace {

template <int OP>
__global__ void k_fp64_chain(double *out, int iters, double a, double b) {
  double x[8];
#pragma unroll
  for (int k = 0; k < 8; k++) x[k] = (double) (threadIdx.x + k) * 1e-3;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int k = 0; k < 8; k++) {
      if (OP == 0) x[k] = fma(x[k], a, b);       // DFMA
      else if (OP == 1) x[k] = x[k] + b;         // DADD
      else x[k] = x[k] * a;                      // DMUL
    }
  }
  double s = 0;
#pragma unroll
  for (int k = 0; k < 8; k++) s += x[k];
  if (s == 12345.678) out[0] = s;  // keeps the chains live
}

template <int OP>
int time_op(double *ops_per_s) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  double *out = nullptr;
  if (cudaMalloc(&out, sizeof(double)) != cudaSuccess) return ABL_DIAG_E_CUDA;
  const int threads = 256, blocks = sms * 8, iters = 4096;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_fp64_chain<OP><<<blocks, threads>>>(out, 64, 1.0000001, 1e-9);  // warm-up
  cudaEventRecord(e0);
  k_fp64_chain<OP><<<blocks, threads>>>(out, iters, 1.0000001, 1e-9);
  cudaEventRecord(e1);
  cudaError_t err = cudaEventSynchronize(e1);
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (err != cudaSuccess || ms <= 0) return ABL_DIAG_E_CUDA;
  *ops_per_s = (double) blocks * threads * iters * 8 / (ms * 1e-3);
  return 0;
}

}  // namespace

extern "C" int abl_diag_fp64_rates(double *dfma_per_s, double *dadd_per_s, double *dmul_per_s) {
  int r = 0;
  if (dfma_per_s && (r = time_op<0>(dfma_per_s)) != 0) return r;
  if (dadd_per_s && (r = time_op<1>(dadd_per_s)) != 0) return r;
  if (dmul_per_s && (r = time_op<2>(dmul_per_s)) != 0) return r;
  return 0;
}
