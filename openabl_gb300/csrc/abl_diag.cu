// Peak-rate probes used to state the FP64 roofline (the GPU's FP64 rate is
// not among the measured HBM / bf16 peaks).  Each thread runs 8 independent
// dependency chains of the instruction under test, long enough to hide
// latency; the grid covers every SM several times.
#include <cuda_runtime.h>

#include "abl_device.cuh"
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
int time_op(double *ops_per_s, double a = 1.0000001) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  double *out = nullptr;
  if (cudaMalloc(&out, sizeof(double)) != cudaSuccess) return ABL_DIAG_E_CUDA;
  const int threads = 256, blocks = sms * 8, iters = 4096;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_fp64_chain<OP><<<blocks, threads>>>(out, 64, a, 1e-9);  // warm-up
  cudaEventRecord(e0);
  k_fp64_chain<OP><<<blocks, threads>>>(out, iters, a, 1e-9);
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

// Operands for the division check: random bit patterns over the whole
// double range (guard cases included), sums of positions in [0, 40), signed
// values, and exact multiples of n.
__device__ double division_operand(uint64_t seed, long i, int n) {
  uint64_t z = seed + 0x9E3779B97F4A7C15ull * (uint64_t) (i + 1);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  switch (i & 3) {
    case 0: return __longlong_as_double((long long) z);
    case 1: return (double) (z >> 11) * 0x1p-53 * 40.0;
    case 2: return ((double) (z >> 11) * 0x1p-53 - 0.5) * 64.0;
    default: return (double) (long) (z % 100000) * 0.001 * n;
  }
}

__global__ void k_division_check(uint64_t seed, long per_n, unsigned long long *bad,
                                 unsigned long long *checked) {
  const long total = per_n * (abl::kRecipN + 7);
  unsigned long long nbad = 0, nchk = 0;
  for (long t = (long) blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (long) gridDim.x * blockDim.x) {
    const int n = (int) (t / per_n) - 3;  // n from -3 to kRecipN + 3: both guard sides
    const double a = division_operand(seed, t, n);
    const double q = abl::div_int(a, n);
    const double r = __ddiv_rn(a, (double) n);
    nchk++;
    // Equal bits, or both NaN (the quotient of a NaN is a NaN either way).
    if (__double_as_longlong(q) != __double_as_longlong(r) && !(q != q && r != r)) nbad++;
  }
  atomicAdd(bad, nbad);
  atomicAdd(checked, nchk);
}

}  // namespace

extern "C" int abl_diag_check_int_division(unsigned long long seed, long per_n,
                                           unsigned long long *checked,
                                           unsigned long long *mismatches) {
  if (per_n <= 0 || !checked || !mismatches) return ABL_DIAG_E_ARG;
  unsigned long long *d = nullptr;
  if (cudaMalloc(&d, 2 * sizeof(unsigned long long)) != cudaSuccess) return ABL_DIAG_E_CUDA;
  cudaMemset(d, 0, 2 * sizeof(unsigned long long));
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  k_division_check<<<sms * 4, 256>>>(seed, per_n, d, d + 1);
  unsigned long long h[2] = {0, 0};
  cudaError_t err = cudaMemcpy(h, d, sizeof h, cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (err != cudaSuccess) return ABL_DIAG_E_CUDA;
  *mismatches = h[0];
  *checked = h[1];
  return 0;
}

// An addition x + b issued as fma(x, 1.0, b): the same correctly rounded
// sum, on the fused-multiply-add path.  The 1.0 is a kernel argument, so the
// compiler cannot turn the fma back into an add.
extern "C" int abl_diag_fp64_add_as_fma_rate(double *per_s) {
  if (!per_s) return ABL_DIAG_E_ARG;
  return time_op<0>(per_s, 1.0);
}

extern "C" int abl_diag_fp64_rates(double *dfma_per_s, double *dadd_per_s, double *dmul_per_s) {
  int r = 0;
  if (dfma_per_s && (r = time_op<0>(dfma_per_s)) != 0) return r;
  if (dadd_per_s && (r = time_op<1>(dadd_per_s)) != 0) return r;
  if (dmul_per_s && (r = time_op<2>(dmul_per_s)) != 0) return r;
  return 0;
}
