// FP64 FMA throughput probe: the denominator of the FP64 roofline (the
// measured-peak file of the machine lists HBM and bf16 rates only).
// Every thread runs 8 independent FMA chains; flops = 2 * 8 * iters * threads.
#include "common.cuh"

__global__ void k_fp64_fma(int64_t iters, double seed, double *out) {
  double a[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) a[k] = seed + threadIdx.x * 1e-9 + k * 1e-7;
  const double m = 0.9999999, c = 1e-9;
  for (int64_t i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = fma(a[k], m, c);
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += a[k];
  if (s == 12345.6789) out[0] = s;  // keeps the chains alive
}

extern "C" int32_t dxtb_fp64_fma_probe(int64_t iters, int32_t blocks, int32_t threads,
                                       double *out, void *stream) {
  if (iters <= 0 || blocks <= 0 || threads <= 0 || threads > 1024 || !out) return DXTB_ERR_ARGS;
  k_fp64_fma<<<blocks, threads, 0, (cudaStream_t)stream>>>(iters, 1.0, out);
  DXTB_CHECK_LAUNCH();
  return DXTB_OK;
}
