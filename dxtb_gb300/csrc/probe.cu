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

// FP64 tensor-core (DMMA) throughput probe: every warp runs 4 independent
// accumulator chains of mma.sync f64 of one shape. Shapes: 0 = m8n8k4
// (sm_80), 1 = m16n8k4, 2 = m16n8k8, 3 = m16n8k16 (sm_90 and later).
// flops per launch = 2 * M * N * K * 4 * iters * (threads / 32) * blocks.
template <int SHAPE>
__global__ void k_fp64_mma(int64_t iters, double seed, double *out) {
  const double a = seed * 1e-3 + (threadIdx.x & 31) * 1e-9, b = 1e-3;
  double c[4][4];
#pragma unroll
  for (int k = 0; k < 4; ++k)
#pragma unroll
    for (int r = 0; r < 4; ++r) c[k][r] = k * 1e-7 + r * 1e-8;
  for (int64_t i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      if constexpr (SHAPE == 0) {
        asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
                     : "+d"(c[k][0]), "+d"(c[k][1])
                     : "d"(a), "d"(b));
      } else if constexpr (SHAPE == 1) {
        asm volatile(
            "mma.sync.aligned.m16n8k4.row.col.f64.f64.f64.f64 {%0,%1,%2,%3}, {%4,%5}, {%6}, "
            "{%0,%1,%2,%3};"
            : "+d"(c[k][0]), "+d"(c[k][1]), "+d"(c[k][2]), "+d"(c[k][3])
            : "d"(a), "d"(a), "d"(b));
      } else if constexpr (SHAPE == 2) {
        asm volatile(
            "mma.sync.aligned.m16n8k8.row.col.f64.f64.f64.f64 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
            "{%8,%9}, {%0,%1,%2,%3};"
            : "+d"(c[k][0]), "+d"(c[k][1]), "+d"(c[k][2]), "+d"(c[k][3])
            : "d"(a), "d"(a), "d"(a), "d"(a), "d"(b), "d"(b));
      } else {
        asm volatile(
            "mma.sync.aligned.m16n8k16.row.col.f64.f64.f64.f64 {%0,%1,%2,%3}, "
            "{%4,%5,%6,%7,%8,%9,%10,%11}, {%12,%13,%14,%15}, {%0,%1,%2,%3};"
            : "+d"(c[k][0]), "+d"(c[k][1]), "+d"(c[k][2]), "+d"(c[k][3])
            : "d"(a), "d"(a), "d"(a), "d"(a), "d"(a), "d"(a), "d"(a), "d"(a), "d"(b), "d"(b),
              "d"(b), "d"(b));
      }
    }
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < 4; ++k)
#pragma unroll
    for (int r = 0; r < 4; ++r) s += c[k][r];
  if (s == 12345.6789) out[0] = s;  // keeps the chains alive
}

extern "C" int32_t dxtb_fp64_mma_probe(int32_t shape, int64_t iters, int32_t blocks, int32_t threads,
                                       double *out, void *stream) {
  if (iters <= 0 || blocks <= 0 || threads <= 0 || threads > 1024 || threads % 32 || !out ||
      shape < 0 || shape > 3)
    return DXTB_ERR_ARGS;
  cudaStream_t st = (cudaStream_t)stream;
  switch (shape) {
    case 0: k_fp64_mma<0><<<blocks, threads, 0, st>>>(iters, 1.0, out); break;
    case 1: k_fp64_mma<1><<<blocks, threads, 0, st>>>(iters, 1.0, out); break;
    case 2: k_fp64_mma<2><<<blocks, threads, 0, st>>>(iters, 1.0, out); break;
    default: k_fp64_mma<3><<<blocks, threads, 0, st>>>(iters, 1.0, out); break;
  }
  DXTB_CHECK_LAUNCH();
  return DXTB_OK;
}
