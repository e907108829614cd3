// Shared device helpers for the dxtb_gb300 kernels (sm_103a, float64).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

#include "../../include/dxtb_gb300.h"

#define DXTB_CHECK_LAUNCH()                                   \
  do {                                                        \
    cudaError_t _e = cudaGetLastError();                      \
    if (_e != cudaSuccess) return DXTB_ERR_LAUNCH;            \
  } while (0)

namespace dxtb {

constexpr double kPi = 3.141592653589793238462643383279502884;
constexpr double kEps = 2.220446049250313080847263336181640625e-16;
constexpr double kTiny = 2.2250738585072014e-308;

__device__ __forceinline__ double pf(const double *p, int off) { return __ldg(p + off); }
__device__ __forceinline__ int pi_(const int32_t *p, int off) { return __ldg(p + off); }

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Block-wide sum; `red` is shared scratch of >= 32 doubles. All threads of
// the block must call it; every thread receives the result.
__device__ __forceinline__ double block_sum(double v, double *red) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nw = (blockDim.x + 31) >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  double t = (threadIdx.x < nw) ? red[threadIdx.x] : 0.0;
  if (wid == 0) t = warp_sum(t);
  if (threadIdx.x == 0) red[0] = t;
  __syncthreads();
  double r = red[0];
  __syncthreads();
  return r;
}

__device__ __forceinline__ double block_max(double v, double *red) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nw = (blockDim.x + 31) >> 5;
  v = warp_max(v);
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  double t = (threadIdx.x < nw) ? red[threadIdx.x] : -1.0e308;
  if (wid == 0) t = warp_max(t);
  if (threadIdx.x == 0) red[0] = t;
  __syncthreads();
  double r = red[0];
  __syncthreads();
  return r;
}

// Size classes of the SCF launch (smallest n of classes 1..5); a filter
// restricts a kernel to the molecules of one class (cls < 0: all).
constexpr int kClasses = 6;
struct ClassFilter {
  int thr[kClasses];
  int cls;
};

__host__ __device__ inline int scf_class(const int *thr, int n) {
  int c = 0;
  for (int k = 1; k < kClasses; ++k)
    if (n >= thr[k]) c = k;
  return c;
}

__device__ __forceinline__ bool in_class(const ClassFilter &f, const dxtb_batch &b, int m) {
  return f.cls < 0 || scf_class(f.thr, (int)(b.ao_off[m + 1] - b.ao_off[m])) == f.cls;
}

// SM count of the current device, cached per device (host side).
inline int32_t device_sms(int *sms) {
  static std::mutex mu;
  static int cache[64] = {0};
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return DXTB_ERR_LAUNCH;
  std::lock_guard<std::mutex> lock(mu);
  if (cache[dev] == 0) {
    int v = 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0)
      return DXTB_ERR_LAUNCH;
    cache[dev] = v;
  }
  *sms = cache[dev];
  return DXTB_OK;
}

// One-time set-up per device (host side). CUDA keeps kernel attributes such
// as the dynamic shared-memory limit per device, so each device runs `setup`
// on its first use; `setup` returns false on a CUDA error, and the next call
// on that device tries again.
struct PerDeviceOnce {
  std::mutex mu;
  bool done[64] = {};
};
template <class F>
inline int32_t per_device_once(PerDeviceOnce &once, F &&setup) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return DXTB_ERR_LAUNCH;
  std::lock_guard<std::mutex> lock(once.mu);
  if (once.done[dev]) return DXTB_OK;
  if (!setup()) {
    cudaGetLastError();
    return DXTB_ERR_LAUNCH;
  }
  once.done[dev] = true;
  return DXTB_OK;
}

// Molecule of a flat index given a prefix array off[0..nmol] (binary search).
__device__ __forceinline__ int find_mol(const int64_t *off, int nmol, int64_t k) {
  int lo = 0, hi = nmol - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (__ldg(off + mid) <= k) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Nuclear-gradient kernels of the molecules selected by a filter (gradient.cu).
int32_t launch_gradient(const dxtb_batch *b, const double *par_f, const int32_t *par_i,
                        const double *cn, const double *mrad, const double *density,
                        const double *wdensity, const double *q, const double *dp, const double *qp,
                        const double *vorb, const double *vdp, const double *vqp,
                        const double *overlap, const double *dipole, double *dedcn, double *grad,
                        const ClassFilter &f, cudaStream_t st);

}  // namespace dxtb
