// CTA-level dense float64 linear algebra for one molecule's AO matrices
// (row-major, leading dimension n, resident in global memory / L2). Every
// routine must be called by all threads of the block.
//
// The symmetric eigenproblem of the SCF is solved as
//   Householder tridiagonalisation  (cta_tridiag)
//   -> eigenvalues by implicit QL without vectors (cta_tql_values)
//   -> eigenvectors of the lowest m eigenvalues only, by inverse iteration
//      with a pivoted tridiagonal LU, one thread per eigenvalue cluster,
//      Gram-Schmidt inside clusters (cta_tri_vectors)
//   -> back-transformation of those m vectors (cta_back_transform).
// The SCF needs only the orbitals with non-vanishing occupation, so the
// O(n^3) accumulation of QL rotations is never done.
#pragma once
#include "common.cuh"

namespace dxtb {

// Shapes of the k-loop for triangular operands.
constexpr int kTriSmem = 512;  // Householder vectors in shared memory up to this order

enum KRange : int {
  kFull = 0,     // k in [0, K)
  kALower = 1,   // op(A)(i,k) = 0 for k > i   -> k < i0 + 4
  kBLowerT = 2,  // op(B)(k,j) = 0 for k > j   -> k < j0 + 4
  kBUpper = 3,   // op(B)(k,j) = 0 for k < j   -> k >= j0
};

// C = alpha * op(A) op(B) + beta * C for M x N outputs and inner size K.
// op(A)(i,k) = TA ? A[k*lda+i] : A[i*lda+k]; op(B)(k,j) = TB ? B[j*ldb+k] : B[k*ldb+j].
// Register tile of 4 x 4 outputs per thread. With lower_only, tiles strictly
// above the diagonal are skipped (symmetric results). The FP64 pipe, not
// memory, is the limit at these sizes.
template <bool TA, bool TB>
__device__ void cta_gemm(int M, int N, int K, double alpha, const double *__restrict__ A, int lda,
                         const double *__restrict__ B, int ldb, double beta, double *__restrict__ C,
                         int ldc, int krange = kFull, bool lower_only = false) {
  const int tm = (M + 3) >> 2, tn = (N + 3) >> 2;
  for (int t = threadIdx.x; t < tm * tn; t += blockDim.x) {
    const int i0 = (t / tn) * 4, j0 = (t % tn) * 4;
    if (lower_only && j0 > i0 + 3) continue;
    double acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int c = 0; c < 4; ++c) acc[a][c] = 0.0;
    int ia[4], jb[4];
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      ia[a] = min(i0 + a, M - 1);
      jb[a] = min(j0 + a, N - 1);
    }
    int k0 = 0, k1 = K;
    if (krange == kALower) k1 = min(K, i0 + 4);
    else if (krange == kBLowerT) k1 = min(K, j0 + 4);
    else if (krange == kBUpper) k0 = j0;
    for (int k = k0; k < k1; ++k) {
      double av[4], bv[4];
#pragma unroll
      for (int a = 0; a < 4; ++a) av[a] = TA ? A[(size_t)k * lda + ia[a]] : A[(size_t)ia[a] * lda + k];
#pragma unroll
      for (int c = 0; c < 4; ++c) bv[c] = TB ? B[(size_t)jb[c] * ldb + k] : B[(size_t)k * ldb + jb[c]];
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[a][c] = fma(av[a], bv[c], acc[a][c]);
    }
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const int i = i0 + a, j = j0 + c;
        if (i < M && j < N && (!lower_only || j <= i)) {
          double *p = C + (size_t)i * ldc + j;
          *p = alpha * acc[a][c] + (beta == 0.0 ? 0.0 : beta * *p);
        }
      }
  }
  __syncthreads();
}

// Copy the lower triangle of a square matrix onto its upper triangle.
__device__ void cta_mirror_lower(int n, double *A) {
  for (int64_t t = threadIdx.x; t < (int64_t)n * n; t += blockDim.x) {
    const int i = (int)(t / n), j = (int)(t % n);
    if (j > i) A[t] = A[(size_t)j * n + i];
  }
  __syncthreads();
}

// In-place lower Cholesky factor of a symmetric positive-definite matrix
// (right-looking). Returns false if a pivot is not positive.
__device__ bool cta_cholesky(int n, double *A) {
  __shared__ int s_bad;
  if (threadIdx.x == 0) s_bad = 0;
  __syncthreads();
  for (int k = 0; k < n; ++k) {
    if (threadIdx.x == 0) {
      const double dkk = A[(size_t)k * n + k];
      if (!(dkk > 0.0)) s_bad = 1;
      A[(size_t)k * n + k] = sqrt(fmax(dkk, kTiny));
    }
    __syncthreads();
    if (s_bad) return false;
    const double lkk = A[(size_t)k * n + k];
    for (int i = k + 1 + threadIdx.x; i < n; i += blockDim.x) A[(size_t)i * n + k] /= lkk;
    __syncthreads();
    const int m = n - k - 1;
    for (int64_t t = threadIdx.x; t < (int64_t)m * m; t += blockDim.x) {
      const int i = k + 1 + (int)(t / m), j = k + 1 + (int)(t % m);
      if (j <= i) A[(size_t)i * n + j] -= A[(size_t)i * n + k] * A[(size_t)j * n + k];
    }
    __syncthreads();
  }
  return true;
}

// X = L^-1 for a lower-triangular L (row-major); upper part of X zeroed.
// Thread j solves column j by forward substitution.
__device__ void cta_trinv(int n, const double *L, double *X) {
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    for (int i = 0; i < j; ++i) X[(size_t)i * n + j] = 0.0;
    X[(size_t)j * n + j] = 1.0 / L[(size_t)j * n + j];
    for (int i = j + 1; i < n; ++i) {
      double s = 0.0;
      for (int k = j; k < i; ++k) s = fma(L[(size_t)i * n + k], X[(size_t)k * n + j], s);
      X[(size_t)i * n + j] = -s / L[(size_t)i * n + i];
    }
  }
  __syncthreads();
}

// Householder reduction of a full symmetric matrix to tridiagonal form
// (lower variant): A = Q T Q^T. On exit d, e hold the diagonal and
// sub-diagonal (e[i] couples i and i+1), the reflector of step k is stored
// in A[k+2..n-1][k] (its leading 1 implicit) with factor tau[k].
__device__ void cta_tridiag(int n, double *A, double *d, double *e, double *tau, double *p,
                            double *vbuf, double *red) {
  // The Householder vector and p live in shared memory when they fit.
  __shared__ double s_v[kTriSmem], s_p[kTriSmem];
  __shared__ double s_part[256];
  double *sv = n <= kTriSmem ? s_v : vbuf;
  double *sp = n <= kTriSmem ? s_p : p;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5, nty = (int)(blockDim.x >> 5);
  for (int k = 0; k < n - 2; ++k) {
    const int m = n - k - 1;
    double *col = A + (size_t)(k + 1) * n + k;  // col[r*n], r < m
    double part = 0.0;
    for (int r = threadIdx.x; r < m; r += blockDim.x) {
      const double x = col[(size_t)r * n];
      sv[r] = x;
      if (r > 0) part += x * x;
    }
    const double sigma = block_sum(part, red);  // also orders the sv writes
    const double alpha = col[0];  // not sv[0]: thread 0 overwrites it below
    double t = 0.0, beta = alpha;
    if (sigma > 0.0) {
      const double nrm = sqrt(alpha * alpha + sigma);
      beta = alpha >= 0.0 ? -nrm : nrm;
      t = (beta - alpha) / beta;
      const double scale = 1.0 / (alpha - beta);
      for (int r = 1 + threadIdx.x; r < m; r += blockDim.x) {
        const double v = sv[r] * scale;
        sv[r] = v;
        col[(size_t)r * n] = v;  // kept for the back-transformation
      }
    }
    if (threadIdx.x == 0) {
      sv[0] = 1.0;
      tau[k] = t;
      e[k] = beta;
      d[k] = A[(size_t)k * n + k];
    }
    __syncthreads();
    if (t != 0.0) {
      // p = t * A22 v; A22 is symmetric, so row r of the product reads
      // column r (coalesced over r). The c range is split into G groups so
      // that all threads work; partials in smem, p^T v fused in.
      const double *A22 = A + (size_t)(k + 1) * n + (k + 1);
      const int G = m < (int)blockDim.x ? max(1, min(256 / m, (int)blockDim.x / m)) : 1;
      for (int q = threadIdx.x; q < G * m; q += blockDim.x) {
        const int r = q % m, g = q / m;
        double s = 0.0;
        for (int c = g; c < m; c += G) s = fma(A22[(size_t)c * n + r], sv[c], s);
        if (G > 1) s_part[g * m + r] = s; else sp[r] = t * s;
      }
      __syncthreads();
      double part2 = 0.0;
      for (int r = threadIdx.x; r < m; r += blockDim.x) {
        double pr;
        if (G > 1) {
          double s = 0.0;
          for (int g = 0; g < G; ++g) s += s_part[g * m + r];
          pr = t * s;
          sp[r] = pr;
        } else {
          pr = sp[r];
        }
        part2 += pr * sv[r];
      }
      const double K = 0.5 * t * block_sum(part2, red);
      for (int r = threadIdx.x; r < m; r += blockDim.x) sp[r] -= K * sv[r];
      __syncthreads();
      // rank-2 update, rows over warps, columns over lanes (coalesced)
      double *W = A + (size_t)(k + 1) * n + (k + 1);
      for (int r = ty; r < m; r += nty) {
        const double vr = sv[r], pr = sp[r];
        double *Wr = W + (size_t)r * n;
        for (int c = tx; c < m; c += 32) Wr[c] -= vr * sp[c] + pr * sv[c];
      }
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    if (n >= 2) {
      d[n - 2] = A[(size_t)(n - 2) * n + (n - 2)];
      e[n - 2] = A[(size_t)(n - 1) * n + (n - 2)];
      tau[n - 2] = 0.0;
    }
    d[n - 1] = A[(size_t)(n - 1) * n + (n - 1)];
    e[n - 1] = 0.0;
    tau[n - 1] = 0.0;
  }
  __syncthreads();
}

// Eigenvalues of the symmetric tridiagonal (d, e) by implicit QL with
// Wilkinson-type shifts (Bowdler, Martin, Reinsch, Wilkinson, Numer. Math.
// 11, 293 (1968)), without eigenvector accumulation. Thread 0 runs the
// scalar recurrence on the scratch copies sd, se (shared memory when they
// fit); lam receives the (unsorted) eigenvalues. False if an eigenvalue
// needs more than 60 sweeps.
__device__ bool cta_tql_values(int n, const double *d, const double *e, double *sd, double *se,
                               double *lam) {
  __shared__ int s_ok;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    sd[i] = d[i];
    se[i] = e[i];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    for (int l = 0; l < n && ok; ++l) {
      int iter = 0;
      while (true) {
        int m = l;
        for (; m < n - 1; ++m) {
          const double dd = fabs(sd[m]) + fabs(sd[m + 1]);
          if (fabs(se[m]) <= kEps * dd) break;
        }
        if (m == l) break;
        if (++iter > 60) {
          ok = 0;
          break;
        }
        double g = (sd[l + 1] - sd[l]) / (2.0 * se[l]);
        double r = sqrt(g * g + 1.0);
        g = sd[m] - sd[l] + se[l] / (g + copysign(r, g));
        double s = 1.0, c = 1.0, p = 0.0;
        int i = m - 1;
        bool early = false;
        for (; i >= l; --i) {
          const double f = s * se[i], bb = c * se[i];
          r = sqrt(f * f + g * g);
          se[i + 1] = r;
          if (r == 0.0) {
            sd[i + 1] -= p;
            se[m] = 0.0;
            early = true;
            break;
          }
          const double ir = 1.0 / r;
          s = f * ir;
          c = g * ir;
          g = sd[i + 1] - p;
          r = (sd[i] - g) * s + 2.0 * c * bb;
          p = s * r;
          sd[i + 1] = g + p;
          g = c * r - bb;
        }
        if (!early) {
          sd[l] -= p;
          se[l] = g;
          se[m] = 0.0;
        }
      }
    }
    s_ok = ok;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) lam[i] = sd[i];
  __syncthreads();
  return s_ok != 0;
}

// Number of eigenvalues of the tridiagonal (d, e) below x (Sturm count of
// the LDL^T pivots, zero pivots replaced by -tiny), in float32.
__device__ __forceinline__ int sturm_count_f32(int n, const float *d, const float *e2, float x,
                                               float tiny) {
  int cnt = 0;
  float q = d[0] - x;
  if (q == 0.0f) q = -tiny;
  cnt += q < 0.0f;
  for (int i = 1; i < n; ++i) {
    q = (d[i] - x) - e2[i - 1] / q;
    if (q == 0.0f) q = -tiny;
    cnt += q < 0.0f;
  }
  return cnt;
}

// The same count in float64 (robust fallback).
__device__ __forceinline__ int sturm_count_f64(int n, const double *d, const double *e, double x,
                                               double tiny) {
  int cnt = 0;
  double q = d[0] - x;
  if (q == 0.0) q = -tiny;
  cnt += q < 0.0;
  for (int i = 1; i < n; ++i) {
    q = (d[i] - x) - e[i - 1] * e[i - 1] / q;
    if (q == 0.0) q = -tiny;
    cnt += q < 0.0;
  }
  return cnt;
}

// Characteristic polynomial p(x) = det(T - x I) of the leading principal
// minors and its derivative, by the three-term recurrence with rescaling
// (no divisions); returns p / p' (the Newton correction is -p/p').
__device__ __forceinline__ double charpoly_ratio(int n, const double *d, const double *e, double x) {
  double p0 = 1.0, p1 = d[0] - x;   // p_{k-1}, p_k
  double q0 = 0.0, q1 = -1.0;       // p'_{k-1}, p'_k
  for (int i = 1; i < n; ++i) {
    const double di = d[i] - x, e2 = e[i - 1] * e[i - 1];
    const double p2 = di * p1 - e2 * p0;
    const double q2 = -p1 + di * q1 - e2 * q0;
    p0 = p1;
    p1 = p2;
    q0 = q1;
    q1 = q2;
    const double big = fmax(fabs(p1), fabs(q1));
    if (big > 1e150) {
      p0 *= 1e-150; p1 *= 1e-150; q0 *= 1e-150; q1 *= 1e-150;
    } else if (big < 1e-150 && big > 0.0) {
      p0 *= 1e150; p1 *= 1e150; q0 *= 1e150; q1 *= 1e150;
    }
  }
  return q1 != 0.0 ? p1 / q1 : 0.0;
}

// All eigenvalues of the symmetric tridiagonal (d, e), ascending, one per
// thread: float32 bisection on Sturm counts isolates eigenvalue k to ~1e-7
// relative, float64 Newton steps on the characteristic polynomial refine it,
// and a float64 Sturm count checks that the result is the k-th eigenvalue;
// eigenvalues that fail (clusters closer than the float32 resolution) are
// recomputed by float64 bisection. df/e2f: float scratch of n each.
__device__ void cta_tri_eigenvalues(int n, const double *d, const double *e, double *lam,
                                    float *df, float *e2f) {
  __shared__ double s_gl, s_gu;
  double gl = 1e308, gu = -1e308;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double r = (i > 0 ? fabs(e[i - 1]) : 0.0) + (i < n - 1 ? fabs(e[i]) : 0.0);
    gl = fmin(gl, d[i] - r);
    gu = fmax(gu, d[i] + r);
    df[i] = (float)d[i];
    e2f[i] = i < n - 1 ? (float)(e[i] * e[i]) : 0.0f;
  }
  gl = -warp_max(-gl);
  gu = warp_max(gu);
  if (threadIdx.x == 0) {
    s_gl = gl;
    s_gu = gu;
  }
  __syncthreads();
  for (int w = 1; w < (int)((blockDim.x + 31) >> 5); ++w) {
    // fold the other warps' bounds (small loop, no extra shared array)
    __syncthreads();
    if ((threadIdx.x >> 5) == w && (threadIdx.x & 31) == 0) {
      s_gl = fmin(s_gl, gl);
      s_gu = fmax(s_gu, gu);
    }
  }
  __syncthreads();
  const double tnorm = fmax(fabs(s_gl), fabs(s_gu));
  const double span = s_gu - s_gl;
  const double glo = s_gl - 1e-6 * span - 1e-12, ghi = s_gu + 1e-6 * span + 1e-12;
  const float tinyf = 1e-30f;
  const double tiny = 1e-300;
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    // --- float32 bisection: count(lo) <= k < count(hi) ---
    float lo = (float)glo, hi = (float)ghi;
    for (int it = 0; it < 60; ++it) {
      const float mid = 0.5f * (lo + hi);
      if (mid <= lo || mid >= hi) break;
      if (sturm_count_f32(n, df, e2f, mid, tinyf) <= k) lo = mid; else hi = mid;
    }
    const double w32 = fmax((double)hi - (double)lo, 4e-7 * tnorm + 1e-12);
    double x = 0.5 * ((double)lo + (double)hi);
    const double blo = x - 4.0 * w32, bhi = x + 4.0 * w32;
    // --- float64 Newton on p(x) ---
    bool ok = true;
    for (int it = 0; it < 4; ++it) {
      const double dx = charpoly_ratio(n, d, e, x);
      x -= dx;
      if (!(x > blo && x < bhi)) { ok = false; break; }
      if (fabs(dx) <= 2.0 * kEps * fmax(fabs(x), 1e-3 * tnorm)) break;
    }
    // --- check the index with float64 Sturm counts (eigenvalues closer than
    // del are interchangeable: their vectors come from one cluster) ---
    const double del = 1e-12 * fmax(tnorm, 1.0);
    if (ok) {
      const int cl = sturm_count_f64(n, d, e, x - del, tiny);
      const int ch = sturm_count_f64(n, d, e, x + del, tiny);
      ok = (cl <= k && k < ch);
    }
    if (!ok) {
      // --- float64 bisection inside the float32 bracket (widened) ---
      double l = glo, h = ghi;
      if (sturm_count_f64(n, d, e, blo, tiny) <= k && sturm_count_f64(n, d, e, bhi, tiny) > k) {
        l = blo;
        h = bhi;
      }
      for (int it = 0; it < 200; ++it) {
        const double mid = 0.5 * (l + h);
        if (mid <= l || mid >= h) break;
        if (sturm_count_f64(n, d, e, mid, tiny) <= k) l = mid; else h = mid;
      }
      x = 0.5 * (l + h);
    }
    lam[k] = x;
  }
  __syncthreads();
}

// Ascending sort by rank (ties broken by index): out[rank(i)] = in[i].
__device__ void cta_rank_sort(int n, const double *in, double *out) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double v = in[i];
    int r = 0;
    for (int j = 0; j < n; ++j) {
      const double u = in[j];
      r += (u < v) || (u == v && j < i);
    }
    out[r] = v;
  }
  __syncthreads();
}

__device__ __forceinline__ double start_vector(int i, int j) {
  // deterministic pseudo-random start in [0.5, 1.5) (any vector with a
  // component along the eigenvector works)
  uint32_t h = 2654435761u * (uint32_t)(i + 1) ^ 40503u * (uint32_t)(j + 7);
  h ^= h >> 13;
  h *= 0x5bd1e995u;
  h ^= h >> 15;
  return 0.5 + (double)(h & 0xffffff) / 16777216.0;
}

// Eigenvectors of the symmetric tridiagonal (d, e) for the m lowest
// (sorted) eigenvalues lam[0..m) by inverse iteration with a partially
// pivoted LU of T - lam I (the scheme of LAPACK's dstein: three solves,
// re-orthogonalisation against the previous members of the cluster).
// Clusters are runs of eigenvalues closer than ctol; each cluster is one
// thread's work. Y: n x m row-major (column j = vector j).
// lu: scratch of 5 * n * blockDim doubles. cl: int scratch of m + 1.
__device__ void cta_tri_vectors(int n, const double *d, const double *e, const double *lam, int m,
                                double tnorm, double *Y, double *lu, int *cl, int *s_ncl) {
  const double ctol = 1e-6 * fmax(tnorm, 1.0);
  const double tiny = kEps * fmax(tnorm, 1.0);
  if (threadIdx.x == 0) {
    int c = 0;
    cl[c++] = 0;
    for (int j = 1; j < m; ++j)
      if (lam[j] - lam[j - 1] > ctol) cl[c++] = j;
    cl[c] = m;
    *s_ncl = c;
  }
  __syncthreads();
  const int ncl = *s_ncl;
  const int nthr = blockDim.x, tid = threadIdx.x;
  double *U0 = lu, *U1 = lu + (size_t)n * nthr, *U2 = lu + 2 * (size_t)n * nthr;
  double *Lm = lu + 3 * (size_t)n * nthr, *Pv = lu + 4 * (size_t)n * nthr;
#define LU(arr, i) arr[(size_t)(i) * nthr + tid]
  for (int c = tid; c < ncl; c += nthr) {
    const int j0 = cl[c], j1 = cl[c + 1];
    for (int j = j0; j < j1; ++j) {
      // separate exactly coincident shifts inside a cluster (dstein)
      const double lmb = lam[j] + (j - j0) * 10.0 * tiny;
      // LU with partial pivoting of T - lmb I; rows hold (diag, super, super2)
      double a = d[0] - lmb, bsup = n > 1 ? e[0] : 0.0;
      for (int i = 0; i < n - 1; ++i) {
        const double low = e[i];
        const double dn = d[i + 1] - lmb, en = (i + 1 < n - 1) ? e[i + 1] : 0.0;
        if (fabs(a) >= fabs(low)) {
          const double piv = a == 0.0 ? tiny : a;
          const double mult = low / piv;
          LU(U0, i) = piv;
          LU(U1, i) = bsup;
          LU(U2, i) = 0.0;
          LU(Lm, i) = mult;
          LU(Pv, i) = 0.0;
          a = dn - mult * bsup;
          bsup = en;
        } else {
          const double mult = a / low;
          LU(U0, i) = low;
          LU(U1, i) = dn;
          LU(U2, i) = en;
          LU(Lm, i) = mult;
          LU(Pv, i) = 1.0;
          a = bsup - mult * dn;
          bsup = -mult * en;
        }
      }
      LU(U0, n - 1) = a;
      // tiny pivots perturbed (sign kept); U0 then holds the reciprocals
      for (int i = 0; i < n; ++i) {
        const double u = LU(U0, i);
        LU(U0, i) = 1.0 / (fabs(u) < tiny ? copysign(tiny, u == 0.0 ? 1.0 : u) : u);
      }
      for (int i = 0; i < n; ++i) Y[(size_t)i * m + j] = start_vector(i, j);
      const int nsolve = (j1 - j0 > 1) ? 3 : 2;
      for (int it = 0; it < nsolve; ++it) {
        // forward: apply the row interchanges and multipliers
        for (int i = 0; i < n - 1; ++i) {
          double xi = Y[(size_t)i * m + j], xn = Y[(size_t)(i + 1) * m + j];
          if (LU(Pv, i) != 0.0) {
            const double t = xi;
            xi = xn;
            xn = t;
          }
          Y[(size_t)i * m + j] = xi;
          Y[(size_t)(i + 1) * m + j] = xn - LU(Lm, i) * xi;
        }
        // back substitution with the upper factor (two super-diagonals)
        double x1 = 0.0, x2 = 0.0;
        for (int i = n - 1; i >= 0; --i) {
          const double v = (Y[(size_t)i * m + j] - LU(U1, i) * x1 - LU(U2, i) * x2) * LU(U0, i);
          Y[(size_t)i * m + j] = v;
          x2 = x1;
          x1 = v;
        }
        // Gram-Schmidt against the earlier members of the cluster
        for (int k = j0; k < j; ++k) {
          double dot = 0.0;
          for (int i = 0; i < n; ++i) dot += Y[(size_t)i * m + k] * Y[(size_t)i * m + j];
          for (int i = 0; i < n; ++i) Y[(size_t)i * m + j] -= dot * Y[(size_t)i * m + k];
        }
        double nrm = 0.0;
        for (int i = 0; i < n; ++i) nrm += Y[(size_t)i * m + j] * Y[(size_t)i * m + j];
        const double inv = 1.0 / sqrt(fmax(nrm, kTiny));
        for (int i = 0; i < n; ++i) Y[(size_t)i * m + j] *= inv;
      }
    }
  }
#undef LU
  __syncthreads();
}

// Y <- Q Y for the reflectors stored by cta_tridiag (Q = H_0 ... H_{n-3});
// Y is n x m row-major. w: scratch of m doubles.
__device__ void cta_back_transform(int n, const double *A, const double *tau, double *Y, int m,
                                   double *w) {
  for (int k = n - 3; k >= 0; --k) {
    const double t = tau[k];
    if (t == 0.0) continue;
    const int mm = n - k - 1;
    const double *col = A + (size_t)(k + 1) * n + k;
    double *Yb = Y + (size_t)(k + 1) * m;
    // w_j = t * v . Y[:, j]; the r range split into G groups (all threads busy)
    __shared__ double s_bpart[256];
    const int G = m < (int)blockDim.x ? max(1, min(256 / m, (int)blockDim.x / m)) : 1;
    for (int q = threadIdx.x; q < G * m; q += blockDim.x) {
      const int j = q % m, g = q / m;
      double s = 0.0;
      for (int r = g; r < mm; r += G) s = fma(r == 0 ? 1.0 : col[(size_t)r * n], Yb[(size_t)r * m + j], s);
      if (G > 1) s_bpart[g * m + j] = s; else w[j] = t * s;
    }
    __syncthreads();
    if (G > 1) {
      for (int j = threadIdx.x; j < m; j += blockDim.x) {
        double s = 0.0;
        for (int g = 0; g < G; ++g) s += s_bpart[g * m + j];
        w[j] = t * s;
      }
      __syncthreads();
    }
    for (int64_t q = threadIdx.x; q < (int64_t)mm * m; q += blockDim.x) {
      const int r = (int)(q / m), j = (int)(q % m);
      const double vr = r == 0 ? 1.0 : col[(size_t)r * n];
      Yb[(size_t)r * m + j] -= vr * w[j];
    }
    __syncthreads();
  }
}

}  // namespace dxtb
