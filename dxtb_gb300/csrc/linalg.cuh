// CTA-level dense float64 linear algebra for one molecule's AO matrices
// (row-major, leading dimension n, resident in global memory / L2). Every
// routine must be called by all threads of the block.
#pragma once
#include "common.cuh"

namespace dxtb {

// C = alpha * op(A) op(B) + beta * C for M x N outputs and inner size K.
// op(A)(i,k) = TA ? A[k*lda+i] : A[i*lda+k]; op(B)(k,j) = TB ? B[j*ldb+k] : B[k*ldb+j].
// Register tile of 4 x 4 outputs per thread; the FP64 pipe, not memory, is
// the limit at these sizes.
template <bool TA, bool TB>
__device__ void cta_gemm(int M, int N, int K, double alpha, const double *__restrict__ A,
                         int lda, const double *__restrict__ B, int ldb, double beta,
                         double *__restrict__ C, int ldc) {
  const int tm = (M + 3) >> 2, tn = (N + 3) >> 2;
  for (int t = threadIdx.x; t < tm * tn; t += blockDim.x) {
    const int i0 = (t / tn) * 4, j0 = (t % tn) * 4;
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
    for (int k = 0; k < K; ++k) {
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
        if (i < M && j < N) {
          double *p = C + (size_t)i * ldc + j;
          *p = alpha * acc[a][c] + (beta == 0.0 ? 0.0 : beta * *p);
        }
      }
  }
  __syncthreads();
}

// In-place lower Cholesky factor of a symmetric positive-definite matrix
// (right-looking). Returns false if a pivot is not positive.
__device__ bool cta_cholesky(int n, double *A, double *red) {
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
  (void)red;
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
                            double *red) {
  for (int k = 0; k < n - 2; ++k) {
    const int m = n - k - 1;
    double *col = A + (size_t)(k + 1) * n + k;  // col[r*n], r < m
    double part = 0.0;
    for (int r = 1 + threadIdx.x; r < m; r += blockDim.x) {
      const double x = col[(size_t)r * n];
      part += x * x;
    }
    const double sigma = block_sum(part, red);
    const double alpha = col[0];
    double t = 0.0, beta = alpha;
    if (sigma > 0.0) {
      const double nrm = sqrt(alpha * alpha + sigma);
      beta = alpha >= 0.0 ? -nrm : nrm;
      t = (beta - alpha) / beta;
      const double scale = 1.0 / (alpha - beta);
      for (int r = 1 + threadIdx.x; r < m; r += blockDim.x) col[(size_t)r * n] *= scale;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      tau[k] = t;
      e[k] = beta;
      d[k] = A[(size_t)k * n + k];
    }
    if (t != 0.0) {
      // p = t * A22 v (v[0] = 1, v[r] = col[r*n])
      const double *A22 = A + (size_t)(k + 1) * n + (k + 1);
      for (int r = threadIdx.x; r < m; r += blockDim.x) {
        double s = A22[r];  // c = 0, v0 = 1 (A22 symmetric: A22[c][r])
        for (int c = 1; c < m; ++c) s = fma(A22[(size_t)c * n + r], col[(size_t)c * n], s);
        p[r] = t * s;
      }
      __syncthreads();
      double part2 = 0.0;
      for (int r = threadIdx.x; r < m; r += blockDim.x)
        part2 += p[r] * (r == 0 ? 1.0 : col[(size_t)r * n]);
      const double K = 0.5 * t * block_sum(part2, red);
      for (int r = threadIdx.x; r < m; r += blockDim.x) p[r] -= K * (r == 0 ? 1.0 : col[(size_t)r * n]);
      __syncthreads();
      double *W = A + (size_t)(k + 1) * n + (k + 1);
      for (int64_t q = threadIdx.x; q < (int64_t)m * m; q += blockDim.x) {
        const int r = (int)(q / m), c = (int)(q % m);
        const double vr = r == 0 ? 1.0 : col[(size_t)r * n];
        const double vc = c == 0 ? 1.0 : col[(size_t)c * n];
        W[(size_t)r * n + c] -= vr * p[c] + p[r] * vc;
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

// Q = H_0 H_1 ... H_{n-3} from the reflectors of cta_tridiag, written
// transposed: Zt[j][r] = Q[r][j] (column j of Q is row j of Zt).
// Backward accumulation on row-major scratch Qs, then transpose.
__device__ void cta_form_q(int n, const double *A, const double *tau, double *Qs, double *Zt,
                           double *w) {
  for (int64_t q = threadIdx.x; q < (int64_t)n * n; q += blockDim.x)
    Qs[q] = (q / n == q % n) ? 1.0 : 0.0;
  __syncthreads();
  for (int k = n - 3; k >= 0; --k) {
    const double t = tau[k];
    if (t == 0.0) continue;
    const int m = n - k - 1;
    const double *col = A + (size_t)(k + 1) * n + k;
    double *Qb = Qs + (size_t)(k + 1) * n + (k + 1);
    for (int c = threadIdx.x; c < m; c += blockDim.x) {
      double s = Qb[c];
      for (int r = 1; r < m; ++r) s = fma(col[(size_t)r * n], Qb[(size_t)r * n + c], s);
      w[c] = t * s;
    }
    __syncthreads();
    for (int64_t q = threadIdx.x; q < (int64_t)m * m; q += blockDim.x) {
      const int r = (int)(q / m), c = (int)(q % m);
      const double vr = r == 0 ? 1.0 : col[(size_t)r * n];
      Qb[(size_t)r * n + c] -= vr * w[c];
    }
    __syncthreads();
  }
  for (int64_t q = threadIdx.x; q < (int64_t)n * n; q += blockDim.x) {
    const int r = (int)(q / n), c = (int)(q % n);
    Zt[(size_t)c * n + r] = Qs[q];
  }
  __syncthreads();
}

// Implicit QL with Wilkinson-type shifts on the tridiagonal (d, e) of order
// n (Bowdler, Martin, Reinsch, Wilkinson, Numer. Math. 11, 293 (1968)),
// applying the plane rotations to the eigenvector rows Zt (Zt[j][:] is
// vector j). Thread 0 runs the scalar recurrence of one sweep and records
// the rotations; then all threads apply them, each to its own components.
// Returns false if an eigenvalue needs more than 60 sweeps.
__device__ bool cta_tql(int n, double *d, double *e, double *Zt, double *rc, double *rs) {
  __shared__ int s_m, s_lo, s_state;  // state: 0 converged l, 1 rotate, 2 fail
  for (int l = 0; l < n; ++l) {
    int iter = 0;
    while (true) {
      if (threadIdx.x == 0) {
        int m = l;
        for (; m < n - 1; ++m) {
          const double dd = fabs(d[m]) + fabs(d[m + 1]);
          if (fabs(e[m]) <= kEps * dd) break;
        }
        if (m == l) {
          s_state = 0;
        } else if (++iter > 60) {
          s_state = 2;
        } else {
          double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
          double r = hypot(g, 1.0);
          g = d[m] - d[l] + e[l] / (g + copysign(r, g));
          double s = 1.0, c = 1.0, p = 0.0;
          int i = m - 1;
          bool early = false;
          for (; i >= l; --i) {
            const double f = s * e[i], bb = c * e[i];
            r = hypot(f, g);
            e[i + 1] = r;
            if (r == 0.0) {
              d[i + 1] -= p;
              e[m] = 0.0;
              early = true;
              break;
            }
            s = f / r;
            c = g / r;
            g = d[i + 1] - p;
            r = (d[i] - g) * s + 2.0 * c * bb;
            p = s * r;
            d[i + 1] = g + p;
            g = c * r - bb;
            rc[i] = c;
            rs[i] = s;
          }
          if (!early) {
            d[l] -= p;
            e[l] = g;
            e[m] = 0.0;
          }
          s_m = m;
          s_lo = early ? i + 1 : l;  // rotations recorded for [s_lo, m-1]
          s_state = 1;
        }
      }
      __syncthreads();
      const int state = s_state;
      if (state == 2) return false;
      if (state == 0) break;
      const int m = s_m, lo = s_lo;
      if (lo <= m - 1) {
        for (int k = threadIdx.x; k < n; k += blockDim.x) {
          double cur = Zt[(size_t)m * n + k];
          for (int i = m - 1; i >= lo; --i) {
            const double zi = Zt[(size_t)i * n + k];
            const double c = rc[i], s = rs[i];
            Zt[(size_t)(i + 1) * n + k] = s * zi + c * cur;
            cur = c * zi - s * cur;
          }
          Zt[(size_t)lo * n + k] = cur;
        }
      }
      __syncthreads();
    }
  }
  return true;
}

}  // namespace dxtb
