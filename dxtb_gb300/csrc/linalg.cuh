// Dense float64 linear algebra for one molecule's AO matrices (row-major,
// leading dimension n, resident in global memory / L2), executed by a TEAM:
// the CTAs of one thread-block cluster (or a single CTA). Every routine must
// be called by all threads of all CTAs of the team, the same number of
// times; each ends with a team barrier unless stated otherwise.
//
// The symmetric eigenproblem of the SCF is solved as
//   Householder tridiagonalisation  (team_tridiag: row i belongs to CTA
//     i mod size and stays in its shared memory where it fits; only vectors
//     move between the CTAs, through distributed shared memory; two team
//     barriers per reflector)
//   -> eigenvalues: float32 bisection + float64 Newton, one thread each
//      (team_tri_eigenvalues)
//   -> eigenvectors of the lowest m eigenvalues only, one thread per
//      eigenvalue cluster: the twisted factorisation for an isolated
//      eigenvalue, inverse iteration with a pivoted tridiagonal LU and
//      Gram-Schmidt inside clusters (team_tri_vectors)
//   -> back-transformation of those m vectors, each CTA a block of
//      vectors (team_back_transform: no team barrier per reflector).
// The SCF needs only the orbitals with non-vanishing occupation, so the
// O(n^3) accumulation of QL rotations is never done.
//
// In a cluster team, data written by another CTA is read with ld.global.cg
// (L2, never a stale L1 line) after a barrier.cluster arrive.release /
// wait.acquire pair, or from that CTA's shared memory (mapa +
// ld/st.shared::cluster, team_tridiag); a one-CTA team uses plain loads and
// __syncthreads.
//
// A float64 instruction costs a warp ~64 cycles on this part whatever its
// active lanes (the SM issues about one warp-instruction per 19 cycles over
// all warps), so the serial and per-thread parts are written for few
// float64 instructions: float32 seeds refined by one Newton-Raphson step
// instead of divisions and square roots, selects instead of per-row
// branches, integer compares on the bit patterns, float32 wherever a
// float64 step checks or refines the result.
#pragma once
#include "common.cuh"

namespace dxtb {

constexpr int kPart = 512;  // shared partial sums of the split dot products
constexpr int kVerifyN = 384;  // eigenvalues are checked by Sturm counts above this order

__device__ __forceinline__ unsigned cluster_ctarank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}

__device__ __forceinline__ unsigned cluster_nctarank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
  return r;
}

__device__ __forceinline__ void cluster_barrier() {
  asm volatile(
      "barrier.cluster.arrive.release.aligned;\n\t"
      "barrier.cluster.wait.acquire.aligned;\n" ::: "memory");
}

// The CTAs that solve one molecule. CL: a thread-block cluster of `size`
// CTAs; otherwise one CTA (size 1).
template <bool CL>
struct Team {
  int rank, size;   // CTA rank in the team, number of CTAs
  int tid, nthr;    // thread index over the team (rank-major), threads of the team
  int stid;         // thread index with consecutive values on different CTAs
  double *gred;     // global scratch [32]: CTA partial sums, two alternating slots
  int *gctl;        // global scratch [16]: words broadcast by rank 0
  int phase;
  __device__ __forceinline__ void sync() {
    if constexpr (CL) cluster_barrier(); else __syncthreads();
  }
  __device__ __forceinline__ bool lead() const { return rank == 0; }
};

// Load of data that another CTA of the team may have written.
template <bool CL>
__device__ __forceinline__ double ld(const double *p) {
  if constexpr (CL) return __ldcg(p); else return *p;
}
template <bool CL>
__device__ __forceinline__ int ldi(const int *p) {
  if constexpr (CL) return __ldcg(p); else return *p;
}

// Sum over the team (every thread gets it); CTA partials combined in rank order.
template <bool CL>
__device__ double team_sum(Team<CL> &tm, double v, double *red) {
  double s = block_sum(v, red);
  if constexpr (CL) {
    if (tm.size > 1) {
      double *slot = tm.gred + 16 * (tm.phase & 1);
      ++tm.phase;
      if (threadIdx.x == 0) slot[tm.rank] = s;
      tm.sync();
      s = 0.0;
      for (int c = 0; c < tm.size; ++c) s += __ldcg(slot + c);
    }
  }
  return s;
}

// Shapes of the k-loop for triangular operands.
enum KRange : int {
  kFull = 0,     // k in [0, K)
  kALower = 1,   // op(A)(i,k) = 0 for k > i   -> k < i0 + 4
  kBLowerT = 2,  // op(B)(k,j) = 0 for k > j   -> k < j0 + 4
  kBUpper = 3,   // op(B)(k,j) = 0 for k < j   -> k >= j0
};

// C = alpha * op(A) op(B) + beta * C for M x N outputs and inner size K.
// op(A)(i,k) = TA ? A[k*lda+i] : A[i*lda+k]; op(B)(k,j) = TB ? B[j*ldb+k] : B[k*ldb+j].
// Register tile of 4 x 4 outputs per thread, tiles spread over the team.
// With lower_only, tiles strictly above the diagonal are skipped
// (symmetric results). The FP64 pipe, not memory, is the limit.
template <bool TA, bool TB, bool CL>
__device__ void team_gemm(Team<CL> &tm, int M, int N, int K, double alpha, const double *A, int lda,
                          const double *B, int ldb, double beta, double *C, int ldc,
                          int krange = kFull, bool lower_only = false) {
  const int tmm = (M + 3) >> 2, tnn = (N + 3) >> 2;
  // Tiles are enumerated so that one round of the team's threads gets tiles
  // of similar k-length (the k-range follows the tile row for kALower and
  // the tile column otherwise); lower_only enumerates the tiles on and below
  // the diagonal only (M == N).
  const bool col_slow = (krange == kBLowerT || krange == kBUpper);
  const int ntile = lower_only ? tmm * (tmm + 1) / 2 : tmm * tnn;
  // consecutive tiles go to different CTAs (stid), so that a cluster's CTAs
  // share the long and the short k-ranges evenly; the triangle indices come
  // from a float32 square root with integer corrections (a float64 square
  // root costs a warp ~700 cycles on this part)
  for (int t = tm.stid; t < ntile; t += tm.nthr) {
    int ti, tj;
    if (lower_only) {
      if (col_slow) {
        // column-major over the lower triangle: column tj holds tmm - tj tiles
        const int u = ntile - 1 - t;  // reverse: count from the short last columns
        int c = (int)((sqrtf(8.0f * (float)u + 1.0f) - 1.0f) * 0.5f);
        while ((c + 1) * (c + 2) / 2 <= u) ++c;
        while (c * (c + 1) / 2 > u) --c;
        tj = tmm - 1 - c;
        ti = tmm - 1 - (u - c * (c + 1) / 2);
      } else {
        int r = (int)((sqrtf(8.0f * (float)t + 1.0f) - 1.0f) * 0.5f);
        while ((r + 1) * (r + 2) / 2 <= t) ++r;
        while (r * (r + 1) / 2 > t) --r;
        ti = r;
        tj = t - r * (r + 1) / 2;
      }
    } else if (col_slow) {
      tj = t / tmm;
      ti = t % tmm;
    } else {
      ti = t / tnn;
      tj = t % tnn;
    }
    const int i0 = ti * 4, j0 = tj * 4;
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
      for (int a = 0; a < 4; ++a)
        av[a] = ld<CL>(TA ? A + (size_t)k * lda + ia[a] : A + (size_t)ia[a] * lda + k);
#pragma unroll
      for (int c = 0; c < 4; ++c)
        bv[c] = ld<CL>(TB ? B + (size_t)jb[c] * ldb + k : B + (size_t)k * ldb + jb[c]);
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
          *p = alpha * acc[a][c] + (beta == 0.0 ? 0.0 : beta * ld<CL>(p));
        }
      }
  }
  tm.sync();
}

// Copy the lower triangle of a square matrix onto its upper triangle.
template <bool CL>
__device__ void team_mirror_lower(Team<CL> &tm, int n, double *A) {
  for (int64_t t = tm.tid; t < (int64_t)n * n; t += tm.nthr) {
    const int i = (int)(t / n), j = (int)(t % n);
    if (j > i) A[t] = ld<CL>(A + (size_t)j * n + i);
  }
  tm.sync();
}

// In-place lower Cholesky factor of a symmetric positive-definite matrix
// (right-looking, the trailing update spread over the team). Returns false
// (on every thread) if a pivot is not positive.
template <bool CL>
__device__ bool team_cholesky(Team<CL> &tm, int n, double *A) {
  for (int k = 0; k < n; ++k) {
    const double dkk = ld<CL>(A + (size_t)k * n + k);
    if (!(dkk > 0.0)) return false;  // every thread read the same value
    const double lkk = sqrt(dkk);
    for (int i = k + 1 + tm.tid; i < n; i += tm.nthr) A[(size_t)i * n + k] = ld<CL>(A + (size_t)i * n + k) / lkk;
    tm.sync();
    if (tm.lead() && threadIdx.x == 0) A[(size_t)k * n + k] = lkk;
    const int m = n - k - 1;
    for (int64_t t = tm.tid; t < (int64_t)m * m; t += tm.nthr) {
      const int i = k + 1 + (int)(t / m), j = k + 1 + (int)(t % m);
      if (j <= i)
        A[(size_t)i * n + j] = ld<CL>(A + (size_t)i * n + j) -
                               ld<CL>(A + (size_t)i * n + k) * ld<CL>(A + (size_t)j * n + k);
    }
    tm.sync();
  }
  return true;
}

// X = L^-1 for a lower-triangular L (row-major); upper part of X zeroed.
// Thread j of the team solves column j by forward substitution.
template <bool CL>
__device__ void team_trinv(Team<CL> &tm, int n, const double *L, double *X) {
  for (int j = tm.stid; j < n; j += tm.nthr) {
    for (int i = 0; i < j; ++i) X[(size_t)i * n + j] = 0.0;
    X[(size_t)j * n + j] = 1.0 / ld<CL>(L + (size_t)j * n + j);
    for (int i = j + 1; i < n; ++i) {
      double s = 0.0;
      for (int k = j; k < i; ++k) s = fma(ld<CL>(L + (size_t)i * n + k), X[(size_t)k * n + j], s);
      X[(size_t)i * n + j] = -s / ld<CL>(L + (size_t)i * n + i);
    }
  }
  tm.sync();
}

// Distributed shared memory of a cluster: the address of a shared variable
// in the CTA of rank r, and stores / loads through it.
__device__ __forceinline__ uint32_t dsmem_addr(const void *p, int r) {
  const uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
  uint32_t o;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(o) : "r"(a), "r"(r));
  return o;
}
__device__ __forceinline__ void dsmem_st(uint32_t a, double v) {
  asm volatile("st.shared::cluster.f64 [%0], %1;" ::"r"(a), "d"(v) : "memory");
}
__device__ __forceinline__ double dsmem_ld(uint32_t a) {
  double v;
  asm volatile("ld.shared::cluster.f64 %0, [%1];" : "=d"(v) : "r"(a) : "memory");
  return v;
}

// Sum of f(0) .. f(C-1) for C in {1, 2, 4, 8, 16} (the team sizes of the
// SCF launches) as a fixed pairwise tree:
// groups of four ((f0 + f1) + (f2 + f3)), then the group sums pairwise.
template <typename F>
__device__ __forceinline__ double rank_tree_sum(int C, F f) {
  if (C == 1) return f(0);
  if (C == 2) return f(0) + f(1);
  double g[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    if (4 * q < C) {
      const double a = f(4 * q), b = f(4 * q + 1), c = f(4 * q + 2), d = f(4 * q + 3);
      g[q] = (a + b) + (c + d);
    } else {
      g[q] = 0.0;
    }
  }
  if (C == 4) return g[0];
  if (C == 8) return g[0] + g[1];
  return (g[0] + g[1]) + (g[2] + g[3]);
}

// v stored into the shared variable *p of every CTA of the team.
template <bool CL>
__device__ __forceinline__ void team_push(const Team<CL> &tm, double *p, double v) {
  if constexpr (CL) {
    for (int r = 0; r < tm.size; ++r) dsmem_st(dsmem_addr(p, r), v);
  } else {
    *p = v;
  }
}

__device__ __forceinline__ bool is_neg(double v) { return __double_as_longlong(v) < 0; }
__device__ __forceinline__ bool is_zero(double v) { return (__double_as_longlong(v) << 1) == 0; }
__device__ __forceinline__ double flip_sign(double v) {
  return __longlong_as_double(__double_as_longlong(v) ^ (long long)0x8000000000000000ull);
}

// 1/x: a float32 seed y (relative error e0 ~ 2^-22) refined by one
// third-order Newton-Raphson step y <- y + y (g + g^2), g = 1 - x y (error
// e0^3, below float64 rounding): three dependent float64 instructions
// instead of a float64 division (about ten); |x| outside [2^-120, 2^120]
// takes the division.
__device__ __forceinline__ double rcp_nr(double x) {
  const int ex = (int)((__double_as_longlong(x) >> 52) & 0x7ff);
  if (ex <= 1023 - 120 || ex >= 1023 + 120) return 1.0 / x;
  const double r = (double)__fdividef(1.0f, (float)x);
  const double g = fma(-x, r, 1.0);
  return fma(r, fma(g, g, g), r);
}

// Scalars of the Householder reflector of a column (alpha, x) with
// sg = |x|^2: beta = -sign(alpha) sqrt(alpha^2 + sg), t = (beta - alpha) / beta
// = 1 + |alpha| / |beta| and scale = 1 / (alpha - beta); sg = 0 gives the
// identity (t = 0, beta = alpha). A float64 instruction costs a warp ~65
// cycles on this part and this chain is serial, so 1/sqrt and the reciprocal
// start from float32 seeds (~2^-23) refined by one third-order
// Newton-Raphson step each in float64 (x^-1/2: y <- y + y (h/2 + 3 h^2/8),
// h = 1 - x y^2; s^-1: rcp_nr), whose error (~2^-69) is below float64
// rounding, instead of the float64 square root and two divisions; squares
// outside [2^-120, 2^120] take the float64 sqrt and division.
__device__ __forceinline__ void householder_scalars(double alpha, double sg, double &t, double &beta,
                                                    double &scale) {
  if (is_zero(sg)) {
    t = 0.0;
    beta = alpha;
    scale = 0.0;
    return;
  }
  const double x = fma(alpha, alpha, sg);
  const double aa = fabs(alpha);
  const int ex = (int)((__double_as_longlong(x) >> 52) & 0x7ff);
  double nrm, rs;
  if (ex > 1023 - 120 && ex < 1023 + 120) {
    const double y0 = (double)rsqrtf((float)x);
    const double h = fma(-x * y0, y0, 1.0);
    const double y = fma(y0 * h, fma(h, 0.375, 0.5), y0);
    nrm = x * y;
    t = fma(aa, y, 1.0);
    rs = rcp_nr(aa + nrm);
  } else {
    nrm = sqrt(x);
    t = (aa + nrm) / nrm;
    rs = 1.0 / (aa + nrm);
  }
  // alpha >= 0: beta = -nrm, alpha - beta = |alpha| + nrm; else the opposite signs
  beta = is_neg(alpha) ? nrm : flip_sign(nrm);
  scale = is_neg(alpha) ? flip_sign(rs) : rs;
}

// Householder reduction of a full symmetric matrix to tridiagonal form
// (lower variant): A = Q T Q^T. On exit d, e hold the diagonal and
// sub-diagonal (e[i] couples i and i+1), the reflector of step k is stored
// in A[k+2..n-1][k] (its leading 1 implicit) with factor tau[k].
//
// Row i of A belongs to CTA i mod size for the whole reduction: the CTA
// keeps its rows in shared memory when `srows` has room for them (and, in a
// cluster, one more row: (ceil(n / size) + 1) * n doubles, `rows_cap`), else
// in place in A (one CTA: in place, served by the L1). It alone reads and
// updates them.
// Every CTA holds the column u of the step (su) and the reflector scalars
// (t, scale), formed one step ahead. Per step k (trailing order
// m = n - k - 1, A22 the trailing matrix):
//   A. v = scale u (v_0 = 1) into sv; q_c = sum_{own r} A22[r][c] v_r for
//      all c (coalesced over c; by symmetry the own rows' share of A22 v);
//   B. the own share of v^T A22 v is pushed to every CTA; the owner of
//      row 0 of A22 (= column 0, the next column before the update) pushes
//      it to every CTA as well (rows in shared memory);
//   --- team barrier ---
//   C. p = t sum_rank q_rank (read from every CTA's shared memory in rank
//      order: the same bits everywhere), K = t^2/2 sum_rank (v.q)_rank,
//      w = p - K v (sp); the next column u' = (A22 - v w^T - w v^T)[1.., 0]
//      formed by every CTA from row 0, v and w;
//   D. warp 0 forms the scalars of step k + 1 from u' while the other warps
//      update the own rows: A22[r][c] -= v_r w_c + w_r v_c (row 0, which
//      leaves the trailing matrix, only on its diagonal);
//   --- team barrier ---
// so a step moves only vectors between the CTAs (distributed shared memory,
// no global round trip), keeps two team barriers, and the serial float64
// chain of the scalars (a warp issues one float64 instruction per ~64
// cycles) runs beside the update. Quantities formed by every CTA come from
// identical inputs in identical order, so they agree bit for bit.
// su, sv, sp, sq: shared [n]; spart: shared [kPart].
template <bool CL>
__device__ void team_tridiag(Team<CL> &tm, int n, double *A, double *d, double *e, double *tau,
                             double *su, double *sv, double *sp, double *sq, double *spart,
                             double *srows, int64_t rows_cap) {
  __shared__ double swarp[32], sscal[4], skq[16];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5, nty = (int)(blockDim.x >> 5);
  const int C = tm.size, rk = tm.rank;
  const int nown = (n + C - 1) / C;  // the same bound on every CTA
  // Own row i = rk + C j lives in shared memory for j >= jsm (the rows that
  // stay in the trailing matrix longest) and in place in A below that. All
  // of them fit up to n ~ 450 at C = 8; above, as many as the shared memory
  // holds beside the broadcast row (a third of them at n ~ 1000, C = 16).
  // nsm and the layout are the same on every CTA of a cluster.
  // A one-CTA team (n < 136 here) keeps all its rows in shared memory or
  // none of them.
  int jsm = nown;
  double *sc0 = nullptr;
  double *R = A + (size_t)rk * n;
  size_t ldr = (size_t)C * n;
  if (srows != nullptr && rows_cap > 0) {
    if constexpr (CL) {
      const int64_t fit = rows_cap / n - 1;  // whole rows beside the broadcast row
      if (fit >= 1) {
        const int nsm = (int)(fit < (int64_t)nown ? fit : (int64_t)nown);
        jsm = nown - nsm;
        sc0 = srows + (size_t)nsm * n;
        for (int64_t t = threadIdx.x; t < (int64_t)nsm * n; t += blockDim.x) {
          const int j = jsm + (int)(t / n), c = (int)(t % n), i = rk + C * j;
          if (i < n) srows[t] = ld<CL>(A + (size_t)i * n + c);
        }
        __syncthreads();
      }
    } else if ((int64_t)nown * n <= rows_cap) {
      R = srows;
      ldr = (size_t)n;
      for (int64_t t = threadIdx.x; t < (int64_t)nown * n; t += blockDim.x) {
        const int j = (int)(t / n), c = (int)(t % n), i = rk + C * j;
        if (i < n) srows[t] = ld<CL>(A + (size_t)i * n + c);
      }
      __syncthreads();
    }
  }
  auto rowp = [&](int i) -> double * {  // own global row i
    if constexpr (CL) {
      const int j = (i - rk) / C;
      return j >= jsm ? srows + (size_t)(j - jsm) * n : A + (size_t)i * n;
    } else {
      return R + (size_t)((i - rk) / C) * ldr;
    }
  };
  // scalars of step k from su[0..m): warp 0 (the lead's lane 0 stores tau, e)
  auto scalars = [&](int k, int m) {
    double p0 = 0.0, p1 = 0.0;
    int r = 1 + tx;
    for (; r + 32 < m; r += 64) {
      p0 = fma(su[r], su[r], p0);
      p1 = fma(su[r + 32], su[r + 32], p1);
    }
    if (r < m) p0 = fma(su[r], su[r], p0);
    const double sg = warp_sum(p0 + p1);
    if (tx == 0) {
      double t, beta, scale;
      householder_scalars(su[0], sg, t, beta, scale);
      sscal[0] = t;
      sscal[1] = scale;
      if (tm.lead()) {
        tau[k] = t;
        e[k] = beta;
      }
    }
  };
  // column 0 below the diagonal
  for (int i = rk + C * threadIdx.x; i < n; i += C * blockDim.x)
    if (i >= 1) team_push(tm, su + (i - 1), rowp(i)[0]);
  tm.sync();
  if (n > 2 && ty == 0) scalars(0, n - 1);
  __syncthreads();
  for (int k = 0; k < n - 2; ++k) {
    const int m = n - k - 1;
    const int rb = ((rk - (k + 1)) % C + C) % C;          // first own local row
    const int mc = rb < m ? (m - rb + C - 1) / C : 0;      // own local rows rb + C jj
    // own row k + 1 + rb + C jj is local row j0 + jj (k + 1 + rb - rk is a multiple of C)
    const int j0 = (k + 1 + rb - rk) / C;
    auto lrow = [&](int jj) -> double * {
      if constexpr (CL) {
        const int j = j0 + jj;
        return (j >= jsm ? srows + (size_t)(j - jsm) * n : A + (size_t)(rk + C * j) * n) + (k + 1);
      } else {
        return rowp(k + 1 + rb + C * jj) + (k + 1);
      }
    };
    if (threadIdx.x == 0 && k % C == rk) d[k] = rowp(k)[k];
    const double t = sscal[0], scale = sscal[1];
    // ---- A ----
    for (int c = threadIdx.x; c < m; c += blockDim.x) {
      const double vc = c == 0 ? 1.0 : scale * su[c];
      sv[c] = vc;
      if (c >= 1 && c >= rb && (c - rb) % C == 0) A[(size_t)(k + 1 + c) * n + k] = vc;
    }
    __syncthreads();
    const int ncg = (m + 31) >> 5;
    const int nrg = max(1, nty / ncg);
    for (int it = ty; it < ncg * nrg; it += nty) {
      const int cg = it % ncg, rg = it / ncg, c = cg * 32 + tx;
      if (c < m) {
        double a0 = 0.0, a1 = 0.0;
        int jj = rg;
        for (; jj + nrg < mc; jj += 2 * nrg) {
          a0 = fma(lrow(jj)[c], sv[rb + C * jj], a0);
          a1 = fma(lrow(jj + nrg)[c], sv[rb + C * (jj + nrg)], a1);
        }
        if (jj < mc) a0 = fma(lrow(jj)[c], sv[rb + C * jj], a0);
        if (nrg > 1) spart[rg * m + c] = a0 + a1;
        else sq[c] = a0 + a1;
      }
    }
    __syncthreads();
    // ---- B ---- (float64 instructions cost pipe time on every warp that
    // issues them, active lanes or not: only the warps that hold entries of
    // q take part in the reduction)
    const int nwq = min(nty, (m + 31) >> 5);
    double kq = 0.0;
    for (int c = threadIdx.x; c < m; c += blockDim.x) {
      double q;
      if (nrg > 1) {
        q = spart[c];
        for (int g = 1; g < nrg; ++g) q += spart[g * m + c];
        sq[c] = q;
      } else {
        q = sq[c];
      }
      kq = fma(q, sv[c], kq);
    }
    if (CL && sc0 != nullptr && rb == 0 && mc > 0) {
      const double *row0 = lrow(0);
      for (int c = 1 + threadIdx.x; c < m; c += blockDim.x) team_push(tm, sc0 + c, row0[c]);
    }
    if (ty < nwq) {
      kq = warp_sum(kq);
      if (tx == 0) swarp[ty] = kq;
    }
    __syncthreads();
    if (ty == 0) {
      // butterfly over the smallest power of two >= nwq lanes only
      double kk = tx < nwq ? swarp[tx] : 0.0;
      for (int o = nwq > 1 ? 1 << (31 - __clz(nwq - 1)) : 0; o > 0; o >>= 1)
        kk += __shfl_xor_sync(0xffffffffu, kk, o);
      kk = __shfl_sync(0xffffffffu, kk, 0);  // lanes past the group hold partial sums
      if constexpr (CL) {
        if (tx < C) dsmem_st(dsmem_addr(skq + rk, tx), kk);
      } else {
        if (tx == 0) sscal[3] = 0.5 * t * t * kk;
      }
    }
    tm.sync();
    // ---- C ----
    if constexpr (CL) {
      // sums over the ranks as fixed pairwise trees (depth log2 size)
      if (threadIdx.x == 0) sscal[3] = 0.5 * t * t * rank_tree_sum(C, [&](int r) { return skq[r]; });
      for (int c = threadIdx.x; c < m; c += blockDim.x)
        sp[c] = t * rank_tree_sum(C, [&](int r) { return dsmem_ld(dsmem_addr(sq + c, r)); });
      __syncthreads();
      const double K = sscal[3];
      for (int c = threadIdx.x; c < m; c += blockDim.x) sp[c] = fma(-K, sv[c], sp[c]);
    } else {
      const double K = sscal[3];
      for (int c = threadIdx.x; c < m; c += blockDim.x) sp[c] = fma(-K, sv[c], t * sq[c]);
    }
    __syncthreads();
    // the next column: u'[r - 1] = A22[0][r] - v_r w_0 - w_r v_0, r >= 1
    {
      const double w0 = sp[0], v0 = sv[0];
      const double *g0 = A + (size_t)(k + 1) * n + (k + 1);  // row 0 of A22 in place
      const double *l0 = (!CL && mc > 0) ? lrow(0) : nullptr;
      for (int r = 1 + threadIdx.x; r < m; r += blockDim.x) {
        const double a0 = CL ? (sc0 != nullptr ? sc0[r] : ld<CL>(g0 + r)) : l0[r];
        su[r - 1] = fma(-sv[r], w0, fma(-sp[r], v0, a0));
      }
    }
    __syncthreads();
    // ---- D ----
    // warp 0 runs the serial chain of the next scalars, the other warps the
    // update (keeping the warps of warp 0's sub-partition idle shortened the
    // chain but cost more update throughput than it saved: measured)
    if (ty == 0) {
      if (k + 1 < n - 2) scalars(k + 1, m - 1);
    } else {
      const int nu = nty - 1, uw = ty - 1;
      for (int it = uw; it < mc * ncg; it += nu) {
        const int jj = it / ncg, c = (it % ncg) * 32 + tx, r = rb + C * jj;
        // row 0 of A22 leaves the trailing matrix: only its diagonal (d of
        // the next step) is kept; the rest is still being read as the next
        // column by the other CTAs
        if (c < m && (r > 0 || c == 0)) {
          double *row = lrow(jj);
          row[c] = fma(-sv[r], sp[c], fma(-sp[r], sv[c], row[c]));
        }
      }
    }
    tm.sync();  // the rows, the next column and its scalars are complete
  }
  if (threadIdx.x == 0) {
    if (n >= 2) {
      if ((n - 2) % C == rk) d[n - 2] = rowp(n - 2)[n - 2];
      if ((n - 1) % C == rk) {
        e[n - 2] = rowp(n - 1)[n - 2];
        d[n - 1] = rowp(n - 1)[n - 1];
      }
    } else if (rk == 0) {
      d[0] = rowp(0)[0];
    }
    if (tm.lead()) {
      if (n >= 2) tau[n - 2] = 0.0;
      tau[n - 1] = 0.0;
      e[n - 1] = 0.0;
    }
  }
  tm.sync();
}

// Number of eigenvalues of the tridiagonal below x, in float32 and without
// divisions: sign changes of the leading principal minors p_k of T - x I
// (three-term recurrence p_{k+1} = (d_k - x) p_k - e2_{k-1} p_{k-1}, e2 = e^2),
// read from the sign bits. An exact zero minor needs no fix-up: the next
// minor is -e2 p_{k-1}, of the sign opposite to p_{k-1}, so a zero of
// either sign adds exactly one change (a zero pivot counted as negative).
// Every fourth row the pair is rescaled by 2^-+64 when the larger magnitude
// leaves [2^-40, 2^40]. No data-dependent branch: the serial chain is one
// float32 FMA per row (a branch per row made the count seven times slower).
__device__ __forceinline__ int sturm_count_f32(int n, const float *d, const float *e2, float x) {
  float p0 = 1.0f, p1 = d[0] - x;
  int cnt = __float_as_int(p1) < 0 ? 1 : 0;
  auto step = [&](float dx, float ee) {
    const float p2 = fmaf(dx, p1, -ee * p0);
    cnt += (__float_as_int(p2) ^ __float_as_int(p1)) < 0 ? 1 : 0;
    p0 = p1;
    p1 = p2;
  };
  int i = 1;
  for (; i + 3 < n; i += 4) {
    const float d0 = d[i] - x, d1 = d[i + 1] - x, d2 = d[i + 2] - x, d3 = d[i + 3] - x;
    const float f0 = e2[i - 1], f1 = e2[i], f2 = e2[i + 1], f3 = e2[i + 2];
    step(d0, f0);
    step(d1, f1);
    step(d2, f2);
    step(d3, f3);
    const int em = max((__float_as_int(p1) >> 23) & 0xff, (__float_as_int(p0) >> 23) & 0xff);
    const float sc = em > 127 + 40 ? 0x1p-64f : (em < 127 - 40 ? 0x1p64f : 1.0f);
    p0 *= sc;
    p1 *= sc;
  }
  for (; i < n; ++i) step(d[i] - x, e2[i - 1]);
  return cnt;
}

// |v| outside [2^-500, 2^500] (biased exponent test, no FP64 instruction)
__device__ __forceinline__ bool out_of_range(double v) {
  const int ex = (int)((__double_as_longlong(v) >> 52) & 0x7ff);
  return ex > 1023 + 500 || (ex < 1023 - 500 && ex != 0);
}

// The same count in float64 without divisions: the pivots of T - x I are
// q_k = p_k / p_{k-1} for the leading principal minors p_k = det(T_k - x I)
// (three-term recurrence, e2 = e^2), so a negative pivot is a sign change
// between p_{k-1} and p_k. A zero minor counts as a change and continues as a
// tiny value of the opposite sign of its predecessor; every eighth row the
// pair is rescaled (by 2^-+500) to stay in range. Selects and sign bits
// only, no data-dependent branch.
__device__ __forceinline__ int sturm_count_f64(int n, const double *d, const double *e2, double x) {
  double p0 = 1.0, p1 = d[0] - x;
  p1 = is_zero(p1) ? -1e-300 : p1;
  int cnt = is_neg(p1) ? 1 : 0;
  for (int i = 1; i < n; ++i) {
    double p2 = fma(d[i] - x, p1, -e2[i - 1] * p0);
    p2 = is_zero(p2) ? (is_neg(p1) ? 1e-300 : -1e-300) : p2;
    cnt += (__double_as_longlong(p2) ^ __double_as_longlong(p1)) < 0 ? 1 : 0;
    p0 = p1;
    p1 = p2;
    if ((i & 7) == 0) {
      const int em = max((int)((__double_as_longlong(p1) >> 52) & 0x7ff), (int)((__double_as_longlong(p0) >> 52) & 0x7ff));
      if (em > 1023 + 500 || em < 1023 - 500) {
        const double sc = em > 1023 ? 0x1p-500 : 0x1p500;
        p0 *= sc;
        p1 *= sc;
      }
    }
  }
  return cnt;
}

// Characteristic polynomial p(x) = det(T - x I) and its derivative by the
// three-term recurrence (e2 = e^2), rescaled every 8 steps; returns p / p'.
__device__ __forceinline__ double charpoly_ratio(int n, const double *d, const double *e2, double x) {
  double p0 = 1.0, p1 = d[0] - x;   // p_{k-1}, p_k
  double q0 = 0.0, q1 = -1.0;       // p'_{k-1}, p'_k
  for (int i = 1; i < n; ++i) {
    const double di = d[i] - x, ee = e2[i - 1];
    const double p2 = fma(di, p1, -ee * p0);
    const double q2 = fma(di, q1, -fma(ee, q0, p1));
    p0 = p1;
    p1 = p2;
    q0 = q1;
    q1 = q2;
    if ((i & 7) == 0 && (out_of_range(p1) || out_of_range(q1) || out_of_range(p0) || out_of_range(q0))) {
      const double big = fmax(fmax(fabs(p1), fabs(q1)), fmax(fabs(p0), fabs(q0)));
      const double sc = big > 1.0 ? 0x1p-500 : 0x1p500;
      p0 *= sc; p1 *= sc; q0 *= sc; q1 *= sc;
    }
  }
  return q1 != 0.0 ? p1 * rcp_nr(q1) : 0.0;
}

// All eigenvalues of the symmetric tridiagonal (d, e) (shared-memory copies
// held by every CTA), one per thread of the team. Float32 bisection on Sturm
// counts isolates eigenvalue k to ~1e-7 relative. Float64 Sturm counts then
// confirm that the bracket holds only the k-th eigenvalue, bisecting a few
// more times where a near-degenerate neighbour shares it. Safeguarded
// float64 Newton steps on the characteristic polynomial refine the isolated
// root. Eigenvalues closer than the float64 resolution of the counts keep
// the bracket midpoint (their vectors come from one cluster). df/e2f: shared
// float scratch of n each, e2: shared double scratch of n. lam: global,
// ascending index k.
template <bool CL>
__device__ void team_tri_eigenvalues(Team<CL> &tm, int n, const double *d, const double *e,
                                     double *e2, double *lam, float *df, float *e2f) {
  __shared__ double s_gl, s_gu;
  double gl = 1e308, gu = -1e308;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double r = (i > 0 ? fabs(e[i - 1]) : 0.0) + (i < n - 1 ? fabs(e[i]) : 0.0);
    gl = fmin(gl, d[i] - r);
    gu = fmax(gu, d[i] + r);
    const double ee = i < n - 1 ? e[i] * e[i] : 0.0;
    e2[i] = ee;
    df[i] = (float)d[i];
    e2f[i] = (float)ee;
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
  // bound on the change of the eigenvalues by the float32 rounding of T
  // (|d|, |e| <= tnorm: 3 2^-24 tnorm) and the backward error of the float32
  // counts (a few 2^-24 (|d| + |x|)); 2^-20 (tnorm + span) covers both
  const double dp = 0x1p-20 * (tnorm + span);
  for (int k = tm.stid; k < n; k += tm.nthr) {
    // --- float32 bisection: count(lo) <= k < count(hi) ---
    float lo = (float)glo, hi = (float)ghi;
    for (int it = 0; it < 60; ++it) {
      const float mid = 0.5f * (lo + hi);
      if (mid <= lo || mid >= hi) break;
      if (sturm_count_f32(n, df, e2f, mid) <= k) lo = mid; else hi = mid;
    }
    const double w32 = fmax((double)hi - (double)lo, 4e-7 * tnorm + 1e-12);
    const double x0 = 0.5 * ((double)lo + (double)hi);
    double l, h;
    int cl, ch;
    // --- isolation by float32 counts: the k-th eigenvalue of T lies within
    // R = w32 + dp of x0, and if the float32 counts at x0 -+ 2R are k and
    // k + 1 no other eigenvalue of T comes closer than R (Weyl), so
    // [x0 - R, x0 + R] brackets it alone without float64 counts ---
    const double R = w32 + dp;
    if (sturm_count_f32(n, df, e2f, (float)(x0 - 2.0 * R)) == k &&
        sturm_count_f32(n, df, e2f, (float)(x0 + 2.0 * R)) == k + 1) {
      l = x0 - R;
      h = x0 + R;
      cl = k;
      ch = k + 1;
    } else {
      // --- float64 bracket [l, h) with count(l) <= k < count(h) ---
      l = x0 - 4.0 * w32;
      h = x0 + 4.0 * w32;
      cl = sturm_count_f64(n, d, e2, l);
      ch = sturm_count_f64(n, d, e2, h);
      if (!(cl <= k && k < ch)) {
        l = glo;
        h = ghi;
        cl = 0;
        ch = n;
      }
    }
    // --- bisect until the bracket holds the k-th eigenvalue alone ---
    for (int it = 0; it < 200 && !(cl == k && ch == k + 1); ++it) {
      const double mid = 0.5 * (l + h);
      if (mid <= l || mid >= h) break;
      const int c = sturm_count_f64(n, d, e2, mid);
      if (c <= k) {
        l = mid;
        cl = c;
      } else {
        h = mid;
        ch = c;
      }
    }
    double x = 0.5 * (l + h);
    const double del = 8.0 * kEps * fmax(tnorm, 1.0);  // resolution of the counts
    if (cl == k && ch == k + 1) {
      // --- safeguarded Newton on p(x): one root in (l, h) ---
      x = fmin(fmax(x0, l), h);
      if (!(x > l && x < h)) x = 0.5 * (l + h);
      // converged when the Newton step is at the rounding level of the
      // recurrence (eps |T|); a step that would leave the bracket becomes a
      // bisection step, and then (or after slow steps) the count at the new
      // point shrinks the bracket
      // a Newton step of size s after one of size s0 (quadratic convergence,
      // error ~ K s^2 with K ~ s / s0^2) leaves an error of about s^3 / s0^2:
      // below tol the next evaluation (~5 n float64 instructions) is skipped
      const double tol = 4.0 * kEps * fmax(tnorm, fabs(x));
      double sprev = 0.0;
      for (int it = 0; it < 16; ++it) {
        double xn = x - charpoly_ratio(n, d, e2, x);
        const bool bis = !(xn > l && xn < h);
        if (bis) xn = 0.5 * (l + h);
        const double step = fabs(xn - x);
        x = xn;
        if (!bis && step <= tol) break;
        if (!bis && sprev > 0.0 && step <= 0.01 * sprev && step * step * step <= tol * sprev * sprev) break;
        sprev = bis ? 0.0 : step;
        if (bis || it >= 3) {
          if (sturm_count_f64(n, d, e2, x) <= k) l = x; else h = x;
          if (h - l <= tol) break;
        }
      }
      // the characteristic-polynomial recurrence loses accuracy for large n
      // (1e-10 |T| at n = 4748): there, accept x only if the
      // (backward-stable) counts put the k-th eigenvalue within del of it,
      // else bisect to that resolution
      const int cxl = n > kVerifyN ? sturm_count_f64(n, d, e2, x - del) : k;
      const int cxh = n > kVerifyN ? sturm_count_f64(n, d, e2, x + del) : k + 1;
      if (!(cxl <= k && k < cxh)) {
        if (cxl > k) h = fmin(h, x - del); else l = fmax(l, x + del);
        for (int it = 0; it < 200 && h - l > 2.0 * del; ++it) {
          const double mid = 0.5 * (l + h);
          if (mid <= l || mid >= h) break;
          if (sturm_count_f64(n, d, e2, mid) <= k) l = mid; else h = mid;
        }
        x = 0.5 * (l + h);
      }
    }
    lam[k] = x;
  }
  tm.sync();
}

// Ascending sort by rank (ties broken by index): out[rank(i)] = in[i]. The
// values go to the shared scratch s (n doubles) as order-preserving int64
// keys (negative numbers with the magnitude bits flipped, -0 as +0), so the
// n^2 comparisons are integer ones instead of float64 (finite inputs).
// out: global.
template <bool CL>
__device__ void team_rank_sort(Team<CL> &tm, int n, const double *in, double *out, double *s) {
  auto key = [](double x) {
    long long b = __double_as_longlong(x);
    if (b == (long long)0x8000000000000000ull) b = 0;
    return b < 0 ? (b ^ 0x7fffffffffffffffll) : b;
  };
  long long *sk = reinterpret_cast<long long *>(s);
  for (int i = threadIdx.x; i < n; i += blockDim.x) sk[i] = key(ld<CL>(in + i));
  __syncthreads();
  for (int i = tm.stid; i < n; i += tm.nthr) {
    const long long v = sk[i];
    int r = 0;
    for (int j = 0; j < n; ++j) {
      const long long u = sk[j];
      r += (u < v) || (u == v && j < i);
    }
    out[r] = __longlong_as_double(v < 0 ? (v ^ 0x7fffffffffffffffll) : v);
  }
  tm.sync();
}

// Deterministic pseudo-random start in [1, 2) (any vector with a component
// along the eigenvector works), assembled from the bits of a hash: no
// float64 instruction.
__device__ __forceinline__ double start_vector(int i, int j) {
  uint32_t h = 2654435761u * (uint32_t)(i + 1) ^ 40503u * (uint32_t)(j + 7);
  h ^= h >> 13;
  h *= 0x5bd1e995u;
  h ^= h >> 15;
  return __longlong_as_double((long long)(0x3ff0000000000000ull | ((uint64_t)h << 20)));
}

// |a| >= |b| for finite doubles, on the bit patterns (integer compare).
__device__ __forceinline__ bool abs_ge(double a, double b) {
  return (__double_as_longlong(a) & 0x7fffffffffffffffll) >= (__double_as_longlong(b) & 0x7fffffffffffffffll);
}

// Eigenvector of an isolated eigenvalue lmb of the tridiagonal (d, e;
// e2 = e^2) by the twisted factorisation of T - lmb I (the vector of one
// optimal inverse-iteration step, as in the MRRR "getvec" step), written
// through the leading minors P[k] = det(T - lmb I)[0:k, 0:k] and trailing
// minors Q[k] = det(T - lmb I)[k:n, k:n] so that no row needs a division:
// the twist index r maximises |P[r] Q[r+1]| (the diagonal of the adjugate,
// proportional to z_r^2), and with z_r = 1
//   z_i = P[i] / P[r] prod_{t=i}^{r-1} (-e_t)          (i < r)
//   z_i = Q[i+1] / Q[r+1] prod_{t=r}^{i-1} (-e_t)      (i > r).
// Both minor sequences are three-term FMA recurrences; they and the running
// products are rescaled by 2^-+400 when they leave [2^-400, 2^400]
// (exponent test on the bits, every fourth row), with the scale counts kept per row
// (as bit patterns in the scratch columns SP, SQ), so no product of two kept
// values overflows; components below 2^-800 of z_r are set to zero. About
// eleven float64 instructions per row in all, against ~20 and four
// memory-bound sweeps of the pivoted LU with two solves. P, Q, SP, SQ: per-thread scratch columns of n doubles (stride
// nslot, column tid). Writes the normalised vector to column j of Y (n x m).
// Returns the Rayleigh-quotient correction gamma_r / |z|^2 of lmb: with
// z_r = 1 the twisted vector satisfies (T - lmb I) z = gamma_r e_r, so a
// correction above the rounding level means lmb was not accurate enough for
// this vector (its error is about |correction| / gap).
__device__ __forceinline__ double tri_vector_twisted(int n, const double *d, const double *e,
                                                     const double *e2, double lmb, double *__restrict__ Y,
                                                     int m, int j, double *__restrict__ P,
                                                     double *__restrict__ Q, double *__restrict__ SP,
                                                     double *__restrict__ SQ, int nslot, int tid) {
#define AT(arr, i) arr[(size_t)(i) * nslot + tid]
  auto expo = [](double v) { return (int)((__double_as_longlong(v) >> 52) & 0x7ff); };
  auto keep = [&](double &a, double &b, int &cnt) {
    const int em = max(expo(a), expo(b));
    if (em > 1023 + 400 || em < 1023 - 400) {
      const bool big = em > 1023;
      const double sc = big ? 0x1p-400 : 0x1p400;
      a *= sc;
      b *= sc;
      cnt += big ? 1 : -1;
    }
  };
  auto cbits = [](int c) { return __longlong_as_double((long long)c); };
  auto cint = [](double v) { return (int)__double_as_longlong(v); };
  // Rows go in blocks of four: the block's loads are issued first and the
  // range test (a branch) runs once per block. Four rows of growth
  // (|minor ratio| <= 2 |T| + |T|^2, |e| <= |T|) stay inside the float64 range
  // for |T| < 2^16, which the caller checks
  // forward: P[k] (k = 0 .. n-1) at slot k
  {
    double pk = 1.0, pkm = 0.0;
    int cnt = 0;
    for (int k0 = 0; k0 < n; k0 += 4) {
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int k = k0 + u;
        if (k < n) {
          AT(P, k) = pk;
          AT(SP, k) = cbits(cnt);
          const double ee = k > 0 ? e2[k - 1] : 0.0;
          const double pn = fma(d[k] - lmb, pk, -ee * pkm);
          pkm = pk;
          pk = pn;
        }
      }
      keep(pk, pkm, cnt);
    }
  }
  // backward: Q[k + 1] at slot k (k = n-1 .. 0); the twist index on the way
  int r = n - 1;
  {
    double q1 = 1.0, q2 = 0.0;  // Q[k+1], Q[k+2]
    int cnt = 0, best = INT_MIN;
    for (int k0 = n - 1; k0 >= 0; k0 -= 4) {
      double pv[4], sv[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int k = k0 - u;
        pv[u] = k >= 0 ? AT(P, k) : 0.0;
        sv[u] = k >= 0 ? AT(SP, k) : 0.0;
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int k = k0 - u;
        if (k >= 0) {
          AT(Q, k) = q1;
          AT(SQ, k) = cbits(cnt);
          // log2 |P[k] Q[k+1]| up to the mantissas (a zero minor counts as tiny)
          const int mag = expo(pv[u]) + expo(q1) + 400 * (cint(sv[u]) + cnt);
          if (mag > best) {
            best = mag;
            r = k;
          }
          const double ee = k < n - 1 ? e2[k] : 0.0;
          const double qn = fma(d[k] - lmb, q1, -ee * q2);
          q2 = q1;
          q1 = qn;
        }
      }
      keep(q1, q2, cnt);
    }
  }
  // the vector from the twist outwards
  auto factor = [](int c) {
    return c < -2 ? 0.0 : (c == -2 ? 0x1p-800 : (c == -1 ? 0x1p-400 : (c == 0 ? 1.0 : (c == 1 ? 0x1p400 : 0x1p800))));
  };
  double nrm = 1.0;
  Y[(size_t)r * m + j] = 1.0;
  {
    double E = rcp_nr(AT(P, r)), one = 1.0;
    int cnt = -cint(AT(SP, r));
    for (int i0 = r - 1; i0 >= 0; i0 -= 4) {
      double pv[4], sv[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        pv[u] = i0 - u >= 0 ? AT(P, i0 - u) : 0.0;
        sv[u] = i0 - u >= 0 ? AT(SP, i0 - u) : 0.0;
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int i = i0 - u;
        if (i >= 0) {
          E *= -e[i];
          const double z = (E * pv[u]) * factor(cnt + cint(sv[u]));
          Y[(size_t)i * m + j] = z;
          nrm = fma(z, z, nrm);
        }
      }
      keep(E, one, cnt);
    }
  }
  {
    double E = rcp_nr(AT(Q, r)), one = 1.0;
    int cnt = -cint(AT(SQ, r));
    for (int i0 = r + 1; i0 < n; i0 += 4) {
      double qv[4], sv[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        qv[u] = i0 + u < n ? AT(Q, i0 + u) : 0.0;
        sv[u] = i0 + u < n ? AT(SQ, i0 + u) : 0.0;
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int i = i0 + u;
        if (i < n) {
          E *= -e[i - 1];
          const double z = (E * qv[u]) * factor(cnt + cint(sv[u]));
          Y[(size_t)i * m + j] = z;
          nrm = fma(z, z, nrm);
        }
      }
      keep(E, one, cnt);
    }
  }
  // residual of the twist row: gamma_r = e_{r-1} z_{r-1} + (d_r - lmb) + e_r z_{r+1}
  double gam = d[r] - lmb;
  if (r > 0) gam = fma(e[r - 1], Y[(size_t)(r - 1) * m + j], gam);
  if (r + 1 < n) gam = fma(e[r], Y[(size_t)(r + 1) * m + j], gam);
  const double inv = 1.0 / sqrt(nrm);
#pragma unroll 4
  for (int i = 0; i < n; ++i) Y[(size_t)i * m + j] *= inv;
  return gam / nrm;
#undef AT
}

// Eigenvectors of the symmetric tridiagonal (d, e) for the m lowest
// (sorted) eigenvalues lam[0..m). Clusters are runs of eigenvalues closer
// than ctol; each cluster is one thread's work (over the team). An isolated
// eigenvalue takes the twisted factorisation (tri_vector_twisted); the
// members of a cluster take inverse iteration with a partially pivoted LU
// of T - lam I (the scheme of LAPACK's dstein: three solves with
// re-orthogonalisation against the previous members of the cluster). A warp issues one float64 instruction per
// ~64 cycles whatever its active lanes, so this serial per-thread work is
// written for few float64 instructions per row: pivots by integer compares,
// no branches (selects), reciprocals of the pivots by rcp_nr (stored, so
// the solves multiply), start vectors from integer bits. Every solve starts
// from a unit vector, and the back substitution rescales by 2^-600 when a
// component passes 2^600 (one solve grows by up to 1 / tiny per
// near-singular pivot, and a tight cluster has several of them).
// d, e, lam: shared copies; e2s: shared scratch of n doubles (e^2). Y: n x m
// row-major global (column j = vector j). lu: global scratch of
// 5 * n * nslot doubles; team threads [0, nslot) factorise (nslot <= team
// threads). cl: global int [m + 1]; the lead CTA lists the clusters, the
// count goes through gctl[2].
template <bool CL>
__device__ void team_tri_vectors(Team<CL> &tm, int n, const double *d, const double *e,
                                 const double *lam, int m, double tnorm, double *Y, double *lu,
                                 int nslot, int *cl, double *e2s) {
  const double ctol = 1e-6 * fmax(tnorm, 1.0);
  const double tiny = kEps * fmax(tnorm, 1.0);
  for (int i = threadIdx.x; i < n; i += blockDim.x) e2s[i] = i < n - 1 ? e[i] * e[i] : 0.0;
  // the twisted vector's range bookkeeping (rescaling every fourth row)
  // assumes |T| within 2^-+16 (a Fock matrix in Hartree: ~1..100)
  // Above 384 orbitals every vector takes inverse iteration: there the
  // twisted vectors of some molecules stalled the SCF near a residual of
  // 1e-2 (n = 743 and 796 in the serving stream, with or without the
  // Rayleigh-quotient step below), where inverse iteration follows the
  // oracle's trajectory exactly; every molecule of the benchmark sets (n <=
  // 377) is verified against the oracle with the twisted path.
  const bool twist_ok = n <= 384 && tnorm < 0x1p16 && tnorm > 0x1p-16;
  if (tm.lead() && threadIdx.x == 0) {
    int c = 0;
    cl[c++] = 0;
    for (int j = 1; j < m; ++j)
      if (lam[j] - lam[j - 1] > ctol) cl[c++] = j;
    cl[c] = m;
    tm.gctl[2] = c;
  }
  tm.sync();
  const int ncl = ldi<CL>(tm.gctl + 2);
  // factorisation slots: the first nslot threads in the spread order, so
  // that the clusters are shared by the CTAs
  const int tid = tm.stid;
  double *U0 = lu, *U1 = lu + (size_t)n * nslot, *U2 = lu + 2 * (size_t)n * nslot;
  double *Lm = lu + 3 * (size_t)n * nslot, *Pv = lu + 4 * (size_t)n * nslot;
#define LU(arr, i) arr[(size_t)(i) * nslot + tid]
  for (int c = tid; tid < nslot && c < ncl; c += nslot) {
    const int j0 = ldi<CL>(cl + c), j1 = ldi<CL>(cl + c + 1);
    if (j1 - j0 == 1 && twist_ok) {
      // one Rayleigh-quotient step when the eigenvalue is off by more than
      // rounding (Newton's root of a long recurrence can be ~1e-10 |T| off,
      // which spoils the vector of an eigenvalue with a gap of ~1e-6 |T|);
      // the refined shift is accurate to ~delta^2 / gap
      double lmb = lam[j0];
      for (int pass = 0; pass < 2; ++pass) {
        const double delta = tri_vector_twisted(n, d, e, e2s, lmb, Y, m, j0, U0, U1, U2, Lm, nslot, tid);
        if (!(fabs(delta) > 8.0 * kEps * fmax(tnorm, 1.0))) break;
        lmb += delta;
      }
      continue;
    }
    for (int j = j0; j < j1; ++j) {
      // separate exactly coincident shifts inside a cluster (dstein)
      const double lmb = lam[j] + (j - j0) * 10.0 * tiny;
      // LU with partial pivoting of T - lmb I; rows hold (1/diag, super, super2).
      // Pivots below tiny in magnitude are replaced by +-tiny (sign kept).
      double a = d[0] - lmb, bsup = n > 1 ? e[0] : 0.0;
      for (int i = 0; i < n - 1; ++i) {
        const double low = e[i];
        const double dn = d[i + 1] - lmb, en = (i + 1 < n - 1) ? e[i + 1] : 0.0;
        const bool swap = !abs_ge(a, low);
        double piv = swap ? low : a;
        if (!abs_ge(piv, tiny)) piv = is_neg(piv) ? -tiny : tiny;
        const double r = rcp_nr(piv);
        const double mult = (swap ? a : low) * r;
        LU(U0, i) = r;
        LU(U1, i) = swap ? dn : bsup;
        LU(U2, i) = swap ? en : 0.0;
        LU(Lm, i) = mult;
        LU(Pv, i) = swap ? 1.0 : 0.0;
        a = fma(-mult, swap ? dn : bsup, swap ? bsup : dn);
        bsup = swap ? flip_sign(mult) * en : en;
      }
      {
        double piv = a;
        if (!abs_ge(piv, tiny)) piv = is_neg(piv) ? -tiny : tiny;
        LU(U0, n - 1) = rcp_nr(piv);
        // the last row has no super-diagonals; its slots may still hold a
        // twisted vector's scale counts (integer bits, NaN patterns when
        // negative), and the back substitution multiplies them by zero
        LU(U1, n - 1) = 0.0;
        LU(U2, n - 1) = 0.0;
      }
      for (int i = 0; i < n; ++i) Y[(size_t)i * m + j] = start_vector(i, j);
      // unit 2-norm of column j, scaled by its largest entry first so that
      // the sum of squares cannot overflow
      auto unit = [&]() {
        double mx = 0.0;
        for (int i = 0; i < n; ++i) mx = fmax(mx, fabs(Y[(size_t)i * m + j]));
        const double s = mx > 0.0 ? 1.0 / mx : 1.0;
        double nrm = 0.0;
        for (int i = 0; i < n; ++i) {
          const double v = Y[(size_t)i * m + j] * s;
          nrm = fma(v, v, nrm);
        }
        const double inv = s / sqrt(fmax(nrm, kTiny));
        for (int i = 0; i < n; ++i) Y[(size_t)i * m + j] *= inv;
      };
      const int nsolve = (j1 - j0 > 1) ? 3 : 2;
      for (int it = 0; it < nsolve; ++it) {
        // every solve starts from a unit vector: one solve grows it by up to
        // ~1/tiny per near-singular pivot, and a cluster of exactly coincident
        // eigenvalues (a split tridiagonal) has several of them
        unit();
        // forward: apply the row interchanges and multipliers (the running
        // row stays in a register; the loads do not depend on the chain)
        double carry = Y[j];
#pragma unroll 4
        for (int i = 0; i < n - 1; ++i) {
          const double yn = Y[(size_t)(i + 1) * m + j];
          const bool sw = LU(Pv, i) != 0.0;
          const double xi = sw ? yn : carry, xn = sw ? carry : yn;
          Y[(size_t)i * m + j] = xi;
          carry = fma(-LU(Lm, i), xi, xn);
        }
        Y[(size_t)(n - 1) * m + j] = carry;
        // back substitution with the upper factor (two super-diagonals)
        double x1 = 0.0, x2 = 0.0;
#pragma unroll 4
        for (int i = n - 1; i >= 0; --i) {
          double v = fma(-LU(U2, i), x2, fma(-LU(U1, i), x1, Y[(size_t)i * m + j])) * LU(U0, i);
          if (!(fabs(v) <= 0x1p600)) {
            // growth beyond 2^600 (one row adds at most ~2^54: |U1|, |U2| <=
            // 2 |T|, |U0| <= 1 / (eps |T|)): rescale the solved rows, the rest
            // of the right-hand side and the carried values alike, and redo
            // this row
            for (int k = 0; k < n; ++k) Y[(size_t)k * m + j] *= 0x1p-600;
            x1 *= 0x1p-600;
            x2 *= 0x1p-600;
            v = fma(-LU(U2, i), x2, fma(-LU(U1, i), x1, Y[(size_t)i * m + j])) * LU(U0, i);
          }
          Y[(size_t)i * m + j] = v;
          x2 = x1;
          x1 = v;
        }
        // Gram-Schmidt against the earlier (normalised) members of the cluster
        for (int k = j0; k < j; ++k) {
          double dot = 0.0;
          for (int i = 0; i < n; ++i) dot = fma(Y[(size_t)i * m + k], Y[(size_t)i * m + j], dot);
          for (int i = 0; i < n; ++i) Y[(size_t)i * m + j] = fma(-dot, Y[(size_t)i * m + k], Y[(size_t)i * m + j]);
        }
      }
      unit();
    }
  }
#undef LU
  tm.sync();
}

// Y <- Q Y for the reflectors stored by team_tridiag (Q = H_0 ... H_{n-3});
// Y is n x m row-major. Each CTA transforms its own block of columns, so no
// team barrier is needed. The reflectors are applied kNB at a time in the
// compact WY form H_k0 ... H_k1-1 = I - V T V^T (T upper triangular, built as
// in LAPACK dlarft, forward / columnwise): W = V^T Y, W <- T W,
// Y <- Y - V W, about five CTA barriers per block instead of two or three
// per reflector. wsc: global scratch of kNB * m doubles (each CTA uses its
// own columns); spart: shared [kPart].
constexpr int kNB = 16;

template <bool CL>
__device__ void team_back_transform(Team<CL> &tm, int n, const double *A, const double *tau, double *Y,
                                    int m, double *wsc, double *spart) {
  __shared__ double sT[kNB][kNB + 1];
  __shared__ double sS[kNB][kNB + 1];
  __shared__ double stau[kNB];
  const int j0 = (int)((int64_t)m * tm.rank / tm.size), j1 = (int)((int64_t)m * (tm.rank + 1) / tm.size);
  const int mc = j1 - j0;
  const int nref = n - 2;  // reflectors 0 .. n-3 (the last ones may be identities)
  double *W = wsc + (size_t)kNB * j0;  // kNB x mc, leading dimension mc
  if (mc > 0 && nref > 0) {
    for (int kb = ((nref - 1) / kNB) * kNB; kb >= 0; kb -= kNB) {
      const int nb = min(kNB, nref - kb);
      const int r0 = kb + 1, L = n - r0;  // rows touched by the block
      // V(rho, i): reflector kb+i at local row rho = r - r0 (implicit 1 at rho = i)
      auto vv = [&](int rho, int i) -> double {
        return rho < i ? 0.0 : (rho == i ? 1.0 : ld<CL>(A + (size_t)(r0 + rho) * n + kb + i));
      };
      // (a) S = V^T V (strictly upper part) for T, rows split in G groups
      const int npair = nb * (nb - 1) / 2;
      if (threadIdx.x < nb) stau[threadIdx.x] = ld<CL>(tau + kb + threadIdx.x);
      if (npair > 0) {
        const int G = max(1, min(kPart / npair, (int)blockDim.x / npair));
        for (int q = threadIdx.x; q < G * npair; q += blockDim.x) {
          const int pr = q % npair, g = q / npair;
          int j = (int)((sqrtf(8.0f * (float)pr + 1.0f) + 1.0f) * 0.5f);  // pr -> (i < j)
          while (j * (j - 1) / 2 > pr) --j;
          while ((j + 1) * j / 2 <= pr) ++j;
          const int i = pr - j * (j - 1) / 2;
          double acc = 0.0;
          for (int rho = j + g; rho < L; rho += G) acc = fma(vv(rho, i), vv(rho, j), acc);
          spart[g * npair + pr] = acc;
        }
        __syncthreads();
        for (int pr = threadIdx.x; pr < npair; pr += blockDim.x) {
          int j = (int)((sqrtf(8.0f * (float)pr + 1.0f) + 1.0f) * 0.5f);
          while (j * (j - 1) / 2 > pr) --j;
          while ((j + 1) * j / 2 <= pr) ++j;
          const int i = pr - j * (j - 1) / 2;
          double acc = 0.0;
          for (int g = 0; g < G; ++g) acc += spart[g * npair + pr];
          sS[i][j] = acc;
        }
      }
      __syncthreads();
      // (b) T: lane i builds row i, T[i][j] = -tau_j sum_{l=i}^{j-1} T[i][l] S[l][j]
      if (threadIdx.x < nb) {
        const int i = threadIdx.x;
        for (int j = 0; j < nb; ++j) {
          if (j < i) {
            sT[i][j] = 0.0;
          } else if (j == i) {
            sT[i][j] = stau[i];
          } else {
            double acc = 0.0;
            for (int l = i; l < j; ++l) acc = fma(sT[i][l], sS[l][j], acc);
            sT[i][j] = -stau[j] * acc;
          }
        }
      }
      // (c) W = V^T Y (nb x mc), rows split in G groups
      {
        const int nout = nb * mc;
        const int G = nout < (int)blockDim.x ? max(1, min(kPart / nout, (int)blockDim.x / nout)) : 1;
        for (int q = threadIdx.x; q < G * nout; q += blockDim.x) {
          const int o = q % nout, g = q / nout;
          const int i = o / mc, j = o % mc;
          double acc = 0.0;
          for (int rho = i + g; rho < L; rho += G)
            acc = fma(vv(rho, i), ld<CL>(Y + (size_t)(r0 + rho) * m + j0 + j), acc);
          if (G > 1) spart[g * nout + o] = acc; else W[(size_t)i * mc + j] = acc;
        }
        __syncthreads();
        if (G > 1) {
          for (int o = threadIdx.x; o < nout; o += blockDim.x) {
            double acc = 0.0;
            for (int g = 0; g < G; ++g) acc += spart[g * nout + o];
            W[(size_t)(o / mc) * mc + o % mc] = acc;
          }
          __syncthreads();
        }
      }
      // (d) W <- T W, one column per thread, rows ascending in place
      for (int j = threadIdx.x; j < mc; j += blockDim.x) {
        for (int i = 0; i < nb; ++i) {
          double acc = 0.0;
          for (int l = i; l < nb; ++l) acc = fma(sT[i][l], W[(size_t)l * mc + j], acc);
          W[(size_t)i * mc + j] = acc;
        }
      }
      __syncthreads();
      // (e) Y <- Y - V W
      for (int64_t q = threadIdx.x; q < (int64_t)L * mc; q += blockDim.x) {
        const int rho = (int)(q / mc), j = (int)(q % mc);
        double *y = Y + (size_t)(r0 + rho) * m + j0 + j;
        double acc = ld<CL>(y);
        const int imax = min(nb - 1, rho);
        for (int i = 0; i <= imax; ++i) acc = fma(-vv(rho, i), W[(size_t)i * mc + j], acc);
        *y = acc;
      }
      __syncthreads();
    }
  }
  tm.sync();
}

}  // namespace dxtb
