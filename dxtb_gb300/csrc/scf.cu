// Persistent self-consistent-field kernels: a TEAM of CTAs runs the whole
// SCF of one molecule (orthogonaliser, Fock build, generalized eigensolve,
// Fermi occupations, density, Mulliken charges and atomic multipoles,
// potentials, limited-memory Broyden root solve) with a per-molecule
// convergence test and iteration cap. No host synchronisation inside the
// loop. Small molecules run one 256-thread CTA each, two per SM; larger ones
// one 512-thread CTA per SM; the largest a thread-block cluster of 2-16
// CTAs (one SM each) that share every O(n^3) phase.
//
// Reference path (src/dxtb/_src): scf/iterator.py:51-195, scf/pure/
// conversions.py:106-366 (charges <-> potential <-> Fock <-> density),
// scf/pure/ovlp_diag.py:36-62 and exlibs/xitorch/_impls/linalg/symeig.py:
// 38-76 (Cholesky orthogonaliser + symmetric eigensolver), wavefunction/
// filling.py:428-742 (Fermi occupations), scf/utils.py:29-52 (density),
// components/interactions/{base,list}.py and coulomb/{secondorder,
// thirdorder,multipole}.py (potentials and energies), scf/base.py:510-619
// (energy and electronic free energy).
#include "linalg.cuh"

namespace dxtb {

constexpr int kScfThreads = 256;     // CTA size for molecules sharing an SM
constexpr int kScfBigThreads = 512;  // CTA size of one-SM and cluster teams
constexpr int kRank = 256;           // Broyden memory (the reference keeps every update; >= maxiter)
constexpr double kOccCut = 1e-15;    // orbitals below this occupation carry no density
constexpr int kLuSlots = 1024;       // concurrent inverse-iteration factorisations per molecule
// size classes (kClasses, common.cuh): 0 small, 1 one SM, 2..5 clusters of 2..16
constexpr int kMaxCluster = 16;
// dynamic shared memory: 32 n bytes, plus the rows of the Householder
// reduction where they fit (one-SM and cluster teams), next to ~10 KB of
// static arrays, within the 227 KB of a CTA
constexpr int kMaxDynSmem = 208 * 1024;

struct MolView {
  int m, n, nat, nsh, N;
  int64_t a0, s0, o0, moff, mtot, n2off, n2tot, g0;
};

__host__ __device__ inline int64_t lu_slots(int64_t n) { return n < kLuSlots ? n : kLuSlots; }
// inverse-iteration factors or the minors of the twisted eigenvectors (5 n per
// slot), reused afterwards by the blocked back-transform (16 n)
__host__ __device__ inline int64_t lu_size(int64_t n) {
  const int64_t a = 5 * n * lu_slots(n), b = 16 * n;
  return a > b ? a : b;
}

// Per-molecule workspace layout (doubles).
__host__ __device__ inline int64_t ws_size_mol(int64_t n, int64_t nat) {
  const int64_t N = n + 9 * nat;
  return 3 * n * n + 10 * n + (2 * kRank + 7) * N + 64 + 16 * nat + lu_size(n) + n + 8 +
         4 * kRank + 64 + 64;
}

struct Ws {
  double *Linv, *A, *Zt, *d, *e, *tau, *p, *rc, *rs, *eps, *fa, *fb, *x, *g, *hx, *hr, *misc;
  double *vsh_tmp, *lu, *sdot, *xold, *rold, *xbest, *team;
  int *cl;
};

__device__ inline Ws ws_carve(double *base, int n, int nat) {
  const int N = n + 9 * nat;
  Ws w;
  double *q = base;
  w.Linv = q; q += (size_t)n * n;
  w.A = q; q += (size_t)n * n;
  w.Zt = q; q += (size_t)n * n;
  w.d = q; q += n;
  w.e = q; q += n;
  w.tau = q; q += n;
  w.p = q; q += n;
  w.rc = q; q += n;
  w.rs = q; q += n;
  w.eps = q; q += n;
  w.fa = q; q += n;
  w.fb = q; q += n;
  w.vsh_tmp = q; q += n;
  w.x = q; q += N;
  w.g = q; q += N;
  w.hx = q; q += (size_t)kRank * N;
  w.hr = q; q += (size_t)kRank * N;
  w.xold = q; q += N;
  w.rold = q; q += N;
  w.xbest = q; q += N;
  w.lu = q; q += (size_t)lu_size(n);
  w.cl = reinterpret_cast<int *>(q); q += n + 8;
  w.sdot = q; q += 4 * kRank + 64;
  w.team = q; q += 64;  // [0, 32) partial sums, [32, 48) broadcast words (int), [48] mixer flag
  w.misc = q;  // 64 + 16 nat + 2N
  return w;
}

// Fermi-Dirac occupations of singly occupied orbitals summing to nel
// (filling.py:428-742 converges to the same unique root): Newton steps on
// the electron count, safeguarded by a bisection bracket; warp 0 only.
// eps is sorted ascending. Returns false on failure.
__device__ bool fermi_warp(int n, const double *eps, double nel, double kt, double *f) {
  const int lane = threadIdx.x & 31;
  if (nel <= 0.0) {
    for (int j = lane; j < n; j += 32) f[j] = 0.0;
    return true;
  }
  if (nel >= (double)n) {
    for (int j = lane; j < n; j += 32) f[j] = 1.0;
    return true;
  }
  double lo = eps[0] - 60.0 * kt, hi = eps[n - 1] + 60.0 * kt;
  const int khomo = min(max((int)ceil(nel) - 1, 0), n - 1);
  double mu = 0.5 * (eps[khomo] + eps[min(khomo + 1, n - 1)]);
  const double ikt = 1.0 / kt;
  // f(x) = 1 / (1 + e^x) from one exp(-|x|) and a reciprocal (rcp_nr: 1 + e
  // lies in [1, 2]); beyond |x| = 40 f is 0 or 1 to 4e-18, below the
  // electron-count threshold, and the exp is skipped (the eigenvalues are
  // sorted, so whole warp iterations far from mu skip it together)
  auto occ = [](double x) {
    if (x > 40.0) return 0.0;
    if (x < -40.0) return 1.0;
    const double ex = exp(-fabs(x));
    const double r = rcp_nr(1.0 + ex);
    return x > 0.0 ? ex * r : r;
  };
  for (int it = 0; it < 200; ++it) {
    double s = 0.0, ds = 0.0;
    for (int j = lane; j < n; j += 32) {
      const double v = occ((eps[j] - mu) * ikt);
      s += v;
      ds = fma(v, 1.0 - v, ds);
    }
    s = warp_sum(s) - nel;
    ds = warp_sum(ds) * ikt;
    if (fabs(s) < 1e-13 * fmax(1.0, nel)) break;
    if (s > 0.0) hi = mu; else lo = mu;
    double next = ds > 0.0 ? mu - s / ds : 0.5 * (lo + hi);
    if (!(next > lo && next < hi)) next = 0.5 * (lo + hi);
    if (hi - lo < 1e-15 * fmax(1.0, fabs(mu))) break;
    mu = next;
  }
  double s = 0.0;
  for (int j = lane; j < n; j += 32) {
    const double v = occ((eps[j] - mu) * ikt);
    f[j] = v;
    s += v;
  }
  s = warp_sum(s);
  return fabs(s - nel) < 1e-6;
}

__device__ __forceinline__ double ent(double f) {
  const double o = fmax(f, kEps), o1 = fmax(1.0 - f, kEps);
  return o * log(o) + o1 * log(o1);
}

struct ScfArgs {
  dxtb_batch b;
  const double *pf;
  const int32_t *pi;
  const double *S, *H0, *D, *Q, *gamma, *hd, *sd, *dd, *sq, *gb, *n0, *nel;
  double kt, xtol, ftol;
  int maxiter;
  // root solver / mixer (dxtb_scf_config)
  int mixer, generations, soft_start;
  double xtol_max, damp, damp_init, offset;
  const int64_t *ws_off;
  const int32_t *order;
  double *ws, *P, *W, *C, *evals, *occ, *q, *dp, *qp, *vorb, *vdp, *vqp, *energies;
  int32_t *status;
  int thr[kClasses];  // smallest n of each size class (thr[0] = 0)
};

// Potential x = (vorb [n], vdp [nat][3], vqp [nat][6]) from the orbital
// charges qo and atomic multipoles dpa/qpa (interactions/base.py:135-181).
// One CTA (the team's lead); qo, dpa, qpa may come from the whole team.
template <bool CL>
__device__ void potential_from_charges(const ScfArgs &a, const MolView &mv, const double *qo,
                                       const double *dpa, const double *qpa, double *qsh,
                                       double *qat, double *vsh, double *vat, double *xout,
                                       int multipole, int es3_shell) {
  const dxtb_batch &b = a.b;
  const int n = mv.n, nat = mv.nat, nsh = mv.nsh;
  for (int s = threadIdx.x; s < nsh; s += blockDim.x) {
    const int t = b.shell_type[mv.s0 + s];
    const int o = b.shell_ao[mv.s0 + s], no = 2 * pi_(a.pi, DXTB_I_L + t) + 1;
    double v = 0.0;
    for (int k = 0; k < no; ++k) v += ld<CL>(qo + o + k);
    qsh[s] = v;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nat; i += blockDim.x) qat[i] = 0.0;
  __syncthreads();
  if (threadIdx.x == 0)
    for (int s = 0; s < nsh; ++s) qat[b.shell_atom[mv.s0 + s]] += qsh[s];
  __syncthreads();
  // shell potential: ES2 gamma q_sh (+ shell-resolved ES3)
  for (int s = threadIdx.x; s < nsh; s += blockDim.x) {
    const double *gr = a.gamma + mv.g0 + (size_t)s * nsh;
    double v = 0.0;
    for (int t = 0; t < nsh; ++t) v = fma(gr[t], qsh[t], v);
    if (es3_shell) v += a.hd[mv.s0 + s] * qsh[s] * qsh[s];
    vsh[s] = v;
  }
  // atom potential: atom-resolved ES3, AES2 monopole terms, GB
  for (int i = threadIdx.x; i < nat; i += blockDim.x) {
    double v = es3_shell ? 0.0 : a.hd[mv.a0 + i] * qat[i] * qat[i];
    if (multipole) {
      for (int j = 0; j < nat; ++j) {
        const int64_t o = mv.n2off + (int64_t)i * nat + j;
        for (int c = 0; c < 3; ++c) v += a.sd[c * mv.n2tot + o] * ld<CL>(dpa + 3 * j + c);
        for (int c = 0; c < 6; ++c) v += a.sq[c * mv.n2tot + o] * ld<CL>(qpa + 6 * j + c);
      }
    }
    if (a.gb != nullptr) {
      const double *gr = a.gb + mv.n2off + (size_t)i * nat;
      for (int j = 0; j < nat; ++j) v += gr[j] * qat[j];
    }
    vat[i] = v;
  }
  __syncthreads();
  for (int o = threadIdx.x; o < n; o += blockDim.x) {
    const int s = b.ao_shell[mv.o0 + o];
    xout[o] = vsh[s] + vat[b.shell_atom[mv.s0 + s]];
  }
  if (multipole) {
    const double qscale[6] = {1.0, 2.0, 1.0, 2.0, 2.0, 1.0};
    for (int j = threadIdx.x; j < nat; j += blockDim.x) {
      const int zj = b.numbers[mv.a0 + j];
      const double dk = pf(a.pf, DXTB_P_DKERNEL + zj), qk = pf(a.pf, DXTB_P_QKERNEL + zj);
      double vd[3], vq[6];
      for (int c = 0; c < 3; ++c) vd[c] = 2.0 * dk * ld<CL>(dpa + 3 * j + c);
      for (int c = 0; c < 6; ++c) vq[c] = 2.0 * qk * ld<CL>(qpa + 6 * j + c) * qscale[c];
      for (int i = 0; i < nat; ++i) {
        const int64_t o = mv.n2off + (int64_t)i * nat + j;
        for (int c = 0; c < 3; ++c) vd[c] += a.sd[c * mv.n2tot + o] * qat[i];
        for (int x = 0; x < 3; ++x)
          for (int y = 0; y < 3; ++y) vd[y] += a.dd[(3 * x + y) * mv.n2tot + o] * ld<CL>(dpa + 3 * i + x);
        for (int c = 0; c < 6; ++c) vq[c] += a.sq[c * mv.n2tot + o] * qat[i];
      }
      for (int c = 0; c < 3; ++c) xout[n + 3 * j + c] = vd[c];
      for (int c = 0; c < 6; ++c) xout[n + 3 * nat + 6 * j + c] = vq[c];
    }
  }
  __syncthreads();
}

// Interaction energy (interactions/base.py:306-360 summed): block result of
// the lead CTA.
template <bool CL>
__device__ double interaction_energy(const ScfArgs &a, const MolView &mv, const double *qsh,
                                     const double *qat, const double *dpa, const double *qpa,
                                     int multipole, int es3_shell, double *red) {
  const dxtb_batch &b = a.b;
  const int nat = mv.nat, nsh = mv.nsh;
  double e = 0.0;
  for (int s = threadIdx.x; s < nsh; s += blockDim.x) {
    const double *gr = a.gamma + mv.g0 + (size_t)s * nsh;
    double v = 0.0;
    for (int t = 0; t < nsh; ++t) v = fma(gr[t], qsh[t], v);
    e += 0.5 * qsh[s] * v;
    if (es3_shell) e += a.hd[mv.s0 + s] * qsh[s] * qsh[s] * qsh[s] / 3.0;
  }
  const double qscale[6] = {1.0, 2.0, 1.0, 2.0, 2.0, 1.0};
  for (int j = threadIdx.x; j < nat; j += blockDim.x) {
    if (!es3_shell) e += a.hd[mv.a0 + j] * qat[j] * qat[j] * qat[j] / 3.0;
    if (multipole) {
      const int zj = b.numbers[mv.a0 + j];
      const double dk = pf(a.pf, DXTB_P_DKERNEL + zj), qk = pf(a.pf, DXTB_P_QKERNEL + zj);
      double vd[3] = {0, 0, 0}, vq[6] = {0, 0, 0, 0, 0, 0};
      for (int i = 0; i < nat; ++i) {
        const int64_t o = mv.n2off + (int64_t)i * nat + j;
        for (int c = 0; c < 3; ++c) vd[c] += a.sd[c * mv.n2tot + o] * qat[i];
        for (int x = 0; x < 3; ++x)
          for (int y = 0; y < 3; ++y)
            vd[y] += 0.5 * a.dd[(3 * x + y) * mv.n2tot + o] * ld<CL>(dpa + 3 * i + x);
        for (int c = 0; c < 6; ++c) vq[c] += a.sq[c * mv.n2tot + o] * qat[i];
      }
      for (int c = 0; c < 3; ++c) {
        const double dj = ld<CL>(dpa + 3 * j + c);
        e += (dk * dj + vd[c]) * dj;
      }
      for (int c = 0; c < 6; ++c) {
        const double qj = ld<CL>(qpa + 6 * j + c);
        e += (qk * qscale[c] * qj + vq[c]) * qj;
      }
    }
    if (a.gb != nullptr) {
      const double *gr = a.gb + mv.n2off + (size_t)j * nat;
      double v = 0.0;
      for (int i = 0; i < nat; ++i) v += gr[i] * qat[i];
      e += 0.5 * qat[j] * v;
    }
  }
  return block_sum(e, red);
}

// State of the root solver, held by the lead CTA only. final_eval: one more
// pass evaluates the energy at the iterate left in x (hit_max: with status
// MAXITER); base: the Anderson history ring's entry 0.
struct Broyden {
  int nrank = 0, final_eval = 0, hit_max = 0, base = 0;
  double resid = 0.0, best_ynorm = 1e308, dx_norm = 0.0;
};

enum ScfAction : int { kNext = 0, kStop = 1 };

// One step of the root solver on F(x) = x - G(x): limited-memory Broyden's
// first method on the inverse Jacobian, Gm = 0.5 I + sum_k c_k d_k^T,
// damped steps x += damp * dx, dx = -Gm F (the broyden1 of exlibs/xitorch/
// _impls/optimize/root/{rootsolver.py:42-265, _jacobian.py:51-120} with
// alpha = -0.5, damp = 0.5, line_search = False, scf/base.py:267-292);
// stop when |dx|_2 < x_tol and |F|_2 < f_tol. Lead CTA only.
__device__ int broyden_step(const ScfArgs &a, Ws &w, int N, int it, Broyden &br, int &status,
                            double *red) {
  double *sdot = w.sdot;         // [kRank] dot products
  double *sdot2 = sdot + kRank;  // [kRank]
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nw = (int)(blockDim.x >> 5);
  // |F|^2 with F = x - G(x)
  double part = 0.0;
  for (int t = threadIdx.x; t < N; t += blockDim.x) {
    const double y = w.x[t] - w.g[t];
    part += y * y;
  }
  const double ynorm = sqrt(block_sum(part, red));
  br.resid = ynorm;
  if (it == 1) {
    if (ynorm <= a.ftol * kEps) return kStop;
    br.nrank = 0;
  } else {
    if (ynorm < br.best_ynorm) {
      br.best_ynorm = ynorm;
      for (int t = threadIdx.x; t < N; t += blockDim.x) w.xbest[t] = w.x[t];
    }
    // Broyden update with dx = x - x_prev, dy = F - F_prev:
    // v = Gm^T dx, c = dx - Gm dy, d = v / (dy . v)
    if (br.nrank >= kRank) br.nrank = 0;  // "restart" reduction of a full memory (not reached: kRank >= maxiter)
    const int nrank = br.nrank;
    // dx and dy once (into the x_prev / F_prev slots, rewritten below): a
    // float64 instruction costs a warp ~64 cycles, so the dot products below
    // read them instead of forming the differences again per history vector
    for (int t = threadIdx.x; t < N; t += blockDim.x) {
      const double xt = w.x[t];
      w.rold[t] = (xt - w.g[t]) - w.rold[t];
      w.xold[t] = xt - w.xold[t];
    }
    __syncthreads();
    for (int k = wid; k < 2 * nrank; k += nw) {
      const int kk = k >> 1;
      double s = 0.0;
      if ((k & 1) == 0) {
        const double *ck = w.hx + (size_t)kk * N;
        for (int t = lane; t < N; t += 32) s = fma(ck[t], w.xold[t], s);
      } else {
        const double *dk = w.hr + (size_t)kk * N;
        for (int t = lane; t < N; t += 32) s = fma(dk[t], w.rold[t], s);
      }
      s = warp_sum(s);
      if (lane == 0) {
        if ((k & 1) == 0) sdot[kk] = s; else sdot2[kk] = s;
      }
    }
    __syncthreads();
    double *cn = w.hx + (size_t)nrank * N, *dn = w.hr + (size_t)nrank * N;
    double pdv = 0.0;
    for (int t = threadIdx.x; t < N; t += blockDim.x) {
      const double dxt = w.xold[t];
      const double dyt = w.rold[t];
      double v = 0.5 * dxt, gdy = 0.5 * dyt;
      for (int k = 0; k < nrank; ++k) {
        v += w.hr[(size_t)k * N + t] * sdot[k];
        gdy += w.hx[(size_t)k * N + t] * sdot2[k];
      }
      cn[t] = dxt - gdy;
      dn[t] = v;
      pdv += dyt * v;
    }
    const double dyv = block_sum(pdv, red);
    if (dyv == 0.0 || !isfinite(dyv)) {
      status = DXTB_ERR_NAN;
      return kStop;
    }
    const double idyv = 1.0 / dyv;
    for (int t = threadIdx.x; t < N; t += blockDim.x) dn[t] *= idyv;
    ++br.nrank;
    __syncthreads();
    if (br.dx_norm < a.xtol && ynorm < a.ftol) return kStop;  // converged at x
  }
  if (it >= a.maxiter) {
    // not converged: evaluate once more at the best iterate, which the root
    // solver returns with a warning (rootsolver.py:250-259)
    if (br.best_ynorm < ynorm) {
      for (int t = threadIdx.x; t < N; t += blockDim.x) w.x[t] = w.xbest[t];
      br.final_eval = 1;
      br.hit_max = 1;
      __syncthreads();
      return kNext;
    }
    br.hit_max = 1;
    return kStop;
  }
  // F_prev = F, x_prev = x; dx = -Gm F = -(0.5 F + sum_k c_k (d_k . F))
  const int nrank = br.nrank;
  for (int k = wid; k < nrank; k += nw) {
    const double *dk = w.hr + (size_t)k * N;
    double s = 0.0;
    for (int t = lane; t < N; t += 32) s += dk[t] * (w.x[t] - w.g[t]);
    s = warp_sum(s);
    if (lane == 0) sdot[k] = s;
  }
  __syncthreads();
  double pdx = 0.0;
  for (int t = threadIdx.x; t < N; t += blockDim.x) {
    const double y = w.x[t] - w.g[t];
    double dx = -0.5 * y;
    for (int k = 0; k < nrank; ++k) dx -= w.hx[(size_t)k * N + t] * sdot[k];
    w.rold[t] = y;
    w.xold[t] = w.x[t];
    w.x[t] += a.damp * dx;
    pdx += dx * dx;
  }
  br.dx_norm = sqrt(block_sum(pdx, red));
  if (br.dx_norm == 0.0) {
    status = DXTB_ERR_NAN;
    return kStop;
  }
  return kNext;
}

// Solves the n x n system A th = r in place (Gaussian elimination with
// partial pivoting, n <= kMaxGen); one thread. False for a zero pivot.
constexpr int kMaxGen = 16;  // Anderson generations (the system and th fit in sdot)
__device__ bool small_solve(int n, double *A, double *r) {
  for (int k = 0; k < n; ++k) {
    int p = k;
    for (int i = k + 1; i < n; ++i)
      if (fabs(A[i * n + k]) > fabs(A[p * n + k])) p = i;
    if (A[p * n + k] == 0.0 || !isfinite(A[p * n + k])) return false;
    if (p != k) {
      for (int j = 0; j < n; ++j) {
        const double t = A[k * n + j];
        A[k * n + j] = A[p * n + j];
        A[p * n + j] = t;
      }
      const double t = r[k];
      r[k] = r[p];
      r[p] = t;
    }
    const double inv = 1.0 / A[k * n + k];
    for (int i = k + 1; i < n; ++i) {
      const double f = A[i * n + k] * inv;
      for (int j = k; j < n; ++j) A[i * n + j] = fma(-f, A[k * n + j], A[i * n + j]);
      r[i] = fma(-f, r[k], r[i]);
    }
  }
  for (int k = n - 1; k >= 0; --k) {
    double v = r[k];
    for (int j = k + 1; j < n; ++j) v = fma(-A[k * n + j], r[j], v);
    r[k] = v / A[k * n + k];
  }
  return true;
}

// One step of the reference's full-mode SCF loop with its Anderson mixer
// (scf/unrolling/default.py:80-140 with mix_guess; scf/mixer/anderson.py:
// 163-317, after Eyert): F = G(x) - x; convergence when |F|_2 < x_atol and
// max |F| < x_atol_max (mixer/base.py:230-256), checked from the second call
// on (the first mixes the guess); then the converged value is G(x), and one
// more pass evaluates the energy there (scf/base.py converged_to_charges).
// Mixing: simple x + damp_init F for the first `generations` calls (soft
// start) or the first call, else x_bar + damp F_bar with the coefficients th
// of (dF_i . dF_j)(1 + offset^2 on the diagonal) th = dF_i . F, dF_i = F -
// F_i over the last min(call - 1, generations) entries. The histories X (in
// hx) and F (in hr) are rings of generations + 1 vectors. Lead CTA only.
__device__ int anderson_step(const ScfArgs &a, Ws &w, int N, int it, Broyden &br, int &status,
                             double *red) {
  const int G = a.generations, H = G + 1;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nw = (int)(blockDim.x >> 5);
  auto X = [&](int h) { return w.hx + (size_t)((br.base + h) % H) * N; };
  auto F = [&](int h) { return w.hr + (size_t)((br.base + h) % H) * N; };
  double *x0 = X(0), *f0 = F(0);
  double p2 = 0.0, pm = 0.0;
  for (int t = threadIdx.x; t < N; t += blockDim.x) {
    const double xt = w.x[t], ft = w.g[t] - xt;
    x0[t] = xt;
    f0[t] = ft;
    p2 = fma(ft, ft, p2);
    pm = fmax(pm, fabs(ft));
  }
  const double l2 = sqrt(block_sum(p2, red));
  const double mx = block_max(pm, red);
  br.resid = l2;
  if (!isfinite(l2)) {
    status = DXTB_ERR_NAN;
    return kStop;
  }
  // the loop ends after maxiter calls beyond the guess-mixing one
  const bool conv = it >= 2 && l2 < a.xtol && mx < a.xtol_max;
  if (conv || it >= a.maxiter + 1) {
    for (int t = threadIdx.x; t < N; t += blockDim.x) w.x[t] = w.g[t];
    br.final_eval = 1;
    br.hit_max = conv ? 0 : 1;
    __syncthreads();
    return kNext;
  }
  double *sdot = w.sdot;  // [0, n(n+1)/2 + n): the system; then th
  if (it > G || (it > 1 && !a.soft_start)) {
    const int n = min(it - 1, G);
    const int npair = n * (n + 1) / 2;
    // task k < npair: (dF_i . dF_j), i <= j; then dF_i . F
    for (int k = wid; k < npair + n; k += nw) {
      int i, j;
      if (k < npair) {
        i = 0;
        while ((i + 1) * (i + 2) / 2 <= k) ++i;
        j = k - i * (i + 1) / 2;  // j <= i
      } else {
        i = k - npair;
        j = -1;
      }
      const double *fi = F(i + 1), *fj = j >= 0 ? F(j + 1) : nullptr;
      double s = 0.0;
      for (int t = lane; t < N; t += 32) {
        const double di = f0[t] - fi[t];
        s = fma(di, j >= 0 ? f0[t] - fj[t] : f0[t], s);
      }
      s = warp_sum(s);
      if (lane == 0) sdot[k] = s;
    }
    __syncthreads();
    double *A = sdot + npair + n, *th = A + n * n;
    if (threadIdx.x == 0) {
      for (int i = 0; i < n; ++i) {
        for (int j = 0; j <= i; ++j) {
          const double v = sdot[i * (i + 1) / 2 + j];
          A[i * n + j] = v;
          A[j * n + i] = v;
        }
        A[i * n + i] *= 1.0 + a.offset * a.offset;
        th[i] = sdot[npair + i];
      }
      w.team[48] = small_solve(n, A, th) ? 1.0 : 0.0;
    }
    __syncthreads();
    if (w.team[48] == 0.0) {
      status = DXTB_ERR_NAN;
      return kStop;
    }
    // x_mix = X0 + damp F0 + sum_i th_i ((X_i - X0) + damp (F_i - F0))
    for (int t = threadIdx.x; t < N; t += blockDim.x) {
      const double xt = x0[t], ft = f0[t];
      double v = fma(a.damp, ft, xt);
      for (int i = 0; i < n; ++i) v = fma(th[i], (X(i + 1)[t] - xt) + a.damp * (F(i + 1)[t] - ft), v);
      w.x[t] = v;
    }
  } else {
    for (int t = threadIdx.x; t < N; t += blockDim.x) w.x[t] = fma(a.damp_init, f0[t], x0[t]);
  }
  br.base = (br.base + H - 1) % H;  // entry 0 of this call becomes entry 1
  __syncthreads();
  return kNext;
}

// The SCF of molecule m_ by the team tm. dsm: dynamic shared memory of
// 3 n doubles + 2 n floats (n of this molecule or larger), then room for
// the rows of the Householder reduction (`rows`: false for teams that
// share an SM, which keep the rows in the L1).
template <bool CL>
__device__ void scf_body(const ScfArgs &a, int m_, Team<CL> &tm, double *dsm, bool rows) {
  __shared__ double red[32];
  __shared__ double spart[kPart];
  const dxtb_batch &b = a.b;
  MolView mv;
  mv.m = m_;
  const int m = mv.m;
  mv.a0 = b.atom_off[m];
  mv.s0 = b.shell_off[m];
  mv.o0 = b.ao_off[m];
  mv.moff = b.mat_off[m];
  mv.mtot = b.mat_off[b.nmol];
  mv.n2off = b.nat2_off[m];
  mv.n2tot = b.nat2_off[b.nmol];
  mv.g0 = b.nsh2_off[m];
  mv.n = (int)(b.ao_off[m + 1] - mv.o0);
  mv.nat = (int)(b.atom_off[m + 1] - mv.a0);
  mv.nsh = (int)(b.shell_off[m + 1] - mv.s0);
  const int n = mv.n, nat = mv.nat;
  const int multipole = pi_(a.pi, DXTB_I_SCAL + DXTB_IS_MULTIPOLE);
  const int es3_shell = pi_(a.pi, DXTB_I_SCAL + DXTB_IS_ES3_SHELL);
  const int N = n + (multipole ? 9 * nat : 0);
  mv.N = N;
  Ws w = ws_carve(a.ws + a.ws_off[m], n, nat);
  tm.gred = w.team;
  tm.gctl = reinterpret_cast<int *>(w.team + 32);
  tm.phase = 0;
  double *qsh = w.misc, *qat = qsh + mv.nsh + 1, *vat = qat + nat + 1;
  double *dpa = vat + nat + 1, *qpa = dpa + 3 * nat + 1, *qo = qpa + 6 * nat + 1;
  double *vsh = w.vsh_tmp;
  // shared copies: tridiagonal (sd, se), sorted eigenvalues (sw), float32 (df, e2f)
  double *sd = dsm, *se = dsm + n, *sw = dsm + 2 * n;
  float *df = reinterpret_cast<float *>(dsm + 3 * n), *e2f = df + n;

  const double *S = a.S + mv.moff, *H0 = a.H0 + mv.moff;
  double *P = a.P + mv.moff, *C = a.C + mv.moff;
  const double *n0 = a.n0 + mv.o0;
  const double nel_a = a.nel[2 * m], nel_b = a.nel[2 * m + 1];
  int status = DXTB_OK;

  // ---- orthogonaliser X = L^-1 (S = L L^T), once per geometry ----
  for (int64_t t = tm.tid; t < (int64_t)n * n; t += tm.nthr) w.A[t] = S[t];
  tm.sync();
  if (!team_cholesky(tm, n, w.A)) status = DXTB_ERR_NOT_POSDEF;
  if (status == DXTB_OK) team_trinv(tm, n, w.A, w.Linv);
  for (int t = tm.tid; t < N; t += tm.nthr) w.x[t] = 0.0;
  tm.sync();

  int it = 0, mo = 1;
  Broyden br;
  while (status == DXTB_OK) {
    ++it;
    // ---- Fock matrix F(x) into Zt (conversions.py:255-297) ----
    // The multipole part -1/2 (T + T^T) with T_ij = sum_c M_c,ij v_c(atom of j)
    // is formed in two coalesced passes (T into A, then the transposed read),
    // the orbital -> atom map and the orbital potential staged in shared
    // memory (free here: df and sd are used later in the iteration).
    {
      int *aoat = reinterpret_cast<int *>(df);
      for (int i = threadIdx.x; i < n; i += blockDim.x) {
        aoat[i] = b.shell_atom[mv.s0 + b.ao_shell[mv.o0 + i]];
        sd[i] = ld<CL>(w.x + i);
      }
      __syncthreads();
      if (multipole) {
        const double *xd = w.x + n, *xq = w.x + n + 3 * nat;
        const double *Dm = a.D + mv.moff, *Qm = a.Q + mv.moff;
        for (int64_t t = tm.tid; t < (int64_t)n * n; t += tm.nthr) {
          const int aj = aoat[(int)(t % n)];
          double acc = 0.0;
#pragma unroll
          for (int c = 0; c < 3; ++c) acc = fma(Dm[c * mv.mtot + t], ld<CL>(xd + 3 * aj + c), acc);
#pragma unroll
          for (int c = 0; c < 6; ++c) acc = fma(Qm[c * mv.mtot + t], ld<CL>(xq + 6 * aj + c), acc);
          w.A[t] = acc;
        }
        tm.sync();
      }
      for (int64_t t = tm.tid; t < (int64_t)n * n; t += tm.nthr) {
        const int i = (int)(t / n), j = (int)(t % n);
        double f = H0[t] - 0.5 * S[t] * (sd[i] + sd[j]);
        if (multipole) f -= 0.5 * (ld<CL>(w.A + t) + ld<CL>(w.A + (size_t)j * n + i));
        w.Zt[t] = f;
      }
      tm.sync();
    }
    // ---- F' = X F X^T (exlibs/xitorch/_impls/linalg/symeig.py:57-61) ----
    // X = L^-1 is lower triangular: A = X F needs k <= i; only the lower
    // triangle of (X F) X^T is formed (k <= j), then mirrored.
    team_gemm<false, false>(tm, n, n, n, 1.0, w.Linv, n, w.Zt, n, 0.0, w.A, n, kALower);
    team_gemm<false, true>(tm, n, n, n, 1.0, w.A, n, w.Linv, n, 0.0, w.Zt, n, kBLowerT, true);
    for (int64_t t = tm.tid; t < (int64_t)n * n; t += tm.nthr) {
      const int i = (int)(t / n), j = (int)(t % n);
      w.A[t] = j <= i ? ld<CL>(w.Zt + t) : ld<CL>(w.Zt + (size_t)j * n + i);
    }
    tm.sync();
    // ---- eigenvalues: Householder tridiagonalisation + bisection/Newton ----
    {
      uint32_t dyn;
      asm("mov.u32 %0, %%dynamic_smem_size;" : "=r"(dyn));
      const int64_t cap = (int64_t)(dyn / sizeof(double)) - 4 * (int64_t)n;
      team_tridiag(tm, n, w.A, w.d, w.e, w.tau, sd, se, sw, reinterpret_cast<double *>(df), spart,
                   rows && cap > 0 ? dsm + 4 * n : nullptr, cap);
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      sd[i] = ld<CL>(w.d + i);
      se[i] = ld<CL>(w.e + i);
    }
    __syncthreads();
    team_tri_eigenvalues(tm, n, sd, se, sw, w.rc, df, e2f);  // sw: e^2 scratch here
    team_rank_sort(tm, n, w.rc, w.eps, sw);  // ascending, like eigh
    for (int i = threadIdx.x; i < n; i += blockDim.x) sw[i] = ld<CL>(w.eps + i);
    double tnorm = 0.0;
    for (int j = threadIdx.x; j < n; j += blockDim.x) tnorm = fmax(tnorm, fabs(sd[j]) + 2.0 * fabs(se[j]));
    tnorm = block_max(tnorm, red);  // also orders the sw writes
    // ---- Fermi occupations (filling.py:428-742), both spin channels ----
    if (tm.lead() && threadIdx.x < 32) {
      bool ok = fermi_warp(n, sw, nel_a, a.kt, w.fa);
      if (nel_b == nel_a) {
        for (int j = threadIdx.x; j < n; j += 32) w.fb[j] = w.fa[j];
      } else {
        ok = ok && fermi_warp(n, sw, nel_b, a.kt, w.fb);
      }
      __syncwarp();
      if (threadIdx.x == 0) {
        // orbitals with non-vanishing occupation (occupations decrease with
        // j), extended to the end of their eigenvalue cluster
        int mm = 0;
        while (mm < n && w.fa[mm] + w.fb[mm] > kOccCut) ++mm;
        mm = mm > 0 ? mm : 1;
        const double ctol = 1e-6 * fmax(tnorm, 1.0);
        while (mm < n && sw[mm] - sw[mm - 1] <= ctol) ++mm;
        tm.gctl[0] = ok ? 1 : 0;
        tm.gctl[1] = mm;
      }
    }
    tm.sync();
    if (!ldi<CL>(tm.gctl + 0)) {
      status = DXTB_ERR_FERMI;
      break;
    }
    mo = ldi<CL>(tm.gctl + 1);
    // ---- eigenvectors of the mo lowest orbitals only ----
    team_tri_vectors(tm, n, sd, se, sw, mo, tnorm, w.Zt, w.lu, (int)min((int64_t)tm.nthr, lu_slots(n)), w.cl,
                     reinterpret_cast<double *>(df));
    team_back_transform(tm, n, w.A, w.tau, w.Zt, mo, w.lu, spart);  // lu: free after the vectors
    // ---- C^T = Y^T X (orbital j is row j; X lower -> k >= i) ----
    team_gemm<true, false>(tm, mo, n, n, 1.0, w.Zt, mo, w.Linv, n, 0.0, C, n, kBUpper);
    // ---- density P = C diag(occ) C^T (scf/utils.py:29-52) ----
    for (int64_t t = tm.tid; t < (int64_t)mo * n; t += tm.nthr) {
      const int j = (int)(t / n);
      w.A[t] = ld<CL>(C + t) * (ld<CL>(w.fa + j) + ld<CL>(w.fb + j));
    }
    tm.sync();
    team_gemm<true, false>(tm, n, n, mo, 1.0, C, n, w.A, n, 0.0, P, n, kFull, true);
    team_mirror_lower(tm, n, P);
    // ---- Mulliken charges and atomic multipoles (conversions.py:203-251) ----
    for (int i = tm.tid; i < n; i += tm.nthr) {
      double pop = 0.0;
      for (int k = 0; k < n; ++k) pop = fma(ld<CL>(P + (size_t)k * n + i), S[(size_t)k * n + i], pop);
      qo[i] = n0[i] - pop;
    }
    if (multipole) {
      for (int t = tm.tid; t < 3 * nat; t += tm.nthr) dpa[t] = 0.0;
      for (int t = tm.tid; t < 6 * nat; t += tm.nthr) qpa[t] = 0.0;
      tm.sync();
      // -sum_k P_ik M[c][k][i] per orbital i, reduced onto the atom of i
      for (int i = tm.tid; i < n; i += tm.nthr) {
        double acc[9];
        for (int c = 0; c < 9; ++c) acc[c] = 0.0;
        for (int k = 0; k < n; ++k) {
          const double pk = ld<CL>(P + (size_t)k * n + i);
          const int64_t e = mv.moff + (int64_t)k * n + i;
          for (int c = 0; c < 3; ++c) acc[c] -= pk * a.D[c * mv.mtot + e];
          for (int c = 0; c < 6; ++c) acc[3 + c] -= pk * a.Q[c * mv.mtot + e];
        }
        const int ai = b.shell_atom[mv.s0 + b.ao_shell[mv.o0 + i]];
        for (int c = 0; c < 3; ++c) atomicAdd(&dpa[3 * ai + c], acc[c]);
        for (int c = 0; c < 6; ++c) atomicAdd(&qpa[6 * ai + c], acc[3 + c]);
      }
    }
    tm.sync();
    // ---- new potential G(x) and the root-solver step (lead CTA) ----
    if (tm.lead()) {
      potential_from_charges<CL>(a, mv, qo, dpa, qpa, qsh, qat, vsh, vat, w.g, multipole, es3_shell);
      int act;
      if (br.final_eval) {
        act = kStop;  // hit_max as set when the final evaluation was scheduled
      } else if (a.mixer == DXTB_MIXER_ANDERSON) {
        act = anderson_step(a, w, N, it, br, status, red);
      } else {
        act = broyden_step(a, w, N, it, br, status, red);
      }
      if (threadIdx.x == 0) {
        tm.gctl[3] = act;
        tm.gctl[4] = (act == kStop && br.hit_max && status == DXTB_OK) ? DXTB_ERR_MAXITER : status;
      }
    }
    tm.sync();
    status = ldi<CL>(tm.gctl + 4);
    if (ldi<CL>(tm.gctl + 3) == kStop) break;
  }

  // ---- outputs ----
  if (status == DXTB_OK || status == DXTB_ERR_MAXITER) {
    // energies (scf/base.py:510-619): E_h0 + E_int and -TS
    double part = 0.0;
    for (int64_t t = tm.tid; t < (int64_t)n * n; t += tm.nthr) part += ld<CL>(P + t) * H0[t];
    const double eh0 = team_sum(tm, part, red);
    if (tm.lead()) {
      const double eint = interaction_energy<CL>(a, mv, qsh, qat, dpa, qpa, multipole, es3_shell, red);
      double ts = 0.0;
      for (int j = threadIdx.x; j < n; j += blockDim.x) ts += ent(w.fa[j]) + ent(w.fb[j]);
      ts = a.kt * block_sum(ts, red);
      if (threadIdx.x == 0) {
        a.energies[4 * m + 0] = eh0 + eint;
        a.energies[4 * m + 1] = ts;
        a.energies[4 * m + 2] = (double)it;
        a.energies[4 * m + 3] = br.resid;
        if (!isfinite(eh0 + eint + ts)) status = DXTB_ERR_NAN;
      }
      for (int j = threadIdx.x; j < n; j += blockDim.x) {
        a.evals[mv.o0 + j] = sw[j];
        a.occ[mv.o0 + j] = w.fa[j] + w.fb[j];
        a.q[mv.o0 + j] = ld<CL>(qo + j);
      }
      // potentials of the final charges (for the gradient)
      for (int t = threadIdx.x; t < n; t += blockDim.x) a.vorb[mv.o0 + t] = w.g[t];
      if (multipole) {
        for (int t = threadIdx.x; t < 3 * nat; t += blockDim.x) {
          a.vdp[3 * mv.a0 + t] = w.g[n + t];
          a.dp[3 * mv.a0 + t] = ld<CL>(dpa + t);
        }
        for (int t = threadIdx.x; t < 6 * nat; t += blockDim.x) {
          a.vqp[6 * mv.a0 + t] = w.g[n + 3 * nat + t];
          a.qp[6 * mv.a0 + t] = ld<CL>(qpa + t);
        }
      }
    }
    // energy-weighted density W = C diag(occ eps) C^T over the mo orbitals
    if (a.W != nullptr) {
      for (int64_t t = tm.tid; t < (int64_t)mo * n; t += tm.nthr) {
        const int j = (int)(t / n);
        w.A[t] = ld<CL>(C + t) * (ld<CL>(w.fa + j) + ld<CL>(w.fb + j)) * sw[j];
      }
      tm.sync();
      team_gemm<true, false>(tm, n, n, mo, 1.0, C, n, w.A, n, 0.0, a.W + mv.moff, n, kFull, true);
      team_mirror_lower(tm, n, a.W + mv.moff);
    }
    // coefficients of orbitals without occupation are not computed
    for (int64_t t = (int64_t)mo * n + tm.tid; t < (int64_t)n * n; t += tm.nthr) C[t] = 0.0;
  }
  if (tm.lead() && threadIdx.x == 0) a.status[m] = status;
  tm.sync();  // the team's workspace may be reused by its next molecule
}

// One CTA per molecule of size class `cls` (0: NT = 256, two per SM;
// 1: NT = 512, one per SM); CTA i takes the i-th molecule of the launch order.
template <int NT, int MINB>
__global__ void __launch_bounds__(NT, MINB) k_scf(ScfArgs a, int cls) {
  extern __shared__ double dsm[];
  const int i = blockIdx.x;
  const int m = a.order ? a.order[i] : i;
  if (scf_class(a.thr, (int)(a.b.ao_off[m + 1] - a.b.ao_off[m])) != cls) return;
  Team<false> tm;
  tm.rank = 0;
  tm.size = 1;
  tm.tid = threadIdx.x;
  tm.stid = threadIdx.x;
  tm.nthr = blockDim.x;
  scf_body<false>(a, m, tm, dsm, MINB == 1);
}

// One thread-block cluster per molecule of size class `cls` (2..5); the
// clusters of the launch take the molecules of the class in launch order,
// round robin. Every CTA of a cluster walks the same list, so the team's
// control flow is uniform.
__global__ void __launch_bounds__(kScfBigThreads, 1) k_scf_cluster(ScfArgs a, int cls) {
  extern __shared__ double dsm[];
  Team<true> tm;
  tm.rank = (int)cluster_ctarank();
  tm.size = (int)cluster_nctarank();
  tm.tid = tm.rank * blockDim.x + threadIdx.x;
  tm.stid = threadIdx.x * tm.size + tm.rank;
  tm.nthr = tm.size * blockDim.x;
  const int q = blockIdx.x / tm.size, nq = gridDim.x / tm.size;
  int cnt = 0;
  for (int i = 0; i < a.b.nmol; ++i) {
    const int m = a.order ? a.order[i] : i;
    if (scf_class(a.thr, (int)(a.b.ao_off[m + 1] - a.b.ao_off[m])) != cls) continue;
    if (cnt++ % nq == q) scf_body<true>(a, m, tm, dsm, true);
  }
}

}  // namespace dxtb

using namespace dxtb;

extern "C" int64_t dxtb_scf_workspace_mol(int64_t n, int64_t nat) { return ws_size_mol(n, nat); }

#include <mutex>

namespace dxtb {

// Size-class thresholds (smallest n of classes 1..5), process-wide.
static std::mutex g_policy_mutex;
static int g_thr[kClasses] = {0, 112, 136, 160, 320, 640};

// Side streams and fork/join events per (device, caller stream), created once
// (no device memory is allocated); all launches stay inside a caller's
// stream capture. Callers on different streams (the serving loop's slots)
// get different side streams, so their large-molecule kernels overlap.
struct SideStream {
  cudaStream_t caller = nullptr;
  cudaStream_t s[kClasses] = {};
  cudaEvent_t fork = nullptr, join[kClasses] = {};
  int prio[kClasses] = {};  // priority of s[c], also set on each class launch
  bool used = false;
};
constexpr int kSidePerDev = 32;
static std::mutex g_side_mutex;
static SideStream g_side[64][kSidePerDev];

// nullptr (and DXTB_OK) when the table is full: all launches then go to
// the caller's stream, one after the other.
static int32_t side_stream(cudaStream_t caller, SideStream **out) {
  *out = nullptr;
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return DXTB_ERR_LAUNCH;
  std::lock_guard<std::mutex> lock(g_side_mutex);
  SideStream *slot = nullptr;
  for (int i = 0; i < kSidePerDev; ++i) {
    SideStream &ss = g_side[dev][i];
    if (ss.used && ss.caller == caller) {
      *out = &ss;
      return DXTB_OK;
    }
    if (!ss.used && slot == nullptr) slot = &ss;
  }
  if (slot == nullptr) return DXTB_OK;
  // By default the larger classes run on the higher-priority streams: their
  // CTAs need whole SMs and bound a batch's makespan, so they are dispatched
  // first. A caller stream with a priority of its own (a serving loop that
  // ranks its lanes) passes it on to every class instead.
  int least = 0, greatest = 0, cprio = 0;
  if (cudaDeviceGetStreamPriorityRange(&least, &greatest) != cudaSuccess) return DXTB_ERR_LAUNCH;
  if (caller == nullptr || cudaStreamGetPriority(caller, &cprio) != cudaSuccess) {
    cudaGetLastError();
    cprio = least;
  }
  for (int c = 0; c < kClasses; ++c) {
    const int prio = cprio != least ? cprio : max(greatest, least - c);  // class 0: the lowest
    if (cudaStreamCreateWithPriority(&slot->s[c], cudaStreamNonBlocking, prio) != cudaSuccess)
      return DXTB_ERR_LAUNCH;
    slot->prio[c] = prio;
    if (cudaEventCreateWithFlags(&slot->join[c], cudaEventDisableTiming) != cudaSuccess) return DXTB_ERR_LAUNCH;
  }
  if (cudaEventCreateWithFlags(&slot->fork, cudaEventDisableTiming) != cudaSuccess) return DXTB_ERR_LAUNCH;
  slot->caller = caller;
  slot->used = true;
  *out = slot;
  return DXTB_OK;
}

// Largest usable cluster size of k_scf_cluster (cached per device). The
// occupancy query uses the largest dynamic shared memory any cluster launch
// asks for (kMaxDynSmem): a size placeable there is placeable at every
// smaller launch size, so no class launch is judged placeable at a smaller
// size than it uses.
static int cluster_cap() {
  static std::mutex mu;
  static int cap_dev[64] = {0};
  const size_t smem = kMaxDynSmem;
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 1;
  std::lock_guard<std::mutex> lock(mu);
  if (cap_dev[dev] != 0) return cap_dev[dev];
  if (cudaFuncSetAttribute(k_scf_cluster, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess ||
      cudaFuncSetAttribute(k_scf_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxDynSmem) !=
          cudaSuccess) {
    cudaGetLastError();
    return 1;
  }
  int cap = 1;
  for (int c = 2; c <= kMaxCluster; c *= 2) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(c);
    cfg.blockDim = dim3(kScfBigThreads);
    cfg.dynamicSmemBytes = smem;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = c;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int nclusters = 0;
    if (cudaOccupancyMaxActiveClusters(&nclusters, k_scf_cluster, &cfg) != cudaSuccess || nclusters < 1) {
      cudaGetLastError();
      break;
    }
    cap = c;
  }
  cap_dev[dev] = cap;
  return cap;
}

// Inputs of the gradient that the SCF arguments do not hold.
struct GradArgs {
  const double *cn, *mrad;
  double *dedcn, *grad;
};

// The gradient kernels of class c, on the stream of that class's SCF launch.
static int32_t class_gradient(const ScfArgs &a, const GradArgs *g, int c, cudaStream_t s) {
  if (g == nullptr) return DXTB_OK;
  ClassFilter f;
  for (int k = 0; k < kClasses; ++k) f.thr[k] = a.thr[k];
  f.cls = c;
  return launch_gradient(&a.b, a.pf, a.pi, g->cn, g->mrad, a.P, a.W, a.q, a.dp, a.qp, a.vorb, a.vdp,
                         a.vqp, a.S, a.D, g->dedcn, g->grad, f, s);
}

static int32_t launch_scf(ScfArgs a, int nmol, cudaStream_t st, const GradArgs *g = nullptr) {
  {
    std::lock_guard<std::mutex> lock(g_policy_mutex);
    for (int c = 0; c < kClasses; ++c) a.thr[c] = g_thr[c];
  }
  int sms = 0;
  if (device_sms(&sms) != DXTB_OK) return DXTB_ERR_LAUNCH;
  const int nmax = a.b.max_nao;
  const size_t smem = (size_t)nmax * (3 * sizeof(double) + 2 * sizeof(float));
  if (smem > kMaxDynSmem) return DXTB_ERR_TOO_LARGE;
  // clusters need the launch order; classes beyond the cluster cap fold down
  int top = a.order ? 5 : 1;
  if (top > 1 && scf_class(a.thr, nmax) >= 2) {
    const int cap = cluster_cap();
    int c = 1;
    while ((2 << (c - 1)) <= cap && c < 5) ++c;  // largest class whose cluster fits
    top = cap >= 2 ? c : 1;
  }
  for (int c = top + 1; c < kClasses; ++c) a.thr[c] = INT32_MAX;
  const int cmax = scf_class(a.thr, nmax);
  SideStream *ss = nullptr;
  int32_t rc = side_stream(st, &ss);
  if (rc != DXTB_OK) return rc;
  // every class waits for the same fork event on its own stream, so all
  // become ready together and the stream priorities order the dispatch (a
  // CTA of class >= 1 needs a whole SM: it must not queue behind the
  // two-per-SM CTAs that would otherwise spread over every SM first)
  if (ss) {
    if (cudaEventRecord(ss->fork, st) != cudaSuccess) return DXTB_ERR_LAUNCH;
    for (int c = 0; c <= cmax; ++c)
      if (cudaStreamWaitEvent(ss->s[c], ss->fork, 0) != cudaSuccess) return DXTB_ERR_LAUNCH;
  }
  static PerDeviceOnce attr;
  if (per_device_once(attr, [] {
        return cudaFuncSetAttribute(k_scf<kScfThreads, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    kMaxDynSmem) == cudaSuccess &&
               cudaFuncSetAttribute(k_scf<kScfBigThreads, 1>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    kMaxDynSmem) == cudaSuccess;
      }) != DXTB_OK)
    return DXTB_ERR_LAUNCH;
  // shared memory of class c: the base plus the rows of the Householder
  // reduction of its largest possible molecule (and, for clusters, one
  // broadcast row). When they do not all fit, the CTA takes the most shared
  // memory if that still holds 60 % of the rows; below that the rows stay in
  // L1/L2 (shared memory is carved out of L1; a carve-out holding a fifth to
  // a third of the rows gained nothing at n ~ 900-1000)
  auto class_smem = [&](int c) -> size_t {
    const int csize = c >= 2 ? 1 << (c - 1) : 1;
    const int nub = (c + 1 < kClasses && a.thr[c + 1] != INT32_MAX) ? min(nmax, a.thr[c + 1] - 1) : nmax;
    const int nown = (nub + csize - 1) / csize;
    const int rows = nown + (c >= 2 ? 1 : 0);
    const size_t full = smem + (size_t)rows * nub * sizeof(double);
    if (full <= (size_t)kMaxDynSmem) return full;
    const int64_t fit = ((int64_t)kMaxDynSmem / 8 - 4 * (int64_t)nub) / nub - (c >= 2 ? 1 : 0);
    return 10 * fit >= 6 * (int64_t)nown ? (size_t)kMaxDynSmem : smem;
  };
  // largest classes first: clusters, then one-SM CTAs, then the shared SMs
  for (int c = cmax; c >= 2; --c) {
    const int csize = 1 << (c - 1);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(min(nmol, max(1, sms / csize)) * csize);
    cfg.blockDim = dim3(kScfBigThreads);
    cfg.dynamicSmemBytes = class_smem(c);
    cfg.stream = ss ? ss->s[c] : st;
    cudaLaunchAttribute at[2];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = csize;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    // the class stream's priority, set on the launch as well so that a
    // captured graph keeps it as a node priority (dxtb_graph_end)
    at[1].id = cudaLaunchAttributePriority;
    at[1].val.priority = ss ? ss->prio[c] : 0;
    cfg.attrs = at;
    cfg.numAttrs = ss ? 2 : 1;
    if (cudaLaunchKernelEx(&cfg, k_scf_cluster, a, c) != cudaSuccess) return DXTB_ERR_LAUNCH;
    const int32_t rc = class_gradient(a, g, c, cfg.stream);
    if (rc != DXTB_OK) return rc;
  }
  // one-SM and shared-SM classes, likewise with their stream's priority
  auto launch_cta_class = [&](auto kernel, int c, int threads, size_t dyn) -> int32_t {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(nmol);
    cfg.blockDim = dim3(threads);
    cfg.dynamicSmemBytes = dyn;
    cfg.stream = ss ? ss->s[c] : st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributePriority;
    at[0].val.priority = ss ? ss->prio[c] : 0;
    cfg.attrs = at;
    cfg.numAttrs = ss ? 1 : 0;
    if (cudaLaunchKernelEx(&cfg, kernel, a, c) != cudaSuccess) return DXTB_ERR_LAUNCH;
    return class_gradient(a, g, c, cfg.stream);
  };
  if (cmax >= 1) {
    const int32_t rc = launch_cta_class(k_scf<kScfBigThreads, 1>, 1, kScfBigThreads, class_smem(1));
    if (rc != DXTB_OK) return rc;
  }
  const size_t smem0 = (size_t)min(nmax, a.thr[1]) * (3 * sizeof(double) + 2 * sizeof(float));
  {
    const int32_t rc = launch_cta_class(k_scf<kScfThreads, 2>, 0, kScfThreads, smem0);
    if (rc != DXTB_OK) return rc;
  }
  if (ss) {
    for (int c = 0; c <= cmax; ++c) {
      if (cudaEventRecord(ss->join[c], ss->s[c]) != cudaSuccess) return DXTB_ERR_LAUNCH;
      if (cudaStreamWaitEvent(st, ss->join[c], 0) != cudaSuccess) return DXTB_ERR_LAUNCH;
    }
  }
  return DXTB_OK;
}

}  // namespace dxtb

extern "C" int32_t dxtb_scf_get_size_classes(int32_t *min_n) {
  if (!min_n) return DXTB_ERR_ARGS;
  std::lock_guard<std::mutex> lock(g_policy_mutex);
  for (int c = 1; c < kClasses; ++c) min_n[c - 1] = g_thr[c];
  return DXTB_OK;
}

extern "C" int32_t dxtb_scf_set_size_classes(const int32_t *min_n) {
  if (!min_n) return DXTB_ERR_ARGS;
  for (int c = 1; c < kClasses; ++c)
    if (min_n[c - 1] < 1 || (c > 1 && min_n[c - 1] < min_n[c - 2])) return DXTB_ERR_ARGS;
  std::lock_guard<std::mutex> lock(g_policy_mutex);
  for (int c = 1; c < kClasses; ++c) g_thr[c] = min_n[c - 1];
  return DXTB_OK;
}

namespace dxtb {

// Checks a configuration and copies it into the kernel arguments.
static int32_t apply_config(const dxtb_scf_config *c, ScfArgs &a) {
  if (!c || c->maxiter <= 0 || !(c->x_atol > 0.0) || !(c->f_atol > 0.0) || !(c->damp > 0.0))
    return DXTB_ERR_ARGS;
  if (c->mixer != DXTB_MIXER_BROYDEN1 && c->mixer != DXTB_MIXER_ANDERSON) return DXTB_ERR_ARGS;
  if (c->mixer == DXTB_MIXER_ANDERSON &&
      (c->generations < 1 || c->generations > kMaxGen || !(c->x_atol_max > 0.0) || !(c->damp_init > 0.0) ||
       !(c->diagonal_offset >= 0.0)))
    return DXTB_ERR_ARGS;
  a.maxiter = c->maxiter;
  a.mixer = c->mixer;
  a.xtol = c->x_atol;
  a.ftol = c->f_atol;
  a.xtol_max = c->x_atol_max;
  a.damp = c->damp;
  a.damp_init = c->damp_init;
  a.generations = c->generations;
  a.soft_start = c->soft_start;
  a.offset = c->diagonal_offset;
  return DXTB_OK;
}

}  // namespace dxtb

extern "C" int32_t dxtb_scf(const dxtb_batch *b, const double *par_f, const int32_t *par_i,
                            const double *overlap, const double *h0, const double *dipole,
                            const double *quadrupole, const double *gamma, const double *hd,
                            const double *amat_sd, const double *amat_dd, const double *amat_sq,
                            const double *gb_mat, const double *n0, const double *nel, double kt,
                            const dxtb_scf_config *cfg, const int64_t *ws_off,
                            const int32_t *order, double *workspace, double *density,
                            double *wdensity, double *coeff, double *evals, double *occ, double *q,
                            double *dp, double *qp, double *vorb, double *vdp, double *vqp,
                            double *energies, int32_t *status, void *stream) {
  if (!b || b->nmol <= 0 || !overlap || !h0 || !gamma || !hd || !n0 || !nel || !ws_off ||
      !workspace || !density || !coeff || !evals || !occ || !q || !vorb || !energies || !status)
    return DXTB_ERR_ARGS;
  if (!(kt > 0.0)) return DXTB_ERR_ARGS;
  ScfArgs a;
  if (apply_config(cfg, a) != DXTB_OK) return DXTB_ERR_ARGS;
  a.b = *b;
  a.pf = par_f;
  a.pi = par_i;
  a.S = overlap;
  a.H0 = h0;
  a.D = dipole;
  a.Q = quadrupole;
  a.gamma = gamma;
  a.hd = hd;
  a.sd = amat_sd;
  a.dd = amat_dd;
  a.sq = amat_sq;
  a.gb = gb_mat;
  a.n0 = n0;
  a.nel = nel;
  a.kt = kt;
  a.ws_off = ws_off;
  a.order = order;
  a.ws = workspace;
  a.P = density;
  a.W = wdensity;
  a.C = coeff;
  a.evals = evals;
  a.occ = occ;
  a.q = q;
  a.dp = dp;
  a.qp = qp;
  a.vorb = vorb;
  a.vdp = vdp;
  a.vqp = vqp;
  a.energies = energies;
  a.status = status;
  return launch_scf(a, b->nmol, (cudaStream_t)stream);
}

extern "C" int32_t dxtb_scf_gradient(
    const dxtb_batch *b, const double *par_f, const int32_t *par_i, const double *overlap,
    const double *h0, const double *dipole, const double *quadrupole, const double *gamma,
    const double *hd, const double *amat_sd, const double *amat_dd, const double *amat_sq,
    const double *gb_mat, const double *n0, const double *nel, double kt, const dxtb_scf_config *cfg,
    const int64_t *ws_off, const int32_t *order, double *workspace, double *density,
    double *wdensity, double *coeff, double *evals, double *occ, double *q, double *dp, double *qp,
    double *vorb, double *vdp, double *vqp, double *energies, int32_t *status, const double *cn,
    const double *mrad, double *dedcn, double *grad, void *stream) {
  if (!b || b->nmol <= 0 || !overlap || !h0 || !gamma || !hd || !n0 || !nel || !ws_off ||
      !workspace || !density || !wdensity || !coeff || !evals || !occ || !q || !vorb || !energies ||
      !status || !cn || !dedcn || !grad)
    return DXTB_ERR_ARGS;
  if (!(kt > 0.0)) return DXTB_ERR_ARGS;
  if (dipole != nullptr && (!vdp || !vqp || !dp || !qp || !mrad)) return DXTB_ERR_ARGS;
  ScfArgs a;
  if (apply_config(cfg, a) != DXTB_OK) return DXTB_ERR_ARGS;
  a.b = *b;
  a.pf = par_f;
  a.pi = par_i;
  a.S = overlap;
  a.H0 = h0;
  a.D = dipole;
  a.Q = quadrupole;
  a.gamma = gamma;
  a.hd = hd;
  a.sd = amat_sd;
  a.dd = amat_dd;
  a.sq = amat_sq;
  a.gb = gb_mat;
  a.n0 = n0;
  a.nel = nel;
  a.kt = kt;
  a.ws_off = ws_off;
  a.order = order;
  a.ws = workspace;
  a.P = density;
  a.W = wdensity;
  a.C = coeff;
  a.evals = evals;
  a.occ = occ;
  a.q = q;
  a.dp = dp;
  a.qp = qp;
  a.vorb = vorb;
  a.vdp = vdp;
  a.vqp = vqp;
  a.energies = energies;
  a.status = status;
  GradArgs g{cn, mrad, dedcn, grad};
  return launch_scf(a, b->nmol, (cudaStream_t)stream, &g);
}

// ---------------------------------------------------------------------------
// SCF entry point for callers that cannot allocate device memory.
//
// Some callers must not call cudaMalloc: hosts that hand the library a fixed
// device-memory pool and forbid allocations outside it, or plugin hosts whose
// allocator is not reachable from the C ABI. dxtb_scf_noalloc serves them: it
// runs the same persistent SCF kernels as dxtb_scf, but its scratch workspace
// is a fixed array in the library's own device memory, so the caller passes
// only the inputs and the output buffers.
//
// The array holds DXTB_NOALLOC_SCRATCH_DOUBLES doubles (16 MiB) and every
// GPU that loads the library keeps it until the process exits. Batches whose
// workspace does not fit are rejected with DXTB_ERR_TOO_LARGE. The size is
// computed on the device from the batch's offset tables and read back once
// per call (one synchronisation of the caller's stream).
// ---------------------------------------------------------------------------
#include <mutex>

namespace dxtb {

static __device__ __align__(256) double g_scf_scratch[DXTB_NOALLOC_SCRATCH_DOUBLES];

// Header of the scratch array: [0] required doubles (int64), [1 .. nmol+1]
// per-molecule workspace offsets (int64, relative to the workspace start).
constexpr int64_t kNoallocHeader = 1;

__global__ void k_noalloc_layout(dxtb_batch b, int64_t *hdr, int64_t ws_start) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  int64_t off = 0;
  for (int m = 0; m < b.nmol; ++m) {
    hdr[kNoallocHeader + m] = off;
    const int64_t n = b.ao_off[m + 1] - b.ao_off[m];
    const int64_t nat = b.atom_off[m + 1] - b.atom_off[m];
    off += ws_size_mol(n, nat);
  }
  hdr[kNoallocHeader + b.nmol] = off;
  hdr[0] = ws_start + off;  // doubles needed from the start of the array
}

static std::mutex g_noalloc_mutex;
static double *g_noalloc_ptr[64] = {nullptr};

// Device address of the scratch array for the current device, looked up
// once per device (host code must not use the symbol itself as a pointer).
static int32_t noalloc_scratch(double **out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return DXTB_ERR_LAUNCH;
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (g_noalloc_ptr[dev] == nullptr) {
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_scf_scratch) != cudaSuccess || p == nullptr)
      return DXTB_ERR_LAUNCH;
    g_noalloc_ptr[dev] = static_cast<double *>(p);
  }
  *out = g_noalloc_ptr[dev];
  return DXTB_OK;
}

}  // namespace dxtb

extern "C" int32_t dxtb_scf_noalloc(
    const dxtb_batch *b, const double *par_f, const int32_t *par_i, const double *overlap,
    const double *h0, const double *dipole, const double *quadrupole, const double *gamma,
    const double *hd, const double *amat_sd, const double *amat_dd, const double *amat_sq,
    const double *gb_mat, const double *n0, const double *nel, double kt, int32_t maxiter,
    double tol, const int32_t *order, double *density, double *wdensity, double *coeff,
    double *evals, double *occ, double *q, double *dp, double *qp, double *vorb, double *vdp,
    double *vqp, double *energies, int32_t *status, void *stream) {
  if (!b || b->nmol <= 0) return DXTB_ERR_ARGS;
  // the header (nmol + 2 int64, rounded up to 32 words) precedes the workspace
  const int64_t ws_start = ((kNoallocHeader + b->nmol + 1) + 31) / 32 * 32;
  if (ws_start >= DXTB_NOALLOC_SCRATCH_DOUBLES) return DXTB_ERR_TOO_LARGE;
  double *scratch = nullptr;
  int32_t rc = noalloc_scratch(&scratch);
  if (rc != DXTB_OK) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  int64_t *hdr = reinterpret_cast<int64_t *>(scratch);
  k_noalloc_layout<<<1, 32, 0, st>>>(*b, hdr, ws_start);
  DXTB_CHECK_LAUNCH();
  int64_t need = 0;
  if (cudaMemcpyAsync(&need, hdr, sizeof(int64_t), cudaMemcpyDeviceToHost, st) != cudaSuccess)
    return DXTB_ERR_LAUNCH;
  if (cudaStreamSynchronize(st) != cudaSuccess) return DXTB_ERR_LAUNCH;
  if (need > DXTB_NOALLOC_SCRATCH_DOUBLES) return DXTB_ERR_TOO_LARGE;
  // the implicit-mode root solver with one tolerance for x_atol and f_atol
  dxtb_scf_config cfg = {};
  cfg.maxiter = maxiter;
  cfg.mixer = DXTB_MIXER_BROYDEN1;
  cfg.x_atol = tol;
  cfg.f_atol = tol;
  cfg.damp = 0.5;
  return dxtb_scf(b, par_f, par_i, overlap, h0, dipole, quadrupole, gamma, hd, amat_sd, amat_dd,
                  amat_sq, gb_mat, n0, nel, kt, &cfg, hdr + kNoallocHeader, order,
                  scratch + ws_start, density, wdensity, coeff, evals, occ, q, dp, qp, vorb, vdp,
                  vqp, energies, status, stream);
}
