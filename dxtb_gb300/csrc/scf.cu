// Persistent self-consistent-field kernel: one CTA per molecule runs the
// whole SCF of that molecule (orthogonaliser, Fock build, generalized
// eigensolve, Fermi occupations, density, Mulliken charges and atomic
// multipoles, potentials, limited-memory Broyden root solve) with a
// per-molecule convergence test and iteration cap. No host synchronisation inside the loop.
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
constexpr int kScfBigThreads = 512;  // CTA size for large molecules on their own SM
constexpr int kRank = 256;        // Broyden inverse-Jacobian memory (the reference keeps all updates; >= maxiter)
constexpr double kDamp = 0.5;     // step damping of the root solver (defaults.DAMP)
constexpr int kSmemTri = 1024;    // tridiagonal copy in shared memory up to this order
constexpr double kOccCut = 1e-15; // orbitals below this occupation carry no density

struct MolView {
  int m, n, nat, nsh, N;
  int64_t a0, s0, o0, moff, mtot, n2off, n2tot, g0;
};

// Per-molecule workspace layout (doubles).
__host__ __device__ inline int64_t ws_size_mol(int64_t n, int64_t nat) {
  const int64_t N = n + 9 * nat;
  return 3 * n * n + 10 * n + (2 * kRank + 7) * N + 64 + 16 * nat + 5 * n * kScfBigThreads + n + 8 +
         4 * kRank + 64;
}

struct Ws {
  double *Linv, *A, *Zt, *d, *e, *tau, *p, *rc, *rs, *eps, *fa, *fb, *x, *g, *hx, *hr, *misc;
  double *vsh_tmp, *lu, *sdot, *xold, *rold, *xbest;
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
  w.lu = q; q += (size_t)5 * n * kScfBigThreads;
  w.cl = reinterpret_cast<int *>(q); q += n + 8;
  w.sdot = q; q += 4 * kRank + 64;
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
  for (int it = 0; it < 200; ++it) {
    double s = 0.0, ds = 0.0;
    for (int j = lane; j < n; j += 32) {
      const double x = (eps[j] - mu) * ikt;
      const double v = x > 0.0 ? exp(-x) / (1.0 + exp(-x)) : 1.0 / (1.0 + exp(x));
      s += v;
      ds += v * (1.0 - v);
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
    const double x = (eps[j] - mu) / kt;
    const double v = x > 0.0 ? exp(-x) / (1.0 + exp(-x)) : 1.0 / (1.0 + exp(x));
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
  const int64_t *ws_off;
  const int32_t *order;
  double *ws, *P, *W, *C, *evals, *occ, *q, *dp, *qp, *vorb, *vdp, *vqp, *energies;
  int32_t *status;
};

// Potential x = (vorb [n], vdp [nat][3], vqp [nat][6]) from the orbital
// charges qo and atomic multipoles dpa/qpa (interactions/base.py:135-181).
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
    for (int k = 0; k < no; ++k) v += qo[o + k];
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
        for (int c = 0; c < 3; ++c) v += a.sd[c * mv.n2tot + o] * dpa[3 * j + c];
        for (int c = 0; c < 6; ++c) v += a.sq[c * mv.n2tot + o] * qpa[6 * j + c];
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
      for (int c = 0; c < 3; ++c) vd[c] = 2.0 * dk * dpa[3 * j + c];
      for (int c = 0; c < 6; ++c) vq[c] = 2.0 * qk * qpa[6 * j + c] * qscale[c];
      for (int i = 0; i < nat; ++i) {
        const int64_t o = mv.n2off + (int64_t)i * nat + j;
        for (int c = 0; c < 3; ++c) vd[c] += a.sd[c * mv.n2tot + o] * qat[i];
        for (int x = 0; x < 3; ++x)
          for (int y = 0; y < 3; ++y) vd[y] += a.dd[(3 * x + y) * mv.n2tot + o] * dpa[3 * i + x];
        for (int c = 0; c < 6; ++c) vq[c] += a.sq[c * mv.n2tot + o] * qat[i];
      }
      for (int c = 0; c < 3; ++c) xout[n + 3 * j + c] = vd[c];
      for (int c = 0; c < 6; ++c) xout[n + 3 * nat + 6 * j + c] = vq[c];
    }
  }
  __syncthreads();
}

// Interaction energy (interactions/base.py:306-360 summed): block result.
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
            vd[y] += 0.5 * a.dd[(3 * x + y) * mv.n2tot + o] * dpa[3 * i + x];
        for (int c = 0; c < 6; ++c) vq[c] += a.sq[c * mv.n2tot + o] * qat[i];
      }
      for (int c = 0; c < 3; ++c) e += (dk * dpa[3 * j + c] + vd[c]) * dpa[3 * j + c];
      for (int c = 0; c < 6; ++c) e += (qk * qscale[c] * qpa[6 * j + c] + vq[c]) * qpa[6 * j + c];
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

// Molecules of at least kBigN orbitals among the first `nbig_max` of the
// launch order run in a 512-thread CTA with an SM of their own; the others
// share SMs two at a time in 256-thread CTAs. The two launches run
// concurrently; every CTA checks which one its molecule belongs to.
constexpr int kBigN = 128;

__device__ __forceinline__ bool scf_is_big(const ScfArgs &a, int i, int nbig_max) {
  const int m = a.order ? a.order[i] : i;
  return i < nbig_max && (a.b.ao_off[m + 1] - a.b.ao_off[m]) >= kBigN;
}

__device__ __forceinline__ void scf_body(const ScfArgs &a, int m);

template <int NT, int MINB>
__global__ void __launch_bounds__(NT, MINB) k_scf(ScfArgs a, int big, int nbig_max) {
  const int i = blockIdx.x;
  if (scf_is_big(a, i, nbig_max) != (big != 0)) return;
  scf_body(a, a.order ? a.order[i] : i);
}

__device__ __forceinline__ void scf_body(const ScfArgs &a, int m_) {
  __shared__ double red[32];
  __shared__ int s_flag, s_m, s_ncl;
  __shared__ double s_tri[2 * kSmemTri];
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
  double *qsh = w.misc, *qat = qsh + mv.nsh + 1, *vat = qat + nat + 1;
  double *dpa = vat + nat + 1, *qpa = dpa + 3 * nat + 1, *qo = qpa + 6 * nat + 1;
  double *vsh = w.vsh_tmp;

  const double *S = a.S + mv.moff, *H0 = a.H0 + mv.moff;
  double *P = a.P + mv.moff, *C = a.C + mv.moff;
  const double *n0 = a.n0 + mv.o0;
  const double nel_a = a.nel[2 * m], nel_b = a.nel[2 * m + 1];
  int status = DXTB_OK;

  // ---- orthogonaliser X = L^-1 (S = L L^T), once per geometry ----
  for (int64_t t = threadIdx.x; t < (int64_t)n * n; t += blockDim.x) w.A[t] = S[t];
  __syncthreads();
  if (!cta_cholesky(n, w.A)) status = DXTB_ERR_NOT_POSDEF;
  if (status == DXTB_OK) cta_trinv(n, w.A, w.Linv);

  for (int t = threadIdx.x; t < N; t += blockDim.x) w.x[t] = 0.0;
  __syncthreads();

  int it = 0, nrank = 0, final_eval = 0, hit_max = 0;
  double resid = 0.0, best_ynorm = 1e308, dx_norm = 0.0;
  while (status == DXTB_OK) {
    ++it;
    // ---- Fock matrix F(x) into Zt (conversions.py:255-297) ----
    for (int64_t t = threadIdx.x; t < (int64_t)n * n; t += blockDim.x) {
      const int i = (int)(t / n), j = (int)(t % n);
      double f = H0[t] - 0.5 * S[t] * (w.x[i] + w.x[j]);
      if (multipole) {
        const int ai = b.shell_atom[mv.s0 + b.ao_shell[mv.o0 + i]];
        const int aj = b.shell_atom[mv.s0 + b.ao_shell[mv.o0 + j]];
        const int64_t e1 = mv.moff + t, e2 = mv.moff + (int64_t)j * n + i;
        double acc = 0.0;
        for (int c = 0; c < 3; ++c)
          acc += a.D[c * mv.mtot + e1] * w.x[n + 3 * aj + c] + a.D[c * mv.mtot + e2] * w.x[n + 3 * ai + c];
        for (int c = 0; c < 6; ++c)
          acc += a.Q[c * mv.mtot + e1] * w.x[n + 3 * nat + 6 * aj + c] +
                 a.Q[c * mv.mtot + e2] * w.x[n + 3 * nat + 6 * ai + c];
        f -= 0.5 * acc;
      }
      w.Zt[t] = f;
    }
    __syncthreads();
    // ---- F' = X F X^T (exlibs/xitorch/_impls/linalg/symeig.py:57-61) ----
    // X = L^-1 is lower triangular: A = X F needs k <= i; only the lower
    // triangle of (X F) X^T is formed (k <= j), then mirrored.
    cta_gemm<false, false>(n, n, n, 1.0, w.Linv, n, w.Zt, n, 0.0, w.A, n, kALower);
    cta_gemm<false, true>(n, n, n, 1.0, w.A, n, w.Linv, n, 0.0, w.Zt, n, kBLowerT, true);
    for (int64_t t = threadIdx.x; t < (int64_t)n * n; t += blockDim.x) {
      const int i = (int)(t / n), j = (int)(t % n);
      w.A[t] = j <= i ? w.Zt[t] : w.Zt[(size_t)j * n + i];
    }
    __syncthreads();
    // ---- eigenvalues: Householder tridiagonalisation + implicit QL ----
    cta_tridiag(n, w.A, w.d, w.e, w.tau, w.p, w.rs, red);
    {
      float *df = n <= 2 * kSmemTri ? reinterpret_cast<float *>(s_tri) : reinterpret_cast<float *>(w.rs);
      float *e2f = n <= 2 * kSmemTri ? reinterpret_cast<float *>(s_tri) + 2 * kSmemTri
                                     : reinterpret_cast<float *>(w.vsh_tmp);
      cta_tri_eigenvalues(n, w.d, w.e, w.rc, df, e2f);
    }
    cta_rank_sort(n, w.rc, w.eps);  // ascending, like eigh
    // ---- Fermi occupations (filling.py:428-742), both spin channels ----
    if (threadIdx.x < 32) {
      bool ok = fermi_warp(n, w.eps, nel_a, a.kt, w.fa);
      if (nel_b == nel_a) {
        for (int j = threadIdx.x; j < n; j += 32) w.fb[j] = w.fa[j];
      } else {
        ok = ok && fermi_warp(n, w.eps, nel_b, a.kt, w.fb);
      }
      __syncwarp();
      if (threadIdx.x == 0) {
        s_flag = ok ? 1 : 0;
        // orbitals with non-vanishing occupation (occupations decrease with j)
        int mv_ = 0;
        while (mv_ < n && w.fa[mv_] + w.fb[mv_] > kOccCut) ++mv_;
        s_m = mv_ > 0 ? mv_ : 1;
      }
    }
    __syncthreads();
    if (!s_flag) {
      status = DXTB_ERR_FERMI;
      break;
    }
    // ---- eigenvectors of the m lowest orbitals only ----
    double tnorm = 0.0;
    for (int j = threadIdx.x; j < n; j += blockDim.x) tnorm = fmax(tnorm, fabs(w.d[j]) + 2.0 * fabs(w.e[j]));
    tnorm = block_max(tnorm, red);
    if (threadIdx.x == 0) {
      // keep a whole eigenvalue cluster together
      int mm = s_m;
      const double ctol = 1e-6 * fmax(tnorm, 1.0);
      while (mm < n && w.eps[mm] - w.eps[mm - 1] <= ctol) ++mm;
      s_m = mm;
    }
    __syncthreads();
    const int mo = s_m;
    cta_tri_vectors(n, w.d, w.e, w.eps, mo, tnorm, w.Zt, w.lu, w.cl, &s_ncl);
    cta_back_transform(n, w.A, w.tau, w.Zt, mo, w.p);
    // ---- C^T = Y^T X (orbital j is row j; X lower -> k >= i) ----
    cta_gemm<true, false>(mo, n, n, 1.0, w.Zt, mo, w.Linv, n, 0.0, C, n, kBUpper);
    for (int j = threadIdx.x; j < n; j += blockDim.x) w.p[j] = w.fa[j] + w.fb[j];
    __syncthreads();
    // ---- density P = C diag(occ) C^T (scf/utils.py:29-52) ----
    for (int64_t t = threadIdx.x; t < (int64_t)mo * n; t += blockDim.x) w.A[t] = C[t] * w.p[t / n];
    __syncthreads();
    cta_gemm<true, false>(n, n, mo, 1.0, C, n, w.A, n, 0.0, P, n, kFull, true);
    cta_mirror_lower(n, P);
    // ---- Mulliken charges and atomic multipoles (conversions.py:203-251) ----
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      double pop = 0.0;
      for (int k = 0; k < n; ++k) pop = fma(P[(size_t)k * n + i], S[(size_t)k * n + i], pop);
      qo[i] = n0[i] - pop;
    }
    if (multipole) {
      for (int t = threadIdx.x; t < 3 * nat; t += blockDim.x) dpa[t] = 0.0;
      for (int t = threadIdx.x; t < 6 * nat; t += blockDim.x) qpa[t] = 0.0;
      __syncthreads();
      // -sum_k P_ik M[c][k][i] per orbital i, reduced onto the atom of i
      for (int i = threadIdx.x; i < n; i += blockDim.x) {
        double acc[9];
        for (int c = 0; c < 9; ++c) acc[c] = 0.0;
        for (int k = 0; k < n; ++k) {
          const double pk = P[(size_t)k * n + i];
          const int64_t e = mv.moff + (int64_t)k * n + i;
          for (int c = 0; c < 3; ++c) acc[c] -= pk * a.D[c * mv.mtot + e];
          for (int c = 0; c < 6; ++c) acc[3 + c] -= pk * a.Q[c * mv.mtot + e];
        }
        const int ai = b.shell_atom[mv.s0 + b.ao_shell[mv.o0 + i]];
        for (int c = 0; c < 3; ++c) atomicAdd(&dpa[3 * ai + c], acc[c]);
        for (int c = 0; c < 6; ++c) atomicAdd(&qpa[6 * ai + c], acc[3 + c]);
      }
    }
    __syncthreads();
    // ---- new potential G(x) ----
    potential_from_charges(a, mv, qo, dpa, qpa, qsh, qat, vsh, vat, w.g, multipole, es3_shell);
    if (final_eval) {
      hit_max = 1;
      break;
    }
    // ---- root solver on F(x) = x - G(x): limited-memory Broyden's first
    // method on the inverse Jacobian, Gm = 0.5 I + sum_k c_k d_k^T, damped
    // steps x += damp * dx, dx = -Gm F (the broyden1 of exlibs/xitorch/
    // _impls/optimize/root/{rootsolver.py:42-265, _jacobian.py:51-120} with
    // alpha = -0.5, damp = 0.5, line_search = False, scf/base.py:267-292);
    // stop when |dx|_2 < x_tol and |F|_2 < f_tol. ----
    {
      double *sdot = w.sdot;                     // [kRank] dot products
      double *sdot2 = sdot + kRank;              // [kRank]
      const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
      const int nw = (int)(blockDim.x >> 5);
      // |F|^2 with F = x - G(x)
      double part = 0.0;
      for (int t = threadIdx.x; t < N; t += blockDim.x) {
        const double y = w.x[t] - w.g[t];
        part += y * y;
      }
      const double ynorm = sqrt(block_sum(part, red));
      resid = ynorm;
      if (it == 1) {
        if (ynorm <= a.ftol * kEps) break;
        nrank = 0;
      } else {
        if (ynorm < best_ynorm) {
          best_ynorm = ynorm;
          for (int t = threadIdx.x; t < N; t += blockDim.x) w.xbest[t] = w.x[t];
        }
        // Broyden update with dx = x - x_prev, dy = F - F_prev:
        // v = Gm^T dx, c = dx - Gm dy, d = v / (dy . v)
        if (nrank >= kRank) nrank = 0;  // "restart" reduction of a full memory
        for (int k = wid; k < 2 * nrank; k += nw) {
          const int kk = k >> 1;
          double s = 0.0;
          if ((k & 1) == 0) {
            const double *ck = w.hx + (size_t)kk * N;
            for (int t = lane; t < N; t += 32) s += ck[t] * (w.x[t] - w.xold[t]);
          } else {
            const double *dk = w.hr + (size_t)kk * N;
            for (int t = lane; t < N; t += 32) s += dk[t] * ((w.x[t] - w.g[t]) - w.rold[t]);
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
          const double dxt = w.x[t] - w.xold[t];
          const double dyt = (w.x[t] - w.g[t]) - w.rold[t];
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
          break;
        }
        const double idyv = 1.0 / dyv;
        for (int t = threadIdx.x; t < N; t += blockDim.x) dn[t] *= idyv;
        ++nrank;
        __syncthreads();
        if (dx_norm < a.xtol && ynorm < a.ftol) break;  // converged at x
      }
      if (it >= a.maxiter) {
        // not converged: evaluate once more at the best iterate, which the
        // root solver returns with a warning (rootsolver.py:250-259)
        if (best_ynorm < ynorm) {
          for (int t = threadIdx.x; t < N; t += blockDim.x) w.x[t] = w.xbest[t];
          final_eval = 1;
          __syncthreads();
          continue;
        }
        hit_max = 1;
        break;
      }
      // F_prev = F, x_prev = x; dx = -Gm F = -(0.5 F + sum_k c_k (d_k . F))
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
        w.x[t] += kDamp * dx;
        pdx += dx * dx;
      }
      dx_norm = sqrt(block_sum(pdx, red));
      if (dx_norm == 0.0) {
        status = DXTB_ERR_NAN;
        break;
      }
    }
    __syncthreads();
  }
  if (hit_max && status == DXTB_OK) status = DXTB_ERR_MAXITER;

  // ---- outputs ----
  if (status == DXTB_OK || status == DXTB_ERR_MAXITER) {
    // energies (scf/base.py:510-619): E_h0 + E_int and -TS
    double part = 0.0;
    for (int64_t t = threadIdx.x; t < (int64_t)n * n; t += blockDim.x) part += P[t] * H0[t];
    const double eh0 = block_sum(part, red);
    const double eint = interaction_energy(a, mv, qsh, qat, dpa, qpa, multipole, es3_shell, red);
    double ts = 0.0;
    for (int j = threadIdx.x; j < n; j += blockDim.x) ts += ent(w.fa[j]) + ent(w.fb[j]);
    ts = a.kt * block_sum(ts, red);
    if (threadIdx.x == 0) {
      a.energies[4 * m + 0] = eh0 + eint;
      a.energies[4 * m + 1] = ts;
      a.energies[4 * m + 2] = (double)it;
      a.energies[4 * m + 3] = resid;
      if (!isfinite(eh0 + eint + ts)) status = DXTB_ERR_NAN;
    }
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
      a.evals[mv.o0 + j] = w.eps[j];
      a.occ[mv.o0 + j] = w.fa[j] + w.fb[j];
      a.q[mv.o0 + j] = qo[j];
    }
    // potentials of the final charges (for the gradient)
    for (int t = threadIdx.x; t < n; t += blockDim.x) a.vorb[mv.o0 + t] = w.g[t];
    if (multipole) {
      for (int t = threadIdx.x; t < 3 * nat; t += blockDim.x) {
        a.vdp[3 * mv.a0 + t] = w.g[n + t];
        a.dp[3 * mv.a0 + t] = dpa[t];
      }
      for (int t = threadIdx.x; t < 6 * nat; t += blockDim.x) {
        a.vqp[6 * mv.a0 + t] = w.g[n + 3 * nat + t];
        a.qp[6 * mv.a0 + t] = qpa[t];
      }
    }
    // energy-weighted density W = C diag(occ eps) C^T over the m orbitals
    const int mo = s_m;
    if (a.W != nullptr) {
      for (int64_t t = threadIdx.x; t < (int64_t)mo * n; t += blockDim.x)
        w.A[t] = C[t] * (w.fa[t / n] + w.fb[t / n]) * w.eps[t / n];
      __syncthreads();
      cta_gemm<true, false>(n, n, mo, 1.0, C, n, w.A, n, 0.0, a.W + mv.moff, n, kFull, true);
      cta_mirror_lower(n, a.W + mv.moff);
    }
    // coefficients of orbitals without occupation are not computed
    for (int64_t t = (int64_t)mo * n + threadIdx.x; t < (int64_t)n * n; t += blockDim.x) C[t] = 0.0;
  }
  if (threadIdx.x == 0) a.status[m] = status;
}

}  // namespace dxtb

using namespace dxtb;

extern "C" int64_t dxtb_scf_workspace_mol(int64_t n, int64_t nat) { return ws_size_mol(n, nat); }

#include <mutex>

namespace dxtb {

// Side stream and fork/join events per (device, caller stream), created once
// (no device memory is allocated); both launches stay inside a caller's
// stream capture. Callers on different streams (the serving loop's slots)
// get different side streams, so their large-molecule kernels overlap.
struct SideStream {
  cudaStream_t caller = nullptr;
  cudaStream_t s = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
  bool used = false;
};
constexpr int kSidePerDev = 32;
static std::mutex g_side_mutex;
static SideStream g_side[64][kSidePerDev];

// nullptr (and DXTB_OK) when the table is full: both launches then go to
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
  if (cudaStreamCreateWithFlags(&slot->s, cudaStreamNonBlocking) != cudaSuccess) return DXTB_ERR_LAUNCH;
  if (cudaEventCreateWithFlags(&slot->fork, cudaEventDisableTiming) != cudaSuccess) return DXTB_ERR_LAUNCH;
  if (cudaEventCreateWithFlags(&slot->join, cudaEventDisableTiming) != cudaSuccess) return DXTB_ERR_LAUNCH;
  slot->caller = caller;
  slot->used = true;
  *out = slot;
  return DXTB_OK;
}

static int32_t launch_scf(const ScfArgs &a, int nmol, cudaStream_t st) {
  SideStream *ss = nullptr;
  int32_t rc = side_stream(st, &ss);
  if (rc != DXTB_OK) return rc;
  int sms = 0;
  if (device_sms(&sms) != DXTB_OK) return DXTB_ERR_LAUNCH;
  const int nbig_max = min(nmol, sms / 2);
  // big molecules on the side stream, the rest on the caller's stream
  cudaStream_t sb = ss ? ss->s : st;
  if (ss) {
    if (cudaEventRecord(ss->fork, st) != cudaSuccess) return DXTB_ERR_LAUNCH;
    if (cudaStreamWaitEvent(ss->s, ss->fork, 0) != cudaSuccess) return DXTB_ERR_LAUNCH;
  }
  if (nbig_max > 0) k_scf<kScfBigThreads, 1><<<nbig_max, kScfBigThreads, 0, sb>>>(a, 1, nbig_max);
  DXTB_CHECK_LAUNCH();
  k_scf<kScfThreads, 2><<<nmol, kScfThreads, 0, st>>>(a, 0, nbig_max);
  DXTB_CHECK_LAUNCH();
  if (ss) {
    if (cudaEventRecord(ss->join, ss->s) != cudaSuccess) return DXTB_ERR_LAUNCH;
    if (cudaStreamWaitEvent(st, ss->join, 0) != cudaSuccess) return DXTB_ERR_LAUNCH;
  }
  return DXTB_OK;
}

}  // namespace dxtb

extern "C" int32_t dxtb_scf(const dxtb_batch *b, const double *par_f, const int32_t *par_i,
                            const double *overlap, const double *h0, const double *dipole,
                            const double *quadrupole, const double *gamma, const double *hd,
                            const double *amat_sd, const double *amat_dd, const double *amat_sq,
                            const double *gb_mat, const double *n0, const double *nel, double kt,
                            int32_t maxiter, double tol, const int64_t *ws_off,
                            const int32_t *order, double *workspace, double *density,
                            double *wdensity, double *coeff, double *evals, double *occ, double *q,
                            double *dp, double *qp, double *vorb, double *vdp, double *vqp,
                            double *energies, int32_t *status, void *stream) {
  if (!b || b->nmol <= 0 || !overlap || !h0 || !gamma || !hd || !n0 || !nel || !ws_off ||
      !workspace || !density || !coeff || !evals || !occ || !q || !vorb || !energies || !status)
    return DXTB_ERR_ARGS;
  if (maxiter <= 0 || !(kt > 0.0)) return DXTB_ERR_ARGS;
  ScfArgs a;
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
  a.xtol = tol;  // x_atol and f_atol of the reference: one tolerance here
  a.ftol = tol;
  a.maxiter = maxiter;
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

// ---------------------------------------------------------------------------
// SCF entry point for callers that cannot allocate device memory.
//
// Some callers cannot call cudaMalloc at all: code that runs while a CUDA
// graph is being captured by someone else, hosts that hand the library a
// fixed memory pool and forbid further device allocations, or plugin hosts
// whose allocator is not reachable from the C ABI. dxtb_scf_noalloc serves
// them: it runs the same persistent SCF kernel as dxtb_scf, but its scratch
// workspace is a fixed array in the library's own device memory, so the
// caller passes only the inputs and the output buffers.
//
// The array holds DXTB_NOALLOC_SCRATCH_DOUBLES doubles (16 MiB) and every
// GPU that loads the library keeps it until the process exits. Batches whose
// workspace does not fit are rejected with DXTB_ERR_TOO_LARGE.
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
  // header (nmol + 2 int64) must fit before the workspace
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
  return dxtb_scf(b, par_f, par_i, overlap, h0, dipole, quadrupole, gamma, hd, amat_sd, amat_dd,
                  amat_sq, gb_mat, n0, nel, kt, maxiter, tol, hdr + kNoallocHeader, order,
                  scratch + ws_start, density, wdensity, coeff, evals, occ, q, dp, qp, vorb, vdp,
                  vqp, energies, status, stream);
}
