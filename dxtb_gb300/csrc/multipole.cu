// Multipole integrals (overlap, dipole, quadrupole) over contracted
// Gaussian shells with the McMurchie-Davidson scheme, fused with the GFN1/
// GFN2 core Hamiltonian.
//
// One warp per shell pair (bra shell i >= ket shell j of one molecule).
// Phase 1: every lane takes one primitive pair, builds its Hermite
//   expansion coefficients E^{ab}_t for the three axes and contracts them
//   with the Hermite moments of (x - C)^e, e <= 2, into 1D tables
//   T[axis][a][b][e]; the tables are staged in shared memory.
// Phase 2: lanes own Cartesian outputs (component pair x multipole order)
//   and sum the staged tables over the primitive pairs of the chunk.
// Phase 3: Cartesian -> spherical transform in shared memory.
// Epilogue: normalised overlap, core Hamiltonian (xtb/base.py:255-372),
//   ket-centred dipole and traceless quadrupole for block (i, j) and the
//   bra-centred ones of the mirrored block (j, i).
//
// Reference: integral/driver/pytorch/impls/pairs.py:228-399 (pair loop,
// mirror), impls/pipeline.py:82-235 (primitive pairs, 3D assembly),
// impls/kernels/md.py (Hermite form), integral/container.py:182-537 and
// integral/types/{dipole,quadrupole}.py (shift, 9->6, traceless).
#include "common.cuh"

namespace dxtb {

constexpr int kWarps = 4;          // warps per CTA
constexpr int kTab = 81;           // 3 axes x 3 x 3 x 3 (a, b, e)
constexpr int kMaxCart = 6;
constexpr int kNComp = 10;         // S, Dx, Dy, Dz, Qxx, Qxy, Qxz, Qyy, Qyz, Qzz

__constant__ int c_cart[3][6][3] = {
    {{0, 0, 0}},
    {{0, 1, 0}, {0, 0, 1}, {1, 0, 0}},  // p in (y, z, x) order
    {{2, 0, 0}, {1, 1, 0}, {1, 0, 1}, {0, 2, 0}, {0, 1, 1}, {0, 0, 2}},
};
__constant__ int c_comp[kNComp][3] = {
    {0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {2, 0, 0},
    {1, 1, 0}, {1, 0, 1}, {0, 2, 0}, {0, 1, 1}, {0, 0, 2},
};

// Cartesian -> spherical rows (m = -l..l) for l <= 2, same convention as
// the reference's trafo.py (CCA order; p is the identity on (y, z, x)).
__device__ __forceinline__ double trafo(int l, int m, int c) {
  if (l < 2) return m == c ? 1.0 : 0.0;
  const double s3 = 1.7320508075688772935274463415058723669;
  switch (m) {
    case 0: return c == 1 ? s3 : 0.0;
    case 1: return c == 4 ? s3 : 0.0;
    case 2: return c == 0 ? -0.5 : (c == 3 ? -0.5 : (c == 5 ? 1.0 : 0.0));
    case 3: return c == 2 ? s3 : 0.0;
    default: return c == 0 ? 0.5 * s3 : (c == 3 ? -0.5 * s3 : 0.0);
  }
}

struct PairGeom {
  int m, i, j;
  int64_t gi, gj, a0;
  int ti, tj, ai, aj, la, lb, na, nb;
  double A[3], B[3];
};

__device__ __forceinline__ void pair_from_index(const dxtb_batch &b, int64_t k, PairGeom &g) {
  g.m = find_mol(b.pair_off, b.nmol, k);
  const int64_t t = k - b.pair_off[g.m];
  // float32 seed with integer corrections (a float64 square root costs a
  // warp ~700 cycles on this part)
  int i = (int)((sqrtf(8.0f * (float)t + 1.0f) - 1.0f) * 0.5f);
  while ((int64_t)(i + 1) * (i + 2) / 2 <= t) ++i;
  while ((int64_t)i * (i + 1) / 2 > t) --i;
  g.i = i;
  g.j = (int)(t - (int64_t)i * (i + 1) / 2);
  const int64_t s0 = b.shell_off[g.m];
  g.a0 = b.atom_off[g.m];
  g.gi = s0 + g.i;
  g.gj = s0 + g.j;
  g.ti = b.shell_type[g.gi];
  g.tj = b.shell_type[g.gj];
  g.ai = b.shell_atom[g.gi];
  g.aj = b.shell_atom[g.gj];
#pragma unroll
  for (int x = 0; x < 3; ++x) {
    g.A[x] = b.positions[3 * (g.a0 + g.ai) + x];
    g.B[x] = b.positions[3 * (g.a0 + g.aj) + x];
  }
}

// 1D tables of one primitive pair for one axis: T[a][b][e] = sum_t
// E^{ab}_t M^e_t with the Hermite moments about xc (unitless: the
// sqrt(pi/p) factors are in the 3D prefactor).
__device__ __forceinline__ void md_table_1d(int la, int lb, int emax, double xpa,
                                            double xpb, double xpc, double x2p,
                                            double *out /* [3][3][3] */) {
  double E[3][3][5];
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int t = 0; t < 5; ++t) E[a][c][t] = 0.0;
  E[0][0][0] = 1.0;
  for (int a = 0; a < la; ++a)
    for (int t = 0; t <= a + 1; ++t) {
      double v = xpa * E[a][0][t];
      if (t > 0) v += x2p * E[a][0][t - 1];
      if (t + 1 <= a) v += (t + 1) * E[a][0][t + 1];
      E[a + 1][0][t] = v;
    }
  for (int a = 0; a <= la; ++a)
    for (int c = 0; c < lb; ++c)
      for (int t = 0; t <= a + c + 1; ++t) {
        double v = xpb * E[a][c][t];
        if (t > 0) v += x2p * E[a][c][t - 1];
        if (t + 1 <= a + c) v += (t + 1) * E[a][c][t + 1];
        E[a][c + 1][t] = v;
      }
  // Hermite moments M^e_t about xc, e <= 2
  const double m10 = xpc, m20 = xpc * xpc + x2p, m21 = 2.0 * xpc;
  for (int a = 0; a <= la; ++a)
    for (int c = 0; c <= lb; ++c) {
      const double *e = E[a][c];
      out[(a * 3 + c) * 3 + 0] = e[0];
      if (emax >= 1) out[(a * 3 + c) * 3 + 1] = m10 * e[0] + e[1];
      if (emax >= 2) out[(a * 3 + c) * 3 + 2] = m20 * e[0] + m21 * e[1] + 2.0 * e[2];
    }
}

// Core-Hamiltonian factor of a shell pair, H0 = hfac * S (xtb/base.py:
// 255-372): mean CN-shifted self-energy, times for pairs of two atoms the
// distance polynomial, the shell scaling (with the GFN2 Slater-exponent
// factor), the pair scaling and the electronegativity term.
__device__ __forceinline__ double h0_factor(const dxtb_batch &b, const double *__restrict__ pf_,
                                            const int32_t *__restrict__ pi_tab,
                                            const double *__restrict__ cn, const PairGeom &g,
                                            double r2) {
  const int la = g.la, lb = g.lb;
  const int zi = b.numbers[g.a0 + g.ai], zj = b.numbers[g.a0 + g.aj];
  const double sei = pf(pf_, DXTB_P_LEVEL + g.ti) - pf(pf_, DXTB_P_KCN + g.ti) * cn[g.a0 + g.ai];
  const double sej = pf(pf_, DXTB_P_LEVEL + g.tj) - pf(pf_, DXTB_P_KCN + g.tj) * cn[g.a0 + g.aj];
  double hfac = 0.5 * (sei + sej);
  if (g.ai != g.aj) {
    const double dist = sqrt(r2);
    const double rr = sqrt(dist / (pf(pf_, DXTB_P_RAD + zi) + pf(pf_, DXTB_P_RAD + zj)));
    const double pi = (1.0 + pf(pf_, DXTB_P_SHPOLY + g.ti) * rr) *
                      (1.0 + pf(pf_, DXTB_P_SHPOLY + g.tj) * rr);
    const int vi = pi_(pi_tab, DXTB_I_VALENCE + g.ti), vj = pi_(pi_tab, DXTB_I_VALENCE + g.tj);
    const double kpol = pf(pf_, DXTB_P_SCAL + DXTB_S_KPOL);
    const double wexp = pf(pf_, DXTB_P_SCAL + DXTB_S_WEXP);
    const double zeta_i = pf(pf_, DXTB_P_SLATER + g.ti), zeta_j = pf(pf_, DXTB_P_SLATER + g.tj);
    const double zfac = wexp == 0.0 ? 1.0 : pow(2.0 * sqrt(zeta_i * zeta_j) / (zeta_i + zeta_j), wexp);
    double kk;
    if (vi && vj) {
      const double en_i = pf(pf_, DXTB_P_EN + zi), en_j = pf(pf_, DXTB_P_EN + zj);
      const double den = en_i - en_j;
      kk = pf(pf_, DXTB_P_KSHELL + la * 5 + lb) * zfac * pf(pf_, DXTB_P_KPAIR + zi * DXTB_MAXZ + zj) *
           (1.0 + pf(pf_, DXTB_P_SCAL + DXTB_S_ENSCALE) * den * den);
    } else {
      const double kii = vi ? pf(pf_, DXTB_P_KSHELL + la * 6) : kpol;
      const double kjj = vj ? pf(pf_, DXTB_P_KSHELL + lb * 6) : kpol;
      kk = 0.5 * (kii + kjj) * zfac;
    }
    hfac *= pi * kk;
  }
  return hfac;
}

// Writes element (mu, nu) = e1 of a shell pair and its mirror (nu, mu) = e2
// from the spherical multipoles v[comp] about the ket centre B (MODE 0) or
// the origin (MODE 1). MODE 0: S, H0 = hfac S, the ket-centred dipole and
// traceless quadrupole at e1 and the bra-centred ones (about A, from the
// exact shift with d = B - A) at e2 (integral/types/dipole.py shift_r0_rj,
// quadrupole.py:41-235). MODE 1: normalised raw moments, quadrupole as 9
// row-major components.
template <int MODE>
__device__ __forceinline__ void write_element(const double *v, int ncomp, int64_t e1, int64_t e2,
                                              int64_t mtot, const double *d, double hfac,
                                              double *__restrict__ S, double *__restrict__ H,
                                              double *__restrict__ D, double *__restrict__ Q) {
  const double s = v[0];
  S[e1] = s;
  S[e2] = s;
  if (MODE == 0 && H != nullptr) {
    H[e1] = hfac * s;
    H[e2] = hfac * s;
  }
  if (ncomp > 1) {
    if (MODE == 0) {
      double dB[3] = {v[1], v[2], v[3]};
      double qB[6] = {v[4], v[5], v[7], v[6], v[8], v[9]};  // xx xy yy xz yz zz
      double dA[3], qA[6];
#pragma unroll
      for (int x = 0; x < 3; ++x) dA[x] = dB[x] + d[x] * s;
      const int qa[6] = {0, 0, 1, 0, 1, 2}, qb[6] = {0, 1, 1, 2, 2, 2};
#pragma unroll
      for (int c = 0; c < 6; ++c) {
        const int x = qa[c], y = qb[c];
        qA[c] = qB[c] + d[y] * dB[x] + d[x] * dB[y] + d[x] * d[y] * s;
      }
#pragma unroll
      for (int x = 0; x < 3; ++x) {
        D[x * mtot + e1] = dB[x];
        D[x * mtot + e2] = dA[x];
      }
      const double trB = 0.5 * (qB[0] + qB[2] + qB[5]);
      const double trA = 0.5 * (qA[0] + qA[2] + qA[5]);
#pragma unroll
      for (int c = 0; c < 6; ++c) {
        const bool diag = (c == 0 || c == 2 || c == 5);
        Q[c * mtot + e1] = 1.5 * qB[c] - (diag ? trB : 0.0);
        Q[c * mtot + e2] = 1.5 * qA[c] - (diag ? trA : 0.0);
      }
    } else {
#pragma unroll
      for (int x = 0; x < 3; ++x) {
        D[x * mtot + e1] = v[1 + x];
        D[x * mtot + e2] = v[1 + x];
      }
      const double q9[9] = {v[4], v[5], v[6], v[5], v[7], v[8], v[6], v[8], v[9]};
#pragma unroll
      for (int c = 0; c < 9; ++c) {
        Q[c * mtot + e1] = q9[c];
        Q[c * mtot + e2] = q9[c];
      }
    }
  }
}

// The shell pairs with no p-p or d product (s-s and s-p: most pairs of an
// organic molecule) take one THREAD each (k_multipole_sp): with a warp per
// pair most lanes of every float64 instruction would idle. The pair is
// evaluated with the s shell on the bra; a p-s pair is computed as its s-p
// mirror (bra and ket exchanged), which yields the same two matrix
// elements. Tables and contraction follow md_table_1d exactly, with the
// p-order (y, z, x) and the spherical transform the identity for l <= 1.
__device__ __forceinline__ bool sp_class(int la, int lb) { return la + lb <= 1; }

template <int LB, int NC>
__device__ __forceinline__ void sp_pair(const PairGeom &g, const double *__restrict__ pf_, double *acc) {
  // acc [(2LB+1) * NC], Cartesian = spherical order for l <= 1
  constexpr int NCB = LB == 0 ? 1 : 3;
  const double AB[3] = {g.A[0] - g.B[0], g.A[1] - g.B[1], g.A[2] - g.B[2]};
  const double r2 = AB[0] * AB[0] + AB[1] * AB[1] + AB[2] * AB[2];
  for (int p1 = 0; p1 < g.na; ++p1) {
    const double a = pf(pf_, DXTB_P_ALPHA + g.ti * DXTB_MAXPRIM + p1);
    const double ca = pf(pf_, DXTB_P_COEFF + g.ti * DXTB_MAXPRIM + p1);
    for (int p2 = 0; p2 < g.nb; ++p2) {
      const double bb = pf(pf_, DXTB_P_ALPHA + g.tj * DXTB_MAXPRIM + p2);
      const double cb = pf(pf_, DXTB_P_COEFF + g.tj * DXTB_MAXPRIM + p2);
      const double oij = 1.0 / (a + bb);
      const double x2p = 0.5 * oij;
      const double sij = exp(-a * bb * oij * r2) * (kPi * sqrt(kPi)) * oij * sqrt(oij) * ca * cb;
      // T[x][c][e]: ket power c (0, or 1 for the p shell), moment e about B
      double T[3][2][3];
#pragma unroll
      for (int x = 0; x < 3; ++x) {
        const double P = (a * g.A[x] + bb * g.B[x]) * oij;
        const double xpb = P - g.B[x], xpc = xpb;
        const double m10 = xpc, m20 = xpc * xpc + x2p, m21 = 2.0 * xpc;
        T[x][0][0] = 1.0;
        T[x][0][1] = m10 * 1.0 + 0.0;
        T[x][0][2] = m20 * 1.0 + m21 * 0.0 + 2.0 * 0.0;
        if (LB == 1) {
          T[x][1][0] = xpb;
          T[x][1][1] = m10 * xpb + x2p;
          T[x][1][2] = m20 * xpb + m21 * x2p + 2.0 * 0.0;
        }
      }
#pragma unroll
      for (int c = 0; c < (LB == 1 ? 2 : 1); ++c)
#pragma unroll
        for (int e = 0; e < 3; ++e) T[0][c][e] *= sij;
#pragma unroll
      for (int cb_ = 0; cb_ < NCB; ++cb_) {
        // p order (y, z, x): component cb_ raises axis (cb_ + 1) % 3
        const int px = LB == 1 && cb_ == 2, py = LB == 1 && cb_ == 0, pz = LB == 1 && cb_ == 1;
#pragma unroll
        for (int comp = 0; comp < NC; ++comp) {
          const int ex = comp == 1 ? 1 : (comp == 4 ? 2 : (comp == 5 || comp == 6 ? 1 : 0));
          const int ey = comp == 2 ? 1 : (comp == 7 ? 2 : (comp == 5 || comp == 8 ? 1 : 0));
          const int ez = comp == 3 ? 1 : (comp == 9 ? 2 : (comp == 6 || comp == 8 ? 1 : 0));
          acc[cb_ * NC + comp] += T[0][px][ex] * T[1][py][ey] * T[2][pz][ez];
        }
      }
    }
  }
}

template <int NC>
__global__ void __launch_bounds__(128)
    k_multipole_sp(dxtb_batch b, const double *__restrict__ pf_, const int32_t *__restrict__ pi_tab,
                   const double *__restrict__ cn, double *__restrict__ S,
                   double *__restrict__ H, double *__restrict__ D, double *__restrict__ Q) {
  const int64_t npairs = b.pair_off[b.nmol];
  const int64_t mtot = b.mat_off[b.nmol];
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < npairs;
       k += (int64_t)gridDim.x * blockDim.x) {
    PairGeom g;
    pair_from_index(b, k, g);
    int la = pi_(pi_tab, DXTB_I_L + g.ti), lb = pi_(pi_tab, DXTB_I_L + g.tj);
    if (!sp_class(la, lb)) continue;
    // the bra of the evaluation is the s shell
    if (la == 1) {
      const int ti = g.ti, ai = g.ai;
      const int64_t gi = g.gi;
      g.ti = g.tj;
      g.ai = g.aj;
      g.gi = g.gj;
      g.tj = ti;
      g.aj = ai;
      g.gj = gi;
#pragma unroll
      for (int x = 0; x < 3; ++x) {
        const double t = g.A[x];
        g.A[x] = g.B[x];
        g.B[x] = t;
      }
      la = 0;
      lb = 1;
    }
    g.la = la;
    g.lb = lb;
    g.na = pi_(pi_tab, DXTB_I_NPRIM + g.ti);
    g.nb = pi_(pi_tab, DXTB_I_NPRIM + g.tj);
    double acc[3 * NC];
#pragma unroll
    for (int r = 0; r < 3 * NC; ++r) acc[r] = 0.0;
    if (lb == 0) sp_pair<0, NC>(g, pf_, acc); else sp_pair<1, NC>(g, pf_, acc);
    const double AB[3] = {g.A[0] - g.B[0], g.A[1] - g.B[1], g.A[2] - g.B[2]};
    const double r2 = AB[0] * AB[0] + AB[1] * AB[1] + AB[2] * AB[2];
    const double hfac = H != nullptr ? h0_factor(b, pf_, pi_tab, cn, g, r2) : 0.0;
    const int64_t moff = b.mat_off[g.m];
    const int n = (int)(b.ao_off[g.m + 1] - b.ao_off[g.m]);
    const int oi = b.shell_ao[g.gi], oj = b.shell_ao[g.gj];
    const double d[3] = {g.B[0] - g.A[0], g.B[1] - g.A[1], g.B[2] - g.A[2]};
#pragma unroll
    for (int mb = 0; mb < 3; ++mb) {
      if (mb > 2 * lb) break;
      const int nu = oj + mb;
      write_element<0>(acc + mb * NC, NC, moff + (int64_t)oi * n + nu, moff + (int64_t)nu * n + oi,
                       mtot, d, hfac, S, H, D, Q);
    }
  }
}

// mode 0: GFN (S + H0 [+ D, Q ket-centred traceless]); mode 1: raw about origin.
// With skip_sp, the s-s and s-p pairs are left to k_multipole_sp.
template <int MODE>
__global__ void __launch_bounds__(kWarps * 32)
    k_multipole(dxtb_batch b, const double *__restrict__ pf_, const int32_t *__restrict__ pi_tab,
                const double *__restrict__ cn, int ncomp_req, int skip_sp,
                double *__restrict__ S, double *__restrict__ H, double *__restrict__ D,
                double *__restrict__ Q) {
  extern __shared__ double smem[];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double(*s_tab)[32][kTab] = reinterpret_cast<double(*)[32][kTab]>(smem);
  double(*s_cart)[kNComp * kMaxCart * kMaxCart] =
      reinterpret_cast<double(*)[kNComp * kMaxCart * kMaxCart]>(smem + kWarps * 32 * kTab);
  double(*s_sph)[kNComp * 25] = reinterpret_cast<double(*)[kNComp * 25]>(
      smem + kWarps * (32 * kTab + kNComp * kMaxCart * kMaxCart));
  const int64_t npairs = b.pair_off[b.nmol];
  // grid-stride over shell pairs: the grid is sized on the host from an
  // upper bound, the exact count is read here (no host synchronisation)
  for (int64_t k = (int64_t)blockIdx.x * kWarps + w; k < npairs; k += (int64_t)gridDim.x * kWarps) {

    PairGeom g;
    pair_from_index(b, k, g);
    g.la = pi_(pi_tab, DXTB_I_L + g.ti);
    g.lb = pi_(pi_tab, DXTB_I_L + g.tj);
    if (skip_sp && sp_class(g.la, g.lb)) continue;  // uniform over the warp
    g.na = pi_(pi_tab, DXTB_I_NPRIM + g.ti);
    g.nb = pi_(pi_tab, DXTB_I_NPRIM + g.tj);
    const int la = g.la, lb = g.lb;
    const int nca = (la + 1) * (la + 2) / 2, ncb = (lb + 1) * (lb + 2) / 2;
    const int ncomp = ncomp_req;  // 1 or 10
    const int emax = ncomp > 1 ? 2 : 0;
    const int nout = nca * ncb * ncomp;

    double acc[12];
  #pragma unroll
    for (int r = 0; r < 12; ++r) acc[r] = 0.0;

    const double AB[3] = {g.A[0] - g.B[0], g.A[1] - g.B[1], g.A[2] - g.B[2]};
    const double r2 = AB[0] * AB[0] + AB[1] * AB[1] + AB[2] * AB[2];
    const int npp = g.na * g.nb;
    for (int c0 = 0; c0 < npp; c0 += 32) {
      const int cnt = min(32, npp - c0);
      if (lane < cnt) {
        const int pp = c0 + lane;
        const int p1 = pp / g.nb, p2 = pp % g.nb;
        const double a = pf(pf_, DXTB_P_ALPHA + g.ti * DXTB_MAXPRIM + p1);
        const double bb = pf(pf_, DXTB_P_ALPHA + g.tj * DXTB_MAXPRIM + p2);
        const double ca = pf(pf_, DXTB_P_COEFF + g.ti * DXTB_MAXPRIM + p1);
        const double cb = pf(pf_, DXTB_P_COEFF + g.tj * DXTB_MAXPRIM + p2);
        const double oij = 1.0 / (a + bb);
        const double x2p = 0.5 * oij;
        const double sij = exp(-a * bb * oij * r2) * (kPi * sqrt(kPi)) * oij * sqrt(oij) * ca * cb;
        double *tab = s_tab[w][lane];
  #pragma unroll
        for (int x = 0; x < 3; ++x) {
          const double P = (a * g.A[x] + bb * g.B[x]) * oij;
          const double xpc = MODE == 0 ? P - g.B[x] : P;  // ket centre or origin
          md_table_1d(la, lb, emax, P - g.A[x], P - g.B[x], xpc, x2p, tab + 27 * x);
        }
        // fold the 3D prefactor into the x table
        for (int q = 0; q < 27; ++q) tab[q] *= sij;
      }
      __syncwarp();
  #pragma unroll
      for (int r = 0; r < 12; ++r) {
        const int o = lane + 32 * r;
        if (o >= nout) break;
        const int comp = o % ncomp;
        const int cb_ = (o / ncomp) % ncb;
        const int ca_ = o / (ncomp * ncb);
        const int *na_ = c_cart[la][ca_], *nb_ = c_cart[lb][cb_], *ec = c_comp[comp];
        const int ix = (na_[0] * 3 + nb_[0]) * 3 + ec[0];
        const int iy = 27 + (na_[1] * 3 + nb_[1]) * 3 + ec[1];
        const int iz = 54 + (na_[2] * 3 + nb_[2]) * 3 + ec[2];
        double s = 0.0;
        for (int q = 0; q < cnt; ++q) {
          const double *tab = s_tab[w][q];
          s += tab[ix] * tab[iy] * tab[iz];
        }
        acc[r] += s;
      }
      __syncwarp();
    }
  #pragma unroll
    for (int r = 0; r < 12; ++r) {
      const int o = lane + 32 * r;
      if (o < nout) s_cart[w][o] = acc[r];
    }
    __syncwarp();
    // spherical transform: sph[comp][ma][mb]
    const int nsa = 2 * la + 1, nsb = 2 * lb + 1;
    for (int o = lane; o < ncomp * nsa * nsb; o += 32) {
      const int comp = o % ncomp, mb = (o / ncomp) % nsb, ma = o / (ncomp * nsb);
      double s = 0.0;
      for (int ca_ = 0; ca_ < nca; ++ca_) {
        const double ta = trafo(la, ma, ca_);
        if (ta == 0.0) continue;
        for (int cb_ = 0; cb_ < ncb; ++cb_) {
          const double tb = trafo(lb, mb, cb_);
          if (tb == 0.0) continue;
          s += ta * tb * s_cart[w][(ca_ * ncb + cb_) * ncomp + comp];
        }
      }
      s_sph[w][(ma * nsb + mb) * ncomp + comp] = s;
    }
    __syncwarp();

    // ---- epilogue ----
    const int64_t moff = b.mat_off[g.m];
    const int n = (int)(b.ao_off[g.m + 1] - b.ao_off[g.m]);
    const int64_t mtot = b.mat_off[b.nmol];
    const int oi = b.shell_ao[g.gi], oj = b.shell_ao[g.gj];

    const double hfac = (MODE == 0 && H != nullptr) ? h0_factor(b, pf_, pi_tab, cn, g, r2) : 0.0;
    const double d[3] = {g.B[0] - g.A[0], g.B[1] - g.A[1], g.B[2] - g.A[2]};  // B - A
    for (int o = lane; o < nsa * nsb; o += 32) {
      const int ma = o / nsb, mb = o % nsb;
      const int mu = oi + ma, nu = oj + mb;
      write_element<MODE>(&s_sph[w][o * ncomp], ncomp, moff + (int64_t)mu * n + nu,
                          moff + (int64_t)nu * n + mu, mtot, d, hfac, S, H, D, Q);
    }
    __syncwarp();  // the next pair reuses this warp's shared tables
  }
}

// ---------------------------------------------------------------------------
// Vector-Jacobian product of the raw integrals (moments about the origin):
// given upstream gradients gS = dL/dS [mat], gD = dL/dD [3][mat] and gQ =
// dL/dQ [9][mat] (any may be null), accumulate dL/dR [natoms][3]. The moment
// operators do not depend on the centres, so a primitive's derivative is the
// raised/lowered Gaussian: d/dA_x <a|x^e|b> = 2 alpha <a+1|..> - a <a-1|..>
// and likewise for the ket. One warp per shell pair; the primitive pairs are
// taken one at a time: three lanes build the three axes' tables in shared
// memory, then the lanes own Cartesian (component pair, moment) outputs.
// This is the backward of integral/wrappers.py:149-215 (autograd there).
constexpr int kVjpWarps = 4;
constexpr int kVjpTab = 3 * 3 * 27;  // (T, dA, dB) x axes x [a][b][e]

__device__ void md_table_vjp(int la, int lb, double alpha, double beta, double xpa, double xpb,
                             double xpc, double x2p, double *out /* [3][27]: T, dA, dB */) {
  double E[4][4][7];
  for (int a = 0; a < 4; ++a)
    for (int c = 0; c < 4; ++c)
      for (int t = 0; t < 7; ++t) E[a][c][t] = 0.0;
  E[0][0][0] = 1.0;
  const int la1 = la + 1, lb1 = lb + 1;
  for (int a = 0; a < la1; ++a)
    for (int t = 0; t <= a + 1; ++t) {
      double v = xpa * E[a][0][t];
      if (t > 0) v += x2p * E[a][0][t - 1];
      if (t + 1 <= a) v += (t + 1) * E[a][0][t + 1];
      E[a + 1][0][t] = v;
    }
  for (int a = 0; a <= la1; ++a)
    for (int c = 0; c < lb1; ++c)
      for (int t = 0; t <= a + c + 1; ++t) {
        double v = xpb * E[a][c][t];
        if (t > 0) v += x2p * E[a][c][t - 1];
        if (t + 1 <= a + c) v += (t + 1) * E[a][c][t + 1];
        E[a][c + 1][t] = v;
      }
  const double m10 = xpc, m20 = xpc * xpc + x2p, m21 = 2.0 * xpc;
  double T[4][4][3];
  for (int a = 0; a <= la1; ++a)
    for (int c = 0; c <= lb1; ++c) {
      const double *e = E[a][c];
      T[a][c][0] = e[0];
      T[a][c][1] = m10 * e[0] + e[1];
      T[a][c][2] = m20 * e[0] + m21 * e[1] + 2.0 * e[2];
    }
  for (int a = 0; a <= la; ++a)
    for (int c = 0; c <= lb; ++c)
      for (int ee = 0; ee < 3; ++ee) {
        const int o = (a * 3 + c) * 3 + ee;
        out[o] = T[a][c][ee];
        double da = 2.0 * alpha * T[a + 1][c][ee];
        if (a > 0) da -= a * T[a - 1][c][ee];
        double db = 2.0 * beta * T[a][c + 1][ee];
        if (c > 0) db -= c * T[a][c - 1][ee];
        out[27 + o] = da;
        out[54 + o] = db;
      }
}

__global__ void __launch_bounds__(kVjpWarps * 32)
    k_multipole_raw_vjp(dxtb_batch b, const double *__restrict__ pf_, const int32_t *__restrict__ pi_tab,
                        const double *__restrict__ gS, const double *__restrict__ gD,
                        const double *__restrict__ gQ, double *__restrict__ grad) {
  __shared__ double s_tab[kVjpWarps][kVjpTab];
  __shared__ double s_g[kVjpWarps][kNComp * kMaxCart * kMaxCart];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t npairs = b.pair_off[b.nmol];
  const int64_t mtot = b.mat_off[b.nmol];
  for (int64_t k = (int64_t)blockIdx.x * kVjpWarps + w; k < npairs; k += (int64_t)gridDim.x * kVjpWarps) {
    PairGeom g;
    pair_from_index(b, k, g);
    const int la = pi_(pi_tab, DXTB_I_L + g.ti), lb = pi_(pi_tab, DXTB_I_L + g.tj);
    const int na = pi_(pi_tab, DXTB_I_NPRIM + g.ti), nb = pi_(pi_tab, DXTB_I_NPRIM + g.tj);
    const int nca = (la + 1) * (la + 2) / 2, ncb = (lb + 1) * (lb + 2) / 2;
    const int nsa = 2 * la + 1, nsb = 2 * lb + 1;
    const int64_t moff = b.mat_off[g.m];
    const int n = (int)(b.ao_off[g.m + 1] - b.ao_off[g.m]);
    const int oi = b.shell_ao[g.gi], oj = b.shell_ao[g.gj];
    const bool same = g.i == g.j;
    // upstream gradient of the pair's Cartesian outputs: the spherical
    // elements (mu, nu) and their mirrors (nu, mu) (counted once in a
    // diagonal block), back through the spherical transform; the 9 raw
    // quadrupole components fold onto the 6 unique ones
    const int nout = nca * ncb * kNComp;
    for (int o = lane; o < nout; o += 32) {
      const int comp = o % kNComp, cb_ = (o / kNComp) % ncb, ca_ = o / (kNComp * ncb);
      double acc = 0.0;
      for (int ma = 0; ma < nsa; ++ma) {
        const double ta = trafo(la, ma, ca_);
        if (ta == 0.0) continue;
        for (int mb = 0; mb < nsb; ++mb) {
          const double tb = trafo(lb, mb, cb_);
          if (tb == 0.0) continue;
          const int64_t e1 = moff + (int64_t)(oi + ma) * n + oj + mb;
          const int64_t e2 = moff + (int64_t)(oj + mb) * n + oi + ma;
          double gv = 0.0;
          auto pick = [&](int64_t e) {
            double v = 0.0;
            if (comp == 0) {
              if (gS) v = gS[e];
            } else if (comp <= 3) {
              if (gD) v = gD[(comp - 1) * mtot + e];
            } else if (gQ) {
              // comps 4..9 = xx, xy, xz, yy, yz, zz; Q9 row-major xx xy xz yx yy yz zx zy zz
              const int c9a[6] = {0, 1, 2, 4, 5, 8}, c9b[6] = {0, 3, 6, 4, 7, 8};
              const int q = comp - 4;
              v = gQ[c9a[q] * mtot + e];
              if (c9b[q] != c9a[q]) v += gQ[c9b[q] * mtot + e];
            }
            return v;
          };
          gv = pick(e1);
          if (!same) gv += pick(e2);
          acc += ta * tb * gv;
        }
      }
      s_g[w][o] = acc;
    }
    __syncwarp();
    double dA[3] = {0.0, 0.0, 0.0}, dB[3] = {0.0, 0.0, 0.0};
    const double AB[3] = {g.A[0] - g.B[0], g.A[1] - g.B[1], g.A[2] - g.B[2]};
    const double r2 = AB[0] * AB[0] + AB[1] * AB[1] + AB[2] * AB[2];
    for (int pp = 0; pp < na * nb; ++pp) {
      const int p1 = pp / nb, p2 = pp % nb;
      const double a = pf(pf_, DXTB_P_ALPHA + g.ti * DXTB_MAXPRIM + p1);
      const double bb = pf(pf_, DXTB_P_ALPHA + g.tj * DXTB_MAXPRIM + p2);
      const double oij = 1.0 / (a + bb);
      const double x2p = 0.5 * oij;
      if (lane < 3) {
        const int x = lane;
        const double P = (a * g.A[x] + bb * g.B[x]) * oij;
        md_table_vjp(la, lb, a, bb, P - g.A[x], P - g.B[x], P, x2p, s_tab[w] + 81 * x);
      }
      __syncwarp();
      const double ca = pf(pf_, DXTB_P_COEFF + g.ti * DXTB_MAXPRIM + p1);
      const double cb = pf(pf_, DXTB_P_COEFF + g.tj * DXTB_MAXPRIM + p2);
      const double sij = exp(-a * bb * oij * r2) * (kPi * sqrt(kPi)) * oij * sqrt(oij) * ca * cb;
      for (int o = lane; o < nout; o += 32) {
        const double gv = s_g[w][o];
        if (gv == 0.0) continue;
        const int comp = o % kNComp, cb_ = (o / kNComp) % ncb, ca_ = o / (kNComp * ncb);
        const int *na_ = c_cart[la][ca_], *nb_ = c_cart[lb][cb_], *ec = c_comp[comp];
        const double *tx = s_tab[w], *ty = s_tab[w] + 81, *tz = s_tab[w] + 162;
        const int ix = (na_[0] * 3 + nb_[0]) * 3 + ec[0];
        const int iy = (na_[1] * 3 + nb_[1]) * 3 + ec[1];
        const int iz = (na_[2] * 3 + nb_[2]) * 3 + ec[2];
        const double f = gv * sij;
        const double Tx = tx[ix], Ty = ty[iy], Tz = tz[iz];
        dA[0] += f * tx[27 + ix] * Ty * Tz;
        dA[1] += f * Tx * ty[27 + iy] * Tz;
        dA[2] += f * Tx * Ty * tz[27 + iz];
        dB[0] += f * tx[54 + ix] * Ty * Tz;
        dB[1] += f * Tx * ty[54 + iy] * Tz;
        dB[2] += f * Tx * Ty * tz[54 + iz];
      }
      __syncwarp();
    }
#pragma unroll
    for (int x = 0; x < 3; ++x) {
      dA[x] = warp_sum(dA[x]);
      dB[x] = warp_sum(dB[x]);
    }
    if (lane == 0) {
#pragma unroll
      for (int x = 0; x < 3; ++x) {
        atomicAdd(&grad[3 * (g.a0 + g.ai) + x], dA[x]);
        atomicAdd(&grad[3 * (g.a0 + g.aj) + x], dB[x]);
      }
    }
  }
}

}  // namespace dxtb

using namespace dxtb;

extern "C" int32_t dxtb_multipole_raw_vjp(const dxtb_batch *b, const double *par_f,
                                          const int32_t *par_i, const double *grad_overlap,
                                          const double *grad_dipole, const double *grad_quadrupole,
                                          double *grad, void *stream) {
  if (!b || b->nmol <= 0 || !par_f || !par_i || !grad || b->max_nsh < 0) return DXTB_ERR_ARGS;
  const int64_t bound = (int64_t)b->nmol * b->max_nsh * (b->max_nsh + 1) / 2;
  if (bound <= 0) return DXTB_OK;
  int sms = 0;
  if (device_sms(&sms) != DXTB_OK) return DXTB_ERR_LAUNCH;
  const int64_t blocks = min((bound + kVjpWarps - 1) / kVjpWarps, (int64_t)sms * 8);
  k_multipole_raw_vjp<<<(unsigned)blocks, kVjpWarps * 32, 0, (cudaStream_t)stream>>>(
      *b, par_f, par_i, grad_overlap, grad_dipole, grad_quadrupole, grad);
  DXTB_CHECK_LAUNCH();
  return DXTB_OK;
}

constexpr size_t kSmem = sizeof(double) * kWarps * (32 * kTab + kNComp * kMaxCart * kMaxCart + kNComp * 25);

static int32_t launch_multipole(const dxtb_batch *b, const double *par_f, const int32_t *par_i,
                                const double *cn, double *S, double *H, double *D, double *Q,
                                int mode, cudaStream_t st) {
  if (!b || b->nmol <= 0 || !S || b->max_nsh < 0) return DXTB_ERR_ARGS;
  const int ncomp = (D != nullptr && Q != nullptr) ? kNComp : 1;
  // upper bound of the pair count from the host descriptor; the kernel reads
  // the exact total pair_off[nmol] on the device
  const int64_t bound = (int64_t)b->nmol * b->max_nsh * (b->max_nsh + 1) / 2;
  if (bound <= 0) return DXTB_OK;
  int sms = 0;
  if (device_sms(&sms) != DXTB_OK) return DXTB_ERR_LAUNCH;
  const int64_t blocks = min((bound + kWarps - 1) / kWarps, (int64_t)sms * 2 * 8);
  static PerDeviceOnce attr;
  if (per_device_once(attr, [] {
        return cudaFuncSetAttribute(k_multipole<0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)kSmem) == cudaSuccess &&
               cudaFuncSetAttribute(k_multipole<1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)kSmem) == cudaSuccess;
      }) != DXTB_OK)
    return DXTB_ERR_LAUNCH;
  if (mode == 0) {
    // s-s and s-p pairs: a thread each; the rest: a warp each
    const int64_t tblocks = min((bound + 127) / 128, (int64_t)sms * 16);
    if (ncomp == 1)
      k_multipole_sp<1><<<(unsigned)tblocks, 128, 0, st>>>(*b, par_f, par_i, cn, S, H, D, Q);
    else
      k_multipole_sp<kNComp><<<(unsigned)tblocks, 128, 0, st>>>(*b, par_f, par_i, cn, S, H, D, Q);
    DXTB_CHECK_LAUNCH();
    k_multipole<0><<<(unsigned)blocks, kWarps * 32, kSmem, st>>>(*b, par_f, par_i, cn, ncomp, 1, S, H, D, Q);
  } else {
    k_multipole<1><<<(unsigned)blocks, kWarps * 32, kSmem, st>>>(*b, par_f, par_i, cn, ncomp, 0, S, nullptr,
                                                             D, Q);
  }
  DXTB_CHECK_LAUNCH();
  return DXTB_OK;
}

extern "C" int32_t dxtb_multipole_h0(const dxtb_batch *b, const double *par_f,
                                     const int32_t *par_i, const double *cn, double *overlap,
                                     double *h0, double *dipole, double *quadrupole,
                                     void *stream) {
  if (h0 != nullptr && cn == nullptr) return DXTB_ERR_ARGS;
  return launch_multipole(b, par_f, par_i, cn, overlap, h0, dipole, quadrupole, 0,
                          (cudaStream_t)stream);
}

extern "C" int32_t dxtb_multipole_raw(const dxtb_batch *b, const double *par_f,
                                      const int32_t *par_i, double *overlap, double *dipole,
                                      double *quadrupole, void *stream) {
  return launch_multipole(b, par_f, par_i, nullptr, overlap, nullptr, dipole, quadrupole, 1,
                          (cudaStream_t)stream);
}
