// Analytic nuclear gradient of the GFN1/GFN2-xTB energy at the converged SCF.
//
// The xTB free energy is variational in the density, so
//   dE/dR = dE/dR |_(P fixed) - sum_{mu nu} W_{mu nu} dS_{mu nu}/dR
// with the energy-weighted density W = C diag(f eps) C^T. The reference
// obtains the same quantity with autograd through the implicit SCF
// (calculators/types/autograd.py:84-196, scf/implicit/fixed_point.py:
// 250-431); GFN1's hand-written form is xtb/gfn1.py:185-408 and
// calculators/types/analytical.py:65-258.
//
// k_grad_pairs: one warp per shell pair. Coefficient blocks for dS, dD, dQ
//   (from P, W, H0 scaling, orbital and multipole potentials) are
//   transformed back to the Cartesian basis, and the McMurchie-Davidson
//   tables with the bra shell raised/lowered give d/dA of every Cartesian
//   integral, contracted on the fly (no derivative integrals are stored).
//   The same warp adds the distance-polynomial term of H0 and the
//   coordination-number derivative of the self-energies.
// k_grad_mol: one CTA per molecule: ES2 (gamma), AES2 kernels and damping
//   radii, repulsion, and the chain rule through the coordination number.
#include "common.cuh"

namespace dxtb {

constexpr int gWarps = 4;
constexpr int gChunk = 16;   // primitive pairs staged per round
constexpr int gTab = 2 * 3 * 36;  // (T, dT) x axes x [a<=3][b<=2][e<=2] -> 216
constexpr int gNComp = 10;

__constant__ int g_cart[3][6][3] = {
    {{0, 0, 0}},
    {{0, 1, 0}, {0, 0, 1}, {1, 0, 0}},
    {{2, 0, 0}, {1, 1, 0}, {1, 0, 1}, {0, 2, 0}, {0, 1, 1}, {0, 0, 2}},
};
__constant__ int g_comp[gNComp][3] = {
    {0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {2, 0, 0},
    {1, 1, 0}, {1, 0, 1}, {0, 2, 0}, {0, 1, 1}, {0, 0, 2},
};

__device__ __forceinline__ double gtrafo(int l, int m, int c) {
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

// 1D Hermite tables T[a][b][e] for a <= la+1, b <= lb, e <= emax (about the
// ket centre), and the bra derivative dT[a][b][e] = 2 alpha T[a+1] - a T[a-1].
__device__ void md_tables_grad(int la, int lb, int emax, double alpha, double xpa, double xpb,
                               double x2p, double pref, double *T /*36*/, double *dT /*36*/) {
  double E[4][3][6];
  for (int a = 0; a < 4; ++a)
    for (int c = 0; c < 3; ++c)
      for (int t = 0; t < 6; ++t) E[a][c][t] = 0.0;
  E[0][0][0] = 1.0;
  const int la1 = la + 1;
  for (int a = 0; a < la1; ++a)
    for (int t = 0; t <= a + 1; ++t) {
      double v = xpa * E[a][0][t];
      if (t > 0) v += x2p * E[a][0][t - 1];
      if (t + 1 <= a) v += (t + 1) * E[a][0][t + 1];
      E[a + 1][0][t] = v;
    }
  for (int a = 0; a <= la1; ++a)
    for (int c = 0; c < lb; ++c)
      for (int t = 0; t <= a + c + 1; ++t) {
        double v = xpb * E[a][c][t];
        if (t > 0) v += x2p * E[a][c][t - 1];
        if (t + 1 <= a + c) v += (t + 1) * E[a][c][t + 1];
        E[a][c + 1][t] = v;
      }
  const double xpc = xpb;
  const double m10 = xpc, m20 = xpc * xpc + x2p, m21 = 2.0 * xpc;
  double Tl[4][3][3];
  for (int a = 0; a <= la1; ++a)
    for (int c = 0; c <= lb; ++c) {
      const double *e = E[a][c];
      Tl[a][c][0] = e[0];
      Tl[a][c][1] = emax >= 1 ? m10 * e[0] + e[1] : 0.0;
      Tl[a][c][2] = emax >= 2 ? m20 * e[0] + m21 * e[1] + 2.0 * e[2] : 0.0;
    }
  for (int a = 0; a <= la; ++a)
    for (int c = 0; c <= lb; ++c)
      for (int ee = 0; ee <= emax; ++ee) {
        const int o = (a * 3 + c) * 3 + ee;
        T[o] = pref * Tl[a][c][ee];
        double d = 2.0 * alpha * Tl[a + 1][c][ee];
        if (a > 0) d -= a * Tl[a - 1][c][ee];
        dT[o] = pref * d;
      }
}

struct GPair {
  int m, i, j, ti, tj, ai, aj, la, lb, na, nb;
  int64_t gi, gj, a0;
  double A[3], B[3];
};

// Shell pairs without a p-p or d product take one thread each
// (k_grad_pairs_sp); the warp kernel leaves them out.
__device__ __forceinline__ bool gsp_class(int la, int lb) { return la + lb <= 1; }

// One shell pair of the integral adjoint (one warp).
__device__ __forceinline__ void grad_pair(
    const dxtb_batch &b, const double *__restrict__ pf_, const int32_t *__restrict__ pi_tab,
    const double *__restrict__ cn, const double *__restrict__ P, const double *__restrict__ W,
    const double *__restrict__ S, const double *__restrict__ D, const double *__restrict__ vorb,
    const double *__restrict__ vdp, const double *__restrict__ vqp, int multipole,
    double *__restrict__ dedcn, double *__restrict__ grad, int64_t k, int lane, double *s_tab,
    double *s_esph, double *s_ecart, bool skip_sp) {

  GPair g;
  g.m = find_mol(b.pair_off, b.nmol, k);
  {
    const int64_t t = k - b.pair_off[g.m];
    int i = (int)((sqrtf(8.0f * (float)t + 1.0f) - 1.0f) * 0.5f);
    while ((int64_t)(i + 1) * (i + 2) / 2 <= t) ++i;
    while ((int64_t)i * (i + 1) / 2 > t) --i;
    g.i = i;
    g.j = (int)(t - (int64_t)i * (i + 1) / 2);
  }
  const int64_t s0 = b.shell_off[g.m];
  g.a0 = b.atom_off[g.m];
  g.gi = s0 + g.i;
  g.gj = s0 + g.j;
  g.ti = b.shell_type[g.gi];
  g.tj = b.shell_type[g.gj];
  g.ai = b.shell_atom[g.gi];
  g.aj = b.shell_atom[g.gj];
  for (int x = 0; x < 3; ++x) {
    g.A[x] = b.positions[3 * (g.a0 + g.ai) + x];
    g.B[x] = b.positions[3 * (g.a0 + g.aj) + x];
  }
  g.la = pi_(pi_tab, DXTB_I_L + g.ti);
  g.lb = pi_(pi_tab, DXTB_I_L + g.tj);
  if (skip_sp && gsp_class(g.la, g.lb)) return;  // uniform over the warp
  g.na = pi_(pi_tab, DXTB_I_NPRIM + g.ti);
  g.nb = pi_(pi_tab, DXTB_I_NPRIM + g.tj);
  const int la = g.la, lb = g.lb, nsa = 2 * la + 1, nsb = 2 * lb + 1;
  const int64_t moff = b.mat_off[g.m], mtot = b.mat_off[b.nmol];
  const int n = (int)(b.ao_off[g.m + 1] - b.ao_off[g.m]);
  const int64_t o0 = b.ao_off[g.m];
  const int oi = b.shell_ao[g.gi], oj = b.shell_ao[g.gj];
  const bool same_atom = (g.ai == g.aj);
  const int zi = b.numbers[g.a0 + g.ai], zj = b.numbers[g.a0 + g.aj];

  // ---- H0 scaling of the pair (xtb/base.py:255-372) ----
  const double sei = pf(pf_, DXTB_P_LEVEL + g.ti) - pf(pf_, DXTB_P_KCN + g.ti) * cn[g.a0 + g.ai];
  const double sej = pf(pf_, DXTB_P_LEVEL + g.tj) - pf(pf_, DXTB_P_KCN + g.tj) * cn[g.a0 + g.aj];
  double fk = 1.0, pi = 1.0, dpi = 0.0, dist = 0.0;  // h = 0.5 (sei + sej) * pi * fk
  double d[3] = {g.B[0] - g.A[0], g.B[1] - g.A[1], g.B[2] - g.A[2]};
  if (!same_atom) {
    dist = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    const double rsum = pf(pf_, DXTB_P_RAD + zi) + pf(pf_, DXTB_P_RAD + zj);
    const double rr = sqrt(dist / rsum);
    const double ki = pf(pf_, DXTB_P_SHPOLY + g.ti), kj = pf(pf_, DXTB_P_SHPOLY + g.tj);
    pi = (1.0 + ki * rr) * (1.0 + kj * rr);
    dpi = (ki * (1.0 + kj * rr) + kj * (1.0 + ki * rr)) * rr / (2.0 * dist);
    const int vi = pi_(pi_tab, DXTB_I_VALENCE + g.ti), vj = pi_(pi_tab, DXTB_I_VALENCE + g.tj);
    const double wexp = pf(pf_, DXTB_P_SCAL + DXTB_S_WEXP);
    const double zti = pf(pf_, DXTB_P_SLATER + g.ti), ztj = pf(pf_, DXTB_P_SLATER + g.tj);
    const double zfac = wexp == 0.0 ? 1.0 : pow(2.0 * sqrt(zti * ztj) / (zti + ztj), wexp);
    if (vi && vj) {
      const double den = pf(pf_, DXTB_P_EN + zi) - pf(pf_, DXTB_P_EN + zj);
      fk = pf(pf_, DXTB_P_KSHELL + la * 5 + lb) * zfac * pf(pf_, DXTB_P_KPAIR + zi * DXTB_MAXZ + zj) *
           (1.0 + pf(pf_, DXTB_P_SCAL + DXTB_S_ENSCALE) * den * den);
    } else {
      const double kpol = pf(pf_, DXTB_P_SCAL + DXTB_S_KPOL);
      const double kii = vi ? pf(pf_, DXTB_P_KSHELL + la * 6) : kpol;
      const double kjj = vj ? pf(pf_, DXTB_P_KSHELL + lb * 6) : kpol;
      fk = 0.5 * (kii + kjj) * zfac;
    }
  }
  const double h = 0.5 * (sei + sej) * pi * fk;

  // ---- coefficient blocks (spherical) ----
  double ps_part = 0.0, gconst[3] = {0.0, 0.0, 0.0};
  const int qa[6] = {0, 0, 1, 0, 1, 2}, qb[6] = {0, 1, 1, 2, 2, 2};
  const int q2comp[6] = {4, 5, 7, 6, 8, 9};  // (xx xy yy xz yz zz) -> component index
  const int64_t A0 = g.a0 + g.ai, B0 = g.a0 + g.aj;
  for (int o = lane; o < nsa * nsb; o += 32) {
    const int ma = o / nsb, mb = o % nsb;
    const int mu = oi + ma, nu = oj + mb;
    const int64_t e1 = moff + (int64_t)mu * n + nu;
    const double Pmn = P[e1], Smn = S[e1];
    ps_part += Pmn * Smn;
    double *es = s_esph + (size_t)o * gNComp;
    for (int c = 0; c < gNComp; ++c) es[c] = 0.0;
    if (same_atom) continue;
    const double cS2 = 2.0 * (Pmn * h - 0.5 * Pmn * (vorb[o0 + mu] + vorb[o0 + nu]) - W[e1]);
    if (!multipole) {
      es[0] = cS2;
      continue;
    }
    double cDA[3], cDB[3], cQA[6], cQB[6];
    for (int x = 0; x < 3; ++x) {
      cDB[x] = -Pmn * vdp[3 * B0 + x];
      cDA[x] = -Pmn * vdp[3 * A0 + x];
    }
    {
      double tA[6], tB[6];
      for (int c = 0; c < 6; ++c) {
        tB[c] = -Pmn * vqp[6 * B0 + c];
        tA[c] = -Pmn * vqp[6 * A0 + c];
      }
      const double trA = 0.5 * (tA[0] + tA[2] + tA[5]), trB = 0.5 * (tB[0] + tB[2] + tB[5]);
      for (int c = 0; c < 6; ++c) {
        const bool diag = (c == 0 || c == 2 || c == 5);
        cQA[c] = 1.5 * tA[c] - (diag ? trA : 0.0);
        cQB[c] = 1.5 * tB[c] - (diag ? trB : 0.0);
      }
    }
    double eS = cS2, eD[3];
    for (int x = 0; x < 3; ++x) {
      eS += cDA[x] * d[x];
      eD[x] = cDB[x] + cDA[x];
    }
    double DB[3];
    for (int x = 0; x < 3; ++x) DB[x] = D[x * mtot + e1];
    for (int c = 0; c < 6; ++c) {
      const int a = qa[c], bq = qb[c];
      eS += cQA[c] * d[a] * d[bq];
      eD[a] += cQA[c] * d[bq];
      eD[bq] += cQA[c] * d[a];
      es[q2comp[c]] = cQB[c] + cQA[c];
      // explicit dependence of the bra-centred moments on A
      gconst[bq] -= cQA[c] * (DB[a] + d[a] * Smn);
      gconst[a] -= cQA[c] * (DB[bq] + d[bq] * Smn);
    }
    for (int x = 0; x < 3; ++x) gconst[x] -= cDA[x] * Smn;
    es[0] = eS;
    for (int x = 0; x < 3; ++x) es[1 + x] = eD[x];
  }
  const double ps = warp_sum(ps_part);
  if (lane == 0) {
    // d E_h0 / d CN (self-energies): -kcn * sum_block P S * (pi * fk off-site)
    const double f = same_atom ? 1.0 : pi * fk;
    atomicAdd(&dedcn[A0], -pf(pf_, DXTB_P_KCN + g.ti) * f * ps);
    if (g.i != g.j) atomicAdd(&dedcn[B0], -pf(pf_, DXTB_P_KCN + g.tj) * f * ps);
  }
  if (same_atom) return;
  __syncwarp();

  // ---- back-transform coefficients to Cartesian: ec[a][b][comp] ----
  const int nca = (la + 1) * (la + 2) / 2, ncb = (lb + 1) * (lb + 2) / 2;
  const int ncomp = multipole ? gNComp : 1;
  const int emax = multipole ? 2 : 0;
  for (int o = lane; o < nca * ncb * ncomp; o += 32) {
    const int comp = o % ncomp, cb = (o / ncomp) % ncb, ca = o / (ncomp * ncb);
    double s = 0.0;
    for (int ma = 0; ma < nsa; ++ma) {
      const double ta = gtrafo(la, ma, ca);
      if (ta == 0.0) continue;
      for (int mb = 0; mb < nsb; ++mb) {
        const double tb = gtrafo(lb, mb, cb);
        if (tb == 0.0) continue;
        s += ta * tb * s_esph[(size_t)(ma * nsb + mb) * gNComp + comp];
      }
    }
    s_ecart[o] = s;
  }
  __syncwarp();

  // ---- contract with d/dA of the Cartesian integrals ----
  double gx = 0.0, gy = 0.0, gz = 0.0;
  const double r2 = dist * dist;
  const int npp = g.na * g.nb;
  const int nout = nca * ncb * ncomp;
  for (int c0 = 0; c0 < npp; c0 += gChunk) {
    const int cnt = min(gChunk, npp - c0);
    if (lane < cnt) {
      const int pp = c0 + lane;
      const int p1 = pp / g.nb, p2 = pp % g.nb;
      const double a = pf(pf_, DXTB_P_ALPHA + g.ti * DXTB_MAXPRIM + p1);
      const double bb = pf(pf_, DXTB_P_ALPHA + g.tj * DXTB_MAXPRIM + p2);
      const double ca = pf(pf_, DXTB_P_COEFF + g.ti * DXTB_MAXPRIM + p1);
      const double cb = pf(pf_, DXTB_P_COEFF + g.tj * DXTB_MAXPRIM + p2);
      const double oij = 1.0 / (a + bb), x2p = 0.5 * oij;
      const double sij = exp(-a * bb * oij * r2) * (kPi * sqrt(kPi)) * oij * sqrt(oij) * ca * cb;
      double *tab = s_tab + (size_t)lane * gTab;
      for (int x = 0; x < 3; ++x) {
        const double Pc = (a * g.A[x] + bb * g.B[x]) * oij;
        md_tables_grad(la, lb, emax, a, Pc - g.A[x], Pc - g.B[x], x2p, x == 0 ? sij : 1.0,
                       tab + 72 * x, tab + 72 * x + 36);
      }
    }
    __syncwarp();
    for (int o = lane; o < nout; o += 32) {
      const int comp = o % ncomp, cb = (o / ncomp) % ncb, ca = o / (ncomp * ncb);
      const double coef = s_ecart[o];
      if (coef == 0.0) continue;
      const int *na_ = g_cart[la][ca], *nb_ = g_cart[lb][cb], *ec = g_comp[comp];
      const int ix = (na_[0] * 3 + nb_[0]) * 3 + ec[0];
      const int iy = (na_[1] * 3 + nb_[1]) * 3 + ec[1];
      const int iz = (na_[2] * 3 + nb_[2]) * 3 + ec[2];
      double sx = 0.0, sy = 0.0, sz = 0.0;
      for (int q = 0; q < cnt; ++q) {
        const double *tab = s_tab + (size_t)q * gTab;
        const double Tx = tab[ix], dTx = tab[36 + ix];
        const double Ty = tab[72 + iy], dTy = tab[108 + iy];
        const double Tz = tab[144 + iz], dTz = tab[180 + iz];
        sx += dTx * Ty * Tz;
        sy += Tx * dTy * Tz;
        sz += Tx * Ty * dTz;
      }
      gx += coef * sx;
      gy += coef * sy;
      gz += coef * sz;
    }
    __syncwarp();
  }
  gx = warp_sum(gx + gconst[0]);
  gy = warp_sum(gy + gconst[1]);
  gz = warp_sum(gz + gconst[2]);
  if (lane == 0) {
    // distance polynomial of H0: 2 sum_block P h S * (dpi/dR) / pi along (A-B)/R
    const double dEdR = 2.0 * ps * h * dpi / pi;
    const double u[3] = {-d[0] / dist, -d[1] / dist, -d[2] / dist};  // (A - B) / R
    const double gv[3] = {gx + dEdR * u[0], gy + dEdR * u[1], gz + dEdR * u[2]};
    for (int x = 0; x < 3; ++x) {
      atomicAdd(&grad[3 * A0 + x], gv[x]);
      atomicAdd(&grad[3 * B0 + x], -gv[x]);
    }
  }
}

__global__ void __launch_bounds__(gWarps * 32)
    k_grad_pairs(dxtb_batch b, const double *__restrict__ pf_, const int32_t *__restrict__ pi_tab,
                 const double *__restrict__ cn, const double *__restrict__ P,
                 const double *__restrict__ W, const double *__restrict__ S,
                 const double *__restrict__ D, const double *__restrict__ vorb,
                 const double *__restrict__ vdp, const double *__restrict__ vqp, int multipole,
                 double *__restrict__ dedcn, double *__restrict__ grad, ClassFilter flt) {
  extern __shared__ double smem[];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double *s_tab = smem + (size_t)w * (gChunk * gTab + 2 * gNComp * 36);
  double *s_esph = s_tab + gChunk * gTab;      // [10][5][5] spherical coefficients
  double *s_ecart = s_esph + gNComp * 36;      // [6][6][10] Cartesian coefficients
  // grid-stride over shell pairs; the exact count is read on the device
  const int64_t npairs = b.pair_off[b.nmol];
  for (int64_t k = (int64_t)blockIdx.x * gWarps + w; k < npairs; k += (int64_t)gridDim.x * gWarps) {
    if (flt.cls >= 0 && !in_class(flt, b, find_mol(b.pair_off, b.nmol, k))) continue;  // warp-uniform
    grad_pair(b, pf_, pi_tab, cn, P, W, S, D, vorb, vdp, vqp, multipole, dedcn, grad, k, lane, s_tab,
              s_esph, s_ecart, true);
    __syncwarp();  // the next pair reuses this warp's shared tables
  }
}

// One s-s or s-p shell pair of the integral adjoint on one thread: the
// coefficient blocks and the bra-derivative contraction of grad_pair, with
// the s shell on the bra (a p-s pair is evaluated as its s-p mirror, which
// holds the same two matrix elements; the pair's contribution is symmetric
// under exchanging bra and ket), the tables written out for l <= 1 and the
// spherical transform the identity.
template <int LB, int NC>
__device__ __forceinline__ void grad_pair_sp(
    const dxtb_batch &b, const double *__restrict__ pf_, const int32_t *__restrict__ pi_tab,
    const double *__restrict__ cn, const double *__restrict__ P, const double *__restrict__ W,
    const double *__restrict__ S, const double *__restrict__ D, const double *__restrict__ vorb,
    const double *__restrict__ vdp, const double *__restrict__ vqp, double *__restrict__ dedcn,
    double *__restrict__ grad, const GPair &g) {
  constexpr int NSB = 2 * LB + 1;
  constexpr bool MP = NC > 1;
  const int64_t moff = b.mat_off[g.m], mtot = b.mat_off[b.nmol];
  const int n = (int)(b.ao_off[g.m + 1] - b.ao_off[g.m]);
  const int64_t o0 = b.ao_off[g.m];
  const int oi = b.shell_ao[g.gi], oj = b.shell_ao[g.gj];
  const bool same_atom = (g.ai == g.aj);
  const int zi = b.numbers[g.a0 + g.ai], zj = b.numbers[g.a0 + g.aj];
  const double sei = pf(pf_, DXTB_P_LEVEL + g.ti) - pf(pf_, DXTB_P_KCN + g.ti) * cn[g.a0 + g.ai];
  const double sej = pf(pf_, DXTB_P_LEVEL + g.tj) - pf(pf_, DXTB_P_KCN + g.tj) * cn[g.a0 + g.aj];
  double fk = 1.0, pi = 1.0, dpi = 0.0, dist = 0.0;
  const double d[3] = {g.B[0] - g.A[0], g.B[1] - g.A[1], g.B[2] - g.A[2]};
  if (!same_atom) {
    dist = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    const double rsum = pf(pf_, DXTB_P_RAD + zi) + pf(pf_, DXTB_P_RAD + zj);
    const double rr = sqrt(dist / rsum);
    const double ki = pf(pf_, DXTB_P_SHPOLY + g.ti), kj = pf(pf_, DXTB_P_SHPOLY + g.tj);
    pi = (1.0 + ki * rr) * (1.0 + kj * rr);
    dpi = (ki * (1.0 + kj * rr) + kj * (1.0 + ki * rr)) * rr / (2.0 * dist);
    const int vi = pi_(pi_tab, DXTB_I_VALENCE + g.ti), vj = pi_(pi_tab, DXTB_I_VALENCE + g.tj);
    const double wexp = pf(pf_, DXTB_P_SCAL + DXTB_S_WEXP);
    const double zti = pf(pf_, DXTB_P_SLATER + g.ti), ztj = pf(pf_, DXTB_P_SLATER + g.tj);
    const double zfac = wexp == 0.0 ? 1.0 : pow(2.0 * sqrt(zti * ztj) / (zti + ztj), wexp);
    if (vi && vj) {
      const double den = pf(pf_, DXTB_P_EN + zi) - pf(pf_, DXTB_P_EN + zj);
      fk = pf(pf_, DXTB_P_KSHELL + g.la * 5 + g.lb) * zfac * pf(pf_, DXTB_P_KPAIR + zi * DXTB_MAXZ + zj) *
           (1.0 + pf(pf_, DXTB_P_SCAL + DXTB_S_ENSCALE) * den * den);
    } else {
      const double kpol = pf(pf_, DXTB_P_SCAL + DXTB_S_KPOL);
      const double kii = vi ? pf(pf_, DXTB_P_KSHELL + g.la * 6) : kpol;
      const double kjj = vj ? pf(pf_, DXTB_P_KSHELL + g.lb * 6) : kpol;
      fk = 0.5 * (kii + kjj) * zfac;
    }
  }
  const double h = 0.5 * (sei + sej) * pi * fk;
  const int64_t A0 = g.a0 + g.ai, B0 = g.a0 + g.aj;
  double ps = 0.0, gconst[3] = {0.0, 0.0, 0.0};
  double es[NSB][NC];
#pragma unroll
  for (int mb = 0; mb < NSB; ++mb) {
    const int mu = oi, nu = oj + mb;
    const int64_t e1 = moff + (int64_t)mu * n + nu;
    const double Pmn = P[e1], Smn = S[e1];
    ps += Pmn * Smn;
#pragma unroll
    for (int c = 0; c < NC; ++c) es[mb][c] = 0.0;
    if (same_atom) continue;
    const double cS2 = 2.0 * (Pmn * h - 0.5 * Pmn * (vorb[o0 + mu] + vorb[o0 + nu]) - W[e1]);
    if constexpr (!MP) {
      es[mb][0] = cS2;
    } else {
      const int qa[6] = {0, 0, 1, 0, 1, 2}, qb[6] = {0, 1, 1, 2, 2, 2};
      const int q2comp[6] = {4, 5, 7, 6, 8, 9};
      double cDA[3], cDB[3], cQA[6], cQB[6], tA[6], tB[6];
#pragma unroll
      for (int x = 0; x < 3; ++x) {
        cDB[x] = -Pmn * vdp[3 * B0 + x];
        cDA[x] = -Pmn * vdp[3 * A0 + x];
      }
#pragma unroll
      for (int c = 0; c < 6; ++c) {
        tB[c] = -Pmn * vqp[6 * B0 + c];
        tA[c] = -Pmn * vqp[6 * A0 + c];
      }
      const double trA = 0.5 * (tA[0] + tA[2] + tA[5]), trB = 0.5 * (tB[0] + tB[2] + tB[5]);
#pragma unroll
      for (int c = 0; c < 6; ++c) {
        const bool diag = (c == 0 || c == 2 || c == 5);
        cQA[c] = 1.5 * tA[c] - (diag ? trA : 0.0);
        cQB[c] = 1.5 * tB[c] - (diag ? trB : 0.0);
      }
      double eS = cS2, eD[3];
#pragma unroll
      for (int x = 0; x < 3; ++x) {
        eS += cDA[x] * d[x];
        eD[x] = cDB[x] + cDA[x];
      }
      double DB[3];
#pragma unroll
      for (int x = 0; x < 3; ++x) DB[x] = D[x * mtot + e1];
#pragma unroll
      for (int c = 0; c < 6; ++c) {
        const int a = qa[c], bq = qb[c];
        eS += cQA[c] * d[a] * d[bq];
        eD[a] += cQA[c] * d[bq];
        eD[bq] += cQA[c] * d[a];
        es[mb][q2comp[c]] = cQB[c] + cQA[c];
        gconst[bq] -= cQA[c] * (DB[a] + d[a] * Smn);
        gconst[a] -= cQA[c] * (DB[bq] + d[bq] * Smn);
      }
#pragma unroll
      for (int x = 0; x < 3; ++x) gconst[x] -= cDA[x] * Smn;
      es[mb][0] = eS;
#pragma unroll
      for (int x = 0; x < 3; ++x) es[mb][1 + x] = eD[x];
    }
  }
  {
    const double f = same_atom ? 1.0 : pi * fk;
    atomicAdd(&dedcn[A0], -pf(pf_, DXTB_P_KCN + g.ti) * f * ps);
    if (g.i != g.j) atomicAdd(&dedcn[B0], -pf(pf_, DXTB_P_KCN + g.tj) * f * ps);
  }
  if (same_atom) return;
  // contraction with d/dA of the Cartesian integrals (moments about B)
  double gx = 0.0, gy = 0.0, gz = 0.0;
  const double r2 = dist * dist;
  for (int p1 = 0; p1 < g.na; ++p1) {
    const double a = pf(pf_, DXTB_P_ALPHA + g.ti * DXTB_MAXPRIM + p1);
    const double ca = pf(pf_, DXTB_P_COEFF + g.ti * DXTB_MAXPRIM + p1);
    for (int p2 = 0; p2 < g.nb; ++p2) {
      const double bb = pf(pf_, DXTB_P_ALPHA + g.tj * DXTB_MAXPRIM + p2);
      const double cb = pf(pf_, DXTB_P_COEFF + g.tj * DXTB_MAXPRIM + p2);
      const double oij = 1.0 / (a + bb), x2p = 0.5 * oij;
      const double sij = exp(-a * bb * oij * r2) * (kPi * sqrt(kPi)) * oij * sqrt(oij) * ca * cb;
      // T[x][c][e] (bra power 0) and dT[x][c][e] = 2 alpha T(bra power 1):
      // E[0][0] = {1}, E[1][0] = {xpa, x2p}, E[0][1] = {xpb, x2p},
      // E[1][1] = {xpb xpa + x2p, xpb x2p + x2p xpa, x2p^2}, moments about B
      double T[3][2][3], dT[3][2][3];
#pragma unroll
      for (int x = 0; x < 3; ++x) {
        const double Pc = (a * g.A[x] + bb * g.B[x]) * oij;
        const double xpa = Pc - g.A[x], xpb = Pc - g.B[x];
        const double m10 = xpb, m20 = xpb * xpb + x2p, m21 = 2.0 * xpb;
        const double pref = x == 0 ? sij : 1.0;
        T[x][0][0] = pref * 1.0;
        T[x][0][1] = MP ? pref * (m10 * 1.0 + 0.0) : 0.0;
        T[x][0][2] = MP ? pref * (m20 * 1.0 + m21 * 0.0 + 2.0 * 0.0) : 0.0;
        dT[x][0][0] = pref * (2.0 * a * xpa);
        dT[x][0][1] = MP ? pref * (2.0 * a * (m10 * xpa + x2p)) : 0.0;
        dT[x][0][2] = MP ? pref * (2.0 * a * (m20 * xpa + m21 * x2p + 2.0 * 0.0)) : 0.0;
        if (LB == 1) {
          const double e0 = xpb * xpa + x2p, e1 = xpb * x2p + x2p * xpa, e2 = x2p * x2p;
          T[x][1][0] = pref * xpb;
          T[x][1][1] = MP ? pref * (m10 * xpb + x2p) : 0.0;
          T[x][1][2] = MP ? pref * (m20 * xpb + m21 * x2p + 2.0 * 0.0) : 0.0;
          dT[x][1][0] = pref * (2.0 * a * e0);
          dT[x][1][1] = MP ? pref * (2.0 * a * (m10 * e0 + e1)) : 0.0;
          dT[x][1][2] = MP ? pref * (2.0 * a * (m20 * e0 + m21 * e1 + 2.0 * e2)) : 0.0;
        }
      }
#pragma unroll
      for (int cb_ = 0; cb_ < NSB; ++cb_) {
        // p order (y, z, x): component cb_ raises axis (cb_ + 1) % 3
        const int px = LB == 1 && cb_ == 2, py = LB == 1 && cb_ == 0, pz = LB == 1 && cb_ == 1;
#pragma unroll
        for (int comp = 0; comp < NC; ++comp) {
          const int ex = comp == 1 ? 1 : (comp == 4 ? 2 : (comp == 5 || comp == 6 ? 1 : 0));
          const int ey = comp == 2 ? 1 : (comp == 7 ? 2 : (comp == 5 || comp == 8 ? 1 : 0));
          const int ez = comp == 3 ? 1 : (comp == 9 ? 2 : (comp == 6 || comp == 8 ? 1 : 0));
          const double coef = es[cb_][comp];
          const double Tx = T[0][px][ex], Ty = T[1][py][ey], Tz = T[2][pz][ez];
          gx = fma(coef, dT[0][px][ex] * Ty * Tz, gx);
          gy = fma(coef, Tx * dT[1][py][ey] * Tz, gy);
          gz = fma(coef, Tx * Ty * dT[2][pz][ez], gz);
        }
      }
    }
  }
  gx += gconst[0];
  gy += gconst[1];
  gz += gconst[2];
  const double dEdR = 2.0 * ps * h * dpi / pi;
  const double u[3] = {-d[0] / dist, -d[1] / dist, -d[2] / dist};
  const double gv[3] = {gx + dEdR * u[0], gy + dEdR * u[1], gz + dEdR * u[2]};
#pragma unroll
  for (int x = 0; x < 3; ++x) {
    atomicAdd(&grad[3 * A0 + x], gv[x]);
    atomicAdd(&grad[3 * B0 + x], -gv[x]);
  }
}

template <int NC>
__global__ void __launch_bounds__(128)
    k_grad_pairs_sp(dxtb_batch b, const double *__restrict__ pf_, const int32_t *__restrict__ pi_tab,
                    const double *__restrict__ cn, const double *__restrict__ P,
                    const double *__restrict__ W, const double *__restrict__ S,
                    const double *__restrict__ D, const double *__restrict__ vorb,
                    const double *__restrict__ vdp, const double *__restrict__ vqp,
                    double *__restrict__ dedcn, double *__restrict__ grad, ClassFilter flt) {
  const int64_t npairs = b.pair_off[b.nmol];
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < npairs;
       k += (int64_t)gridDim.x * blockDim.x) {
    GPair g;
    g.m = find_mol(b.pair_off, b.nmol, k);
    if (flt.cls >= 0 && !in_class(flt, b, g.m)) continue;
    const int64_t t = k - b.pair_off[g.m];
    int i = (int)((sqrtf(8.0f * (float)t + 1.0f) - 1.0f) * 0.5f);
    while ((int64_t)(i + 1) * (i + 2) / 2 <= t) ++i;
    while ((int64_t)i * (i + 1) / 2 > t) --i;
    int j = (int)(t - (int64_t)i * (i + 1) / 2);
    const int64_t s0 = b.shell_off[g.m];
    g.a0 = b.atom_off[g.m];
    int ti = b.shell_type[s0 + i], tj = b.shell_type[s0 + j];
    int la = pi_(pi_tab, DXTB_I_L + ti), lb = pi_(pi_tab, DXTB_I_L + tj);
    if (!gsp_class(la, lb)) continue;
    if (la == 1) {  // evaluate the s-p mirror: the s shell on the bra
      const int ii = i, tt = ti;
      i = j;
      j = ii;
      ti = tj;
      tj = tt;
      la = 0;
      lb = 1;
    }
    g.i = i;
    g.j = j;
    g.gi = s0 + i;
    g.gj = s0 + j;
    g.ti = ti;
    g.tj = tj;
    g.la = la;
    g.lb = lb;
    g.ai = b.shell_atom[g.gi];
    g.aj = b.shell_atom[g.gj];
#pragma unroll
    for (int x = 0; x < 3; ++x) {
      g.A[x] = b.positions[3 * (g.a0 + g.ai) + x];
      g.B[x] = b.positions[3 * (g.a0 + g.aj) + x];
    }
    g.na = pi_(pi_tab, DXTB_I_NPRIM + ti);
    g.nb = pi_(pi_tab, DXTB_I_NPRIM + tj);
    if (lb == 0)
      grad_pair_sp<0, NC>(b, pf_, pi_tab, cn, P, W, S, D, vorb, vdp, vqp, dedcn, grad, g);
    else
      grad_pair_sp<1, NC>(b, pf_, pi_tab, cn, P, W, S, D, vorb, vdp, vqp, dedcn, grad, g);
  }
}

__device__ __forceinline__ double exp_count_d(double r, double r0, double k, double *dc) {
  const double c = 1.0 / (1.0 + exp(-k * (r0 / r - 1.0)));
  *dc = -c * (1.0 - c) * k * r0 / (r * r);
  return c;
}

// Per molecule: ES2, AES2, repulsion, then the coordination-number chain rule.
__global__ void k_grad_mol(dxtb_batch b, const double *__restrict__ pf_,
                           const int32_t *__restrict__ pi_tab, const double *__restrict__ cn,
                           const double *__restrict__ mrad, const double *__restrict__ q,
                           const double *__restrict__ dp, const double *__restrict__ qp,
                           int multipole, double *__restrict__ dedcn, double *__restrict__ grad,
                           ClassFilter flt) {
  extern __shared__ double sm[];
  const int m = blockIdx.x;
  if (!in_class(flt, b, m)) return;
  const int64_t a0 = b.atom_off[m], s0 = b.shell_off[m], o0 = b.ao_off[m];
  const int nat = (int)(b.atom_off[m + 1] - a0), nsh = (int)(b.shell_off[m + 1] - s0);
  const int cn_kind = pi_(pi_tab, DXTB_I_SCAL + DXTB_IS_CN_KIND);
  double *qsh = sm;              // [nsh]
  double *qat = qsh + nsh;       // [nat]
  double *dmr = qat + nat;       // [nat] dE/d mrad
  int *sfirst = reinterpret_cast<int *>(dmr + nat);  // [nat + 1] first shell of each atom
  for (int s = threadIdx.x; s < nsh; s += blockDim.x) {
    const int t = b.shell_type[s0 + s];
    const int o = b.shell_ao[s0 + s], no = 2 * pi_(pi_tab, DXTB_I_L + t) + 1;
    double v = 0.0;
    for (int k = 0; k < no; ++k) v += q[o0 + o + k];
    qsh[s] = v;
  }
  for (int i = threadIdx.x; i < nat; i += blockDim.x) dmr[i] = 0.0;
  if (threadIdx.x == 0) {
    int s = 0;
    for (int i = 0; i < nat; ++i) {
      sfirst[i] = s;
      while (s < nsh && b.shell_atom[s0 + s] == i) ++s;
    }
    sfirst[nat] = nsh;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nat; i += blockDim.x) {
    double v = 0.0;
    for (int s = sfirst[i]; s < sfirst[i + 1]; ++s) v += qsh[s];
    qat[i] = v;
  }
  __syncthreads();
  const double gexp = pf(pf_, DXTB_P_SCAL + DXTB_S_GEXP);
  const int avg_kind = pi_(pi_tab, DXTB_I_SCAL + DXTB_IS_AVERAGE);
  const double kexp = pf(pf_, DXTB_P_SCAL + DXTB_S_REP_KEXP);
  const double klight = pf(pf_, DXTB_P_SCAL + DXTB_S_REP_KLIGHT);
  const double rcut = pf(pf_, DXTB_P_SCAL + DXTB_S_REP_CUTOFF);
  const double dmp3 = pf(pf_, DXTB_P_SCAL + DXTB_S_DMP3), dmp5 = pf(pf_, DXTB_P_SCAL + DXTB_S_DMP5);

  // atom i accumulates d/dR_i of every ordered pair (i, j) and (j, i)
  for (int i = threadIdx.x; i < nat; i += blockDim.x) {
    const double *pa = b.positions + 3 * (a0 + i);
    const int zi = b.numbers[a0 + i];
    double gi[3] = {0.0, 0.0, 0.0};
    double dmr_i = 0.0;
    for (int j = 0; j < nat; ++j) {
      if (j == i) continue;
      const double *pb = b.positions + 3 * (a0 + j);
      const int zj = b.numbers[a0 + j];
      const double r[3] = {pa[0] - pb[0], pa[1] - pb[1], pa[2] - pb[2]};
      const double R = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
      double dEdR = 0.0;
      // ES2 (coulomb/secondorder.py:799-872): E = 1/2 q gamma q
      for (int si = sfirst[i]; si < sfirst[i + 1]; ++si) {
        const int ti = b.shell_type[s0 + si];
        const double hi = pf(pf_, DXTB_P_LGAM + ti) * pf(pf_, DXTB_P_GAM + zi) + kEps;
        for (int sj = sfirst[j]; sj < sfirst[j + 1]; ++sj) {
          const int tj = b.shell_type[s0 + sj];
          const double hj = pf(pf_, DXTB_P_LGAM + tj) * pf(pf_, DXTB_P_GAM + zj) + kEps;
          double avg;
          if (avg_kind == 0) avg = 2.0 / (1.0 / hi + 1.0 / hj);
          else if (avg_kind == 1) avg = 0.5 * (hi + hj);
          else avg = sqrt(hi * hj);
          const double re = R + kEps;
          const double dg = gexp == 2.0 ? re * re : pow(re, gexp);
          const double tmp = dg + (gexp == 2.0 ? 1.0 / (avg * avg) : pow(avg, -gexp));
          const double dgam = -pow(tmp, -1.0 / gexp - 1.0) * (gexp == 2.0 ? re : pow(re, gexp - 1.0));
          dEdR += qsh[si] * qsh[sj] * dgam;  // both orderings: 2 * 1/2
        }
      }
      // repulsion (classicals/repulsion/base.py:351-430)
      if (R <= rcut) {
        const double a = sqrt(pf(pf_, DXTB_P_AREP + zi) * pf(pf_, DXTB_P_AREP + zj) + kTiny);
        const double k = (klight >= 0.0 && zi <= 2 && zj <= 2) ? klight : kexp;
        const double rk = pow(R, k);
        const double e = pf(pf_, DXTB_P_ZEFF + zi) * pf(pf_, DXTB_P_ZEFF + zj) * exp(-a * rk) / R;
        dEdR += -(a * rk * k + 1.0) * e / R;
      }
      for (int x = 0; x < 3; ++x) gi[x] += dEdR * r[x] / R;
      // AES2 pair terms e_ij + e_ji (coulomb/multipole.py:373-640)
      if (multipole) {
        const double M = 0.5 * (mrad[a0 + i] + mrad[a0 + j]);
        const double rr = M / R;
        const double r3d = pow(rr, dmp3), r5d = pow(rr, dmp5);
        const double f3 = 1.0 / (1.0 + 6.0 * r3d), f5 = 1.0 / (1.0 + 6.0 * r5d);
        const double df3 = f3 * f3 * 6.0 * dmp3 * r3d / R, df5 = f5 * f5 * 6.0 * dmp5 * r5d / R;
        const double df3M = -f3 * f3 * 6.0 * dmp3 * r3d / M, df5M = -f5 * f5 * 6.0 * dmp5 * r5d / M;
        const double iR = 1.0 / R, iR3 = iR * iR * iR, iR5 = iR3 * iR * iR;
        const double h3 = iR3 * f3, dh3 = -3.0 * iR3 * iR * f3 + iR3 * df3;
        const double dk3 = -3.0 * iR3 * iR * f5 + iR3 * df5;  // d/dR of k3 = f5 / R^3
        const double k5 = iR5 * f5, dk5 = -5.0 * iR5 * iR * f5 + iR5 * df5;
        double gr[3] = {0.0, 0.0, 0.0};
        double dM = 0.0;
        // two orderings: (i, j) with vector r and (j, i) with -r
        for (int ord = 0; ord < 2; ++ord) {
          const int I = ord == 0 ? i : j, J = ord == 0 ? j : i;
          const double sgn = ord == 0 ? 1.0 : -1.0;
          const double rv[3] = {sgn * r[0], sgn * r[1], sgn * r[2]};
          const double qI = qat[I];
          const double *u = dp + 3 * (a0 + J), *av = dp + 3 * (a0 + I);
          const double *wq = qp + 6 * (a0 + J);
          const double ru = rv[0] * u[0] + rv[1] * u[1] + rv[2] * u[2];
          const double ra = rv[0] * av[0] + rv[1] * av[1] + rv[2] * av[2];
          const double ab = av[0] * u[0] + av[1] * u[1] + av[2] * u[2];
          const double Wm[3][3] = {{wq[0], wq[1], wq[3]}, {wq[1], wq[2], wq[4]}, {wq[3], wq[4], wq[5]}};
          double Wr[3];
          for (int x = 0; x < 3; ++x) Wr[x] = Wm[x][0] * rv[0] + Wm[x][1] * rv[1] + Wm[x][2] * rv[2];
          const double rWr = rv[0] * Wr[0] + rv[1] * Wr[1] + rv[2] * Wr[2];
          double gv[3];
          for (int x = 0; x < 3; ++x) {
            // A: q_I (r.u) h3
            double v = qI * (u[x] * h3 + ru * dh3 * rv[x] * iR);
            // B: 1/2 [(a.b) k3 - 3 (r.a)(r.b) k5]
            v += 0.5 * (ab * dk3 * rv[x] * iR - 3.0 * (av[x] * ru + u[x] * ra) * k5 -
                        3.0 * ra * ru * dk5 * rv[x] * iR);
            // C: q_I (r W r) k5
            v += qI * (2.0 * Wr[x] * k5 + rWr * dk5 * rv[x] * iR);
            gv[x] = v;
          }
          // d e / d r (r = R_I - R_J); atom i gets +gv for ord 0, -gv for ord 1 (r = R_j - R_i)
          for (int x = 0; x < 3; ++x) gr[x] += sgn * gv[x];
          dM += qI * ru * iR3 * df3M + 0.5 * (ab * iR3 - 3.0 * ra * ru * iR5) * df5M + qI * rWr * iR5 * df5M;
        }
        for (int x = 0; x < 3; ++x) gi[x] += gr[x];
        dmr_i += 0.5 * dM;  // e_ij and e_ji both depend on M = (m_i + m_j) / 2
      }
    }
    for (int x = 0; x < 3; ++x) atomicAdd(&grad[3 * (a0 + i) + x], gi[x]);
    if (multipole) dmr[i] = dmr_i;
  }
  __syncthreads();
  // AES2 damping radius -> dE/dCN (coulomb/multipole.py:330-335)
  if (multipole) {
    const double kx = pf(pf_, DXTB_P_SCAL + DXTB_S_MP_KEXP), sh = pf(pf_, DXTB_P_SCAL + DXTB_S_MP_SHIFT);
    const double rmax = pf(pf_, DXTB_P_SCAL + DXTB_S_MP_RMAX);
    for (int i = threadIdx.x; i < nat; i += blockDim.x) {
      const int z = b.numbers[a0 + i];
      const double rad = pf(pf_, DXTB_P_MPRAD + z), vcn = pf(pf_, DXTB_P_MPVCN + z);
      const double t1 = exp(-kx * (cn[a0 + i] - vcn - sh));
      const double dmdcn = (rmax - rad) * kx * t1 / ((1.0 + t1) * (1.0 + t1));
      atomicAdd(&dedcn[a0 + i], dmr[i] * dmdcn);
    }
  }
  __syncthreads();
  // coordination number chain rule (tad_mctc cn_d3 restated)
  const double cutoff = pf(pf_, DXTB_P_SCAL + DXTB_S_CN_CUTOFF);
  for (int i = threadIdx.x; i < nat; i += blockDim.x) {
    const double *pa = b.positions + 3 * (a0 + i);
    const double rci = pf(pf_, DXTB_P_RCOV + b.numbers[a0 + i]);
    const double di = dedcn[a0 + i];
    double gi[3] = {0.0, 0.0, 0.0};
    for (int j = 0; j < nat; ++j) {
      if (j == i) continue;
      const double *pb = b.positions + 3 * (a0 + j);
      const double r[3] = {pa[0] - pb[0], pa[1] - pb[1], pa[2] - pb[2]};
      const double R = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
      if (R > cutoff) continue;
      const double r0 = rci + pf(pf_, DXTB_P_RCOV + b.numbers[a0 + j]);
      double dc;
      if (cn_kind == 0) {
        exp_count_d(R, r0, 16.0, &dc);
      } else {
        double d1, d2;
        const double c1 = exp_count_d(R, r0, 10.0, &d1);
        const double c2 = exp_count_d(R, r0 + 2.0, 20.0, &d2);
        dc = d1 * c2 + c1 * d2;
      }
      const double f = (di + dedcn[a0 + j]) * dc / R;
      for (int x = 0; x < 3; ++x) gi[x] += f * r[x];
    }
    for (int x = 0; x < 3; ++x) atomicAdd(&grad[3 * (a0 + i) + x], gi[x]);
  }
}

}  // namespace dxtb

using namespace dxtb;

constexpr size_t gSmem = sizeof(double) * gWarps * (gChunk * gTab + 2 * gNComp * 36);

namespace dxtb {

int32_t launch_gradient(const dxtb_batch *b, const double *par_f, const int32_t *par_i,
                        const double *cn, const double *mrad, const double *density,
                        const double *wdensity, const double *q, const double *dp, const double *qp,
                        const double *vorb, const double *vdp, const double *vqp,
                        const double *overlap, const double *dipole, double *dedcn, double *grad,
                        const ClassFilter &f, cudaStream_t st) {
  if (!b || b->nmol <= 0 || !cn || !density || !wdensity || !q || !vorb || !overlap || !dedcn ||
      !grad)
    return DXTB_ERR_ARGS;
  // The multipole (GFN2) terms are taken iff the dipole integrals are given.
  const int multipole = dipole != nullptr;
  if (multipole && (!vdp || !vqp || !dp || !qp || !mrad)) return DXTB_ERR_ARGS;
  static PerDeviceOnce attr;
  if (per_device_once(attr, [] {
        return cudaFuncSetAttribute(k_grad_pairs, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)gSmem) == cudaSuccess;
      }) != DXTB_OK)
    return DXTB_ERR_LAUNCH;
  const int64_t bound = (int64_t)b->nmol * b->max_nsh * (b->max_nsh + 1) / 2;
  if (bound > 0) {
    int sms = 0;
    if (device_sms(&sms) != DXTB_OK) return DXTB_ERR_LAUNCH;
    const int64_t blocks = min((bound + gWarps - 1) / gWarps, (int64_t)sms * 16);
    k_grad_pairs<<<(unsigned)blocks, gWarps * 32, gSmem, st>>>(*b, par_f, par_i, cn, density, wdensity,
                                                               overlap, dipole, vorb, vdp, vqp, multipole,
                                                               dedcn, grad, f);
    DXTB_CHECK_LAUNCH();
    // s-s and s-p pairs: a thread each
    const int64_t tblocks = min((bound + 127) / 128, (int64_t)sms * 16);
    if (multipole)
      k_grad_pairs_sp<gNComp><<<(unsigned)tblocks, 128, 0, st>>>(*b, par_f, par_i, cn, density, wdensity,
                                                                 overlap, dipole, vorb, vdp, vqp, dedcn,
                                                                 grad, f);
    else
      k_grad_pairs_sp<1><<<(unsigned)tblocks, 128, 0, st>>>(*b, par_f, par_i, cn, density, wdensity, overlap,
                                                            dipole, vorb, vdp, vqp, dedcn, grad, f);
    DXTB_CHECK_LAUNCH();
  }
  const size_t smem = sizeof(double) * (size_t)(b->max_nsh + 3 * b->max_nat + 8);
  if (smem > 200 * 1024) return DXTB_ERR_TOO_LARGE;
  if (smem > 48 * 1024 &&
      cudaFuncSetAttribute(k_grad_mol, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return DXTB_ERR_LAUNCH;
  k_grad_mol<<<b->nmol, 128, smem, st>>>(*b, par_f, par_i, cn, mrad, q, dp, qp, multipole, dedcn, grad, f);
  DXTB_CHECK_LAUNCH();
  return DXTB_OK;
}

}  // namespace dxtb

extern "C" int32_t dxtb_gradient(const dxtb_batch *b, const double *par_f, const int32_t *par_i,
                                 const double *cn, const double *cn_mp, const double *mrad,
                                 const double *density, const double *wdensity, const double *q,
                                 const double *dp, const double *qp, const double *vorb,
                                 const double *vdp, const double *vqp, const double *overlap,
                                 const double *dipole, const double *unused0,
                                 const double *unused1, double *dedcn, double *dedcn_mp,
                                 double *grad, void *stream) {
  (void)cn_mp;
  (void)unused0;
  (void)unused1;
  (void)dedcn_mp;
  ClassFilter all;
  for (int c = 0; c < kClasses; ++c) all.thr[c] = 0;
  all.cls = -1;
  return launch_gradient(b, par_f, par_i, cn, mrad, density, wdensity, q, dp, qp, vorb, vdp, vqp,
                         overlap, dipole, dedcn, grad, all, (cudaStream_t)stream);
}
