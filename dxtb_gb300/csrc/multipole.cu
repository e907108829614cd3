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
  int i = (int)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
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

// mode 0: GFN (S + H0 [+ D, Q ket-centred traceless]); mode 1: raw about origin.
template <int MODE>
__global__ void __launch_bounds__(kWarps * 32)
    k_multipole(dxtb_batch b, const double *__restrict__ pf_, const int32_t *__restrict__ pi_tab,
                const double *__restrict__ cn, int ncomp_req,
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

    double hfac = 0.0;
    if (MODE == 0 && H != nullptr) {
      const int zi = b.numbers[g.a0 + g.ai], zj = b.numbers[g.a0 + g.aj];
      const double sei = pf(pf_, DXTB_P_LEVEL + g.ti) - pf(pf_, DXTB_P_KCN + g.ti) * cn[g.a0 + g.ai];
      const double sej = pf(pf_, DXTB_P_LEVEL + g.tj) - pf(pf_, DXTB_P_KCN + g.tj) * cn[g.a0 + g.aj];
      hfac = 0.5 * (sei + sej);
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
    }

    const double d[3] = {g.B[0] - g.A[0], g.B[1] - g.A[1], g.B[2] - g.A[2]};  // B - A
    for (int o = lane; o < nsa * nsb; o += 32) {
      const int ma = o / nsb, mb = o % nsb;
      const double *v = &s_sph[w][o * ncomp];
      const int mu = oi + ma, nu = oj + mb;
      const int64_t e1 = moff + (int64_t)mu * n + nu, e2 = moff + (int64_t)nu * n + mu;
      const double s = v[0];
      S[e1] = s;
      S[e2] = s;
      if (MODE == 0 && H != nullptr) {
        H[e1] = hfac * s;
        H[e2] = hfac * s;
      }
      if (ncomp > 1) {
        if (MODE == 0) {
          // ket-centred (about B) for (mu, nu); bra-centred (about A) for (nu, mu)
          double dB[3] = {v[1], v[2], v[3]};
          double qB[6] = {v[4], v[5], v[7], v[6], v[8], v[9]};  // xx xy yy xz yz zz
          double dA[3], qA[6];
          for (int x = 0; x < 3; ++x) dA[x] = dB[x] + d[x] * s;
          const int qa[6] = {0, 0, 1, 0, 1, 2}, qb[6] = {0, 1, 1, 2, 2, 2};
          for (int c = 0; c < 6; ++c) {
            const int x = qa[c], y = qb[c];
            qA[c] = qB[c] + d[y] * dB[x] + d[x] * dB[y] + d[x] * d[y] * s;
          }
          for (int x = 0; x < 3; ++x) {
            D[x * mtot + e1] = dB[x];
            D[x * mtot + e2] = dA[x];
          }
          const double trB = 0.5 * (qB[0] + qB[2] + qB[5]);
          const double trA = 0.5 * (qA[0] + qA[2] + qA[5]);
          for (int c = 0; c < 6; ++c) {
            const bool diag = (c == 0 || c == 2 || c == 5);
            Q[c * mtot + e1] = 1.5 * qB[c] - (diag ? trB : 0.0);
            Q[c * mtot + e2] = 1.5 * qA[c] - (diag ? trA : 0.0);
          }
        } else {
          for (int x = 0; x < 3; ++x) {
            D[x * mtot + e1] = v[1 + x];
            D[x * mtot + e2] = v[1 + x];
          }
          // raw 9 components, row-major (xx, xy, xz, yx, yy, yz, zx, zy, zz)
          const double q9[9] = {v[4], v[5], v[6], v[5], v[7], v[8], v[6], v[8], v[9]};
          for (int c = 0; c < 9; ++c) {
            Q[c * mtot + e1] = q9[c];
            Q[c * mtot + e2] = q9[c];
          }
        }
      }
    }
    __syncwarp();  // the next pair reuses this warp's shared tables
  }
}

}  // namespace dxtb

using namespace dxtb;

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
  if (mode == 0)
    k_multipole<0><<<(unsigned)blocks, kWarps * 32, kSmem, st>>>(*b, par_f, par_i, cn, ncomp, S, H, D, Q);
  else
    k_multipole<1><<<(unsigned)blocks, kWarps * 32, kSmem, st>>>(*b, par_f, par_i, cn, ncomp, S, nullptr,
                                                             D, Q);
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
