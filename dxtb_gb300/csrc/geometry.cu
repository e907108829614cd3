// Geometry-only terms of the GFN-xTB single point: coordination numbers and
// the interaction caches that stay fixed during the SCF (ES2 gamma, ES3
// Hubbard derivatives, AES2 damping radii and kernels, repulsion energy).
// One CTA per molecule; threads stride over atom or shell pairs.
#include "common.cuh"

namespace dxtb {

// D3-type counting functions (tad_mctc exp_count / gfn2_count restated from
// Grimme et al., JCP 132, 154104 (2010) and the GFN2-xTB paper).
__device__ __forceinline__ double exp_count(double r, double r0, double k) {
  return 1.0 / (1.0 + exp(-k * (r0 / r - 1.0)));
}

__device__ __forceinline__ double count_fn(int kind, double r, double r0) {
  if (kind == 0) return exp_count(r, r0, 16.0);
  return exp_count(r, r0, 10.0) * exp_count(r, r0 + 2.0, 20.0);
}

__global__ void k_coordination_number(dxtb_batch b, const double *__restrict__ pf_,
                                      int kind, double *__restrict__ cn) {
  const int m = blockIdx.x;
  const int64_t a0 = b.atom_off[m];
  const int nat = (int)(b.atom_off[m + 1] - a0);
  const double cutoff = pf(pf_, DXTB_P_SCAL + DXTB_S_CN_CUTOFF);
  for (int i = threadIdx.x; i < nat; i += blockDim.x) {
    const double *pi = b.positions + 3 * (a0 + i);
    const double rci = pf(pf_, DXTB_P_RCOV + b.numbers[a0 + i]);
    double s = 0.0;
    for (int j = 0; j < nat; ++j) {
      if (j == i) continue;
      const double *pj = b.positions + 3 * (a0 + j);
      const double dx = pi[0] - pj[0], dy = pi[1] - pj[1], dz = pi[2] - pj[2];
      const double r = sqrt(dx * dx + dy * dy + dz * dz);
      if (r > cutoff) continue;
      s += count_fn(kind, r, rci + pf(pf_, DXTB_P_RCOV + b.numbers[a0 + j]));
    }
    cn[a0 + i] = s;
  }
}

__device__ __forceinline__ double powg(double x, double g) {
  return g == 2.0 ? x * x : pow(x, g);
}

__global__ void k_interaction_cache(dxtb_batch b, const double *__restrict__ pf_,
                                    const int32_t *__restrict__ pi_tab,
                                    const double *__restrict__ cn_mp,
                                    double *__restrict__ gamma, double *__restrict__ hd,
                                    double *__restrict__ mrad, double *__restrict__ amat_sd,
                                    double *__restrict__ amat_dd, double *__restrict__ amat_sq,
                                    double *__restrict__ erep) {
  extern __shared__ double sm[];
  const int m = blockIdx.x;
  const int64_t a0 = b.atom_off[m], s0 = b.shell_off[m];
  const int nat = (int)(b.atom_off[m + 1] - a0);
  const int nsh = (int)(b.shell_off[m + 1] - s0);
  const int64_t g0 = b.nsh2_off[m], n2off = b.nat2_off[m], n2tot = b.nat2_off[b.nmol];
  const int avg_kind = pi_(pi_tab, DXTB_I_SCAL + DXTB_IS_AVERAGE);
  const int es3_shell = pi_(pi_tab, DXTB_I_SCAL + DXTB_IS_ES3_SHELL);
  const int multipole = pi_(pi_tab, DXTB_I_SCAL + DXTB_IS_MULTIPOLE);
  const double gexp = pf(pf_, DXTB_P_SCAL + DXTB_S_GEXP);

  // ---- ES2 gamma, shell resolved (coulomb/secondorder.py:799-872) ----
  for (int64_t t = threadIdx.x; t < (int64_t)nsh * nsh; t += blockDim.x) {
    const int i = (int)(t / nsh), j = (int)(t % nsh);
    const int ti = b.shell_type[s0 + i], tj = b.shell_type[s0 + j];
    const int ai = b.shell_atom[s0 + i], aj = b.shell_atom[s0 + j];
    const double hi = pf(pf_, DXTB_P_LGAM + ti) * pf(pf_, DXTB_P_GAM + b.numbers[a0 + ai]) + kEps;
    const double hj = pf(pf_, DXTB_P_LGAM + tj) * pf(pf_, DXTB_P_GAM + b.numbers[a0 + aj]) + kEps;
    double avg;
    if (avg_kind == 0) avg = 2.0 / (1.0 / hi + 1.0 / hj);
    else if (avg_kind == 1) avg = 0.5 * (hi + hj);
    else avg = sqrt(hi * hj);
    double dg;
    if (ai == aj) {
      dg = kEps;
    } else {
      const double *pa = b.positions + 3 * (a0 + ai), *pb = b.positions + 3 * (a0 + aj);
      const double dx = pa[0] - pb[0], dy = pa[1] - pb[1], dz = pa[2] - pb[2];
      dg = powg(sqrt(dx * dx + dy * dy + dz * dz) + kEps, gexp);
    }
    const double tmp = dg + powg(avg, -gexp);
    gamma[g0 + t] = gexp == 2.0 ? 1.0 / sqrt(tmp) : 1.0 / pow(tmp, 1.0 / gexp);
  }

  // ---- ES3 Hubbard derivatives (coulomb/thirdorder.py get_cache) ----
  if (es3_shell) {
    for (int i = threadIdx.x; i < nsh; i += blockDim.x) {
      const int ti = b.shell_type[s0 + i];
      const int l = pi_(pi_tab, DXTB_I_L + ti);
      hd[s0 + i] = pf(pf_, DXTB_P_GAM3 + b.numbers[a0 + b.shell_atom[s0 + i]]) *
                   pf(pf_, DXTB_P_ES3SCALE + l);
    }
  } else {
    for (int i = threadIdx.x; i < nat; i += blockDim.x)
      hd[a0 + i] = pf(pf_, DXTB_P_GAM3 + b.numbers[a0 + i]);
  }

  // ---- AES2 damping radii (coulomb/multipole.py:323-335) ----
  double *smrad = sm;  // [nat]
  if (multipole) {
    const double kexp = pf(pf_, DXTB_P_SCAL + DXTB_S_MP_KEXP);
    const double shift = pf(pf_, DXTB_P_SCAL + DXTB_S_MP_SHIFT);
    const double rmax = pf(pf_, DXTB_P_SCAL + DXTB_S_MP_RMAX);
    for (int i = threadIdx.x; i < nat; i += blockDim.x) {
      const int z = b.numbers[a0 + i];
      const double rad = pf(pf_, DXTB_P_MPRAD + z), vcn = pf(pf_, DXTB_P_MPVCN + z);
      const double t1 = exp(-kexp * (cn_mp[a0 + i] - vcn - shift));
      const double r = rad + (rmax - rad) / (1.0 + t1);
      smrad[i] = r;
      mrad[a0 + i] = r;
    }
  }
  __syncthreads();

  // ---- AES2 interaction matrices (coulomb/multipole.py:373-448) ----
  if (multipole) {
    const double dmp3 = pf(pf_, DXTB_P_SCAL + DXTB_S_DMP3);
    const double dmp5 = pf(pf_, DXTB_P_SCAL + DXTB_S_DMP5);
    for (int64_t t = threadIdx.x; t < (int64_t)nat * nat; t += blockDim.x) {
      const int i = (int)(t / nat), j = (int)(t % nat);
      const int64_t o = n2off + t;
      if (i == j) {
        for (int c = 0; c < 3; ++c) amat_sd[c * n2tot + o] = 0.0;
        for (int c = 0; c < 9; ++c) amat_dd[c * n2tot + o] = 0.0;
        for (int c = 0; c < 6; ++c) amat_sq[c * n2tot + o] = 0.0;
        continue;
      }
      const double *pa = b.positions + 3 * (a0 + i), *pb = b.positions + 3 * (a0 + j);
      const double r[3] = {pa[0] - pb[0], pa[1] - pb[1], pa[2] - pb[2]};
      const double dist = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
      const double g1 = 1.0 / dist, g3 = g1 * g1 * g1, g5 = g3 * g1 * g1;
      const double rr = 0.5 * (smrad[i] + smrad[j]) * g1;
      const double f3 = 1.0 / (1.0 + 6.0 * pow(rr, dmp3));
      const double f5 = 1.0 / (1.0 + 6.0 * pow(rr, dmp5));
      for (int c = 0; c < 3; ++c) amat_sd[c * n2tot + o] = r[c] * g3 * f3;
      const double g5f5 = g5 * f5;
      for (int x = 0; x < 3; ++x)
        for (int y = 0; y < 3; ++y)
          amat_dd[(3 * x + y) * n2tot + o] =
              (x == y ? g3 * f5 : 0.0) - r[x] * r[y] * 3.0 * g5f5;
      amat_sq[0 * n2tot + o] = r[0] * r[0] * g5f5;
      amat_sq[1 * n2tot + o] = 2.0 * r[0] * r[1] * g5f5;
      amat_sq[2 * n2tot + o] = r[1] * r[1] * g5f5;
      amat_sq[3 * n2tot + o] = 2.0 * r[0] * r[2] * g5f5;
      amat_sq[4 * n2tot + o] = 2.0 * r[1] * r[2] * g5f5;
      amat_sq[5 * n2tot + o] = r[2] * r[2] * g5f5;
    }
  }

  // ---- repulsion (classicals/repulsion/base.py:240-348, rep.py) ----
  const double kexp = pf(pf_, DXTB_P_SCAL + DXTB_S_REP_KEXP);
  const double klight = pf(pf_, DXTB_P_SCAL + DXTB_S_REP_KLIGHT);
  const double rcut = pf(pf_, DXTB_P_SCAL + DXTB_S_REP_CUTOFF);
  for (int i = threadIdx.x; i < nat; i += blockDim.x) {
    const int zi = b.numbers[a0 + i];
    const double *pa = b.positions + 3 * (a0 + i);
    double e = 0.0;
    for (int j = 0; j < nat; ++j) {
      if (j == i) continue;
      const int zj = b.numbers[a0 + j];
      const double *pb = b.positions + 3 * (a0 + j);
      const double dx = pa[0] - pb[0], dy = pa[1] - pb[1], dz = pa[2] - pb[2];
      const double r = sqrt(dx * dx + dy * dy + dz * dz);
      if (r > rcut) continue;
      const double a = sqrt(pf(pf_, DXTB_P_AREP + zi) * pf(pf_, DXTB_P_AREP + zj) + kTiny);
      const double k = (klight >= 0.0 && zi <= 2 && zj <= 2) ? klight : kexp;
      e += pf(pf_, DXTB_P_ZEFF + zi) * pf(pf_, DXTB_P_ZEFF + zj) * exp(-a * pow(r, k)) / r;
    }
    erep[a0 + i] = 0.5 * e;
  }
}

}  // namespace dxtb

using namespace dxtb;

extern "C" int32_t dxtb_coordination_number(const dxtb_batch *b, const double *par_f,
                                            const int32_t *par_i, int32_t kind,
                                            double *cn, void *stream) {
  (void)par_i;
  if (!b || b->nmol <= 0 || !cn) return DXTB_ERR_ARGS;
  k_coordination_number<<<b->nmol, 128, 0, (cudaStream_t)stream>>>(*b, par_f, kind, cn);
  DXTB_CHECK_LAUNCH();
  return DXTB_OK;
}

extern "C" int32_t dxtb_interaction_cache(const dxtb_batch *b, const double *par_f,
                                          const int32_t *par_i, const double *cn_mp,
                                          double *gamma, double *hd, double *mrad,
                                          double *amat_sd, double *amat_dd,
                                          double *amat_sq, double *erep, void *stream) {
  if (!b || b->nmol <= 0 || !gamma || !hd || !erep) return DXTB_ERR_ARGS;
  const size_t smem = sizeof(double) * (size_t)(b->max_nat > 0 ? b->max_nat : 1);
  if (smem > 48 * 1024) return DXTB_ERR_TOO_LARGE;
  k_interaction_cache<<<b->nmol, 256, smem, (cudaStream_t)stream>>>(
      *b, par_f, par_i, cn_mp, gamma, hd, mrad, amat_sd, amat_dd, amat_sq, erep);
  DXTB_CHECK_LAUNCH();
  return DXTB_OK;
}
