// Molecular properties of converged single points (packed batches).
//
// dxtb_dipole_moment: the electric dipole moment of every molecule,
// mu = sum_mu n0_mu R_atom(mu) - sum_{mu nu} P_{mu nu} <mu| r |nu>, with the
// reference occupations n0 summing to the valence charge of each atom and
// the normalised dipole integral about the origin (calculators/properties/
// moments/dip.py, dipole_xtb). One CTA per molecule; the n^2 contraction
// reads P and the three integral components once, coalesced (HBM bound).

#include "common.cuh"

namespace dxtb {

constexpr int kDipThreads = 256;

__global__ void __launch_bounds__(kDipThreads)
k_dipole_moment(dxtb_batch b, const double *__restrict__ n0, const double *__restrict__ density,
                const double *__restrict__ dip0, double *__restrict__ out) {
  __shared__ double red[32];
  const int m = blockIdx.x;
  const int64_t a0 = b.ao_off[m], n = b.ao_off[m + 1] - a0;
  const int64_t m0 = b.mat_off[m], nn = n * n;
  const int64_t mat = b.mat_off[b.nmol];
  const int64_t at0 = b.atom_off[m], sh0 = b.shell_off[m];
  double e[3] = {0.0, 0.0, 0.0};
  for (int64_t i = threadIdx.x; i < nn; i += blockDim.x) {
    const double p = density[m0 + i];
    e[0] = fma(p, dip0[m0 + i], e[0]);
    e[1] = fma(p, dip0[mat + m0 + i], e[1]);
    e[2] = fma(p, dip0[2 * mat + m0 + i], e[2]);
  }
  double c[3] = {0.0, 0.0, 0.0};
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
    const int64_t at = at0 + b.shell_atom[sh0 + b.ao_shell[a0 + i]];
    const double z = n0[a0 + i];
    for (int k = 0; k < 3; ++k) c[k] = fma(z, b.positions[3 * at + k], c[k]);
  }
  for (int k = 0; k < 3; ++k) {
    const double v = block_sum(c[k] - e[k], red);
    if (threadIdx.x == 0) out[3 * m + k] = v;
  }
}

}  // namespace dxtb

using namespace dxtb;

extern "C" int32_t dxtb_dipole_moment(const dxtb_batch *b, const double *n0,
                                      const double *density, const double *dipole_origin,
                                      double *dipole, void *stream) {
  if (!b || b->nmol <= 0 || !n0 || !density || !dipole_origin || !dipole) return DXTB_ERR_ARGS;
  k_dipole_moment<<<b->nmol, kDipThreads, 0, (cudaStream_t)stream>>>(*b, n0, density,
                                                                      dipole_origin, dipole);
  DXTB_CHECK_LAUNCH();
  return DXTB_OK;
}
