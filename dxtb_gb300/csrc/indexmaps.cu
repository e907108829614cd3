// IndexHelper maps on the device, bit-exact with
// IndexHelper.from_numbers_angular (basis/indexhelper.py:338-492) for a single
// molecule (batch mode 0) and a zero-padded batch (batch mode 1).
//
// Padding conventions of the reference: shells_to_ushell pads with -1; the
// shell/orbital offsets and the shells_to_atom / orbitals_to_shell maps pad
// with -999; padding atoms (Z = 0) own no shells in batch mode but keep one
// "unique shell" of angular momentum -1 in unique_angular.
#include "common.cuh"

namespace dxtb {

constexpr int64_t kPad = -999;

// Unique species and per-unique-shell maps (single CTA).
__global__ void k_index_unique(const int64_t *__restrict__ numbers, int64_t total, int batch,
                               const int32_t *__restrict__ el_nsh, const int32_t *__restrict__ el_ang,
                               int64_t *__restrict__ unique_angular,
                               int64_t *__restrict__ ushells_to_unique,
                               int64_t *__restrict__ ushells_per_unique,
                               int64_t *__restrict__ unique_out, int64_t *__restrict__ zmap /*[MAXZ*4]*/) {
  __shared__ int present[DXTB_MAXZ];
  for (int z = threadIdx.x; z < DXTB_MAXZ; z += blockDim.x) present[z] = 0;
  __syncthreads();
  for (int64_t k = threadIdx.x; k < total; k += blockDim.x) {
    const int64_t z = numbers[k];
    if (z >= 0 && z < DXTB_MAXZ) present[z] = 1;
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  // zmap[z] = unique index, zmap[MAXZ + u] = ushell offset (before zeroing),
  // zmap[2 MAXZ + u] = shell count (after batch zeroing)
  int64_t u = 0, off = 0;
  for (int z = 0; z < DXTB_MAXZ; ++z) {
    if (!present[z]) continue;
    const int nsh = el_nsh[z] > 0 ? el_nsh[z] : 1;  // unknown species: one shell of l = -1
    unique_out[u] = z;
    zmap[z] = u;
    zmap[DXTB_MAXZ + u] = off;
    for (int s = 0; s < nsh; ++s) {
      unique_angular[off + s] = el_nsh[z] > 0 ? el_ang[z * 8 + s] : -1;
      ushells_to_unique[off + s] = u;
    }
    const int64_t cnt = (batch && z == 0) ? 0 : nsh;
    ushells_per_unique[u] = cnt;
    zmap[2 * DXTB_MAXZ + u] = cnt;
    off += nsh;
    ++u;
  }
}

// Per row (molecule) maps; thread 0 runs the prefix sums, all threads fill.
__global__ void k_index_rows(const int64_t *__restrict__ numbers, int nat_max, int64_t nsh_max,
                             int64_t nao_max, const int64_t *__restrict__ unique_angular,
                             const int64_t *__restrict__ zmap, int64_t *__restrict__ angular,
                             int64_t *__restrict__ atom_to_unique,
                             int64_t *__restrict__ shells_to_ushell,
                             int64_t *__restrict__ shells_per_atom, int64_t *__restrict__ shell_index,
                             int64_t *__restrict__ shells_to_atom,
                             int64_t *__restrict__ orbitals_per_shell,
                             int64_t *__restrict__ orbital_index,
                             int64_t *__restrict__ orbitals_to_shell) {
  const int r = blockIdx.x;
  const int64_t *num = numbers + (int64_t)r * nat_max;
  int64_t *a2u = atom_to_unique + (int64_t)r * nat_max;
  int64_t *spa = shells_per_atom + (int64_t)r * nat_max;
  int64_t *sidx = shell_index + (int64_t)r * nat_max;
  int64_t *s2u = shells_to_ushell + r * nsh_max;
  int64_t *s2a = shells_to_atom + r * nsh_max;
  int64_t *ang = angular + r * nsh_max;
  int64_t *ops = orbitals_per_shell + r * nsh_max;
  int64_t *oidx = orbital_index + r * nsh_max;
  int64_t *o2s = orbitals_to_shell + r * nao_max;
  for (int a = threadIdx.x; a < nat_max; a += blockDim.x) {
    const int64_t u = zmap[num[a]];
    a2u[a] = u;
    spa[a] = zmap[2 * DXTB_MAXZ + u];
  }
  for (int64_t s = threadIdx.x; s < nsh_max; s += blockDim.x) {
    s2u[s] = -1;
    s2a[s] = kPad;
  }
  for (int64_t o = threadIdx.x; o < nao_max; o += blockDim.x) o2s[o] = kPad;
  __syncthreads();
  if (threadIdx.x == 0) {
    int64_t sh = 0;
    for (int a = 0; a < nat_max; ++a) {
      const int64_t cnt = spa[a];
      sidx[a] = cnt == 0 ? kPad : sh;
      const int64_t uoff = zmap[DXTB_MAXZ + a2u[a]];
      for (int64_t k = 0; k < cnt; ++k) {
        s2u[sh + k] = uoff + k;
        s2a[sh + k] = a;
      }
      sh += cnt;
    }
    int64_t ao = 0;
    for (int64_t s = 0; s < nsh_max; ++s) {
      const int64_t l = s2u[s] >= 0 ? unique_angular[s2u[s]] : kPad;
      ang[s] = l;
      const int64_t no = l >= 0 ? 2 * l + 1 : 0;
      ops[s] = no;
      oidx[s] = no == 0 ? kPad : ao;
      for (int64_t k = 0; k < no; ++k) o2s[ao + k] = s;
      ao += no;
    }
  }
}

}  // namespace dxtb

using namespace dxtb;

extern "C" int32_t dxtb_index_sizes(const int64_t *numbers_host, int32_t nbatch, int32_t nat_max,
                                    int32_t batch_mode, const int32_t *el_nsh_host,
                                    const int32_t *el_ang_host, int64_t *sizes_out) {
  if (!numbers_host || !el_nsh_host || !el_ang_host || !sizes_out || nbatch <= 0 || nat_max < 0)
    return DXTB_ERR_ARGS;
  const bool batch = batch_mode > 0;
  int present[DXTB_MAXZ] = {0};
  for (int64_t k = 0; k < (int64_t)nbatch * nat_max; ++k) {
    const int64_t z = numbers_host[k];
    if (z < 0 || z >= DXTB_MAXZ) return DXTB_ERR_ARGS;
    present[z] = 1;
  }
  int64_t nunique = 0, nushell = 0;
  for (int z = 0; z < DXTB_MAXZ; ++z)
    if (present[z]) {
      ++nunique;
      nushell += el_nsh_host[z] > 0 ? el_nsh_host[z] : 1;
    }
  int64_t nsh_max = 0, nao_max = 0;
  for (int r = 0; r < nbatch; ++r) {
    int64_t nsh = 0, nao = 0;
    for (int a = 0; a < nat_max; ++a) {
      const int64_t z = numbers_host[(int64_t)r * nat_max + a];
      if (batch && z == 0) continue;
      const int ns = el_nsh_host[z] > 0 ? el_nsh_host[z] : 1;
      nsh += ns;
      for (int s = 0; s < ns && el_nsh_host[z] > 0; ++s) nao += 2 * el_ang_host[z * 8 + s] + 1;
    }
    if (nsh > nsh_max) nsh_max = nsh;
    if (nao > nao_max) nao_max = nao;
  }
  sizes_out[0] = nunique;
  sizes_out[1] = nushell;
  sizes_out[2] = nsh_max;
  sizes_out[3] = nao_max;
  return DXTB_OK;
}

extern "C" int32_t dxtb_index_maps(const int64_t *numbers, int32_t nbatch, int32_t nat_max,
                                   int32_t batch_mode, const int32_t *el_nsh, const int32_t *el_ang,
                                   int64_t nsh_max, int64_t nao_max, int64_t *unique_angular,
                                   int64_t *angular, int64_t *atom_to_unique,
                                   int64_t *ushells_to_unique, int64_t *ushells_per_unique,
                                   int64_t *shells_to_ushell, int64_t *shells_per_atom,
                                   int64_t *shell_index, int64_t *shells_to_atom,
                                   int64_t *orbitals_per_shell, int64_t *orbital_index,
                                   int64_t *orbitals_to_shell, int64_t *unique_out,
                                   int64_t *zmap_scratch, void *stream) {
  if (!numbers || nbatch <= 0 || nat_max <= 0 || !el_nsh || !el_ang || !zmap_scratch)
    return DXTB_ERR_ARGS;
  cudaStream_t st = (cudaStream_t)stream;
  k_index_unique<<<1, 256, 0, st>>>(numbers, (int64_t)nbatch * nat_max, batch_mode > 0, el_nsh,
                                     el_ang, unique_angular, ushells_to_unique, ushells_per_unique,
                                     unique_out, zmap_scratch);
  DXTB_CHECK_LAUNCH();
  k_index_rows<<<nbatch, 128, 0, st>>>(numbers, nat_max, nsh_max, nao_max, unique_angular,
                                        zmap_scratch, angular, atom_to_unique, shells_to_ushell,
                                        shells_per_atom, shell_index, shells_to_atom,
                                        orbitals_per_shell, orbital_index, orbitals_to_shell);
  DXTB_CHECK_LAUNCH();
  return DXTB_OK;
}
