// Generalized-Born / ALPB implicit solvation: Born radii (Onufriev-Bashford-
// Case descreening integral), the interaction matrix the SCF adds to its
// atomic potential, and the nuclear gradient of E = 1/2 q^T A q at the
// converged charges. One CTA per molecule; positions, radii and per-atom
// intermediates sit in shared memory, threads stride over atoms or pairs.
//
// Reference: src/dxtb/_src/components/interactions/solvation/born.py:60-239
// (get_born_radii, compute_psi) and alpb.py:94-184 (p16 / Still kernels,
// shape descriptor), :227-321 (keps, alpbet, cache matrix). The reference
// differentiates the solvation energy with autograd; the adjoint here is
// derived by hand from the same expressions.
#include "common.cuh"

namespace dxtb {

constexpr double kObc0 = 1.0, kObc1 = 0.8, kObc2 = 4.85;  // born.py:67
constexpr double kDescreen = 0.8;                         // born.py:66
constexpr double kBornCutoff = 66.0;                      // born.py:63, Bohr
constexpr double kAlphaAlpb = 0.571412;                   // alpb.py:79
constexpr double kP16 = 1.028 / 16.0;                     // alpb.py:106

struct GbPar {
  double keps, alpbet, scale, offset;
  int kernel;  // 0 p16, 1 Still
};

__host__ __device__ inline GbPar gb_par(double epsilon, int kernel, int alpb, double scale,
                                         double offset) {
  GbPar p;
  p.alpbet = alpb ? kAlphaAlpb / epsilon : 0.0;
  p.keps = (1.0 / epsilon - 1.0) / (1.0 + p.alpbet);
  p.scale = scale;
  p.offset = offset;
  p.kernel = kernel;
  return p;
}

// Descreening term h(r; rho_i, R_j) of psi_j and its r-derivative
// (born.py:196-239: overlapping form when r < R_j + rho_i and r + rho_i > R_j).
__device__ __forceinline__ void psi_term(double r, double rho, double rv, double &h, double &dh) {
  const double dpl = r + rho, dmi = r - rho;
  if (r < rv + rho && r + rho > rv) {
    const double ip = 1.0 / dpl, irv = 1.0 / rv, ratio = dpl * irv;
    const double lnr = log(ratio);
    const double u = 0.5 * dmi * (ip - ratio * irv) - lnr;
    const double du = 0.5 * (ip - ratio * irv) + 0.5 * dmi * (-ip * ip - irv * irv) - ip;
    const double ir = 1.0 / r;
    h = irv - ip + 0.5 * ir * u;
    dh = ip * ip - 0.5 * u * ir * ir + 0.5 * du * ir;
  } else {
    const double pr = dpl * dmi, qu = dmi / dpl, ir = 1.0 / r;
    h = rho / pr;
    dh = -2.0 * r * rho / (pr * pr);
    if (qu > 0.0) {
      const double lq = log(qu);
      h += 0.5 * lq * ir;
      dh += 0.5 * (2.0 * rho / (pr * r) - lq * ir * ir);
    }
  }
}

// Interaction kernel f(r, ab) and its partial derivatives (alpb.py:94-142).
__device__ __forceinline__ double gb_kernel(int kind, double r, double ab, double *fr, double *fa) {
  if (kind == 0) {
    const double s = sqrt(ab), den = s + r * kP16, x = s / den;
    const double x2 = x * x, x4 = x2 * x2, x8 = x4 * x4, g = x8 * x8;
    const double f = 1.0 / (r + s * g);
    if (fr) {
      *fr = -f * f * (1.0 - 16.0 * s * g * kP16 / den);
      // d f / d s * d s / d ab
      *fa = -f * f * g * (1.0 + 16.0 * r * kP16 / den) * (0.5 / s);
    }
    return f;
  }
  const double r2 = r * r, e = exp(-0.25 * r2 / ab);
  const double f = 1.0 / sqrt(r2 + ab * e), f3 = f * f * f;
  if (fr) {
    *fr = -f3 * r * (1.0 - 0.25 * e);
    *fa = -0.5 * f3 * e * (1.0 + 0.25 * r2 / ab);
  }
  return f;
}

// Born radius from psi and d B / d psi (born.py:128-151).
__device__ __forceinline__ double born_of_psi(double psi, double rv, const GbPar &p, double *dbdpsi) {
  const double srv = rv - p.offset, r1 = 1.0 / rv, s1 = 1.0 / srv;
  const double x = 0.5 * psi * srv;
  const double t = x * (kObc0 + x * (kObc2 * x - kObc1));
  const double th = tanh(t);
  const double den = s1 - r1 * th;
  const double born = p.scale / den;
  if (dbdpsi) {
    const double dt = kObc0 - 2.0 * kObc1 * x + 3.0 * kObc2 * x * x;
    *dbdpsi = p.scale * r1 * (1.0 - th * th) * dt * 0.5 * srv / (den * den);
  }
  return born;
}

// Inertia tensor of solid spheres about the volume centre (alpb.py:144-184):
// returns det(I) and fills the 3x3 adjugate (symmetric) and the centre.
__device__ double inertia_det(int nat, const double *sx, const double *sy, const double *sz,
                              const double *rv, double *red, double *adj, double *cen,
                              double *vtot) {
  double v = 0.0, cx = 0.0, cy = 0.0, cz = 0.0;
  for (int i = threadIdx.x; i < nat; i += blockDim.x) {
    const double vol = rv[i] * rv[i] * rv[i];
    v += vol;
    cx += vol * sx[i];
    cy += vol * sy[i];
    cz += vol * sz[i];
  }
  const double V = block_sum(v, red);
  cen[0] = block_sum(cx, red) / V;
  cen[1] = block_sum(cy, red) / V;
  cen[2] = block_sum(cz, red) / V;
  double t[6] = {0, 0, 0, 0, 0, 0};  // xx yy zz xy xz yz
  for (int i = threadIdx.x; i < nat; i += blockDim.x) {
    const double vol = rv[i] * rv[i] * rv[i];
    const double dx = sx[i] - cen[0], dy = sy[i] - cen[1], dz = sz[i] - cen[2];
    const double dg = dx * dx + dy * dy + dz * dz + 0.4 * rv[i] * rv[i];
    t[0] += vol * (dg - dx * dx);
    t[1] += vol * (dg - dy * dy);
    t[2] += vol * (dg - dz * dz);
    t[3] -= vol * dx * dy;
    t[4] -= vol * dx * dz;
    t[5] -= vol * dy * dz;
  }
  double I[6];
  for (int c = 0; c < 6; ++c) I[c] = block_sum(t[c], red);
  const double a = I[0], b = I[1], c = I[2], d = I[3], e = I[4], f = I[5];
  // symmetric [[a d e] [d b f] [e f c]]
  adj[0] = b * c - f * f;
  adj[4] = a * c - e * e;
  adj[8] = a * b - d * d;
  adj[1] = adj[3] = e * f - d * c;
  adj[2] = adj[6] = d * f - b * e;
  adj[5] = adj[7] = d * e - a * f;
  *vtot = V;
  return a * adj[0] + d * adj[1] + e * adj[2];
}

__global__ void k_born_matrix(dxtb_batch b, const double *__restrict__ pf_, GbPar p,
                              double *__restrict__ born, double *__restrict__ psi_out,
                              double *__restrict__ gbm) {
  extern __shared__ double sm[];
  __shared__ double red[32];
  const int m = blockIdx.x;
  const int64_t a0 = b.atom_off[m], n2 = b.nat2_off[m];
  const int nat = (int)(b.atom_off[m + 1] - a0);
  double *sx = sm, *sy = sx + nat, *sz = sy + nat, *rv = sz + nat, *sb = rv + nat;
  for (int i = threadIdx.x; i < nat; i += blockDim.x) {
    sx[i] = b.positions[3 * (a0 + i) + 0];
    sy[i] = b.positions[3 * (a0 + i) + 1];
    sz[i] = b.positions[3 * (a0 + i) + 2];
    rv[i] = pf(pf_, DXTB_P_VDW + b.numbers[a0 + i]);
  }
  __syncthreads();
  for (int j = threadIdx.x; j < nat; j += blockDim.x) {
    double s = 0.0, h, dh;
    for (int i = 0; i < nat; ++i) {
      if (i == j) continue;
      const double dx = sx[i] - sx[j], dy = sy[i] - sy[j], dz = sz[i] - sz[j];
      const double r = sqrt(dx * dx + dy * dy + dz * dz);
      if (r > kBornCutoff) continue;
      psi_term(r, kDescreen * rv[i], rv[j], h, dh);
      s += h;
    }
    const double bj = born_of_psi(s, rv[j], p, nullptr);
    sb[j] = bj;
    born[a0 + j] = bj;
    psi_out[a0 + j] = s;
  }
  __syncthreads();
  double shift = 0.0;
  if (p.alpbet > 0.0) {
    __shared__ double adj[9], cen[3];
    double V;
    const double det = inertia_det(nat, sx, sy, sz, rv, red, adj, cen, &V);
    shift = p.keps * p.alpbet * sqrt(5.0 * cbrt(det) / (2.0 * V));
  }
  for (int64_t k = threadIdx.x; k < (int64_t)nat * nat; k += blockDim.x) {
    const int i = (int)(k / nat), j = (int)(k % nat);
    double r = 0.0;
    if (i != j) {
      const double dx = sx[i] - sx[j], dy = sy[i] - sy[j], dz = sz[i] - sz[j];
      r = sqrt(dx * dx + dy * dy + dz * dz);
    }
    gbm[n2 + k] = p.keps * gb_kernel(p.kernel, r, sb[i] * sb[j], nullptr, nullptr) + shift;
  }
}

__global__ void k_born_grad(dxtb_batch b, const double *__restrict__ pf_, GbPar p,
                            const double *__restrict__ q, const double *__restrict__ born,
                            const double *__restrict__ psi, double *__restrict__ grad) {
  extern __shared__ double sm[];
  __shared__ double red[32];
  const int m = blockIdx.x;
  const int64_t a0 = b.atom_off[m], s0 = b.shell_off[m], o0 = b.ao_off[m];
  const int nat = (int)(b.atom_off[m + 1] - a0);
  const int nsh = (int)(b.shell_off[m + 1] - s0);
  const int n = (int)(b.ao_off[m + 1] - o0);
  double *sx = sm, *sy = sx + nat, *sz = sy + nat, *rv = sz + nat, *sb = rv + nat;
  double *qa = sb + nat, *dpsi = qa + nat;
  int *first = reinterpret_cast<int *>(dpsi + nat);  // [nat + 1] first orbital of each atom
  for (int i = threadIdx.x; i < nat; i += blockDim.x) {
    sx[i] = b.positions[3 * (a0 + i) + 0];
    sy[i] = b.positions[3 * (a0 + i) + 1];
    sz[i] = b.positions[3 * (a0 + i) + 2];
    rv[i] = pf(pf_, DXTB_P_VDW + b.numbers[a0 + i]);
    sb[i] = born[a0 + i];
  }
  for (int s = threadIdx.x; s < nsh; s += blockDim.x) {
    const int at = b.shell_atom[s0 + s];
    if (s == 0 || b.shell_atom[s0 + s - 1] != at) first[at] = b.shell_ao[s0 + s];
  }
  if (threadIdx.x == 0) first[nat] = n;
  __syncthreads();
  double qpart = 0.0;
  for (int i = threadIdx.x; i < nat; i += blockDim.x) {
    double s = 0.0;
    for (int o = first[i]; o < first[i + 1]; ++o) s += q[o0 + o];
    qa[i] = s;
    qpart += s;
  }
  const double qtot = block_sum(qpart, red);  // also orders the qa writes
  // d E / d psi_k = keps q_k sum_j q_j f_a(r_kj, B_k B_j) B_j * d B_k / d psi_k
  for (int k = threadIdx.x; k < nat; k += blockDim.x) {
    double s = 0.0, fr, fa;
    for (int j = 0; j < nat; ++j) {
      double r = 0.0;
      if (j != k) {
        const double dx = sx[k] - sx[j], dy = sy[k] - sy[j], dz = sz[k] - sz[j];
        r = sqrt(dx * dx + dy * dy + dz * dz);
      }
      gb_kernel(p.kernel, r, sb[k] * sb[j], &fr, &fa);
      // an infinite Born radius (saturated OBC tanh, buried atoms of dense
      // systems) decouples the pair: f and its derivatives vanish faster than
      // B grows, so the limit of the term is 0 (the product would be 0 * inf)
      if (isfinite(sb[j]) && isfinite(sb[k])) s += qa[j] * fa * sb[j];
    }
    double dbdpsi;
    born_of_psi(psi[a0 + k], rv[k], p, &dbdpsi);
    dpsi[k] = isfinite(dbdpsi) && isfinite(sb[k]) ? p.keps * qa[k] * s * dbdpsi : 0.0;
  }
  __syncthreads();
  // ALPB shape term 1/2 keps alpbet adet (sum q)^2 (zero for neutral molecules)
  double cshape = 0.0, tradj = 0.0;
  __shared__ double adj[9], cen[3];
  if (p.alpbet > 0.0) {
    double V;
    const double det = inertia_det(nat, sx, sy, sz, rv, red, adj, cen, &V);
    const double adet = sqrt(5.0 * cbrt(det) / (2.0 * V));
    cshape = 0.5 * p.keps * p.alpbet * qtot * qtot * adet / (6.0 * det);  // * d det / d R
    tradj = adj[0] + adj[4] + adj[8];
  }
  for (int i = threadIdx.x; i < nat; i += blockDim.x) {
    double g[3] = {0.0, 0.0, 0.0};
    const double rhoi = kDescreen * rv[i];
    for (int j = 0; j < nat; ++j) {
      if (j == i) continue;
      const double d[3] = {sx[i] - sx[j], sy[i] - sy[j], sz[i] - sz[j]};
      const double r = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
      double fr, fa;
      gb_kernel(p.kernel, r, sb[i] * sb[j], &fr, &fa);
      double G = isfinite(fr) ? p.keps * qa[i] * qa[j] * fr : 0.0;
      if (r <= kBornCutoff) {
        double h, dh;
        psi_term(r, rhoi, rv[j], h, dh);  // i descreens j
        G += dpsi[j] * dh;
        psi_term(r, kDescreen * rv[j], rv[i], h, dh);  // j descreens i
        G += dpsi[i] * dh;
      }
      const double ir = G / r;
      for (int x = 0; x < 3; ++x) g[x] += ir * d[x];
    }
    if (cshape != 0.0) {
      const double vol = rv[i] * rv[i] * rv[i];
      const double dv[3] = {sx[i] - cen[0], sy[i] - cen[1], sz[i] - cen[2]};
      for (int x = 0; x < 3; ++x) {
        const double ad = adj[3 * x] * dv[0] + adj[3 * x + 1] * dv[1] + adj[3 * x + 2] * dv[2];
        g[x] += cshape * vol * (2.0 * dv[x] * tradj - 2.0 * ad);
      }
    }
    for (int x = 0; x < 3; ++x) grad[3 * (a0 + i) + x] += g[x];
  }
}

}  // namespace dxtb

using namespace dxtb;

static int32_t gb_check(const dxtb_batch *b, double epsilon, int32_t kernel, size_t smem) {
  if (!b || b->nmol <= 0 || !(epsilon > 0.0) || (kernel != 0 && kernel != 1)) return DXTB_ERR_ARGS;
  if (smem > 220 * 1024) return DXTB_ERR_TOO_LARGE;
  return DXTB_OK;
}

extern "C" int32_t dxtb_born_matrix(const dxtb_batch *b, const double *par_f, const int32_t *par_i,
                                    double epsilon, int32_t kernel, int32_t alpb, double born_scale,
                                    double born_offset, double *born, double *psi, double *gb_mat,
                                    void *stream) {
  (void)par_i;
  if (!born || !psi || !gb_mat || !par_f) return DXTB_ERR_ARGS;
  const size_t smem = sizeof(double) * 5 * (size_t)(b ? b->max_nat : 0);
  const int32_t rc = gb_check(b, epsilon, kernel, smem);
  if (rc != DXTB_OK) return rc;
  if (smem > 48 * 1024 &&
      cudaFuncSetAttribute(k_born_matrix, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return DXTB_ERR_LAUNCH;
  const GbPar p = gb_par(epsilon, kernel, alpb, born_scale, born_offset);
  k_born_matrix<<<b->nmol, 256, smem, (cudaStream_t)stream>>>(*b, par_f, p, born, psi, gb_mat);
  DXTB_CHECK_LAUNCH();
  return DXTB_OK;
}

extern "C" int32_t dxtb_born_gradient(const dxtb_batch *b, const double *par_f,
                                      const int32_t *par_i, double epsilon, int32_t kernel,
                                      int32_t alpb, double born_scale, double born_offset,
                                      const double *q, const double *born, const double *psi,
                                      double *grad, void *stream) {
  (void)par_i;
  if (!q || !born || !psi || !grad || !par_f) return DXTB_ERR_ARGS;
  const size_t smem =
      sizeof(double) * 7 * (size_t)(b ? b->max_nat : 0) + sizeof(int) * (size_t)((b ? b->max_nat : 0) + 1);
  const int32_t rc = gb_check(b, epsilon, kernel, smem);
  if (rc != DXTB_OK) return rc;
  if (smem > 48 * 1024 &&
      cudaFuncSetAttribute(k_born_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return DXTB_ERR_LAUNCH;
  const GbPar p = gb_par(epsilon, kernel, alpb, born_scale, born_offset);
  k_born_grad<<<b->nmol, 256, smem, (cudaStream_t)stream>>>(*b, par_f, p, q, born, psi, grad);
  DXTB_CHECK_LAUNCH();
  return DXTB_OK;
}
