/*
 * dxtb_gb300 — C ABI of the GB300 (sm_103a) GFN1/GFN2-xTB single-point path.
 *
 * Every entry point takes plain device pointers and sizes, runs on the CUDA
 * stream it is given, allocates nothing, and returns an int32 status
 * (DXTB_OK or one of the DXTB_ERR_* codes). All floating-point data is
 * float64; all index data is int32 or int64 as declared.
 *
 * Batches are PACKED, not padded: molecule m owns atoms
 * [atom_off[m], atom_off[m+1]), shells [shell_off[m], shell_off[m+1]),
 * orbitals [ao_off[m], ao_off[m+1]), a dense n_m x n_m block of every AO
 * matrix at mat_off[m] (row-major, n_m = ao_off[m+1]-ao_off[m]), a
 * nat_m x nat_m block of every atom-pair matrix at nat2_off[m] and a
 * nsh_m x nsh_m block of the shell-resolved Coulomb matrix at nsh2_off[m].
 * Multi-component AO matrices (dipole: 3, quadrupole: 6) are stored
 * component-major: component k of molecule m starts at
 * k * mat_off[nmol] + mat_off[m].
 *
 * Reference interfaces these entry points replace (paths relative to
 * src/dxtb/_src of marvinfriede/dxtb) are cited at each declaration.
 */
#ifndef DXTB_GB300_H
#define DXTB_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define DXTB_OK 0
#define DXTB_ERR_ARGS 1          /* invalid sizes or null pointers          */
#define DXTB_ERR_LAUNCH 2        /* CUDA launch or runtime error            */
#define DXTB_ERR_NOT_POSDEF 3    /* overlap matrix not positive definite     */
#define DXTB_ERR_MAXITER 4       /* SCF did not converge within maxiter      */
#define DXTB_ERR_FERMI 5         /* Fermi level search failed                */
#define DXTB_ERR_NAN 6           /* NaN/Inf in a per-molecule result         */
#define DXTB_ERR_TOO_LARGE 7     /* size beyond a compiled-in maximum        */

/* ---- parameter tables ---------------------------------------------------
 * Flat float64 / int32 arrays filled by the host from the GFN parameter
 * files (the TOML tables under param/gfn{1,2}). A "shell type" is one shell of one
 * element; element Z owns shell types [EL_SH0[Z], EL_SH0[Z] + EL_NSH[Z]).
 */
#define DXTB_MAXZ 87
#define DXTB_MAXSHT 320
#define DXTB_MAXPRIM 8

/* float64 table offsets */
#define DXTB_P_ALPHA 0                                          /* [SHT][8] */
#define DXTB_P_COEFF (DXTB_P_ALPHA + DXTB_MAXSHT * DXTB_MAXPRIM) /* [SHT][8] */
#define DXTB_P_LEVEL (DXTB_P_COEFF + DXTB_MAXSHT * DXTB_MAXPRIM) /* Eh      */
#define DXTB_P_KCN (DXTB_P_LEVEL + DXTB_MAXSHT)                   /* Eh      */
#define DXTB_P_SHPOLY (DXTB_P_KCN + DXTB_MAXSHT)
#define DXTB_P_REFOCC (DXTB_P_SHPOLY + DXTB_MAXSHT)
#define DXTB_P_LGAM (DXTB_P_REFOCC + DXTB_MAXSHT)
#define DXTB_P_SLATER (DXTB_P_LGAM + DXTB_MAXSHT)
#define DXTB_P_EN (DXTB_P_SLATER + DXTB_MAXSHT)   /* per element [MAXZ]      */
#define DXTB_P_GAM (DXTB_P_EN + DXTB_MAXZ)
#define DXTB_P_GAM3 (DXTB_P_GAM + DXTB_MAXZ)
#define DXTB_P_ZEFF (DXTB_P_GAM3 + DXTB_MAXZ)
#define DXTB_P_AREP (DXTB_P_ZEFF + DXTB_MAXZ)
#define DXTB_P_DKERNEL (DXTB_P_AREP + DXTB_MAXZ)
#define DXTB_P_QKERNEL (DXTB_P_DKERNEL + DXTB_MAXZ)
#define DXTB_P_MPRAD (DXTB_P_QKERNEL + DXTB_MAXZ)
#define DXTB_P_MPVCN (DXTB_P_MPRAD + DXTB_MAXZ)
#define DXTB_P_RCOV (DXTB_P_MPVCN + DXTB_MAXZ)    /* Bohr, D3 (4/3 scaled)  */
#define DXTB_P_RAD (DXTB_P_RCOV + DXTB_MAXZ)      /* Bohr, H0 polynomial    */
#define DXTB_P_VDW (DXTB_P_RAD + DXTB_MAXZ)       /* Bohr, Born radii       */
#define DXTB_P_KPAIR (DXTB_P_VDW + DXTB_MAXZ)     /* [MAXZ][MAXZ]           */
#define DXTB_P_KSHELL (DXTB_P_KPAIR + DXTB_MAXZ * DXTB_MAXZ) /* [5][5]      */
#define DXTB_P_ES3SCALE (DXTB_P_KSHELL + 25)      /* [5] per angular momentum */
#define DXTB_P_SCAL (DXTB_P_ES3SCALE + 5)         /* scalars, see below     */
#define DXTB_S_KPOL 0
#define DXTB_S_WEXP 1
#define DXTB_S_ENSCALE 2
#define DXTB_S_GEXP 3
#define DXTB_S_REP_KEXP 4
#define DXTB_S_REP_KLIGHT 5   /* < 0: not used (GFN1)                      */
#define DXTB_S_DMP3 6
#define DXTB_S_DMP5 7
#define DXTB_S_MP_KEXP 8
#define DXTB_S_MP_SHIFT 9
#define DXTB_S_MP_RMAX 10
#define DXTB_S_CN_CUTOFF 11
#define DXTB_S_REP_CUTOFF 12
#define DXTB_NSCAL 16
#define DXTB_P_SIZE (DXTB_P_SCAL + DXTB_NSCAL)

/* int32 table offsets */
#define DXTB_I_L 0                                   /* [SHT] angular momentum */
#define DXTB_I_NPRIM (DXTB_I_L + DXTB_MAXSHT)        /* [SHT]                  */
#define DXTB_I_VALENCE (DXTB_I_NPRIM + DXTB_MAXSHT)  /* [SHT] 0/1              */
#define DXTB_I_ELEM (DXTB_I_VALENCE + DXTB_MAXSHT)   /* [SHT]                  */
#define DXTB_I_EL_NSH (DXTB_I_ELEM + DXTB_MAXSHT)    /* [MAXZ]                 */
#define DXTB_I_EL_SH0 (DXTB_I_EL_NSH + DXTB_MAXZ)    /* [MAXZ]                 */
#define DXTB_I_SCAL (DXTB_I_EL_SH0 + DXTB_MAXZ)
#define DXTB_IS_METHOD 0      /* 1 = GFN1, 2 = GFN2                         */
#define DXTB_IS_CN_KIND 1     /* 0 = exp (GFN1), 1 = gfn (GFN2)             */
#define DXTB_IS_AVERAGE 2     /* 0 harmonic, 1 arithmetic, 2 geometric      */
#define DXTB_IS_ES3_SHELL 3   /* 1: shell-resolved third order (GFN2)       */
#define DXTB_IS_MULTIPOLE 4   /* 1: AES2 anisotropic electrostatics (GFN2)  */
#define DXTB_NISCAL 8
#define DXTB_I_SIZE (DXTB_I_SCAL + DXTB_NISCAL)

/* ---- packed batch descriptor ------------------------------------------- */
typedef struct dxtb_batch {
  int32_t nmol;
  int32_t max_nao;             /* largest n_m in the batch                  */
  int32_t max_nat;
  int32_t max_nsh;
  const int64_t *atom_off;     /* [nmol+1]                                  */
  const int64_t *shell_off;    /* [nmol+1]                                  */
  const int64_t *ao_off;       /* [nmol+1]                                  */
  const int64_t *mat_off;      /* [nmol+1] prefix of n_m^2                  */
  const int64_t *nat2_off;     /* [nmol+1] prefix of nat_m^2                */
  const int64_t *nsh2_off;     /* [nmol+1] prefix of nsh_m^2                */
  const int64_t *pair_off;     /* [nmol+1] prefix of nsh_m (nsh_m+1) / 2    */
  const int32_t *numbers;      /* [natoms] atomic numbers                   */
  const double *positions;     /* [natoms][3] Bohr                          */
  const int32_t *shell_atom;   /* [nshells] atom index local to molecule    */
  const int32_t *shell_type;   /* [nshells] global shell type               */
  const int32_t *shell_ao;     /* [nshells] first AO, local to molecule     */
  const int32_t *ao_shell;     /* [naos] shell index local to molecule      */
} dxtb_batch;

/* ---- entry points ------------------------------------------------------ */

/* IndexHelper maps, bit-exact with IndexHelper.from_numbers_angular
 * (basis/indexhelper.py:338-492) for batch_mode 0 (one molecule, nbatch = 1)
 * and batch mode 1 (nbatch zero-padded rows of nat_max atoms).
 * dxtb_index_sizes is host-only: numbers_host [nbatch][nat_max], el_nsh_host
 * [MAXZ] shells per element (0: no parameters), el_ang_host [MAXZ][8] their
 * angular momenta; sizes_out [4] = (nunique, nushell, nsh_max, nao_max).
 * dxtb_index_maps fills, on the stream: unique_angular [nushell],
 * ushells_to_unique [nushell], ushells_per_unique [nunique], unique_out
 * [nunique] (sorted atomic numbers), and per row: atom_to_unique,
 * shells_per_atom, shell_index [nat_max]; angular, shells_to_ushell,
 * shells_to_atom, orbitals_per_shell, orbital_index [nsh_max];
 * orbitals_to_shell [nao_max]. zmap_scratch: device int64 [3 * MAXZ]. */
int32_t dxtb_index_sizes(const int64_t *numbers_host, int32_t nbatch,
                         int32_t nat_max, int32_t batch_mode,
                         const int32_t *el_nsh_host, const int32_t *el_ang_host,
                         int64_t *sizes_out);
int32_t dxtb_index_maps(const int64_t *numbers, int32_t nbatch, int32_t nat_max,
                        int32_t batch_mode, const int32_t *el_nsh,
                        const int32_t *el_ang, int64_t nsh_max, int64_t nao_max,
                        int64_t *unique_angular, int64_t *angular,
                        int64_t *atom_to_unique, int64_t *ushells_to_unique,
                        int64_t *ushells_per_unique, int64_t *shells_to_ushell,
                        int64_t *shells_per_atom, int64_t *shell_index,
                        int64_t *shells_to_atom, int64_t *orbitals_per_shell,
                        int64_t *orbital_index, int64_t *orbitals_to_shell,
                        int64_t *unique_out, int64_t *zmap_scratch, void *stream);

/* Coordination numbers (tad_mctc cn_d3 as called at xtb/gfn1.py:62-64,
 * xtb/gfn2.py:58-62, coulomb/multipole.py:323-328). kind 0 = exp, 1 = gfn.
 * cn: [natoms]. */
int32_t dxtb_coordination_number(const dxtb_batch *b, const double *par_f,
                                 const int32_t *par_i, int32_t kind, double *cn,
                                 void *stream);

/* Geometry-only interaction caches: ES2 gamma (coulomb/secondorder.py:
 * 799-872) [nsh2_off], ES3 Hubbard derivatives (thirdorder.py get_cache)
 * [nshells], AES2 damping radii and matrices (coulomb/multipole.py:270-448)
 * mrad [natoms], sd [3][nat2], dd [9][nat2], sq [6][nat2] (component-major
 * over nat2_off[nmol]; null for GFN1), and the atom-resolved repulsion
 * energy (classicals/repulsion/base.py:293-348) erep [natoms]. */
int32_t dxtb_interaction_cache(const dxtb_batch *b, const double *par_f,
                               const int32_t *par_i, const double *cn_mp,
                               double *gamma, double *hd, double *mrad,
                               double *amat_sd, double *amat_dd,
                               double *amat_sq, double *erep, void *stream);

/* Multipole integrals and core Hamiltonian for every shell pair of the
 * batch: the PyTorch integral driver (integral/driver/pytorch/impls/
 * pairs.py:228-399 with kernels/md.py) followed by normalisation, the
 * r0 -> rj shifts and the traceless transform (integral/container.py:
 * 182-537) and BaseHamiltonian.build (xtb/base.py:255-372). Outputs:
 * overlap [mat], h0 [mat] (may be null), dipole [3][mat] and quadrupole
 * [6][mat] (ket-centred, traceless; null to skip). cn: [natoms] from
 * dxtb_coordination_number with the method's counting function. */
int32_t dxtb_multipole_h0(const dxtb_batch *b, const double *par_f,
                          const int32_t *par_i, const double *cn,
                          double *overlap, double *h0, double *dipole,
                          double *quadrupole, void *stream);

/* Raw multipole integrals about the origin as returned by the integral
 * wrappers overlap/dipint/quadint (integral/wrappers.py:149-315):
 * overlap [mat], dipole [3][mat], quadrupole [9][mat] (row-major xx..zz),
 * all normalised, not shifted, not made traceless. The moments are written
 * together: with dipole or quadrupole null, only the overlap is. */
int32_t dxtb_multipole_raw(const dxtb_batch *b, const double *par_f,
                           const int32_t *par_i, double *overlap,
                           double *dipole, double *quadrupole, void *stream);

/* ---- SCF configuration (calculators/config/scf.py ConfigSCF) -----------
 * mixer DXTB_MIXER_BROYDEN1: the implicit-mode root solver (scf_mode
 * "implicit": xitorch broyden1 on F(x) = x - G(x), exlibs/xitorch/_impls/
 * optimize/root/rootsolver.py:42-265 with alpha = -0.5 and damp), stopping
 * when |dx|_2 < x_atol and |F|_2 < f_atol, returning the best iterate after
 * maxiter iterations. DXTB_MIXER_ANDERSON: the full-mode loop (scf_mode
 * "full", scf/unrolling/default.py:71-140, mix_guess) with the Anderson
 * mixer of scf/mixer/anderson.py:163-317 (damp, damp_init, generations
 * <= 16, soft_start, diagonal_offset), converged when |G(x) - x|_2 < x_atol
 * and max |G(x) - x| < x_atol_max (scf/mixer/base.py:230-256), the energy
 * evaluated at G(x). Reference defaults (constants/defaults.py): maxiter
 * 100, x_atol = f_atol = 1e-4, x_atol_max = 1e-5, damp 0.5, damp_init 0.1,
 * generations 5, soft_start 1, diagonal_offset 0.01. */
#define DXTB_MIXER_BROYDEN1 0
#define DXTB_MIXER_ANDERSON 1
typedef struct dxtb_scf_config {
  int32_t maxiter;
  int32_t mixer;
  double x_atol;
  double f_atol;
  double x_atol_max;
  double damp;
  double damp_init;
  int32_t generations;
  int32_t soft_start;
  double diagonal_offset;
} dxtb_scf_config;

/* Backward of dxtb_multipole_raw: accumulates into grad [natoms][3] the
 * vector-Jacobian product dL/dR = sum dL/dM_k dM_k/dR of the normalised
 * integrals about the origin for the upstream gradients grad_overlap [mat],
 * grad_dipole [3][mat] and grad_quadrupole [9][mat] (row-major xx..zz; any
 * may be null). The reference obtains it by autograd through the integral
 * wrappers (integral/wrappers.py:149-215). */
int32_t dxtb_multipole_raw_vjp(const dxtb_batch *b, const double *par_f,
                               const int32_t *par_i, const double *grad_overlap,
                               const double *grad_dipole,
                               const double *grad_quadrupole, double *grad,
                               void *stream);

/* Electric dipole moment of every molecule, dipole [nmol][3] in e a0:
 * sum_A Z_A R_A - tr(P D0) (calculators/properties/moments/dip.py,
 * dipole_xtb), with n0 [naos] the reference occupations (summing to the
 * valence charge Z_A of each atom), density [mat] and dipole_origin
 * [3][mat] the normalised dipole integrals about the origin from
 * dxtb_multipole_raw. The reference's calculator obtains the same moment
 * as dE/dF through its electric-field interaction (calculators/types/
 * autograd.py:399-472, dipole). */
int32_t dxtb_dipole_moment(const dxtb_batch *b, const double *n0,
                           const double *density, const double *dipole_origin,
                           double *dipole, void *stream);

/* CUDA graph of a sequence of this library's calls on one stream (the
 * reference has no counterpart: it re-dispatches its PyTorch operators on
 * every call). dxtb_graph_begin starts a thread-local capture on `stream`
 * (not the legacy default stream); the entry points called on it
 * afterwards, with the same buffers, are recorded instead of run, including
 * the work dxtb_scf/dxtb_scf_gradient fork onto their per-class streams.
 * Their first call on `stream` must come before the capture (it creates
 * those streams and sets per-device kernel attributes). dxtb_graph_end ends
 * the capture and returns an executable graph in *exec, instantiated with
 * node priorities so the SCF's class priorities hold on replay.
 * dxtb_graph_launch replays it on a stream; dxtb_graph_destroy frees it.
 * Replays read and write the buffers given at capture time. */
int32_t dxtb_graph_begin(void *stream);
int32_t dxtb_graph_end(void *stream, void **exec);
int32_t dxtb_graph_launch(void *exec, void *stream);
int32_t dxtb_graph_destroy(void *exec);

/* SCF workspace of one molecule in doubles (n AOs, nat atoms); the caller
 * lays the molecules' workspaces out at ws_off[m] (prefix of these sizes). */
int64_t dxtb_scf_workspace_mol(int64_t n, int64_t nat);

/* Self-consistent field for every molecule of the batch, one persistent
 * launch per size class and one team per molecule (a CTA, or a thread-block
 * cluster for the larger classes) (scf/iterator.py:51-144 with the scf/pure modules,
 * wavefunction/filling.py:428-742, exlibs/xitorch symeig): Fock build,
 * generalized eigensolve, Fermi occupations at kT, density, Mulliken
 * charges and multipole moments, potentials, and the limited-memory
 * root solve of x - G(x) on the potential configured by cfg (the
 * implicit-mode broyden1 or the full-mode Anderson mixer, see
 * dxtb_scf_config) with per-molecule convergence and iteration cap.
 * order: [nmol] launch order (largest first) or null. Inputs are the
 * integrals and caches of the calls above, n0 [naos] reference occupation,
 * nel [nmol][2] alpha/beta electrons, gb_mat [nat2] or null. Outputs:
 * density [mat], wdensity [mat] (energy-weighted, may be null), coeff [mat]
 * (orbital j is row j of the block), evals and occ [naos] (unsorted), q
 * [naos] orbital charges, dp [natoms][3], qp [natoms][6] atomic multipoles,
 * vorb [naos], vdp [natoms][3], vqp [natoms][6] potentials of the final
 * charges, energies [nmol][4] = (E_h0 + E_interaction, -TS, iterations,
 * final residual) and status [nmol]. Molecules run by size class (see
 * dxtb_scf_set_size_classes); order lists them by non-increasing n. */
int32_t dxtb_scf(const dxtb_batch *b, const double *par_f, const int32_t *par_i,
                 const double *overlap, const double *h0, const double *dipole,
                 const double *quadrupole, const double *gamma,
                 const double *hd, const double *amat_sd, const double *amat_dd,
                 const double *amat_sq, const double *gb_mat, const double *n0,
                 const double *nel, double kt, const dxtb_scf_config *cfg,
                 const int64_t *ws_off, const int32_t *order,
                 double *workspace, double *density, double *wdensity,
                 double *coeff, double *evals, double *occ, double *q,
                 double *dp, double *qp, double *vorb, double *vdp,
                 double *vqp, double *energies, int32_t *status, void *stream);

/* Size classes of the SCF launch (process-wide): molecules with n orbitals
 * run, by class, one 256-thread CTA each two per SM (class 0), one
 * 512-thread CTA on its own SM (class 1), or a thread-block cluster of 2, 4,
 * 8 or 16 CTAs on as many SMs (classes 2-5) that share every O(n^3) phase.
 * min_n[c-1] is the smallest n of class c (non-decreasing); the default is
 * {112, 136, 160, 320, 640}. Clusters need the launch order of dxtb_scf;
 * cluster sizes the GPU cannot place fold into the largest one it can.
 * Each class runs on a stream of its own, forked from the caller's stream:
 * larger classes get higher stream priorities, unless the caller's stream
 * has a non-default priority, which every class then inherits. */
int32_t dxtb_scf_set_size_classes(const int32_t *min_n);
/* The current thresholds (min_n [5]). */
int32_t dxtb_scf_get_size_classes(int32_t *min_n);

/* dxtb_scf followed by dxtb_gradient, fused per size class: the gradient of
 * a class's molecules is launched on that class's stream right after its
 * SCF launch, so it overlaps the SCF of the larger classes. Arguments: those
 * of dxtb_scf (wdensity required), then cn (the Hamiltonian coordination
 * numbers), mrad (GFN2 damping radii, else NULL), dedcn [natoms] and grad
 * [natoms][3], both zeroed by the caller before the call. No counterpart in
 * the reference (its forces are autograd after the SCF). */
int32_t dxtb_scf_gradient(const dxtb_batch *b, const double *par_f,
                          const int32_t *par_i, const double *overlap,
                          const double *h0, const double *dipole,
                          const double *quadrupole, const double *gamma,
                          const double *hd, const double *amat_sd,
                          const double *amat_dd, const double *amat_sq,
                          const double *gb_mat, const double *n0,
                          const double *nel, double kt, const dxtb_scf_config *cfg,
                          const int64_t *ws_off, const int32_t *order,
                          double *workspace, double *density, double *wdensity,
                          double *coeff, double *evals, double *occ, double *q,
                          double *dp, double *qp, double *vorb, double *vdp,
                          double *vqp, double *energies, int32_t *status,
                          const double *cn, const double *mrad, double *dedcn,
                          double *grad, void *stream);

/* Nuclear gradient dE/dR [natoms][3] at the converged SCF (analytic
 * adjoint; the reference differentiates with autograd through
 * calculators/types/autograd.py:84-196 and scf/implicit/fixed_point.py).
 * Accumulates into grad (caller zeroes it). The GFN2 multipole terms are
 * included iff dipole is non-null; then mrad, dp, qp, vdp and vqp are
 * required. No host synchronisation. */
int32_t dxtb_gradient(const dxtb_batch *b, const double *par_f,
                      const int32_t *par_i, const double *cn,
                      const double *cn_mp, const double *mrad,
                      const double *density, const double *wdensity,
                      const double *q, const double *dp, const double *qp,
                      const double *vorb, const double *vdp, const double *vqp,
                      const double *overlap, const double *dipole,
                      const double *reserved0, const double *reserved1,
                      double *dedcn, double *dedcn_mp, double *grad,
                      void *stream);

/* Generalized-Born / ALPB solvation cache (one CTA per molecule): Born
 * radii by the Onufriev-Bashford-Case descreening integral (solvation/
 * born.py:60-239, obc = 1.0/0.8/4.85, descreening 0.8, cutoff 66 Bohr,
 * D3 van-der-Waals radii from par_f) and the matrix
 * A_ij = keps f(R_ij, B_i B_j) [+ keps alpbet adet] of solvation/alpb.py:
 * 94-184, 227-321 with alpbet = 0.571412 / epsilon (alpb != 0) or 0,
 * keps = (1/epsilon - 1) / (1 + alpbet); kernel 0 = P16, 1 = Still.
 * Outputs: born [natoms], psi [natoms] (kept for the gradient), gb_mat
 * [nat2] for dxtb_scf. The reference keeps the same matrix in
 * GeneralizedBornCache.mat. */
int32_t dxtb_born_matrix(const dxtb_batch *b, const double *par_f,
                         const int32_t *par_i, double epsilon, int32_t kernel,
                         int32_t alpb, double born_scale, double born_offset,
                         double *born, double *psi, double *gb_mat, void *stream);

/* Nuclear gradient of E_GB = 1/2 q_at^T A q_at at the converged orbital
 * charges q [naos] (atom sums taken here), with born and psi from
 * dxtb_born_matrix: explicit distance dependence of the kernel, the Born
 * radii through psi, and the ALPB shape term (zero for neutral molecules).
 * Accumulates into grad [natoms][3]. The reference obtains it by autograd
 * through GeneralizedBorn.get_cache. */
int32_t dxtb_born_gradient(const dxtb_batch *b, const double *par_f,
                           const int32_t *par_i, double epsilon, int32_t kernel,
                           int32_t alpb, double born_scale, double born_offset,
                           const double *q, const double *born, const double *psi,
                           double *grad, void *stream);

/* SCF without any device allocation. No counterpart in the reference: it is
 * for callers that must not call cudaMalloc, such as hosts that hand the
 * library a fixed device-memory pool and forbid allocations outside it, or
 * plugin hosts whose allocator cannot be reached through a C ABI. It runs
 * the kernels of dxtb_scf with the same inputs and outputs, but takes its
 * scratch workspace from a fixed array inside the library
 * (DXTB_NOALLOC_SCRATCH_DOUBLES doubles = 16 MiB on every GPU that loads
 * the library, held until the process exits) instead of caller memory.
 * The array starts with a header of H = 32 * ceil((nmol + 2) / 32) int64
 * words (the total size and the per-molecule offsets); a batch whose
 * H + sum over molecules of dxtb_scf_workspace_mol exceeds the array
 * returns DXTB_ERR_TOO_LARGE without running the SCF.
 * Every call computes that size on the device, copies it to the host and
 * synchronises the caller's stream once before it launches the SCF.
 * The first call on a device looks up the array's device address, and the
 * first call from each CUDA stream creates that stream's side streams and
 * fork/join events for the larger size classes (set-up only, no device
 * memory); make that first call before any stream capture begins. All calls
 * share the one array, which keeps the last call's contents (nothing in it
 * needs to start at zero): calls that overlap on the GPU (other streams,
 * other threads) race and must be serialised by the caller. */
#define DXTB_NOALLOC_SCRATCH_DOUBLES (1 << 21)
int32_t dxtb_scf_noalloc(const dxtb_batch *b, const double *par_f,
                         const int32_t *par_i, const double *overlap,
                         const double *h0, const double *dipole,
                         const double *quadrupole, const double *gamma,
                         const double *hd, const double *amat_sd,
                         const double *amat_dd, const double *amat_sq,
                         const double *gb_mat, const double *n0,
                         const double *nel, double kt, int32_t maxiter,
                         double tol, const int32_t *order, double *density,
                         double *wdensity, double *coeff, double *evals,
                         double *occ, double *q, double *dp, double *qp,
                         double *vorb, double *vdp, double *vqp,
                         double *energies, int32_t *status, void *stream);

/* FP64 FMA throughput probe used as the measured FP64 roofline denominator:
 * blocks x threads threads each run 8 independent FMA chains of iters
 * steps (2 * 8 * iters flops per thread). No counterpart in the reference. */
int32_t dxtb_fp64_fma_probe(int64_t iters, int32_t blocks, int32_t threads,
                            double *out, void *stream);

/* FP64 tensor-core (DMMA) throughput probe: every warp of blocks x threads
 * runs 4 independent accumulator chains of iters mma.sync f64 instructions
 * of one shape (0 = m8n8k4, 1 = m16n8k4, 2 = m16n8k8, 3 = m16n8k16);
 * flops = 2 M N K * 4 * iters * threads / 32 * blocks. threads must be a
 * multiple of 32. No counterpart in the reference. */
int32_t dxtb_fp64_mma_probe(int32_t shape, int64_t iters, int32_t blocks,
                            int32_t threads, double *out, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* DXTB_GB300_H */
