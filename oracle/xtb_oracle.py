"""
CPU oracle: float64 restatement of dxtb's GFN1/GFN2-xTB single-point path.

TEST INFRASTRUCTURE ONLY (the checker and the timed CPU reference); the
``dxtb_gb300`` package never imports it.

Written from the behaviour of the reference (paths below are relative to
``src/dxtb/_src`` of marvinfriede/dxtb). PyTorch on the CPU is used only so
that forces come from autograd, as they do in the reference.

Pieces owned by the missing dependency ``tad-mctc`` 0.7.0 (coordination
numbers, radii, unit constants) are restated from their published
definitions; ``dxtb_gb300/data/radii.py`` names the sources.
"""

from __future__ import annotations

import json
import math
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np
import torch

from dxtb_gb300.data import radii as _radii

DATA = Path(__file__).resolve().parents[1] / "dxtb_gb300" / "data"
DT = torch.float64
EPS = torch.finfo(DT).eps
PAD = -999
CN_CUTOFF = 25.0
REP_CUTOFF = 25.0


# --------------------------------------------------------------------------
# parameters
# --------------------------------------------------------------------------


def load_par(method: str) -> dict:
    """Parameter file converted from ``param/gfn{1,2}/*.toml``."""
    with open(DATA / f"{method}.json") as fh:
        par = json.load(fh)
    par["element"] = {int(k): v for k, v in par["element"].items()}
    return par


_STONG = None


def stong(ng: int) -> np.ndarray:
    global _STONG
    if _STONG is None:
        _STONG = dict(np.load(DATA / "stong.npz"))
    return _STONG[f"sto{ng}g"]


# --------------------------------------------------------------------------
# IndexHelper (basis/indexhelper.py:338-492)
# --------------------------------------------------------------------------


def _fill(index: np.ndarray, repeat: np.ndarray) -> np.ndarray:
    """``indexhelper.py:_fill``: position k of block b gets value b."""
    out = np.zeros(int(repeat.sum()), dtype=np.int64)
    for idx, (off, cnt) in enumerate(zip(index.tolist(), repeat.tolist())):
        if cnt > 0:
            out[off : off + cnt] = idx
    return out


def _expand(index: np.ndarray, repeat: np.ndarray) -> np.ndarray:
    """``indexhelper.py:_expand``: concatenated ranges [off, off+cnt)."""
    parts = [
        np.arange(o, o + c, dtype=np.int64)
        for o, c in zip(index.tolist(), repeat.tolist())
    ]
    return np.concatenate(parts) if parts else np.zeros(0, dtype=np.int64)


def _pack(arrs: list[np.ndarray], value: int) -> np.ndarray:
    n = max((a.shape[0] for a in arrs), default=0)
    out = np.full((len(arrs), n), value, dtype=np.int64)
    for i, a in enumerate(arrs):
        out[i, : a.shape[0]] = a
    return out


def index_helper(numbers, angular: dict[int, list[int]]) -> dict[str, np.ndarray]:
    """
    The twelve IndexHelper maps (``indexhelper.py:382-492``) for a single
    molecule (1D ``numbers``) or a zero-padded batch (2D, batch mode 1).
    """
    numbers = np.asarray(numbers, dtype=np.int64)
    batch = numbers.ndim > 1
    unique, atom_to_unique = np.unique(numbers, return_inverse=True)
    atom_to_unique = atom_to_unique.reshape(numbers.shape)
    unique_angular = np.array(
        [l for z in unique.tolist() for l in angular.get(z, [-1])], dtype=np.int64
    )
    ushells_per_unique = np.array(
        [len(angular.get(z, [-1])) for z in unique.tolist()], dtype=np.int64
    )
    ushell_index = np.cumsum(ushells_per_unique) - ushells_per_unique
    ushells_to_unique = _fill(ushell_index, ushells_per_unique)

    if batch:
        if (unique == 0).any():
            ushells_per_unique[0] = 0
        shells_to_ushell = _pack(
            [
                _expand(ushell_index[a], ushells_per_unique[a])
                for a in atom_to_unique
            ],
            -1,
        )
    else:
        shells_to_ushell = _expand(
            ushell_index[atom_to_unique], ushells_per_unique[atom_to_unique]
        )

    shells_per_atom = ushells_per_unique[atom_to_unique]
    shell_index = np.cumsum(shells_per_atom, -1) - shells_per_atom
    shell_index[shells_per_atom == 0] = PAD
    if batch:
        shells_to_atom = _pack(
            [_fill(si, sp) for si, sp in zip(shell_index, shells_per_atom)], PAD
        )
    else:
        shells_to_atom = _fill(shell_index, shells_per_atom)

    lsh = np.where(
        shells_to_ushell >= 0,
        unique_angular[np.clip(shells_to_ushell, 0, None)],
        PAD,
    )
    orbitals_per_shell = np.where(lsh >= 0, 2 * lsh + 1, 0)
    orbital_index = np.cumsum(orbitals_per_shell, -1) - orbitals_per_shell
    orbital_index[orbitals_per_shell == 0] = PAD
    if batch:
        orbitals_to_shell = _pack(
            [_fill(oi, op) for oi, op in zip(orbital_index, orbitals_per_shell)],
            PAD,
        )
    else:
        orbitals_to_shell = _fill(orbital_index, orbitals_per_shell)

    return {
        "unique_angular": unique_angular,
        "angular": lsh.astype(np.int64),
        "atom_to_unique": atom_to_unique.astype(np.int64),
        "ushells_to_unique": ushells_to_unique,
        "ushells_per_unique": ushells_per_unique,
        "shells_to_ushell": shells_to_ushell.astype(np.int64),
        "shells_per_atom": shells_per_atom.astype(np.int64),
        "shell_index": shell_index.astype(np.int64),
        "shells_to_atom": shells_to_atom.astype(np.int64),
        "orbitals_per_shell": orbitals_per_shell.astype(np.int64),
        "orbital_index": orbital_index.astype(np.int64),
        "orbitals_to_shell": orbitals_to_shell.astype(np.int64),
    }


# --------------------------------------------------------------------------
# basis (basis/slater.py, basis/ortho.py, basis/bas.py:124-168)
# --------------------------------------------------------------------------

_DFACT = [1.0, 1.0, 3.0, 15.0, 105.0, 945.0]


def slater_to_gauss(ng: int, n: int, l: int, zeta: float):
    """STO-nG expansion with normalisation (``basis/slater.py:69-146``)."""
    itype = n + [0, 4, 7, 9, 10][l] - 1
    if n == 6 and ng == 6:
        itype = 15 + l
    tab = stong(ng)
    coeff = torch.tensor(tab[0, itype, :], dtype=DT)
    alpha = torch.tensor(tab[1, itype, :], dtype=DT) * zeta**2
    coeff = coeff * (
        (2.0 / math.pi * alpha) ** 0.75
        * torch.sqrt(4 * alpha) ** l
        / math.sqrt(_DFACT[l])
    )
    p = alpha[:, None] + alpha[None, :]
    pref = (math.pi / p) ** 1.5 * _DFACT[l] / (2 * p) ** l
    s = (coeff[:, None] * coeff[None, :] * pref).sum()
    return alpha, coeff / torch.sqrt(s)


def _gauss_s_overlap(ai, aj, ci, cj):
    """``basis/ortho.py:gaussian_integral``."""
    oij = 1.0 / (ai[:, None] + aj[None, :])
    return (torch.sqrt(math.pi * oij) ** 3 * ci[:, None] * cj[None, :]).sum()


def orthogonalize(alpha, coeff):
    """Second s function orthonormalised to the first (``basis/ortho.py:74-110``)."""
    (ai, aj), (ci, cj) = alpha, coeff
    ov = _gauss_s_overlap(ai, aj, ci, cj)
    a_new = torch.cat((aj, ai))
    c_new = torch.cat((cj, -ov * ci))
    so = _gauss_s_overlap(a_new, a_new, c_new, c_new)
    return a_new, c_new / torch.sqrt(so)


# --------------------------------------------------------------------------
# integrals (integral/driver/pytorch/impls/{pairs,pipeline,kernels/os,trafo}.py)
# --------------------------------------------------------------------------

S3 = math.sqrt(3.0)
TRAFO = [
    torch.tensor([[1.0]], dtype=DT),
    torch.eye(3, dtype=DT),
    torch.tensor(
        [
            [0.0, S3, 0.0, 0.0, 0.0, 0.0],
            [0.0, 0.0, 0.0, 0.0, S3, 0.0],
            [-0.5, 0.0, 0.0, -0.5, 0.0, 1.0],
            [0.0, 0.0, S3, 0.0, 0.0, 0.0],
            [S3 * 0.5, 0.0, 0.0, -S3 * 0.5, 0.0, 0.0],
        ],
        dtype=DT,
    ),
]
"""Cartesian → spherical rows (m = -l..l); p in (y, z, x) order (trafo.py)."""
NLM = [
    [(0, 0, 0)],
    [(0, 1, 0), (0, 0, 1), (1, 0, 0)],
    [(2, 0, 0), (1, 1, 0), (1, 0, 1), (0, 2, 0), (0, 1, 1), (0, 0, 2)],
]
COMP_S = [(0, 0, 0)]
COMP_D = [(1, 0, 0), (0, 1, 0), (0, 0, 1)]
COMP_Q9 = [
    (2, 0, 0), (1, 1, 0), (1, 0, 1),
    (1, 1, 0), (0, 2, 0), (0, 1, 1),
    (1, 0, 1), (0, 1, 1), (0, 0, 2),
]


def os_table(la, lb, emax, xij, rpi, rpj, rpc):
    """Three-index Obara–Saika 1D recursion (``kernels/os.py:80-163``)."""
    t = {(0, 0, 0): torch.ones_like(rpi)}
    for e in range(emax + 1):
        for i in range(la + 1):
            for j in range(lb + 1):
                if (i, j, e) in t:
                    continue
                if i > 0:
                    v = rpi * t[(i - 1, j, e)]
                    if i > 1:
                        v = v + (i - 1) * xij * t[(i - 2, j, e)]
                    if j > 0:
                        v = v + j * xij * t[(i - 1, j - 1, e)]
                    if e > 0:
                        v = v + e * xij * t[(i - 1, j, e - 1)]
                elif j > 0:
                    v = rpj * t[(0, j - 1, e)]
                    if j > 1:
                        v = v + (j - 1) * xij * t[(0, j - 2, e)]
                    if e > 0:
                        v = v + e * xij * t[(0, j - 1, e - 1)]
                else:
                    v = rpc * t[(0, 0, e - 1)]
                    if e > 1:
                        v = v + (e - 1) * xij * t[(0, 0, e - 2)]
                t[(i, j, e)] = v
    return t


def shell_pair_blocks(lb, lk, ab, ak, cb, ck, pos_a, vec, comps):
    """
    Multipole blocks about the origin for a class of shell pairs
    (``pipeline.py:151-235``): shape (npair, ncomp, 2lb+1, 2lk+1).
    """
    ai = ab[:, None]
    aj = ak[None, :]
    oij = 1.0 / (ai + aj)
    xij = 0.5 * oij
    r2 = (vec * vec).sum(-1)[:, None, None]
    sij = (
        torch.exp(-ai * aj * oij * r2)
        * math.sqrt(math.pi) ** 3
        * oij**1.5
        * cb[:, None]
        * ck[None, :]
    )  # (np, pi, pj)
    rpi = vec[:, :, None, None] * (aj * oij)  # (np, 3, pi, pj)
    rpj = -vec[:, :, None, None] * (ai * oij)
    rpc = rpi + pos_a[:, :, None, None]
    emax = max(max(c) for c in comps)
    t = os_table(lb, lk, emax, xij, rpi, rpj, rpc)
    out = []
    for comp in comps:
        cart = torch.zeros(vec.shape[0], len(NLM[lb]), len(NLM[lk]), dtype=DT)
        for a, na in enumerate(NLM[lb]):
            for b, nb in enumerate(NLM[lk]):
                prod = sij
                for ax in range(3):
                    prod = prod * t[(na[ax], nb[ax], comp[ax])][:, ax]
                cart[:, a, b] = prod.sum((-2, -1))
        out.append(TRAFO[lb] @ cart @ TRAFO[lk].T)
    return torch.stack(out, 1)


@dataclass
class System:
    """Everything about one molecule that does not depend on positions."""

    method: str
    numbers: np.ndarray
    par: dict
    ih: dict
    nat: int
    nsh: int
    nao: int
    ush_l: list
    ush_z: list
    ush_idx_in_elem: list
    alphas: list = field(default_factory=list)
    coeffs: list = field(default_factory=list)


def make_system(method: str, numbers) -> System:
    par = load_par(method)
    numbers = np.asarray(numbers, dtype=np.int64)
    angular = {z: e["angular"] for z, e in par["element"].items()}
    ih = index_helper(numbers, angular)
    unique = np.unique(numbers)
    ush_l, ush_z, ush_k = [], [], []
    for z in unique.tolist():
        for k, l in enumerate(par["element"][z]["angular"]):
            ush_l.append(l)
            ush_z.append(z)
            ush_k.append(k)
    sysm = System(
        method, numbers, par, ih, len(numbers), len(ih["angular"]),
        int(ih["orbitals_per_shell"].sum()), ush_l, ush_z, ush_k,
    )
    # bas.py:124-168
    for u, (l, z, k) in enumerate(zip(ush_l, ush_z, ush_k)):
        e = par["element"][z]
        a, c = slater_to_gauss(e["ngauss"][k], e["pqn"][k], l, e["slater"][k])
        if method in ("gfn1",) and not e["valence"][k]:
            a, c = orthogonalize((sysm.alphas[u - 1], a), (sysm.coeffs[u - 1], c))
        sysm.alphas.append(a)
        sysm.coeffs.append(c)
    # pairs.py:181-204 (unit self-overlap with the integral kernel itself)
    for u, l in enumerate(ush_l):
        a, c = sysm.alphas[u], sysm.coeffs[u]
        z3 = torch.zeros(1, 3, dtype=DT)
        s = shell_pair_blocks(l, l, a, a, c, c, z3, z3, COMP_S)[0, 0, 0, 0]
        sysm.coeffs[u] = c / (torch.sqrt(torch.clamp(s, min=EPS)) + EPS)
    return sysm


def multipole_raw(sysm: System, positions: torch.Tensor, comps) -> torch.Tensor:
    """Assemble (ncomp, nao, nao) about the origin (``pairs.py:228-399``)."""
    ih = sysm.ih
    sh_atom = ih["shells_to_atom"]
    sh_ush = ih["shells_to_ushell"]
    ang = ih["angular"]
    off = ih["orbital_index"]
    nao = sysm.nao
    mat = torch.zeros(len(comps), nao, nao, dtype=DT)
    bra, ket = np.tril_indices(sysm.nsh)
    classes: dict[tuple[int, int], list[int]] = {}
    for p, (b, k) in enumerate(zip(bra, ket)):
        classes.setdefault((int(sh_ush[b]), int(sh_ush[k])), []).append(p)
    for (ub, uk), plist in classes.items():
        ib = bra[plist]
        jk = ket[plist]
        lb, lk = sysm.ush_l[ub], sysm.ush_l[uk]
        pos_a = positions[sh_atom[ib]]
        vec = positions[sh_atom[jk]] - pos_a
        blk = shell_pair_blocks(
            lb, lk, sysm.alphas[ub], sysm.alphas[uk], sysm.coeffs[ub],
            sysm.coeffs[uk], pos_a, vec, comps,
        )
        w = torch.tensor(np.where(ib == jk, 0.5, 1.0), dtype=DT)
        blk = blk * w[:, None, None, None]
        for n, (b, k) in enumerate(zip(ib, jk)):
            rb = slice(off[b], off[b] + 2 * lb + 1)
            rk = slice(off[k], off[k] + 2 * lk + 1)
            mat[:, rb, rk] = mat[:, rb, rk] + blk[n]
    return mat + mat.transpose(-1, -2)


def snorm(s: torch.Tensor) -> torch.Tensor:
    """``integral/utils.py:31-34``."""
    d = s.diagonal()
    return torch.where(d == 0.0, torch.zeros_like(d), d.clamp(min=1e-300) ** -0.5)


def integrals(sysm: System, positions: torch.Tensor, level: int):
    """
    Normalised overlap, and for GFN2 the ket-centred dipole (3) and traceless
    quadrupole (6) integrals (``integral/container.py:182-537``,
    ``types/dipole.py:40-86``, ``types/quadrupole.py``).
    """
    s_raw = multipole_raw(sysm, positions, COMP_S)[0]
    norm = snorm(s_raw)
    nn = norm[:, None] * norm[None, :]
    s = s_raw * nn
    if level < 2:
        return s, None, None
    d0 = multipole_raw(sysm, positions, COMP_D) * nn
    q9 = multipole_raw(sysm, positions, COMP_Q9) * nn
    q = q9[[0, 3, 4, 6, 7, 8]]  # xx yx yy zx zy zz
    porb = positions[_orb_atom(sysm)]  # (nao, 3)
    x, y, z = porb[:, 0], porb[:, 1], porb[:, 2]
    dx, dy, dz = d0[0], d0[1], d0[2]

    def sdiag(c, dc):
        return -2 * c[None, :] * dc + (c * c)[None, :] * s

    def soff(a, b, da, db):
        return -b[None, :] * da - a[None, :] * db + (a * b)[None, :] * s

    q = torch.stack(
        [
            q[0] + sdiag(x, dx),
            q[1] + soff(y, x, dy, dx),
            q[2] + sdiag(y, dy),
            q[3] + soff(z, x, dz, dx),
            q[4] + soff(z, y, dz, dy),
            q[5] + sdiag(z, dz),
        ]
    )
    d = d0 - porb.T[:, None, :] * s[None]
    tr = 0.5 * (q[0] + q[2] + q[5])
    q = torch.stack(
        [1.5 * q[0] - tr, 1.5 * q[1], 1.5 * q[2] - tr, 1.5 * q[3], 1.5 * q[4],
         1.5 * q[5] - tr]
    )
    return s, d, q


def _orb_atom(sysm: System) -> np.ndarray:
    return sysm.ih["shells_to_atom"][sysm.ih["orbitals_to_shell"]]


# --------------------------------------------------------------------------
# coordination numbers (tad_mctc.ncoord.cn_d3 with exp_count / gfn2_count)
# --------------------------------------------------------------------------


def _exp_count(r, r0, k):
    return 1.0 / (1.0 + torch.exp(-k * (r0 / r - 1.0)))


def coordination_number(numbers, positions, kind: str) -> torch.Tensor:
    """
    D3-type coordination number (Grimme et al., JCP 132, 154104 (2010)):
    CN_A = sum_{B != A, R_AB <= 25} count(R_AB, Rcov_A + Rcov_B), with
    count = 1/(1+exp(-16 (R0/R - 1))) for GFN1 (``xtb/gfn1.py:62-64``) and the
    double-exponential GFN2 form count(10, R0) * count(20, R0 + 2)
    (``xtb/gfn2.py:58-62``, ``coulomb/multipole.py:323-328``).
    """
    rcov = torch.tensor(_radii.lookup(_radii.COV_D3, numbers, "covalent"), dtype=DT)
    nat = len(numbers)
    diff = positions[:, None, :] - positions[None, :, :]
    eye = torch.eye(nat, dtype=torch.bool)
    r = torch.sqrt(torch.where(eye[..., None], 1.0, diff * diff).sum(-1))
    r0 = rcov[:, None] + rcov[None, :]
    if kind == "exp":
        cnt = _exp_count(r, r0, 16.0)
    else:
        cnt = _exp_count(r, r0, 10.0) * _exp_count(r, r0 + 2.0, 20.0)
    mask = (~eye) & (r <= CN_CUTOFF)
    return torch.where(mask, cnt, torch.zeros_like(cnt)).sum(-1)


def _distances(positions):
    nat = positions.shape[0]
    eye = torch.eye(nat, dtype=torch.bool)
    diff = positions[:, None, :] - positions[None, :, :]
    r = torch.sqrt(torch.where(eye[..., None], 1.0, diff * diff).sum(-1))
    return torch.where(eye, torch.zeros_like(r), r), eye


# --------------------------------------------------------------------------
# core Hamiltonian (xtb/base.py:255-372, xtb/gfn1.py:66-165, xtb/gfn2.py:67-156)
# --------------------------------------------------------------------------


def _ush_hscale(sysm: System) -> torch.Tensor:
    par = sysm.par
    shell = par["hamiltonian"]["xtb"]["shell"]
    lab = "spdfg"
    n = len(sysm.ush_l)
    ksh = torch.ones(n, n, dtype=DT)
    val = [par["element"][z]["valence"][k] for z, k in zip(sysm.ush_z, sysm.ush_idx_in_elem)]
    if sysm.method == "gfn1":
        kpol = par["hamiltonian"]["xtb"]["kpol"]
        kii = []
        for u, l in enumerate(sysm.ush_l):
            kii.append(kpol if not val[u] else shell.get(lab[l] * 2, 1.0))
        for i in range(n):
            for j in range(n):
                li, lj = lab[sysm.ush_l[i]], lab[sysm.ush_l[j]]
                if val[i] and val[j]:
                    v = shell.get(li + lj, shell.get(lj + li, (kii[i] + kii[j]) / 2))
                else:
                    v = (kii[i] + kii[j]) / 2
                ksh[i, j] = v
    else:
        wexp = par["hamiltonian"]["xtb"]["wexp"]
        zeta = torch.tensor(
            [par["element"][z]["slater"][k] for z, k in zip(sysm.ush_z, sysm.ush_idx_in_elem)],
            dtype=DT,
        )
        zi, zj = zeta[:, None], zeta[None, :]
        zmat = (2 * torch.sqrt(zi * zj) / (zi + zj)) ** wexp
        for i in range(n):
            for j in range(n):
                li, lj = lab[sysm.ush_l[i]], lab[sysm.ush_l[j]]
                if li + lj in shell:
                    v = shell[li + lj]
                elif lj + li in shell:
                    v = shell[lj + li]
                else:
                    v = 0.5 * (shell[li * 2] + shell[lj * 2])
                ksh[i, j] = v * zmat[i, j]
    return ksh


def _kpair(par, za, zb) -> float:
    for a, b, v in par["hamiltonian"]["xtb"].get("kpair", []):
        if (a == za and b == zb) or (a == zb and b == za):
            return v
    return 1.0


def shell_params(sysm: System):
    """Per-shell parameter vectors spread from the element tables."""
    par = sysm.par
    ih = sysm.ih
    out = {k: [] for k in ("levels", "kcn", "shpoly", "refocc", "lgam", "slater", "valence")}
    for s in range(sysm.nsh):
        u = ih["shells_to_ushell"][s]
        z, k = sysm.ush_z[u], sysm.ush_idx_in_elem[u]
        e = par["element"][z]
        for key in out:
            out[key].append(float(e[key][k]))
    return {k: torch.tensor(v, dtype=DT) for k, v in out.items()}


def hamiltonian(sysm: System, positions, s, cn) -> torch.Tensor:
    ih = sysm.ih
    par = sysm.par
    sh_atom = torch.as_tensor(ih["shells_to_atom"])
    sp = shell_params(sysm)
    kcn = sp["kcn"] * _radii.EV2AU
    se = sp["levels"] * _radii.EV2AU - kcn * cn[sh_atom]
    numbers = sysm.numbers
    rad = torch.tensor(_radii.lookup(_radii.ATOMIC_RADII, numbers, "atomic"), dtype=DT)
    dist, eye = _distances(positions)
    rr = dist / (rad[:, None] + rad[None, :])
    rr_sh = torch.where(eye, torch.zeros_like(rr), torch.sqrt(torch.where(eye, 1.0, rr)))
    rr_sh = rr_sh[sh_atom][:, sh_atom]
    pi = (1.0 + sp["shpoly"][:, None] * rr_sh) * (1.0 + sp["shpoly"][None, :] * rr_sh)
    en = torch.tensor([par["element"][int(z)]["en"] for z in numbers], dtype=DT)[sh_atom]
    offsite = ~torch.eye(sysm.nat, dtype=torch.bool)[sh_atom][:, sh_atom]
    enscale = par["hamiltonian"]["xtb"]["enscale"]
    var_x = torch.where(offsite, 1.0 + enscale * (en[:, None] - en[None, :]) ** 2, 0.0)
    z_sh = [int(numbers[a]) for a in ih["shells_to_atom"]]
    kp = torch.tensor([[_kpair(par, a, b) for b in z_sh] for a in z_sh], dtype=DT)
    hs_u = _ush_hscale(sysm)
    ush = torch.as_tensor(ih["shells_to_ushell"])
    hs = hs_u[ush][:, ush]
    val = sp["valence"] > 0.5
    var_k = torch.where(val[:, None] & val[None, :], hs * kp * var_x, hs)
    var_h = 0.5 * (se[:, None] + se[None, :])
    hsh = torch.where(offsite, pi * var_k * var_h, var_h)
    o2s = torch.as_tensor(ih["orbitals_to_shell"])
    h = hsh[o2s][:, o2s] * s
    return 0.5 * (h + h.T)


# --------------------------------------------------------------------------
# interactions
# --------------------------------------------------------------------------


@dataclass
class Caches:
    gamma: torch.Tensor  # (nsh, nsh)
    hd: torch.Tensor  # ES3: per atom (GFN1) or per shell (GFN2)
    es3_shell: bool
    aes2: dict | None = None
    gb: torch.Tensor | None = None  # (nat, nat) generalized Born matrix


def es2_gamma(sysm: System, positions) -> torch.Tensor:
    """Shell-resolved Coulomb matrix (``coulomb/secondorder.py:799-872``)."""
    par = sysm.par
    ih = sysm.ih
    sh_atom = torch.as_tensor(ih["shells_to_atom"])
    sp = shell_params(sysm)
    gam = torch.tensor([par["element"][int(z)]["gam"] for z in sysm.numbers], dtype=DT)
    h = sp["lgam"] * gam[sh_atom] + EPS
    g = par["charge"]["effective"]["gexp"]
    avg_kind = par["charge"]["effective"]["average"]
    if avg_kind == "harmonic":
        hi = 1.0 / h
        avg = 2.0 / (hi[:, None] + hi[None, :])
    elif avg_kind == "arithmetic":
        avg = 0.5 * (h[:, None] + h[None, :])
    else:
        avg = torch.sqrt(h[:, None] * h[None, :])
    dist, eye = _distances(positions)
    dg = torch.where(eye, torch.full_like(dist, EPS), (dist + EPS) ** g)[sh_atom][:, sh_atom]
    return 1.0 / (dg + avg ** (-g)) ** (1.0 / g)


def es3_hd(sysm: System):
    """``coulomb/thirdorder.py:get_cache``."""
    par = sysm.par
    to = par["thirdorder"]
    gam3 = torch.tensor([par["element"][int(z)]["gam3"] for z in sysm.numbers], dtype=DT)
    if to.get("shell", False) is False:
        return gam3, False
    scale = [to["shell"]["s"], to["shell"]["p"], to["shell"]["d"]]
    sh_atom = torch.as_tensor(sysm.ih["shells_to_atom"])
    sc = torch.tensor([scale[l] for l in sysm.ih["angular"]], dtype=DT)
    return gam3[sh_atom] * sc, True


def aes2_cache(sysm: System, positions, cn2) -> dict:
    """``coulomb/multipole.py:270-448``; ``cn2`` is the GFN2 coordination number."""
    par = sysm.par
    mp = par["multipole"]["damped"]
    el = [par["element"][int(z)] for z in sysm.numbers]
    rad = torch.tensor([e["mprad"] for e in el], dtype=DT)
    vcn = torch.tensor([e["mpvcn"] for e in el], dtype=DT)
    dk = torch.tensor([e["dkernel"] for e in el], dtype=DT)
    qk = torch.tensor([e["qkernel"] for e in el], dtype=DT)
    t1 = torch.exp(-mp["kexp"] * (cn2 - vcn - mp["shift"]))
    mrad = rad + (mp["rmax"] - rad) / (1.0 + t1)
    dist, eye = _distances(positions)
    g1 = torch.where(eye, torch.zeros_like(dist), 1.0 / torch.where(eye, 1.0, dist))
    g3 = g1**3
    g5 = g3 * g1 * g1
    rr = 0.5 * (mrad[:, None] + mrad[None, :]) * g1
    f3 = 1.0 / (1.0 + 6.0 * rr ** mp["dmp3"])
    f5 = 1.0 / (1.0 + 6.0 * rr ** mp["dmp5"])
    rij = torch.where(eye[..., None], EPS, positions[:, None, :] - positions[None, :, :])
    sd = rij * (g3 * f3)[..., None]
    g5f5 = (g5 * f5)[..., None, None]
    dd = torch.eye(3, dtype=DT) * (g3 * f5)[..., None, None] - rij[..., :, None] * rij[..., None, :] * 3 * g5f5
    x, y, z = rij[..., 0], rij[..., 1], rij[..., 2]
    sq = torch.stack([x * x, 2 * x * y, y * y, 2 * x * z, 2 * y * z, z * z], -1) * (g5 * f5)[..., None]
    return {"sd": sd, "dd": dd, "sq": sq, "dk": dk, "qk": qk, "mrad": mrad}


QSCALE = torch.tensor([1.0, 2.0, 1.0, 2.0, 2.0, 1.0], dtype=DT)


def potentials(sysm: System, c: Caches, q_orb, dp, qp):
    """Orbital monopole and atomic multipole potentials (``interactions/base.py:135-181``)."""
    ih = sysm.ih
    o2s = torch.as_tensor(ih["orbitals_to_shell"])
    s2a = torch.as_tensor(ih["shells_to_atom"])
    qsh = torch.zeros(sysm.nsh, dtype=DT).index_add(0, o2s, q_orb)
    qat = torch.zeros(sysm.nat, dtype=DT).index_add(0, s2a, qsh)
    vsh = c.gamma @ qsh
    vat = torch.zeros(sysm.nat, dtype=DT)
    if c.es3_shell:
        vsh = vsh + c.hd * qsh**2
    else:
        vat = vat + c.hd * qat**2
    vdp = vqp = None
    if c.aes2 is not None:
        a = c.aes2
        vat = vat + torch.einsum("ijx,jx->i", a["sd"], dp) + torch.einsum("ijx,jx->i", a["sq"], qp)
        vdp = torch.einsum("ijx,i->jx", a["sd"], qat) + torch.einsum("ijxy,ix->jy", a["dd"], dp) + 2 * a["dk"][:, None] * dp
        vqp = torch.einsum("ijx,i->jx", a["sq"], qat) + 2 * a["qk"][:, None] * qp * QSCALE
    if c.gb is not None:
        vat = vat + c.gb @ qat
    vsh = vsh + vat[s2a]
    return vsh[o2s], vdp, vqp


def interaction_energy(sysm: System, c: Caches, q_orb, dp, qp) -> torch.Tensor:
    """``interactions/base.py:306-360`` summed over atoms and components."""
    ih = sysm.ih
    o2s = torch.as_tensor(ih["orbitals_to_shell"])
    s2a = torch.as_tensor(ih["shells_to_atom"])
    qsh = torch.zeros(sysm.nsh, dtype=DT).index_add(0, o2s, q_orb)
    qat = torch.zeros(sysm.nat, dtype=DT).index_add(0, s2a, qsh)
    e = 0.5 * (qsh * (c.gamma @ qsh)).sum()
    if c.es3_shell:
        e = e + (c.hd * qsh**3 / 3.0).sum()
    else:
        e = e + (c.hd * qat**3 / 3.0).sum()
    if c.aes2 is not None:
        a = c.aes2
        vdp_sd = torch.einsum("ijx,i->jx", a["sd"], qat)
        vdp_dd = 0.5 * torch.einsum("ijxy,ix->jy", a["dd"], dp)
        e = e + (a["dk"][:, None] * dp * dp).sum() + ((vdp_sd + vdp_dd) * dp).sum()
        vqp = torch.einsum("ijx,i->jx", a["sq"], qat)
        e = e + (a["qk"][:, None] * qp * QSCALE * qp).sum() + (vqp * qp).sum()
    if c.gb is not None:
        e = e + 0.5 * (qat * (c.gb @ qat)).sum()
    return e


def repulsion_energy(sysm: System, positions) -> torch.Tensor:
    """``classicals/repulsion/base.py:240-430`` and ``rep.py`` (0.5 sum over pairs)."""
    par = sysm.par
    rp = par["repulsion"]["effective"]
    el = [par["element"][int(z)] for z in sysm.numbers]
    arep = torch.tensor([e["arep"] for e in el], dtype=DT)
    zeff = torch.tensor([e["zeff"] for e in el], dtype=DT)
    dist, eye = _distances(positions)
    a = torch.sqrt(arep[:, None] * arep[None, :] + torch.finfo(DT).tiny)
    z = zeff[:, None] * zeff[None, :]
    k = torch.full_like(dist, rp["kexp"])
    if "klight" in rp:
        light = torch.as_tensor(sysm.numbers <= 2)
        k = torch.where(light[:, None] & light[None, :], torch.full_like(k, rp["klight"]), k)
    dsafe = torch.where(eye, 1.0, dist)
    e = z * torch.exp(-a * dsafe**k) / dsafe
    e = torch.where((~eye) & (dist <= REP_CUTOFF), e, torch.zeros_like(e))
    return 0.5 * e.sum()


# --------------------------------------------------------------------------
# SCF (scf/iterator.py, scf/pure/conversions.py, wavefunction/filling.py)
# --------------------------------------------------------------------------


def reference_occupation(sysm: System, chrg: float = 0.0, spin: int | None = None):
    """``scf/iterator.py:147-195`` and ``filling.py:180-259``: ``spin``
    unpaired electrons (None: the parity of the electron count); a count
    above the electrons or of the wrong parity raises ValueError."""
    sp = shell_params(sysm)
    nsph = torch.as_tensor(sysm.ih["orbitals_per_shell"]).to(DT)
    o2s = torch.as_tensor(sysm.ih["orbitals_to_shell"])
    n0 = (sp["refocc"] / nsph)[o2s]
    nel = float(sp["refocc"].sum()) - chrg
    uhf = math.floor(nel + 0.5) % 2
    if spin is not None:
        if spin > math.floor(nel + 0.5) or spin % 2 != uhf:
            raise ValueError(f"{spin} unpaired electrons do not fit {nel} electrons")
        uhf = int(spin)
    diff = min(uhf, nel)
    nb = (nel - diff) / 2.0
    return n0, (nb + diff, nb)


def fermi_occupation(eps: torch.Tensor, nel: float, kt: float) -> torch.Tensor:
    """
    Fermi–Dirac occupation of singly-occupied orbitals summing to ``nel``
    (the fixed point of ``filling.py:428-742``): bisection on the electron
    count to machine precision.
    """
    n = eps.shape[0]
    if nel <= 0.0:
        return torch.zeros_like(eps)
    if nel >= n:
        return torch.ones_like(eps)
    lo = float(eps.min()) - 60 * kt
    hi = float(eps.max()) + 60 * kt
    e = eps.detach()

    def count(mu):
        x = (e - mu) / kt
        return torch.where(x > 0, torch.exp(-x) / (1 + torch.exp(-x)), 1 / (1 + torch.exp(x))).sum()

    for _ in range(200):
        mu = 0.5 * (lo + hi)
        if float(count(mu)) > nel:
            hi = mu
        else:
            lo = mu
        if hi - lo < 1e-16 * max(1.0, abs(mu)):
            break
    mu = 0.5 * (lo + hi)
    x = (e - mu) / kt
    return torch.where(x > 0, torch.exp(-x) / (1 + torch.exp(-x)), 1 / (1 + torch.exp(x)))


def moments(sysm: System, p, s, d, q):
    """``conversions.py:203-251``: Mulliken charges and atomic multipoles."""
    pop = (p * s).sum(0)  # diag(P S) for symmetric P, S
    dp = qp = None
    if d is not None:
        oa = torch.as_tensor(_orb_atom(sysm))
        # -sum_k P_ik D[m, k, i]
        dpo = -torch.einsum("ik,mki->im", p, d)
        qpo = -torch.einsum("ik,mki->im", p, q)
        dp = torch.zeros(sysm.nat, 3, dtype=DT).index_add(0, oa, dpo)
        qp = torch.zeros(sysm.nat, 6, dtype=DT).index_add(0, oa, qpo)
    return pop, dp, qp


def fock(sysm: System, h0, s, d, q, vorb, vdp, vqp):
    """``conversions.py:255-297``."""
    f = h0 - 0.5 * s * (vorb[:, None] + vorb[None, :])
    oa = torch.as_tensor(_orb_atom(sysm))
    for mp, v in ((d, vdp), (q, vqp)):
        if mp is not None and v is not None:
            vo = v[oa]  # (nao, ncomp)
            tmp = 0.5 * torch.einsum("kij,jk->ij", mp, vo)
            f = f - (tmp + tmp.T)
    return f


@dataclass
class Result:
    energy: float
    e_elec: float
    e_rep: float
    e_free: float
    iterations: int
    p: torch.Tensor
    w: torch.Tensor
    q: torch.Tensor
    eps: torch.Tensor
    occ: torch.Tensor
    cn: torch.Tensor
    extra: dict


def _geometry_terms(sysm: System, positions, solvation=None):
    level = 2 if sysm.method == "gfn2" else 1
    s, d, q = integrals(sysm, positions, level)
    cn = coordination_number(
        sysm.numbers, positions, sysm.par["hamiltonian"]["xtb"]["cn"]
    ) if sysm.nat > 0 else None
    h0 = hamiltonian(sysm, positions, s, cn)
    gamma = es2_gamma(sysm, positions)
    hd, es3_shell = es3_hd(sysm)
    aes = None
    if sysm.method == "gfn2":
        cn2 = coordination_number(sysm.numbers, positions, "gfn")
        aes = aes2_cache(sysm, positions, cn2)
    gb = None
    if solvation is not None:
        from oracle import solvation_oracle

        gb = solvation_oracle.born_matrix(sysm.numbers, positions, **solvation)
    return s, d, q, h0, cn, Caches(gamma, hd, es3_shell, aes, gb)


def singlepoint(
    method: str,
    numbers,
    positions,
    chrg: float = 0.0,
    spin: int | None = None,
    etemp: float = 300.0,
    maxiter: int = 250,
    tol: float = 1e-11,
    solvation: dict | None = None,
    grad: bool = False,
    exclude: tuple = (),
    mixer: str = "broyden1",
    anderson: dict | None = None,
) -> Result:
    """
    GFN1/GFN2 single point: SCF on the potential, energy as in
    ``scf/base.py:510-619`` + repulsion; with ``grad`` the forces are
    ``-dE/dR`` from autograd of the energy functional at the final density
    (variational: ``E[P, R] - tr(W S(R))``).

    mixer "broyden1": the implicit mode's root solver to ``tol`` (x_atol =
    f_atol), ``broyden1_loop``. mixer "anderson": the full mode's loop with
    the Anderson mixer, ``anderson_loop``, with the options of ``anderson``
    (reference defaults: x_atol 1e-4, x_atol_max 1e-5, damp 0.5, damp_init
    0.1, generations 5, soft_start, diagonal_offset 0.01) and ``maxiter``.
    """
    sysm = make_system(method, numbers)
    pos = torch.as_tensor(positions, dtype=DT).clone()
    kt = etemp * _radii.KELVIN2AU
    with torch.no_grad():
        s, d, q, h0, cn, c = _geometry_terms(sysm, pos, solvation)
        n0, (na, nb) = reference_occupation(sysm, chrg, spin)
        lchol = torch.linalg.cholesky(s)
        linv = torch.linalg.inv(lchol)
        nat = sysm.nat
        ncomp = 1 + (9 if d is not None else 0)

        def f_map(x):
            vo = x[: sysm.nao]
            vdp = x[sysm.nao : sysm.nao + 3 * nat].reshape(nat, 3) if d is not None else None
            vqp = x[sysm.nao + 3 * nat :].reshape(nat, 6) if d is not None else None
            fm = fock(sysm, h0, s, d, q, vo, vdp, vqp)
            ev, y = torch.linalg.eigh(linv @ fm @ linv.T)
            cmat = linv.T @ y
            fa = fermi_occupation(ev, na, kt)
            fb = fermi_occupation(ev, nb, kt)
            occ = fa + fb
            p = (cmat * occ) @ cmat.T
            pop, dp, qp = moments(sysm, p, s, d, q)
            qo = n0 - pop
            v, vd, vq = potentials(sysm, c, qo, dp, qp)
            parts = [v] + ([vd.reshape(-1), vq.reshape(-1)] if d is not None else [])
            return torch.cat(parts), (p, cmat, ev, fa, fb, qo, dp, qp)

        x = torch.zeros(sysm.nao + (9 * nat if d is not None else 0), dtype=DT)
        if mixer == "anderson":
            x, it, conv = anderson_loop(lambda v: f_map(v)[0], x, maxiter, anderson or {})
            hit_max = not conv
        else:
            x, it, hit_max = broyden1_loop(lambda v: f_map(v)[0], x, maxiter, tol)
        gx, aux = f_map(x)
        p, cmat, ev, fa, fb, qo, dp, qp = aux
        occ = fa + fb
        e_h0 = (p * h0).sum()
        e_int = interaction_energy(sysm, c, qo, dp, qp)

        def ts(f):
            o = f.clamp(min=EPS)
            o1 = (1 - f).clamp(min=EPS)
            return (o * torch.log(o) + o1 * torch.log(o1)).sum()

        e_free = kt * (ts(fa) + ts(fb))
        e_rep = repulsion_energy(sysm, pos) if "rep" not in exclude else torch.zeros((), dtype=DT)
        w = (cmat * (occ * ev)) @ cmat.T
    energy = float(e_h0 + e_int + e_free + e_rep)
    extra = {"e_h0": float(e_h0), "e_int": float(e_int), "s": s, "h0": h0, "converged": not hit_max}
    res = Result(
        energy, float(e_h0 + e_int), float(e_rep), float(e_free), it, p, w, qo,
        ev, occ, cn, extra,
    )
    if grad:
        res.extra["gradient"] = gradient(sysm, pos, p, w, n0, solvation, exclude)
    return res


def broyden1_loop(g_map, x, maxiter: int, tol: float, alpha: float = -0.5, damp: float = 0.5):
    """
    The implicit mode's root solver on F(x) = x - G(x): xitorch broyden1
    (exlibs/xitorch/_impls/optimize/root/rootsolver.py:42-265 and
    _jacobian.py:51-120 with alpha = -0.5, damp = 0.5, no line search;
    scf/base.py:267-292), inverse Jacobian Gm = -alpha I + C D^T, stop when
    |dx|_2 < tol and |F|_2 < tol; after maxiter the best iterate is returned.
    Returns (x, iterations, hit_maxiter).
    """
    cs, ds = [], []
    best = None
    x_old = y_old = None
    dx_norm = float("inf")
    it = 0
    for it in range(1, maxiter + 1):
        y = x - g_map(x)
        ynorm = float(torch.linalg.norm(y))
        if it == 1:
            best = (ynorm, x.clone())
        else:
            if ynorm < best[0]:
                best = (ynorm, x.clone())
            dxx, dyy = x - x_old, y - y_old

            def gm(v):
                out = -alpha * v
                for c_, d_ in zip(cs, ds):
                    out = out + c_ * torch.dot(d_, v)
                return out

            def gmt(v):
                out = -alpha * v
                for c_, d_ in zip(cs, ds):
                    out = out + d_ * torch.dot(c_, v)
                return out

            v = gmt(dxx)
            cs.append(dxx - gm(dyy))
            ds.append(v / torch.dot(dyy, v))
            if dx_norm < tol and ynorm < tol:
                return x, it, False
        if it == maxiter:
            return best[1], it, True
        dxv = alpha * y
        for c_, d_ in zip(cs, ds):
            dxv = dxv - c_ * torch.dot(d_, y)
        dx_norm = float(torch.linalg.norm(dxv))
        x_old, y_old = x.clone(), y.clone()
        x = x + damp * dxv
    return x, it, True


def anderson_loop(g_map, guess, maxiter: int, opts: dict):
    """
    The full mode's SCF loop (scf/unrolling/default.py:80-140: mix_guess,
    then up to maxiter calls, convergence tested after each mixing on the
    current difference) with the Anderson mixer (scf/mixer/anderson.py:
    163-317, Eyert's method without theta_0; mixer/base.py:230-256 for the
    convergence test |F|_2 < x_atol and max|F| < x_atol_max). Returns
    (G(x) at the last call, loop iterations, converged): the reference
    evaluates the energy at that converged value (converged_to_charges).
    """
    damp = opts.get("damp", 0.5)
    damp_init = opts.get("damp_init", 0.1)
    gens = opts.get("generations", 5)
    offset = opts.get("diagonal_offset", 0.01)
    soft = opts.get("soft_start", True)
    x_tol = opts.get("x_atol", 1e-4)
    x_tol_max = opts.get("x_atol_max", 1e-5)
    xh = torch.zeros(gens + 1, len(guess), dtype=DT)  # x history, entry 0 = current input
    fh = torch.zeros(gens + 1, len(guess), dtype=DT)  # difference history
    step = 0

    def mix(x_new, x_old):
        nonlocal step, xh, fh
        xh[0] = x_old
        step += 1
        fh[0] = x_new - x_old
        if step > gens or (step > 1 and not soft):
            n = min(step - 1, gens)
            df = fh[0] - fh[1 : n + 1]
            a = df @ df.T
            b = df @ fh[0]
            eye = torch.eye(n, dtype=DT)
            a = a * torch.where(eye != 0, eye + offset**2, torch.ones((), dtype=DT))
            th = torch.linalg.solve(a, b)
            x_bar = th @ (xh[1 : n + 1] - xh[0]) + xh[0]
            f_bar = th @ (-df) + fh[0]
            x_mix = x_bar + damp * f_bar
        else:
            x_mix = xh[0] + damp_init * fh[0]
        delta = fh[0].clone()
        fh = torch.roll(fh, 1, 0)
        xh = torch.roll(xh, 1, 0)
        xh[0] = x_mix
        return x_mix, delta

    q_new = g_map(guess)
    q, _ = mix(q_new, guess)
    for it in range(1, maxiter + 1):
        q_new = g_map(q)
        q, delta = mix(q_new, q)
        if float(torch.linalg.norm(delta)) < x_tol and float(delta.abs().max()) < x_tol_max:
            return q_new, it, True
    return q_new, maxiter, False


def gradient(sysm: System, positions, p, w, n0, solvation=None, exclude=()) -> torch.Tensor:
    """dE/dR at fixed converged P and W (Hellmann–Feynman + Pulay terms)."""
    pos = positions.clone().requires_grad_(True)
    s, d, q, h0, cn, c = _geometry_terms(sysm, pos, solvation)
    pop, dp, qp = moments(sysm, p, s, d, q)
    e = (p * h0).sum() + interaction_energy(sysm, c, n0 - pop, dp, qp)
    if "rep" not in exclude:
        e = e + repulsion_energy(sysm, pos)
    e = e - (w * s).sum()
    (g,) = torch.autograd.grad(e, pos)
    return g


HALOGENS = (17, 35, 53, 85)   # components/classicals/halogen/hal.py: donors
XB_BASES = (7, 8, 15, 16)     # and acceptors
XB_CUTOFF = 20.0              # constants/xtb.py DEFAULT_XB_CUTOFF


def halogen_energy(par: dict, numbers, positions) -> torch.Tensor:
    """
    GFN1 halogen-bond correction (``components/classicals/halogen/hal.py``,
    ``_xbond_list`` and ``_xbond_energy``): for every donor X and acceptor J
    within the cutoff, with K the nearest other atom of X,
    E_X += xbond_X (l12 - damp l6) / (1 + l12) (1/2 - cos(J-X-K) / 4)^6,
    l6 = ((R_X + R_J) rscale / r_XJ)^6 with the atomic radii of the H0
    distance polynomial. Differentiable in ``positions``.
    """
    z = [int(v) for v in np.asarray(numbers).ravel()]
    pos = torch.as_tensor(positions, dtype=DT)
    xb = par["halogen"]["classical"]
    damp, rscale = float(xb["damping"]), float(xb["rscale"])
    e = torch.zeros((), dtype=DT)
    for x, zx in enumerate(z):
        if zx not in HALOGENS:
            continue
        strength = float(par["element"][zx].get("xbond", 0.0))
        d = ((pos - pos[x]) ** 2).sum(-1)
        dk = d.detach().clone()
        dk[x] = float("inf")
        k = int(torch.argmin(dk))
        for j, zj in enumerate(z):
            if zj not in XB_BASES or float(dk[j].sqrt()) > XB_CUTOFF:
                continue
            r0 = (_radii.ATOMIC_RADII[zx] + _radii.ATOMIC_RADII[zj]) * rscale
            l6 = (r0**2 / d[j]) ** 3
            l12 = l6 * l6
            lj = (l12 - damp * l6) / (1.0 + l12)
            dkj = ((pos[k] - pos[j]) ** 2).sum()
            cosa = (d[k] + d[j] - dkj) / torch.sqrt(d[k] * d[j])
            e = e + strength * lj * (0.5 - 0.25 * cosa) ** 6
    return e


def dipole_moment(sysm: System, positions, p) -> torch.Tensor:
    """
    Electric dipole moment (e a0) at the density ``p``: the valence charges
    at the nuclei minus the electronic moment about the origin,
    sum_A Z_A R_A - tr(P D0) (``calculators/properties/moments/dip.py``
    ``dipole_xtb``, with ``integral`` the normalised dipole integral about
    the origin). Z_A = sum of the reference occupations of A's shells (the
    neutral atom's valence electrons).
    """
    pos = torch.as_tensor(positions, dtype=DT)
    s_raw = multipole_raw(sysm, pos, COMP_S)[0]
    norm = snorm(s_raw)
    d0 = multipole_raw(sysm, pos, COMP_D) * (norm[:, None] * norm[None, :])
    n0, _ = reference_occupation(sysm, 0.0)
    zval = torch.zeros(sysm.nat, dtype=DT).index_add_(0, torch.as_tensor(_orb_atom(sysm)), n0)
    return (zval[:, None] * pos).sum(0) - torch.einsum("xij,ij->x", d0, p)


# --------------------------------------------------------------------------
# Turbomole ``coord`` reader (the format of test/test_singlepoint/mols/*/coord)
# --------------------------------------------------------------------------


def read_coord(path) -> tuple[np.ndarray, np.ndarray]:
    """Atomic numbers and positions (Bohr) from a Turbomole ``$coord`` block."""
    syms = [e["symbol"].lower() for _, e in sorted(load_par("gfn2")["element"].items())]
    numbers, pos = [], []
    active = False
    for line in Path(path).read_text().splitlines():
        t = line.strip()
        if t.startswith("$"):
            active = t.startswith("$coord")
            continue
        if active and t:
            f = t.split()
            pos.append([float(v) for v in f[:3]])
            numbers.append(syms.index(f[3].lower()) + 1)
    return np.array(numbers, dtype=np.int64), np.array(pos, dtype=np.float64)
