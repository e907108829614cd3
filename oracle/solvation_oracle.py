"""
CPU restatement of dxtb's generalized-Born / ALPB solvation (test
infrastructure only: the CUDA path never imports this module).

Follows ``src/dxtb/_src/components/interactions/solvation/born.py`` and
``alpb.py`` of the reference:

- ``compute_psi``: born.py:153-239, the dielectric descreening integral.
  ``psi_j = sum_{i != j, r_ij <= cutoff} h(r_ij; rho_i = 0.8 rvdw_i, rvdw_j)``
  has two forms. The overlapping form is used when ``r < rvdw_j + rho_i``
  and ``r + rho_i > rvdw_j``; otherwise the non-overlapping one is used.
- ``born_radii``: born.py:60-151, the Onufriev-Bashford-Case radii with
  obc = (1.0, 0.8, 4.85).
- ``p16_kernel`` / ``still_kernel``: alpb.py:94-142.
- ``adet``: alpb.py:144-184, the ALPB shape descriptor from the inertia
  tensor of solid spheres.
- ``born_matrix``: alpb.py:257-321,
  ``A = keps * kernel(R, B_i B_j) [+ keps * alpbet * adet]``.
  Here ``alpbet = 0.571412 / eps`` (ALPB) or 0 (GB), and
  ``keps = (1/eps - 1) / (1 + alpbet)``.

Everything is float64 torch and differentiable, so the oracle's autograd
gradient covers the solvation term (the reference differentiates it with
autograd as well).
"""

from __future__ import annotations

import numpy as np
import torch

ALPHA_ALPB = 0.571412
OBC = (1.0, 0.8, 4.85)
DESCREENING = 0.8
CUTOFF = 66.0


def _rvdw(numbers) -> torch.Tensor:
    from dxtb_gb300.data import radii

    return torch.as_tensor(radii.lookup(radii.VDW_D3, numbers, "van-der-Waals"), dtype=torch.float64)


def _pair_dist(positions: torch.Tensor) -> tuple[torch.Tensor, torch.Tensor]:
    """Distances with an exact 0 on the diagonal (and a finite derivative there)."""
    nat = positions.shape[0]
    off = ~torch.eye(nat, dtype=torch.bool)
    d = positions.unsqueeze(-2) - positions.unsqueeze(-3)
    r2 = (d * d).sum(-1)
    r = torch.sqrt(torch.where(off, r2, torch.ones_like(r2)))
    return torch.where(off, r, torch.zeros_like(r)), off


def compute_psi(positions: torch.Tensor, rvdw: torch.Tensor, cutoff: float = CUTOFF,
                descreening: float = DESCREENING) -> torch.Tensor:
    """Descreening integral psi_j (born.py:153-239); index i = rows (descreener)."""
    r, off = _pair_dist(positions)
    rs = torch.where(off, r, torch.ones_like(r))
    rho = (rvdw * descreening).unsqueeze(-1)      # rho_i (rows)
    rv = rvdw.unsqueeze(-2)                      # rvdw_j (columns)
    d_pl = rs + rho
    d_mi = rs - rho
    d_pr = d_pl * d_mi
    d_qu = d_mi / d_pl
    one = torch.ones_like(rs)
    non_ovlp = rho / torch.where(off, d_pr, one) + torch.where(
        off & (d_qu > 0), 0.5 * torch.log(torch.where(d_qu > 0, d_qu, one)) / rs, torch.zeros_like(rs)
    )
    ratio = d_pl / rv
    ovlp = 1.0 / rv - 1.0 / d_pl + 0.5 / rs * (0.5 * d_mi * (1.0 / d_pl - ratio / rv) - torch.log(ratio))
    use_ovlp = (rs < rv + rho) & (rs + rho > rv)
    term = torch.where(use_ovlp, ovlp, non_ovlp)
    term = torch.where(off & (rs <= cutoff), term, torch.zeros_like(term))
    return term.sum(-2)


def born_radii(positions: torch.Tensor, rvdw: torch.Tensor, born_scale: float = 1.0,
               born_offset: float = 0.0) -> tuple[torch.Tensor, torch.Tensor]:
    """(Born radii, psi) by the OBC integrator (born.py:60-151)."""
    psi = compute_psi(positions, rvdw)
    srvdw = rvdw - born_offset
    r1 = 1.0 / rvdw
    s1 = 1.0 / srvdw
    x = 0.5 * psi * srvdw
    t = x * (OBC[0] + x * (OBC[2] * x - OBC[1]))
    return born_scale / (s1 - r1 * torch.tanh(t)), psi


def p16_kernel(r: torch.Tensor, ab: torch.Tensor) -> torch.Tensor:
    s = torch.sqrt(ab)
    arg = (s / (s + r * 1.028 / 16)) ** 16
    return 1.0 / (r + s * arg)


def still_kernel(r: torch.Tensor, ab: torch.Tensor) -> torch.Tensor:
    r2 = r * r
    return 1.0 / torch.sqrt(r2 + ab * torch.exp(-0.25 * r2 / ab))


def adet(positions: torch.Tensor, rad: torch.Tensor) -> torch.Tensor:
    """ALPB shape descriptor (alpb.py:144-184)."""
    vol = rad**3
    center = (positions * vol.unsqueeze(-1)).sum(-2) / vol.sum()
    d = positions - center
    diag = (d * d).sum(-1) + 0.4 * rad**2
    inertia = (vol[:, None, None] * (torch.diag_embed(diag.unsqueeze(-1).expand(-1, 3))
                                     - d.unsqueeze(-1) * d.unsqueeze(-2))).sum(0)
    det = torch.linalg.det(inertia)
    return torch.sqrt(5.0 * det ** (1.0 / 3.0) / (2.0 * vol.sum()))


def born_matrix(numbers, positions: torch.Tensor, epsilon: float = 78.9, alpb: bool = True,
                kernel: str = "p16", born_scale: float = 1.0, born_offset: float = 0.0,
                rvdw: torch.Tensor | None = None, **_) -> torch.Tensor:
    """A_ij of alpb.py:257-321 (diagonal included, r_ii = 0)."""
    pos = positions if torch.is_tensor(positions) else torch.as_tensor(positions, dtype=torch.float64)
    if rvdw is None:
        rvdw = _rvdw(np.asarray(numbers))
    born, _ = born_radii(pos, rvdw, born_scale, born_offset)
    alpbet = ALPHA_ALPB / epsilon if alpb else 0.0
    keps = (1.0 / epsilon - 1.0) / (1.0 + alpbet)
    r, _ = _pair_dist(pos)
    ab = born.unsqueeze(-1) * born.unsqueeze(-2)
    f = {"p16": p16_kernel, "still": still_kernel}[kernel](r, ab)
    mat = keps * f
    if alpbet > 0:
        mat = mat + keps * alpbet * adet(pos, rvdw)
    return mat


def atom_energies(numbers, positions, charges, **kw) -> torch.Tensor:
    """E_i = 1/2 q_i (A q)_i (alpb.py:323-341)."""
    A = born_matrix(numbers, positions, **kw)
    q = torch.as_tensor(charges, dtype=torch.float64)
    return 0.5 * q * (A @ q)
