"""
Molecular properties on top of the GPU single point: the electric dipole
moment, the harmonic vibrational analysis and IR intensities.

Reference interfaces (paths relative to ``src/dxtb/_src``):

- ``calculators/properties/moments/dip.py`` (``dipole_xtb``): mu = sum_A Z_A
  R_A - tr(P D0), with D0 the normalised dipole integral about the origin and
  Z_A the valence charge. Here ``dxtb_dipole_moment`` evaluates it for every
  molecule of a packed batch in one launch.
- ``calculators/properties/vibration/analysis.py`` (``vib_analysis``,
  ``VibResult``): mass-weighted Hessian, translations and rotations
  projected out, frequencies sqrt(lambda) (signed) in atomic units and
  un-mass-weighted normal modes.
- ``calculators/properties/vibration/ir.py`` (``ir_ints``, ``IRResult``):
  intensities sum_x (d mu_x / dQ)^2 from the nuclear dipole derivative and
  the normal modes.
- ``calculators/properties/vibration/result.py`` (``BaseResult``): results
  stored in atomic units, converted on request.

The Hessian and the dipole derivative come from the same packed batch of the
6 nat displaced geometries (``dxtb_gb300.hessian``): analytic gradients and
dipole moments of every displaced single point, central differences.
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib
from .data.masses import AU2KMMOL, AU2RCM, atomic_mass

LINDEP_THRESHOLD = 1e-7


def dipole_moments(pb, density: torch.Tensor, stream=None) -> torch.Tensor:
    """
    Dipole moments (nmol, 3) in e a0 of every molecule of the packed batch
    ``pb`` at the densities ``density`` (packed n_m x n_m blocks), from one
    launch of the raw integrals about the origin and one of
    ``dxtb_dipole_moment``.
    """
    L = _lib.lib()
    nm = int(pb.total["mat"])
    dev = pb.device
    s = torch.empty(nm, dtype=torch.float64, device=dev)
    d0 = torch.empty(3 * nm, dtype=torch.float64, device=dev)
    q9 = torch.empty(9 * nm, dtype=torch.float64, device=dev)  # the kernel writes D and Q together
    out = torch.empty(pb.nmol * 3, dtype=torch.float64, device=dev)
    st = _lib.stream_ptr() if stream is None else stream
    _lib.check(L.dxtb_multipole_raw(C.byref(pb.struct), pb.t["par_f"].data_ptr(),
                                    pb.t["par_i"].data_ptr(), s.data_ptr(), d0.data_ptr(),
                                    q9.data_ptr(), st),
               "dipole integrals")
    _lib.check(L.dxtb_dipole_moment(C.byref(pb.struct), pb.t["n0"].data_ptr(), density.data_ptr(),
                                    d0.data_ptr(), out.data_ptr(), st),
               "dipole moment")
    return out.view(pb.nmol, 3)


class BaseResult:
    """Frequencies stored in atomic units, returned in ``freqs_unit``."""

    converter_freqs = {"a.u.": 1.0, "cm^-1": AU2RCM}

    def __init__(self, freqs: torch.Tensor):
        self._freqs = freqs
        self._freqs_unit = "a.u."

    @property
    def freqs(self) -> torch.Tensor:
        return self._freqs * self.converter_freqs[self._freqs_unit]

    @freqs.setter
    def freqs(self, *_):
        raise RuntimeError("Setting frequencies is not supported; they are stored in atomic "
                           "units. Use `to_unit` or set `freqs_unit`.")

    @property
    def freqs_unit(self) -> str:
        return self._freqs_unit

    @freqs_unit.setter
    def freqs_unit(self, value: str) -> None:
        if value not in self.converter_freqs:
            raise ValueError(f"Unsupported frequency unit: {value}")
        self._freqs_unit = value

    @staticmethod
    def _convert(value, unit, converter):
        if unit not in converter:
            raise ValueError(f"Unsupported unit for conversion: {unit}")
        return value * converter[unit]


class VibResult(BaseResult):
    """Frequencies (atomic units) and normal modes (3 nat, nfreqs)."""

    def __init__(self, freqs: torch.Tensor, modes: torch.Tensor):
        super().__init__(freqs)
        self._modes = modes

    @property
    def modes(self) -> torch.Tensor:
        return self._modes

    def to_unit(self, value: str, unit: str) -> torch.Tensor:
        if value == "freqs":
            return self._convert(self._freqs, unit, self.converter_freqs)
        raise ValueError(f"Unsupported value for conversion: {value}")

    def use_common_units(self) -> None:
        self.freqs_unit = "cm^-1"

    def __iter__(self):
        return iter((self.freqs, self.modes))


class IRResult(BaseResult):
    """Frequencies and IR intensities (stored in atomic units)."""

    converter_ints = {"a.u.": 1.0, "km/mol": AU2KMMOL}

    def __init__(self, freqs: torch.Tensor, ints: torch.Tensor):
        super().__init__(freqs)
        self._ints = ints
        self._ints_unit = "a.u."

    @property
    def ints(self) -> torch.Tensor:
        return self._ints * self.converter_ints[self._ints_unit]

    @property
    def ints_unit(self) -> str:
        return self._ints_unit

    @ints_unit.setter
    def ints_unit(self, value: str) -> None:
        if value not in self.converter_ints:
            raise ValueError(f"Unsupported intensity unit: {value}")
        self._ints_unit = value

    def to_unit(self, value: str, unit: str) -> torch.Tensor:
        if value == "freqs":
            return self._convert(self._freqs, unit, self.converter_freqs)
        if value == "ints":
            return self._convert(self._ints, unit, self.converter_ints)
        raise ValueError(f"Unsupported value for conversion: {value}")

    def use_common_units(self) -> None:
        self.freqs_unit = "cm^-1"
        self.ints_unit = "km/mol"

    def __iter__(self):
        return iter((self.freqs, self.ints))


def is_linear(positions: torch.Tensor, tol: float = 1e-6) -> bool:
    """True for one or two atoms or when every atom lies on the line of the
    first two (all cross products below ``tol`` times the bond lengths)."""
    pos = positions.reshape(-1, 3)
    if pos.shape[0] <= 2:
        return True
    axis = pos[1] - pos[0]
    axis = axis / torch.linalg.norm(axis)
    rel = pos - pos[0]
    cross = torch.linalg.cross(rel, axis.expand_as(rel))
    scale = torch.linalg.norm(rel, dim=-1).max().clamp(min=1.0)
    return bool((torch.linalg.norm(cross, dim=-1) <= tol * scale).all())


def _rigid_modes(mass: torch.Tensor, positions: torch.Tensor, linear: bool) -> torch.Tensor:
    """Mass-weighted translations and rotations as rows (k, 3 nat)."""
    nat = mass.shape[0]
    msq = mass.sqrt()
    rows = []
    for x in range(3):
        t = torch.zeros(nat, 3, dtype=mass.dtype, device=mass.device)
        t[:, x] = msq
        rows.append(t.reshape(-1))
    com = (mass[:, None] * positions).sum(0) / mass.sum()
    rel = positions - com
    inertia = (mass * (rel * rel).sum(-1)).sum() * torch.eye(3, dtype=mass.dtype, device=mass.device)
    inertia = inertia - torch.einsum("a,ax,ay->xy", mass, rel, rel)
    _, axes = torch.linalg.eigh(inertia)
    axes = torch.flip(axes, [-1])  # last axis: smallest moment (the molecular axis if linear)
    ex, ey, ez = axes.T
    c = rel @ axes
    cx, cy, cz = c[:, 0:1], c[:, 1:2], c[:, 2:3]
    m = msq[:, None]
    rot = [m * (cy * ez - cz * ey), m * (cz * ex - cx * ez), m * (cx * ey - cy * ex)]
    if linear:
        rot = rot[:2]
    rows.extend(r.reshape(-1) for r in rot)
    return torch.stack(rows)


def vib_analysis(numbers, positions: torch.Tensor, hessian: torch.Tensor,
                 project_translational: bool = True, project_rotational: bool = True) -> VibResult:
    """
    Harmonic frequencies and normal modes of one molecule from its Hessian
    (nat, 3, nat, 3) in Eh/Bohr^2 (``vibration/analysis.py``, ``vib_analysis``).

    Translations (and rotations; two for a linear molecule) are projected out
    before the mass-weighted Hessian is diagonalised in the complementary
    space, so a non-linear molecule has 3 nat - 6 frequencies. Frequencies
    are sqrt(|lambda|) with the sign of lambda, in atomic units (Hartree);
    ``VibResult.use_common_units`` gives cm^-1. Modes are un-mass-weighted,
    shape (3 nat, nfreqs).
    """
    z = np.asarray(numbers.cpu() if torch.is_tensor(numbers) else numbers, dtype=np.int64).ravel()
    z = z[z > 0]
    nat = len(z)
    if hessian.shape == (nat * 3, nat * 3):
        raise ValueError(
            "The Hessian matrix must have shape (nat, 3, nat, 3); got "
            f"{tuple(hessian.shape)} for {nat} atoms."
        )
    if hessian.shape != (nat, 3, nat, 3):
        raise ValueError(f"Hessian of shape {tuple(hessian.shape)} for {nat} atoms")
    dt, dev = hessian.dtype, hessian.device
    pos = torch.as_tensor(positions, dtype=dt, device=dev).reshape(-1, 3)[:nat]
    mass = torch.as_tensor(atomic_mass(z), dtype=dt, device=dev)
    ism = mass.rsqrt().repeat_interleave(3)
    h = hessian.reshape(3 * nat, 3 * nat)
    h = ism[:, None] * h * ism[None, :]
    h = 0.5 * (h + h.T)
    rows = []
    if nat > 1 and (project_translational or project_rotational):
        rig = _rigid_modes(mass, pos, is_linear(pos))
        if project_translational:
            rows.append(rig[:3])
        if project_rotational:
            rows.append(rig[3:])
    if rows:
        q, _ = torch.linalg.qr(torch.cat(rows).T)
        proj = torch.eye(3 * nat, dtype=dt, device=dev) - q @ q.T
        w, v = torch.linalg.eigh(proj)
        bvec = v[:, w > LINDEP_THRESHOLD]
        if bvec.shape[-1] == 0:
            raise RuntimeError("The projection onto internal coordinates is empty.")
        fc, m = torch.linalg.eigh(bvec.T @ h @ bvec)
        mode = bvec @ m
    else:
        fc, mode = torch.linalg.eigh(h)
    freqs = torch.sqrt(fc.abs()) * torch.sign(fc)
    return VibResult(freqs, ism[:, None] * mode)


def ir_ints(dmu_dr: torch.Tensor, modes: torch.Tensor) -> torch.Tensor:
    """IR intensities (atomic units) from the nuclear dipole derivative
    (3, nat, 3) and the normal modes (3 nat, nfreqs) (``vibration/ir.py``)."""
    dq = dmu_dr.reshape(3, -1) @ modes
    return (dq * dq).sum(0)
