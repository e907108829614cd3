"""
Overlap, dipole and quadrupole integrals with the interface of dxtb's
integral wrappers and PyTorch driver classes.

- ``overlap(numbers, positions, par)``, ``dipint``, ``quadint``:
  ``integral/wrappers.py:149-315``.
- ``IntDriver`` (alias ``IntDriverPytorch``), with ``Overlap``,
  ``Dipole`` and ``Quadrupole`` (aliases ``OverlapPytorch`` etc.) and
  their ``build(driver)``: ``integral/driver/pytorch/{driver,overlap,
  dipole,quadrupole}.py``.

All three come from one launch of the McMurchie-Davidson kernel
(``dxtb_multipole_raw``, one warp per shell pair). With
``positions.requires_grad`` the wrappers return tensors whose backward is
the integral VJP kernel (``dxtb_multipole_raw_vjp``), as the reference's
wrappers carry autograd. The dipole is (3, nao,
nao) and the quadrupole (9, nao, nao) in the order xx xy xz yx yy yz zx zy
zz. The moment operators are taken about the origin, as the reference
wrappers return them. A batch (2D zero-padded ``numbers``) gives
zero-padded (B, ..., nao_max, nao_max) tensors. The contracted Gaussians
are normalised to unit self-overlap when the parameter tables are built.
The reference's ``normalize`` step (division by sqrt(S_ii S_jj)) is
therefore the identity to rounding, and ``normalize=False`` returns the
same matrices.
"""

from __future__ import annotations

import ctypes as C

import torch

from . import _lib
from .params import Tables

__all__ = ["overlap", "dipint", "quadint", "IntDriver", "IntDriverPytorch", "Overlap", "Dipole",
           "Quadrupole", "OverlapPytorch", "DipolePytorch", "QuadrupolePytorch"]


def _method(par) -> str:
    if isinstance(par, Tables):
        return par.method
    name = par if isinstance(par, str) else str(getattr(getattr(par, "meta", None), "name", par))
    name = name.lower().replace("-", "").replace("_", "")
    for m in ("gfn1", "gfn2"):
        if m in name:
            return m
    raise ValueError(f"cannot tell the GFN method of {par!r}")


class IntDriver:
    """Integral driver: packs the molecules once, ``setup(positions)`` per geometry."""

    def __init__(self, numbers, par, ihelp=None, *, device=None, dtype=None, **_):
        from .calculators import tables

        if dtype is not None and dtype != torch.float64:
            raise TypeError("the GB300 integrals are float64")
        self.tables = par if isinstance(par, Tables) else tables(_method(par))
        self.numbers = numbers if torch.is_tensor(numbers) else torch.as_tensor(numbers)
        self.batched = self.numbers.ndim > 1
        nums = self.numbers.reshape(-1, self.numbers.shape[-1]).cpu().numpy()
        self._mols = [n[n > 0] for n in nums]
        self.device = torch.device(device) if device is not None else torch.device("cuda")
        self.ihelp = ihelp
        self._pb = None
        self._out = None

    def setup(self, positions: torch.Tensor, **_) -> None:
        from .engine import PackedBatch

        pos = positions.detach().reshape(-1, positions.shape[-2], 3)
        plist = [pos[i, : len(m)] for i, m in enumerate(self._mols)]
        if self._pb is None:
            self._pb = PackedBatch(self.tables, self._mols, plist, self.device)
        else:
            self._pb.set_positions(plist)
        self._out = None

    def _compute(self) -> dict:
        """S, D (3) and Q (9) for every molecule, one kernel launch."""
        if self._pb is None:
            raise RuntimeError("call setup(positions) first")
        if self._out is None:
            pb = self._pb
            L = _lib.lib()
            nm = pb.total["mat"]
            S = torch.empty(max(nm, 1), dtype=torch.float64, device=self.device)
            D = torch.empty(3 * max(nm, 1), dtype=torch.float64, device=self.device)
            Q = torch.empty(9 * max(nm, 1), dtype=torch.float64, device=self.device)
            _lib.check(L.dxtb_multipole_raw(C.byref(pb.struct), pb.t["par_f"].data_ptr(),
                                            pb.t["par_i"].data_ptr(), S.data_ptr(), D.data_ptr(),
                                            Q.data_ptr(), _lib.stream_ptr()), "multipole integrals")
            self._out = {"S": S, "D": D, "Q": Q, "mtot": nm}
        return self._out

    def matrices(self, kind: str) -> torch.Tensor:
        out = self._compute()
        pb = self._pb
        ncomp = {"S": 1, "D": 3, "Q": 9}[kind]
        flat = out[kind][: ncomp * out["mtot"]].view(ncomp, out["mtot"])
        blocks = []
        for i in range(pb.nmol):
            n = int(pb.nao[i])
            m0 = int(pb.mat_off[i])
            blocks.append(flat[:, m0 : m0 + n * n].view(ncomp, n, n))
        if not self.batched:
            b = blocks[0]
            return b[0] if ncomp == 1 else b
        nmax = int(pb.nao.max())
        res = torch.zeros(pb.nmol, ncomp, nmax, nmax, dtype=torch.float64, device=self.device)
        for i, b in enumerate(blocks):
            n = b.shape[-1]
            res[i, :, :n, :n] = b
        return res[:, 0] if ncomp == 1 else res


class _Integral:
    kind = "S"

    def __init__(self, *_, **__):
        self.matrix: torch.Tensor | None = None

    def build(self, driver: IntDriver) -> torch.Tensor:
        self.matrix = driver.matrices(self.kind)
        return self.matrix

    @property
    def norm(self) -> torch.Tensor | None:
        """1/sqrt(S_ii): ones, the basis is normalised when the tables are built."""
        if self.matrix is None:
            return None
        return torch.ones(self.matrix.shape[-1], dtype=self.matrix.dtype, device=self.matrix.device)

    def normalize(self, norm=None) -> None:
        """Identity (see the module docstring)."""


class Overlap(_Integral):
    kind = "S"


class Dipole(_Integral):
    kind = "D"


class Quadrupole(_Integral):
    kind = "Q"


IntDriverPytorch = IntDriver
OverlapPytorch, DipolePytorch, QuadrupolePytorch = Overlap, Dipole, Quadrupole


class _RawIntegral(torch.autograd.Function):
    """Integral matrices with the VJP kernel as backward."""

    @staticmethod
    def forward(ctx, positions, drv, kind):
        drv.setup(positions.detach())
        ctx.drv, ctx.kind, ctx.shape = drv, kind, positions.shape
        return drv.matrices(kind).clone()

    @staticmethod
    def backward(ctx, gout):
        drv, kind = ctx.drv, ctx.kind
        pb = drv._pb
        ncomp = {"S": 1, "D": 3, "Q": 9}[kind]
        mtot = pb.total["mat"]
        flat = torch.zeros(ncomp, max(mtot, 1), dtype=torch.float64, device=drv.device)
        g = gout.reshape(pb.nmol if drv.batched else 1, ncomp, gout.shape[-2], gout.shape[-1]) \
            if ncomp > 1 else gout.reshape(-1, 1, gout.shape[-2], gout.shape[-1])
        for i in range(pb.nmol):
            n, m0 = int(pb.nao[i]), int(pb.mat_off[i])
            flat[:, m0 : m0 + n * n] = g[i, :, :n, :n].reshape(ncomp, n * n)
        grad = torch.zeros(pb.total["atoms"], 3, dtype=torch.float64, device=drv.device)
        ptrs = {"S": None, "D": None, "Q": None}
        ptrs[kind] = flat.data_ptr()
        L = _lib.lib()
        _lib.check(L.dxtb_multipole_raw_vjp(C.byref(pb.struct), pb.t["par_f"].data_ptr(),
                                            pb.t["par_i"].data_ptr(), ptrs["S"], ptrs["D"], ptrs["Q"],
                                            grad.data_ptr(), _lib.stream_ptr()), "integral VJP")
        out = torch.zeros(ctx.shape, dtype=torch.float64, device=drv.device).reshape(-1, ctx.shape[-2], 3)
        for i in range(pb.nmol):
            a0, a1 = int(pb.atom_off[i]), int(pb.atom_off[i + 1])
            out[i, : a1 - a0] = grad[a0:a1]
        return out.reshape(ctx.shape), None, None


def _integral(kind: str, numbers, positions, par, **kwargs) -> torch.Tensor:
    kwargs.pop("normalize", None)
    kwargs.pop("driver", None)
    drv = IntDriver(numbers, par, device=positions.device if positions.is_cuda else None)
    if positions.requires_grad:
        return _RawIntegral.apply(positions, drv, kind)
    drv.setup(positions)
    return drv.matrices(kind)


def overlap(numbers, positions, par, **kwargs) -> torch.Tensor:
    """Overlap (nao, nao), or (B, nao, nao) for a batch (wrappers.py:149-168)."""
    return _integral("S", numbers, positions, par, **kwargs)


def dipint(numbers, positions, par, **kwargs) -> torch.Tensor:
    """Dipole integrals about the origin, (3, nao, nao) (wrappers.py:171-190)."""
    return _integral("D", numbers, positions, par, **kwargs)


def quadint(numbers, positions, par, **kwargs) -> torch.Tensor:
    """Quadrupole integrals about the origin, (9, nao, nao) (wrappers.py:193-212)."""
    return _integral("Q", numbers, positions, par, **kwargs)
