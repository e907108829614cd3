"""
IndexHelper with the interface of dxtb's (basis/indexhelper.py:123-969).

The twelve maps are built on the GPU by ``dxtb_index_maps`` (bit-exact with
``IndexHelper.from_numbers_angular``, batch modes 0 and 1); spread and reduce
follow ``utils/scattergather.py:262-419`` (gathers and scatter-sums in which
negative padding indices read zero and are dropped).
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib

__all__ = ["IndexHelper"]

PAD = -999
MAXZ = 87


def _angular_tables(angular: dict[int, list[int]]):
    nsh = np.zeros(MAXZ, dtype=np.int32)
    ang = np.zeros((MAXZ, 8), dtype=np.int32)
    for z, ls in angular.items():
        if 0 < z < MAXZ:
            nsh[z] = len(ls)
            ang[z, : len(ls)] = ls
    return nsh, ang


def _gather(src: torch.Tensor, idx: torch.Tensor, dim: int) -> torch.Tensor:
    """Gather along ``dim``; negative (padding) indices give zero."""
    mask = idx >= 0
    safe = torch.where(mask, idx, torch.zeros_like(idx))
    out = torch.index_select(src, dim, safe.reshape(-1)).reshape(
        *src.shape[:dim], *idx.shape, *src.shape[dim + 1 :]
    ) if idx.ndim == 1 else None
    if out is None:
        raise ValueError("batched gathers go through the per-row helpers")
    shape = [1] * out.ndim
    shape[dim] = idx.shape[0]
    return torch.where(mask.reshape(shape), out, torch.zeros((), dtype=out.dtype, device=out.device))


def _scatter_sum(src: torch.Tensor, idx: torch.Tensor, size: int, dim: int) -> torch.Tensor:
    """Scatter-add along ``dim``; entries with negative indices are dropped."""
    mask = idx >= 0
    shape = list(src.shape)
    shape[dim] = size
    out = torch.zeros(shape, dtype=src.dtype, device=src.device)
    keep = torch.nonzero(mask).reshape(-1)
    return out.index_add(dim, idx[keep], torch.index_select(src, dim, keep))


class IndexHelper:
    """Index maps between atoms, shells and orbitals."""

    PAD = PAD

    def __init__(self, maps: dict[str, torch.Tensor], batch_mode: int, unique: torch.Tensor):
        for k, v in maps.items():
            setattr(self, k, v)
        self.batch_mode = batch_mode
        self.unique = unique

    # ---- construction ---------------------------------------------------
    @classmethod
    def from_numbers(cls, numbers: torch.Tensor, par="gfn2", batch_mode: int | None = None):
        """Maps for the shells of the GFN parametrisation ``par``."""
        from .params import load_par

        if isinstance(par, str):
            p = load_par(par.lower().replace("-xtb", "").replace("_xtb", ""))
            angular = {z: e["angular"] for z, e in p["element"].items()}
        else:
            angular = par
        return cls.from_numbers_angular(numbers, angular, batch_mode)

    @classmethod
    def from_numbers_angular(cls, numbers: torch.Tensor, angular: dict[int, list[int]],
                             batch_mode: int | None = None):
        if not torch.is_tensor(numbers):
            numbers = torch.as_tensor(numbers)
        if batch_mode is None:
            batch_mode = int(numbers.ndim > 1)
        device = numbers.device if numbers.device.type == "cuda" else torch.device("cuda")
        rows = numbers.reshape(-1, numbers.shape[-1]).to(torch.int64)
        nbatch, nat_max = rows.shape
        nsh_el, ang_el = _angular_tables(angular)
        host = np.ascontiguousarray(rows.cpu().numpy())
        sizes = np.zeros(4, dtype=np.int64)
        L = _lib.lib()
        _lib.check(
            L.dxtb_index_sizes(host.ctypes.data, nbatch, nat_max, batch_mode,
                               nsh_el.ctypes.data, ang_el.ctypes.data, sizes.ctypes.data),
            "index sizes",
        )
        nunique, nushell, nsh_max, nao_max = (int(v) for v in sizes)
        dev = rows.to(device).contiguous()
        i64 = dict(dtype=torch.int64, device=device)
        t_nsh = torch.as_tensor(nsh_el, device=device)
        t_ang = torch.as_tensor(ang_el, device=device)
        m = {
            "unique_angular": torch.empty(nushell, **i64),
            "angular": torch.empty(nbatch, nsh_max, **i64),
            "atom_to_unique": torch.empty(nbatch, nat_max, **i64),
            "ushells_to_unique": torch.empty(nushell, **i64),
            "ushells_per_unique": torch.empty(nunique, **i64),
            "shells_to_ushell": torch.empty(nbatch, nsh_max, **i64),
            "shells_per_atom": torch.empty(nbatch, nat_max, **i64),
            "shell_index": torch.empty(nbatch, nat_max, **i64),
            "shells_to_atom": torch.empty(nbatch, nsh_max, **i64),
            "orbitals_per_shell": torch.empty(nbatch, nsh_max, **i64),
            "orbital_index": torch.empty(nbatch, nsh_max, **i64),
            "orbitals_to_shell": torch.empty(nbatch, nao_max, **i64),
        }
        unique = torch.empty(nunique, **i64)
        zmap = torch.empty(3 * MAXZ, **i64)
        order = ["unique_angular", "angular", "atom_to_unique", "ushells_to_unique",
                 "ushells_per_unique", "shells_to_ushell", "shells_per_atom", "shell_index",
                 "shells_to_atom", "orbitals_per_shell", "orbital_index", "orbitals_to_shell"]
        _lib.check(
            L.dxtb_index_maps(dev.data_ptr(), nbatch, nat_max, batch_mode, t_nsh.data_ptr(),
                              t_ang.data_ptr(), nsh_max, nao_max,
                              *[m[k].data_ptr() for k in order], unique.data_ptr(),
                              zmap.data_ptr(), _lib.stream_ptr()),
            "index maps",
        )
        if numbers.ndim == 1:
            for k in ("angular", "atom_to_unique", "shells_to_ushell", "shells_per_atom",
                      "shell_index", "shells_to_atom", "orbitals_per_shell", "orbital_index",
                      "orbitals_to_shell"):
                m[k] = m[k][0]
        return cls(m, batch_mode, unique)

    # ---- sizes ----------------------------------------------------------
    @property
    def nao(self) -> int:
        return int(self.orbitals_per_shell.sum(-1).max())

    @property
    def nsh(self) -> int:
        return int(self.shells_per_atom.sum(-1).max())

    @property
    def nat(self) -> int:
        return int(self.atom_to_unique.shape[-1])

    @property
    def orbitals_per_atom(self) -> torch.Tensor:
        return self.reduce_shell_to_atom(self.orbitals_per_shell)

    # ---- spread (gather) --------------------------------------------------
    def _spread(self, x: torch.Tensor, idx: torch.Tensor, dim: int) -> torch.Tensor:
        if idx.ndim == 1:
            return _gather(x, idx, dim % x.ndim)
        return torch.stack([_gather(x[b], idx[b], (dim % x.ndim) - 1) for b in range(idx.shape[0])])

    def _spread_2d(self, x, idx, dims):
        out = x
        for d in dims:
            out = self._spread(out, idx, d)
        return out

    def spread_atom_to_shell(self, x, dim=-1, extra=False):
        if isinstance(dim, tuple):
            return self._spread_2d(x, self.shells_to_atom, dim)
        return self._spread(x, self.shells_to_atom, dim if not extra else dim)

    def spread_shell_to_orbital(self, x, dim=-1, extra=False):
        if isinstance(dim, tuple):
            return self._spread_2d(x, self.orbitals_to_shell, dim)
        return self._spread(x, self.orbitals_to_shell, dim)

    def spread_atom_to_orbital(self, x, dim=-1, extra=False):
        if isinstance(dim, tuple):
            return self.spread_shell_to_orbital(self.spread_atom_to_shell(x, dim), dim)
        return self.spread_shell_to_orbital(self.spread_atom_to_shell(x, dim), dim)

    def spread_uspecies_to_atom(self, x, dim=-1):
        return self._spread(x, self.atom_to_unique, dim)

    def spread_uspecies_to_shell(self, x, dim=-1):
        return self.spread_atom_to_shell(self.spread_uspecies_to_atom(x, dim), dim)

    def spread_uspecies_to_orbital(self, x, dim=-1):
        return self.spread_atom_to_orbital(self.spread_uspecies_to_atom(x, dim), dim)

    def spread_ushell_to_shell(self, x, dim=-1):
        if isinstance(dim, tuple):
            return self._spread_2d(x, self.shells_to_ushell, dim)
        return self._spread(x, self.shells_to_ushell, dim)

    def spread_ushell_to_orbital(self, x, dim=-1):
        return self.spread_shell_to_orbital(self.spread_ushell_to_shell(x, dim), dim)

    # ---- reduce (scatter-sum) --------------------------------------------
    def _reduce(self, x, idx, size, dim):
        if idx.ndim == 1:
            return _scatter_sum(x, idx, size, dim % x.ndim)
        return torch.stack(
            [_scatter_sum(x[b], idx[b], size, (dim % x.ndim) - 1) for b in range(idx.shape[0])]
        )

    def reduce_orbital_to_shell(self, x, dim=-1, extra=False):
        size = self.orbitals_per_shell.shape[-1]
        if isinstance(dim, tuple):
            for d in dim:
                x = self._reduce(x, self.orbitals_to_shell, size, d)
            return x
        return self._reduce(x, self.orbitals_to_shell, size, dim)

    def reduce_shell_to_atom(self, x, dim=-1, extra=False):
        size = self.shells_per_atom.shape[-1]
        if isinstance(dim, tuple):
            for d in dim:
                x = self._reduce(x, self.shells_to_atom, size, d)
            return x
        return self._reduce(x, self.shells_to_atom, size, dim)

    def reduce_orbital_to_atom(self, x, dim=-1, extra=False):
        return self.reduce_shell_to_atom(self.reduce_orbital_to_shell(x, dim), dim)
