"""
ctypes binding of ``libdxtb_gb300.so`` (C ABI in ``include/dxtb_gb300.h``).

The library is the only compute path: if it is missing, or no CUDA device is
visible, every entry raises instead of falling back to anything else.
"""

from __future__ import annotations

import ctypes as C
import threading

import torch

from . import build as _build

_lock = threading.Lock()
_lib = None

i32, i64, f64, vp = C.c_int32, C.c_int64, C.c_double, C.c_void_p

STATUS = {
    0: "ok",
    1: "invalid arguments",
    2: "CUDA launch error",
    3: "overlap matrix not positive definite",
    4: "SCF not converged (maxiter)",
    5: "Fermi level search failed",
    6: "NaN/Inf in result",
    7: "size beyond compiled-in maximum",
}


class Batch(C.Structure):
    """Mirror of ``dxtb_batch``."""

    _fields_ = [
        ("nmol", i32), ("max_nao", i32), ("max_nat", i32), ("max_nsh", i32),
        ("atom_off", vp), ("shell_off", vp), ("ao_off", vp), ("mat_off", vp),
        ("nat2_off", vp), ("nsh2_off", vp), ("pair_off", vp),
        ("numbers", vp), ("positions", vp), ("shell_atom", vp), ("shell_type", vp),
        ("shell_ao", vp), ("ao_shell", vp),
    ]


class ScfConfig(C.Structure):
    """Mirror of ``dxtb_scf_config``."""

    _fields_ = [
        ("maxiter", i32), ("mixer", i32), ("x_atol", f64), ("f_atol", f64), ("x_atol_max", f64),
        ("damp", f64), ("damp_init", f64), ("generations", i32), ("soft_start", i32),
        ("diagonal_offset", f64),
    ]


MIXERS = {"broyden1": 0, "anderson": 1}


_SIGS = {
    "dxtb_coordination_number": (i32, [vp, vp, vp, i32, vp, vp]),
    "dxtb_interaction_cache": (i32, [vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp]),
    "dxtb_multipole_h0": (i32, [vp, vp, vp, vp, vp, vp, vp, vp, vp]),
    "dxtb_multipole_raw": (i32, [vp, vp, vp, vp, vp, vp, vp]),
    "dxtb_multipole_raw_vjp": (i32, [vp] * 8),
    "dxtb_dipole_moment": (i32, [vp] * 6),
    "dxtb_graph_begin": (i32, [vp]),
    "dxtb_graph_end": (i32, [vp, vp]),
    "dxtb_graph_launch": (i32, [vp, vp]),
    "dxtb_graph_destroy": (i32, [vp]),
    "dxtb_scf_workspace_mol": (i64, [i64, i64]),
    "dxtb_scf": (i32, [vp] * 15 + [f64, vp] + [vp] * 17),
    "dxtb_gradient": (i32, [vp] * 22),
    "dxtb_scf_gradient": (i32, [vp] * 15 + [f64, vp] + [vp] * 21),
    "dxtb_index_sizes": (i32, [vp, i32, i32, i32, vp, vp, vp]),
    "dxtb_index_maps": (i32, [vp, i32, i32, i32, vp, vp, i64, i64] + [vp] * 14 + [vp]),
    "dxtb_scf_set_size_classes": (i32, [vp]),
    "dxtb_scf_get_size_classes": (i32, [vp]),
    "dxtb_born_matrix": (i32, [vp, vp, vp, f64, i32, i32, f64, f64, vp, vp, vp, vp]),
    "dxtb_born_gradient": (i32, [vp, vp, vp, f64, i32, i32, f64, f64, vp, vp, vp, vp, vp]),
    "dxtb_fp64_fma_probe": (i32, [i64, i32, i32, vp, vp]),
    "dxtb_fp64_mma_probe": (i32, [i32, i64, i32, i32, vp, vp]),
    "dxtb_scf_noalloc": (i32, [vp] * 15 + [f64, i32, f64] + [vp] * 15),
}


def lib():
    """Load (building first if needed) the CUDA library."""
    global _lib
    with _lock:
        if _lib is None:
            if not torch.cuda.is_available():
                raise RuntimeError(
                    "dxtb_gb300 needs a CUDA device (GB300, sm_103a); none is visible"
                )
            path = _build.LIB
            if not path.exists():
                _build.build()
            handle = C.CDLL(str(path))
            for name, sig in _SIGS.items():
                if sig is None or not hasattr(handle, name):
                    continue
                fn = getattr(handle, name)
                fn.restype, fn.argtypes = sig[0], sig[1]
            _lib = handle
    return _lib


def check(code: int, what: str) -> None:
    if code != 0:
        raise RuntimeError(f"{what}: {STATUS.get(code, code)}")


def ptr(t: torch.Tensor | None) -> int | None:
    return None if t is None else t.data_ptr()


def stream_ptr() -> int:
    return torch.cuda.current_stream().cuda_stream
