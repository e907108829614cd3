"""Host-side checks that need no GPU: the C-ABI library builds, loads and
exports every entry point the header declares; parameter layout; workloads."""

import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


def _declared() -> list[str]:
    src = (ROOT / "include" / "dxtb_gb300.h").read_text()
    return sorted(set(re.findall(r"^(?:int32_t|int64_t)\s+(dxtb_\w+)\(", src, re.M)))


def test_library_exports_header_symbols():
    from dxtb_gb300 import build

    lib = build.build()
    handle = ctypes.CDLL(str(lib))
    missing = [s for s in _declared() if not hasattr(handle, s)]
    assert not missing, missing


def test_bindings_cover_header_symbols():
    """Every declared entry point has ctypes argtypes (doubles and int64
    arguments would otherwise be passed as C ints)."""
    from dxtb_gb300 import _lib

    missing = [s for s in _declared() if s not in _lib._SIGS]
    assert not missing, missing


def test_layout_parsed_from_header():
    from dxtb_gb300.params import layout

    L = layout()
    assert L["DXTB_P_SIZE"] > L["DXTB_P_KPAIR"] > L["DXTB_P_ALPHA"]
    assert L["DXTB_I_SIZE"] == L["DXTB_I_SCAL"] + L["DXTB_NISCAL"]


@pytest.mark.parametrize("method", ["gfn1", "gfn2"])
def test_tables(method):
    from dxtb_gb300.params import Tables, layout

    t = Tables(method)
    L = layout()
    # every contracted shell is normalised: recompute the self-overlap
    import math

    for z, types in t.el_shells.items():
        for ty in types:
            n = t.i32[L["DXTB_I_NPRIM"] + ty]
            l = t.i32[L["DXTB_I_L"] + ty]
            a = t.f64[L["DXTB_P_ALPHA"] + 8 * ty : L["DXTB_P_ALPHA"] + 8 * ty + n]
            c = t.f64[L["DXTB_P_COEFF"] + 8 * ty : L["DXTB_P_COEFF"] + 8 * ty + n]
            p = a[:, None] + a[None, :]
            df = [1.0, 1.0, 3.0][l]
            s = (c[:, None] * c[None, :] * (math.pi / p) ** 1.5 * df / (2 * p) ** l).sum()
            assert abs(s - 1.0) < 1e-13


def test_cgto_matches_oracle():
    """The package's host-side STO-nG contraction equals the oracle's."""
    from dxtb_gb300.params import Tables, layout
    from oracle import xtb_oracle as X

    t = Tables("gfn1")
    L = layout()
    sysm = X.make_system("gfn1", np.array([1, 6, 16]))
    for u, (z, k) in enumerate(zip(sysm.ush_z, sysm.ush_idx_in_elem)):
        ty = t.el_shells[z][k]
        n = t.i32[L["DXTB_I_NPRIM"] + ty]
        a = t.f64[L["DXTB_P_ALPHA"] + 8 * ty : L["DXTB_P_ALPHA"] + 8 * ty + n]
        c = t.f64[L["DXTB_P_COEFF"] + 8 * ty : L["DXTB_P_COEFF"] + 8 * ty + n]
        assert np.allclose(a, sysm.alphas[u].numpy(), rtol=1e-14)
        assert np.allclose(c, sysm.coeffs[u].numpy(), rtol=1e-12)


def test_workloads_deterministic_and_valid():
    from dxtb_gb300.workloads import VALENCE, config_molecules, random_molecule

    a = random_molecule(2001, 40)
    b = random_molecule(2001, 40)
    assert np.array_equal(a[0], b[0]) and np.allclose(a[1], b[1])
    for num, pos in config_molecules(2, count=16):
        assert sum(VALENCE[int(z)] for z in num) % 2 == 0
        d = np.linalg.norm(pos[:, None] - pos[None], axis=-1) + 10 * np.eye(len(num))
        assert d.min() >= 2.0 - 1e-12
    (num, pos), = config_molecules(1)
    assert sorted(num.tolist()).count(1) == 12 and len(num) == 24


def test_size_class_policy_host_calls():
    """The size-class thresholds are host state: defaults, validation and
    restore work without a GPU (no CUDA call is made)."""
    import ctypes as C

    from dxtb_gb300 import build

    L = C.CDLL(str(build.build()))
    L.dxtb_scf_get_size_classes.restype = C.c_int32
    L.dxtb_scf_set_size_classes.restype = C.c_int32
    cur = (C.c_int32 * 5)()
    assert L.dxtb_scf_get_size_classes(cur) == 0
    saved = list(cur)
    assert saved == sorted(saved) and saved[0] >= 1
    try:
        assert L.dxtb_scf_set_size_classes((C.c_int32 * 5)(100, 90, 200, 300, 400)) == 1  # decreasing
        assert L.dxtb_scf_set_size_classes((C.c_int32 * 5)(0, 90, 200, 300, 400)) == 1  # below 1
        assert L.dxtb_scf_set_size_classes((C.c_int32 * 5)(64, 96, 128, 256, 512)) == 0
        got = (C.c_int32 * 5)()
        assert L.dxtb_scf_get_size_classes(got) == 0
        assert list(got) == [64, 96, 128, 256, 512]
    finally:
        assert L.dxtb_scf_set_size_classes((C.c_int32 * 5)(*saved)) == 0


def test_scf_workspace_grows_with_size():
    import ctypes as C

    from dxtb_gb300 import build

    L = C.CDLL(str(build.build()))
    L.dxtb_scf_workspace_mol.restype = C.c_int64
    L.dxtb_scf_workspace_mol.argtypes = [C.c_int64, C.c_int64]
    a, b = L.dxtb_scf_workspace_mol(90, 30), L.dxtb_scf_workspace_mol(172, 60)
    assert 0 < a < b
    # at least the three n x n matrices of the molecule
    assert a >= 3 * 90 * 90 and b >= 3 * 172 * 172


def test_alpha_beta_split_and_errors():
    """Alpha/beta electrons as in wavefunction/filling.py:180-259, with its
    ValueErrors for too many unpaired electrons and a wrong parity."""
    from dxtb_gb300.engine import alpha_beta

    assert alpha_beta(10.0) == (5.0, 5.0)
    assert alpha_beta(9.0) == (5.0, 4.0)
    assert alpha_beta(10.0, 2) == (6.0, 4.0)
    assert alpha_beta(9.0, 3) == (6.0, 3.0)
    for nel, spin in [(10.0, 1), (9.0, 2), (2.0, 4)]:
        with pytest.raises(ValueError):
            alpha_beta(nel, spin)
