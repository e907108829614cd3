"""
Extract the dxtb test fixtures that pin the GFN-xTB path into ``golden.npz``.

Run once in a checkout that has the dxtb source tree (read-only)::

    python tests/golden/make_golden.py /path/to/dxtb

Everything written here is copied verbatim from the dxtb test suite (fixture
files and inline reference tensors, read as data); nothing is computed. The
file records, per entry, which dxtb file it came from.
"""

from __future__ import annotations

import ast
import json
import re
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).parent
MOLS = ["H2", "LiH", "H2O", "CH4", "SiH4", "LYS_xao"]
KEYS = {"H2": "h2", "LiH": "lih", "H2O": "h2o", "CH4": "ch4", "SiH4": "sih4", "LYS_xao": "lys_xao"}


def _coord(path: Path, symbols: list[str]):
    numbers, pos, active = [], [], False
    for line in path.read_text().splitlines():
        t = line.strip()
        if t.startswith("$"):
            active = t.startswith("$coord")
            continue
        if active and t:
            f = t.split()
            pos.append([float(v) for v in f[:3]])
            numbers.append(symbols.index(f[3].lower()) + 1)
    return np.array(numbers), np.array(pos)


def _tensor_literals(src: str, func: str) -> dict[str, np.ndarray]:
    """Literal ``torch.tensor([...])`` assignments inside one test function."""
    tree = ast.parse(src)
    out = {}
    for node in ast.walk(tree):
        if isinstance(node, ast.FunctionDef) and node.name == func:
            for stmt in ast.walk(node):
                if (
                    isinstance(stmt, ast.Assign)
                    and isinstance(stmt.targets[0], ast.Name)
                    and isinstance(stmt.value, ast.Call)
                    and getattr(stmt.value.func, "attr", "") == "tensor"
                ):
                    try:
                        out[stmt.targets[0].id] = np.array(
                            ast.literal_eval(stmt.value.args[0]), dtype=np.float64
                        )
                    except ValueError:
                        pass
    return out


def _ref_vector(src: str) -> np.ndarray:
    m = re.search(r"ref = torch.tensor\(\s*\[(.*?)\]", src, re.S)
    return np.array(
        [float(v) for v in re.findall(r"-?\d+\.\d+(?:[eE][-+]?\d+)?", m.group(1))]
    )


def _refs_dict(src: str, var: str = "refs") -> dict[str, dict[str, np.ndarray]]:
    """The literal ``{name: {key: torch.tensor([...]), ...}}`` dict ``var`` of a samples file."""
    tree = ast.parse(src)
    for node in ast.walk(tree):
        tgt = getattr(node, "target", None) or (getattr(node, "targets", [None]) or [None])[0]
        if isinstance(node, (ast.Assign, ast.AnnAssign)) and isinstance(tgt, ast.Name) and tgt.id == var:
            out = {}
            for kn, vn in zip(node.value.keys, node.value.values):
                rec = {}
                for kk, vv in zip(vn.keys, vn.values):
                    if isinstance(vv, ast.Call) and vv.args:
                        arr = np.array(ast.literal_eval(vv.args[0]), dtype=np.float64)
                        if arr.size:
                            rec[kk.value] = arr
                out[kn.value] = rec
            return out
    raise KeyError(var)


def _flat_literal(node) -> list[float]:
    """Numbers of a list literal whose items may be starred sub-lists."""
    out: list[float] = []
    for el in node.elts:
        if isinstance(el, ast.Starred):
            out.extend(_flat_literal(el.value))
        elif isinstance(el, (ast.List, ast.Tuple)):
            out.extend(_flat_literal(el))
        else:
            out.append(float(ast.literal_eval(el)))
    return out


def _reshaped_tensor_dict(src: str, var: str = "ref") -> dict[str, np.ndarray]:
    """The module-level ``{name: torch.tensor([...]).reshape(r, c)}`` dict ``var``."""
    tree = ast.parse(src)
    for node in tree.body:
        tgt = getattr(node, "target", None) or (getattr(node, "targets", [None]) or [None])[0]
        if isinstance(node, (ast.Assign, ast.AnnAssign)) and isinstance(tgt, ast.Name) and tgt.id == var:
            out = {}
            for kn, vn in zip(node.value.keys, node.value.values):
                shape = tuple(int(ast.literal_eval(a)) for a in vn.args)
                vals = _flat_literal(vn.func.value.args[0])
                out[kn.value] = np.array(vals, dtype=np.float64).reshape(shape)
            return out
    raise KeyError(var)


def main(ref_root: str) -> None:
    root = Path(ref_root)
    test = root / "test"
    symbols = [
        e["symbol"].lower()
        for _, e in sorted(
            json.load(open(HERE.parents[1] / "dxtb_gb300" / "data" / "gfn2.json"))[
                "element"
            ].items(),
            key=lambda kv: int(kv[0]),
        )
    ]
    g: dict[str, np.ndarray] = {}
    src: dict[str, str] = {}
    ov = np.load(test / "test_overlap" / "overlap.npz")
    h0 = np.load(test / "test_hamiltonian" / "h0.npz")
    gr = np.load(test / "test_scf" / "grad.npz")
    for m in MOLS:
        k = KEYS[m]
        num, pos = _coord(test / "test_singlepoint" / "mols" / m / "coord", symbols)
        g[f"{m}/numbers"] = num
        g[f"{m}/positions"] = pos
        g[f"{m}/overlap_gfn1"] = ov[k].astype(np.float64)
        g[f"{m}/h0_gfn1"] = h0[k].astype(np.float64)
        g[f"{m}/grad_elec_gfn1"] = gr[f"{k}_full"].astype(np.float64)
    src["*/numbers,positions"] = "test/test_singlepoint/mols/*/coord"
    src["*/overlap_gfn1"] = "test/test_overlap/overlap.npz (tblite 0.3.0)"
    src["*/h0_gfn1"] = "test/test_hamiltonian/h0.npz (tblite 0.3.0)"
    src["*/grad_elec_gfn1"] = (
        "test/test_scf/grad.npz '<name>_full' (GFN1, rep/disp/hal excluded)"
    )
    for meth in ("gfn1", "gfn2"):
        f = test / "test_scf" / f"test_elements_{meth}.py"
        g[f"atoms/{meth}"] = _ref_vector(f.read_text())
        src[f"atoms/{meth}"] = f"{f.relative_to(root)}: ref (tblite, E_scf - TS)"
    aes = (test / "test_coulomb" / "test_aes2.py").read_text()
    for func in ("test_energy", "test_potential"):
        for name, arr in _tensor_literals(aes, func).items():
            g[f"aes2_{func}/{name}"] = arr
    src["aes2_*"] = "test/test_coulomb/test_aes2.py (LiH, inline tensors)"
    # generalized Born / ALPB solvation (tblite reference values)
    solv = _refs_dict((test / "test_solvation" / "samples.py").read_text())
    for m in ("MB16_43_01", "SiH4"):
        for key, arr in solv[m].items():
            g[f"solv/{m}/{key}"] = arr
    num, pos = _coord(test / "test_singlepoint" / "mols" / "MB16_43_01" / "coord", symbols)
    g["MB16_43_01/numbers"] = num
    g["MB16_43_01/positions"] = pos
    src["solv/*"] = (
        "test/test_solvation/samples.py refs (tblite): psi, born, energies (ALPB p16, "
        "eps 78.9), energies_still (GB Still), charges, gsolv and gradient (GFN1 + ALPB)"
    )
    src["MB16_43_01/*"] = "test/test_singlepoint/mols/MB16_43_01/coord"
    # GFN2 H0 without the overlap factor (tblite 0.3.0), H2, LiH and SiH4
    h2 = _reshaped_tensor_dict((test / "test_hamiltonian" / "test_gfn2.py").read_text())
    for m in ("H2", "LiH", "SiH4"):
        g[f"{m}/h0scale_gfn2"] = h2[m]
    src["*/h0scale_gfn2"] = (
        "test/test_hamiltonian/test_gfn2.py ref (tblite 0.3.0): GFN2 H0 built with overlap=None"
    )
    # GFN1 properties: dipole moment without field (e a0), harmonic
    # frequencies (cm^-1) and IR intensities (km/mol)
    props = _refs_dict((test / "test_properties" / "samples.py").read_text())
    for m in ("H2", "LiH", "H2O", "CH4", "SiH4"):
        for key in ("dipole", "freqs", "ints"):
            g[f"props/{m}/{key}"] = props[m][key]
    src["props/*"] = (
        "test/test_properties/samples.py refs (GFN1): dipole (no field), freqs, ints; used by "
        "test_dipole.py (atol 1e-3) and test_vibration_ref.py (atol 10 cm^-1, rtol 1e-3)"
    )
    # SCF energies of multi-atom molecules (E_scf - TS): GFN1 from tblite
    # 0.2.1 with repulsion and dispersion disabled; GFN2 from tblite 0.4.0
    # ("electronic energy", which holds the self-consistent D4 part)
    scf = _refs_dict((test / "test_scf" / "samples.py").read_text())
    for m in ("H2", "LiH", "H2O", "CH4", "SiH4", "MB16_43_01", "LYS_xao"):
        for key in ("egfn1", "egfn2"):
            g[f"scf/{m}/{key}"] = scf[m][key]
    chg = _refs_dict((test / "test_scf" / "samples_charged.py").read_text())
    num, pos = _coord(test / "test_singlepoint" / "mols" / "AD7en+" / "coord", symbols)
    g["AD7en+/numbers"] = num
    g["AD7en+/positions"] = pos
    for key in ("charge", "egfn1", "egfn2"):
        g[f"scf/AD7en+/{key}"] = chg["AD7en+"][key]
    src["scf/*"] = (
        "test/test_scf/samples.py and samples_charged.py (AD7en+, charge +1): egfn1 (tblite "
        "0.2.1, repulsion and dispersion disabled), egfn2 (tblite 0.4.0 electronic energy, with "
        "the self-consistent D4 part); used by test_scf.py / test_charged.py with "
        "tol sqrt(eps) * 10"
    )
    src["AD7en+/*"] = "test/test_singlepoint/mols/AD7en+/coord"
    np.savez_compressed(HERE / "golden.npz", **g)
    (HERE / "golden_sources.json").write_text(json.dumps(src, indent=1))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path to the dxtb source tree>")
    main(sys.argv[1])
