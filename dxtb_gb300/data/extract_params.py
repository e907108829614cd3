"""
Regenerate the packaged parameter files from a dxtb source tree.

The GFN1-xTB and GFN2-xTB parameters are published data (Grimme, Bannwarth,
Shushkov, JCTC 13, 1989 (2017); Bannwarth, Ehlert, Grimme, JCTC 15, 1652
(2019)). dxtb ships them as TOML (``src/dxtb/_src/param/gfn{1,2}/*.toml``)
and the STO-nG expansion tables of Stewart (JCP 52, 431 (1970)) as ``.npy``
(``src/dxtb/_src/basis/sto-ng/sto-{1..6}g.npy``). This script reads those
files once and writes the compact, dense per-element layout that the GPU
path consumes (``gfn1.json``, ``gfn2.json``, ``stong.npz`` next to this
file), so the package does not need the dxtb tree at run time.

Usage::

    python -m dxtb_gb300.data.extract_params /path/to/dxtb
"""

from __future__ import annotations

import json
import sys
import tomllib
from pathlib import Path

import numpy as np

HERE = Path(__file__).parent
LABEL2L = {"s": 0, "p": 1, "d": 2, "f": 3, "g": 4}
ELEM_KEYS_SHELL = ("levels", "slater", "ngauss", "refocc", "shpoly", "kcn", "lgam")
ELEM_KEYS_ATOM = (
    "gam", "gam3", "zeff", "arep", "xbond", "en", "dkernel", "qkernel",
    "mprad", "mpvcn",
)


def _valence(angular: list[int]) -> list[bool]:
    """First shell of every angular momentum is valence, repeats are not
    (dxtb ``param/module/utils.py:480-530``)."""
    seen: set[int] = set()
    out = []
    for l in angular:
        out.append(l not in seen)
        seen.add(l)
    return out


def convert(toml_path: Path) -> dict:
    with open(toml_path, "rb") as fh:
        raw = tomllib.load(fh)
    symbols = list(raw["element"].keys())
    elements = {}
    for z, sym in enumerate(symbols, start=1):
        e = raw["element"][sym]
        ang = [LABEL2L[s[-1]] for s in e["shells"]]
        rec = {
            "symbol": sym,
            "shells": e["shells"],
            "angular": ang,
            "pqn": [int(s[0]) for s in e["shells"]],
            "valence": _valence(ang),
        }
        for k in ELEM_KEYS_SHELL:
            rec[k] = list(e.get(k, [0.0] * len(ang)))
        for k in ELEM_KEYS_ATOM:
            rec[k] = float(e.get(k, 0.0))
        elements[z] = rec

    out = {k: v for k, v in raw.items() if k != "element"}
    # pair scaling of the Hamiltonian: symbol pairs to atomic-number pairs
    kpair = raw["hamiltonian"]["xtb"].get("kpair", {})
    sym2z = {s: i + 1 for i, s in enumerate(symbols)}
    out["hamiltonian"]["xtb"]["kpair"] = [
        [sym2z[a], sym2z[b], float(v)]
        for a, b, v in ((*key.split("-"), val) for key, val in kpair.items())
    ]
    out["element"] = elements
    return out


def main(ref_root: str) -> None:
    root = Path(ref_root) / "src" / "dxtb" / "_src"
    for name in ("gfn1", "gfn2"):
        data = convert(root / "param" / name / f"{name}-xtb.toml")
        with open(HERE / f"{name}.json", "w") as fh:
            json.dump(data, fh, indent=0, sort_keys=True)
    tabs = {
        f"sto{ng}g": np.load(root / "basis" / "sto-ng" / f"sto-{ng}g.npy")
        for ng in range(1, 7)
    }
    np.savez(HERE / "stong.npz", **tabs)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python -m dxtb_gb300.data.extract_params <path to the dxtb source tree>")
    main(sys.argv[1])
