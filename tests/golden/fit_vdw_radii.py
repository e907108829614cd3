"""
Least-squares fit of the D3 van-der-Waals radii to the tblite descreening
integrals psi of dxtb's solvation fixtures (``golden.npz`` entries
``solv/MB16_43_01/psi`` and ``solv/SiH4/psi``), using the oracle's
restatement of ``compute_psi``. Prints the fitted radii in Angstrom and
the relative residual; the table in ``dxtb_gb300/data/radii.py`` holds the
values rounded to the 5 digits of the published table.

    python tests/golden/fit_vdw_radii.py
"""

from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import torch
from scipy.optimize import least_squares

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from dxtb_gb300.data import radii  # noqa: E402
from oracle import solvation_oracle as S  # noqa: E402

G = np.load(Path(__file__).parent / "golden.npz")


def fit(name: str, known: dict[int, float]) -> dict[int, float]:
    z = G[f"{name}/numbers"]
    x = torch.tensor(G[f"{name}/positions"])
    psi = G[f"solv/{name}/psi"]
    unknown = [e for e in sorted(set(z.tolist())) if e not in known]

    def rvdw(p):
        d = {**known, **dict(zip(unknown, p))}
        return torch.tensor([d[int(e)] for e in z], dtype=torch.float64)

    def res(p):
        return (S.compute_psi(x, rvdw(p)).numpy() - psi) / np.abs(psi)

    sol = least_squares(res, np.full(len(unknown), 3.0), xtol=1e-15, ftol=1e-15, gtol=1e-15)
    print(f"{name}: max relative residual {np.abs(sol.fun).max():.2e}")
    for e, v in zip(unknown, sol.x):
        print(f"  Z={e:3d}  {v / radii.AA2AU:.6f} AA")
    return {**known, **dict(zip(unknown, sol.x))}


if __name__ == "__main__":
    mb = fit("MB16_43_01", {})
    fit("SiH4", {1: mb[1]})
