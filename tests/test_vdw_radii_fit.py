"""
The D3 van-der-Waals radii of ``dxtb_gb300/data/radii.py`` are pinned by the
reference's solvation fixtures: a free least-squares fit of every radius of
MB16_43_01 (H, B, N, O, F, Na, Al, Si and Cl) to its 16 tblite descreening
integrals psi (``golden.npz`` entry ``solv/MB16_43_01/psi``, through the
oracle's restatement of ``compute_psi``) returns the table's values, which
hold the 5 digits of the published table.
"""

from pathlib import Path

import numpy as np
import pytest
import torch

G = np.load(Path(__file__).parent / "golden" / "golden.npz")


def test_fit_reproduces_the_table():
    scipy_opt = pytest.importorskip("scipy.optimize")
    from dxtb_gb300.data import radii
    from oracle import solvation_oracle as S

    z = G["MB16_43_01/numbers"]
    x = torch.tensor(G["MB16_43_01/positions"])
    psi = G["solv/MB16_43_01/psi"]
    elems = sorted(set(int(e) for e in z))

    def res(p):
        d = dict(zip(elems, p))
        r = torch.tensor([d[int(e)] for e in z], dtype=torch.float64)
        return (S.compute_psi(x, r).numpy() - psi) / np.abs(psi)

    sol = scipy_opt.least_squares(res, np.full(len(elems), 3.0), xtol=1e-15, ftol=1e-15, gtol=1e-15)
    assert np.abs(sol.fun).max() < 1e-12
    table = radii.lookup(radii.VDW_D3, elems, "vdw")
    # the table rounds to 5 significant digits in Angstrom
    assert np.abs(sol.x / table - 1.0).max() < 1e-5
