"""
Parity above n = 1000 orbitals: one seeded random-walk molecule of 401 atoms
(n = 1145, GFN2), which runs as a 16-CTA cluster (the largest size class):
the Sturm-count verification above 384 orbitals, inverse-iteration
eigenvectors and the Householder rows in global memory are exercised at this
size. Energies in vacuum and with generalized Born (Still kernel, epsilon =
78.4, the solvation of the large-system configuration) against the oracle
fixture of ``golden/make_large_fixture.py``; forces against central
differences of the GPU energy in vacuum. (With solvation, 17 buried atoms of
this dense blob have saturated, infinite Born radii and others radii of
1e15 Bohr that move in rounding-sized steps, so finite differences of the
solvated energy carry ~1e-5 of noise.)
"""

from pathlib import Path

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

E_TOL = 1e-8   # Eh
F_TOL = 1e-6   # Eh/Bohr
GB = {"epsilon": 78.4, "alpb": False, "kernel": "still"}


def _data():
    return np.load(Path(__file__).parent / "golden" / "large_gb.npz")


def test_large_molecule_energies():
    from dxtb_gb300.calculators import tables
    from dxtb_gb300.engine import PackedBatch, run

    d = _data()
    assert bool(d["converged"]) and bool(d["converged_vacuum"])
    pb = PackedBatch(tables("gfn2"), [d["numbers"]], [torch.tensor(d["positions"])])
    assert int(pb.nao[0]) >= 1000
    res = run(pb, forces=True, gb=GB, tol=1e-10, maxiter=250)
    assert int(res.status.cpu()[0]) == 0
    assert abs(float(res.energy[0]) - float(d["energy"])) < E_TOL
    assert torch.isfinite(res.gradient).all()
    vac = run(pb, tol=1e-10, maxiter=250)
    assert int(vac.status.cpu()[0]) == 0
    assert abs(float(vac.energy[0]) - float(d["energy_vacuum"])) < E_TOL


def test_large_molecule_forces_by_finite_differences():
    from dxtb_gb300.calculators import tables
    from dxtb_gb300.engine import PackedBatch, run

    d = _data()
    z, p0 = d["numbers"], d["positions"]
    pb = PackedBatch(tables("gfn2"), [z], [torch.tensor(p0)])
    res = run(pb, forces=True, tol=1e-10, maxiter=250)
    assert int(res.status.cpu()[0]) == 0
    g = res.gradient.cpu().numpy()
    # central differences (h = 1e-4 Bohr) on three coordinates, all displaced
    # geometries in one packed batch
    h = 1e-4
    where = [(0, 0), (len(z) // 2, 1), (len(z) - 1, 2)]
    pos = []
    for a, x in where:
        for sgn in (1.0, -1.0):
            q = p0.copy()
            q[a, x] += sgn * h
            pos.append(torch.tensor(q))
    pbd = PackedBatch(tables("gfn2"), [z] * len(pos), pos)
    rd = run(pbd, tol=1e-10, maxiter=250)
    assert (rd.status.cpu() == 0).all()
    e = rd.energy.cpu().numpy()
    for k, (a, x) in enumerate(where):
        assert abs((e[2 * k] - e[2 * k + 1]) / (2 * h) - g[a, x]) < F_TOL, (a, x)
