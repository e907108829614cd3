"""
Parity above n = 1000 orbitals: one seeded random-walk molecule of 401 atoms
(n = 1145; GFN2, generalized Born with the Still kernel at epsilon = 78.4,
the solvation of the large-system configuration) against the oracle fixture
of ``golden/make_large_fixture.py``. The molecule runs as a 16-CTA cluster
(the largest size class): the Sturm-count verification above 384 orbitals,
the 2^-+400 rescaling of the twisted factorisation and the Householder rows
in global memory are exercised at this size. Energy against the oracle;
forces against central differences of the GPU energy.
"""

from pathlib import Path

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

E_TOL = 1e-8   # Eh
F_TOL = 1e-6   # Eh/Bohr
GB = {"epsilon": 78.4, "alpb": False, "kernel": "still"}


def test_large_molecule_with_born_solvation():
    from dxtb_gb300.calculators import tables
    from dxtb_gb300.engine import PackedBatch, run

    d = np.load(Path(__file__).parent / "golden" / "large_gb.npz")
    assert bool(d["converged"])
    pb = PackedBatch(tables("gfn2"), [d["numbers"]], [torch.tensor(d["positions"])])
    assert int(pb.nao[0]) >= 1000
    res = run(pb, forces=True, gb=GB, tol=1e-10, maxiter=250)
    assert int(res.status.cpu()[0]) == 0
    assert abs(float(res.energy[0]) - float(d["energy"])) < E_TOL
    g = res.gradient.cpu().numpy()
    # forces: central differences (h = 1e-4 Bohr) of the GPU energy on three
    # coordinates, all displaced geometries in one packed batch
    h = 1e-4
    z, p0 = d["numbers"], d["positions"]
    where = [(0, 0), (len(z) // 2, 1), (len(z) - 1, 2)]
    pos = []
    for a, x in where:
        for sgn in (1.0, -1.0):
            q = p0.copy()
            q[a, x] += sgn * h
            pos.append(torch.tensor(q))
    pbd = PackedBatch(tables("gfn2"), [z] * len(pos), pos)
    rd = run(pbd, gb=GB, tol=1e-10, maxiter=250)
    assert (rd.status.cpu() == 0).all()
    e = rd.energy.cpu().numpy()
    for k, (a, x) in enumerate(where):
        assert abs((e[2 * k] - e[2 * k + 1]) / (2 * h) - g[a, x]) < F_TOL, (a, x)
