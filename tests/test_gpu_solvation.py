"""
Generalized-Born / ALPB solvation on the CUDA path against the reference's
fixtures (tblite values in dxtb's test/test_solvation/samples.py) and the
oracle: Born radii and psi, the interaction matrix, GFN1 + ALPB solvation
energy and gradient of MB16_43_01, GFN2 + GB energies and forces.
"""

from pathlib import Path

import numpy as np
import pytest
import torch

from oracle import solvation_oracle as S
from oracle import xtb_oracle as X

pytestmark = pytest.mark.gpu

G = np.load(Path(__file__).parent / "golden" / "golden.npz")
E_TOL, F_TOL = 1e-8, 1e-6


def _batch(method, mols, charges=None):
    from dxtb_gb300.calculators import tables
    from dxtb_gb300.engine import PackedBatch

    return PackedBatch(tables(method), [m[0] for m in mols], [torch.tensor(m[1]) for m in mols],
                       charges=charges)


@pytest.mark.parametrize("kernel,alpb", [("p16", True), ("p16", False), ("still", False)])
def test_born_radii_and_matrix(kernel, alpb):
    from dxtb_gb300 import _lib
    from dxtb_gb300.engine import gb_args

    names = ["MB16_43_01", "SiH4"]
    mols = [(G[f"{n}/numbers"], G[f"{n}/positions"]) for n in names]
    pb = _batch("gfn1", mols)
    L = _lib.lib()
    na, n2 = pb.total["atoms"], pb.total["nat2"]
    born = torch.empty(na, dtype=torch.float64, device="cuda")
    psi = torch.empty_like(born)
    A = torch.empty(n2, dtype=torch.float64, device="cuda")
    gb = {"epsilon": 78.9, "alpb": alpb, "kernel": kernel}
    _lib.check(L.dxtb_born_matrix(__import__("ctypes").byref(pb.struct), pb.t["par_f"].data_ptr(),
                                  pb.t["par_i"].data_ptr(), *gb_args(gb), born.data_ptr(),
                                  psi.data_ptr(), A.data_ptr(), _lib.stream_ptr()), "born")
    born, psi, A = born.cpu().numpy(), psi.cpu().numpy(), A.cpu().numpy()
    for i, n in enumerate(names):
        a0, a1 = pb.atom_off[i], pb.atom_off[i + 1]
        assert np.abs(psi[a0:a1] / G[f"solv/{n}/psi"] - 1).max() < 1e-10
        assert np.abs(born[a0:a1] / G[f"solv/{n}/born"] - 1).max() < 1e-10
        ref = S.born_matrix(mols[i][0], torch.tensor(mols[i][1]), **gb).numpy()
        nat = a1 - a0
        got = A[pb.nat2_off[i] : pb.nat2_off[i] + nat * nat].reshape(nat, nat)
        assert np.abs(got - ref).max() < 1e-13


def test_gfn1_alpb_mb16_43_01_energy_and_gradient():
    """Solvation energy against the reference fixture; energy and gradient against the oracle."""
    from dxtb_gb300 import GFN1Calculator
    from dxtb_gb300.solvation import GeneralizedBorn

    z = torch.tensor(G["MB16_43_01/numbers"])
    pos = torch.tensor(G["MB16_43_01/positions"], device="cuda")
    opts = {"exclude": ["disp", "hal"], "scf_mode": "implicit", "x_atol": 1e-10, "f_atol": 1e-10,
            "maxiter": 250, "guess": "sad"}
    vac = GFN1Calculator(z, opts=opts, device="cuda").singlepoint(pos)
    gb = GeneralizedBorn(z, 78.9)
    calc = GFN1Calculator(z, interaction=[gb], opts=opts, device="cuda")
    sol = calc.singlepoint(pos)
    gsolv = float(sol.scf - vac.scf)
    assert abs(gsolv - G["solv/MB16_43_01/gsolv"].sum()) < 1e-7
    ref = X.singlepoint("gfn1", z.numpy(), pos.cpu().numpy(), tol=1e-12, solvation={"epsilon": 78.9},
                        grad=True)
    e = float(calc.get_energy(pos))
    f = calc.get_forces(pos).cpu().numpy()
    assert abs(e - ref.energy) < E_TOL
    assert np.abs(f + ref.extra["gradient"].numpy()).max() < F_TOL


@pytest.mark.parametrize("alpb,chrg", [(False, 0.0), (True, 1.0)])
def test_gfn2_gb_energy_forces_vs_oracle(alpb, chrg):
    """GFN2 + GB (eps 78.4) on synthetic molecules; a cation exercises the ALPB shape gradient."""
    from dxtb_gb300.engine import run
    from dxtb_gb300.workloads import random_molecule

    mols = [random_molecule(5000 + i, n) for i, n in enumerate([12, 21, 30])]
    gb = {"epsilon": 78.4, "alpb": alpb, "kernel": "p16"}
    pb = _batch("gfn2", mols, charges=[chrg] * len(mols))
    res = run(pb, forces=True, gb=gb)
    assert (res.status.cpu() == 0).all()
    g = res.gradient.cpu().numpy()
    for i, (num, x) in enumerate(mols):
        ref = X.singlepoint("gfn2", num, x, chrg=chrg, tol=1e-12, solvation=gb, grad=True)
        assert abs(float(res.energy[i]) - ref.energy) < E_TOL
        gi = g[pb.atom_off[i] : pb.atom_off[i + 1]]
        assert np.abs(gi - ref.extra["gradient"].numpy()).max() < F_TOL
