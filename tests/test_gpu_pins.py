"""
The CUDA path against the reference's own fixtures, directly (not only
through the oracle):

- free atoms H-Ar, GFN1 and GFN2, against the tblite energies of
  test/test_scf/test_elements_gfn{1,2}.py (E_scf - TS). This runs the device
  eigensolver at n = 1 (H in GFN2), on exactly degenerate shells and on
  fractional Fermi occupations (open-shell C, N, O, F, Si, S, ...);
- the GFN2 H0 of H2, LiH and SiH4 against the inline tblite 0.3.0 matrices
  of test/test_hamiltonian/test_gfn2.py (built there with overlap=None, the
  scaling matrix): the device H0 must equal that matrix times the device S.
"""

from pathlib import Path

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

G = np.load(Path(__file__).parent / "golden" / "golden.npz")
CLOSED = {2, 4, 10, 12, 18}


@pytest.mark.parametrize("method", ["gfn1", "gfn2"])
def test_free_atoms_vs_tblite(method):
    from dxtb_gb300.calculators import tables
    from dxtb_gb300.engine import PackedBatch, run

    zs = list(range(1, 19))
    pb = PackedBatch(tables(method), [np.array([z]) for z in zs], [torch.zeros(1, 3, dtype=torch.float64)] * len(zs))
    if method == "gfn2":
        assert int(pb.nao[0]) == 1  # the H atom: a 1 x 1 eigenproblem
    res = run(pb, tol=1e-12, maxiter=250)
    assert (res.status.cpu() == 0).all()
    e = (res.e_scf + res.e_free).cpu().numpy()
    ref = G[f"atoms/{method}"][: len(zs)]
    for k, z in enumerate(zs):
        tol = 1e-9 if z in CLOSED else 2e-8  # the oracle's pins use the same bars
        assert abs(e[k] - ref[k]) < tol, (z, e[k], ref[k])
    assert float(res.e_rep.abs().max()) == 0.0


@pytest.mark.parametrize("name", ["H2", "LiH", "SiH4"])
def test_gfn2_h0_vs_inline_reference(name):
    from dxtb_gb300.calculators import tables
    from dxtb_gb300.engine import PackedBatch, run

    num = G[f"{name}/numbers"].astype(np.int64)
    pos = G[f"{name}/positions"]
    pb = PackedBatch(tables("gfn2"), [num], [torch.tensor(pos)])
    res = run(pb)
    n = int(pb.nao[0])
    S = res.state["S"][: n * n].view(n, n).cpu().numpy()
    H = res.state["H"][: n * n].view(n, n).cpu().numpy()
    ref = G[f"{name}/h0scale_gfn2"]
    assert ref.shape == (n, n)
    assert np.abs(H - ref * S).max() < np.sqrt(np.finfo(np.float64).eps) * 10


def test_gfn1_scf_energies_vs_tblite():
    """The GFN1 SCF energies (E_scf - TS) of test/test_scf/samples.py and the
    cation AD7en+ of samples_charged.py (tblite 0.2.1, repulsion and
    dispersion disabled) on the device, all eight molecules in one packed
    batch with their charges. The reference's own tolerance is sqrt(eps) * 10
    (1.5e-7); the oracle reproduces these values to 5e-10, so the device is
    held to the parity bar of 1e-8 Eh."""
    from dxtb_gb300.calculators import tables
    from dxtb_gb300.engine import PackedBatch, run

    names = ["H2", "LiH", "H2O", "CH4", "SiH4", "MB16_43_01", "LYS_xao", "AD7en+"]
    chrg = [float(G[f"scf/{n}/charge"]) if f"scf/{n}/charge" in G.files else 0.0 for n in names]
    assert chrg[-1] == 1.0
    pb = PackedBatch(tables("gfn1"), [G[f"{n}/numbers"] for n in names],
                     [torch.tensor(G[f"{n}/positions"]) for n in names], charges=chrg)
    res = run(pb, tol=1e-10, maxiter=250)
    assert (res.status.cpu() == 0).all()
    e = (res.e_scf + res.e_free).cpu().numpy()
    for k, n in enumerate(names):
        assert abs(e[k] - float(G[f"scf/{n}/egfn1"])) < 1e-8, n
