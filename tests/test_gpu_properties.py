"""
Properties through the GPU calculator against the reference's property
fixtures (``test/test_properties/samples.py``, GFN1, under ``props/`` in
``tests/golden/golden.npz``) and the oracle:

- ``dipole``: one ``dxtb_dipole_moment`` launch at the converged density;
  fixture tolerance of ``test_dipole.py`` (1e-3 e a0), and the oracle's
  moment at the same geometry to 1e-7 (both SCFs converged to 1e-10), GFN1
  and GFN2 (a random 30-atom molecule);
- ``vibration``: frequencies from the GPU Hessian (one packed batch of the
  6 nat displaced single points) at the tolerance of
  ``test_vibration_ref.py`` (10 cm^-1 absolute, 1e-3 relative);
- ``ir``: intensities from the dipole derivative of the same displaced
  batch, within 1 % of the fixture.

The calculator options are those of the reference tests: full-mode SCF with
the Anderson mixer, x_atol = f_atol = 1e-10.
"""

from pathlib import Path

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

G = np.load(Path(__file__).parent / "golden" / "golden.npz")
OPTS = {"scf_mode": "full", "mixer": "anderson", "maxiter": 100, "x_atol": 1e-10,
        "f_atol": 1e-10, "guess": "sad", "exclude": ["disp", "d4sc"]}


def calc(method, name):
    from dxtb_gb300.calculators import GFN1Calculator, GFN2Calculator

    z = torch.tensor(G[f"{name}/numbers"].astype(np.int64))
    pos = torch.tensor(G[f"{name}/positions"], device="cuda")
    cls = GFN1Calculator if method == "gfn1" else GFN2Calculator
    return cls(z, opts=OPTS), pos


@pytest.mark.parametrize("name", ["H2", "LiH", "H2O", "CH4", "SiH4"])
def test_dipole_vs_fixture_and_oracle(name):
    from oracle import xtb_oracle as X

    c, pos = calc("gfn1", name)
    mu = c.dipole(pos).cpu().numpy()
    assert np.abs(mu - G[f"props/{name}/dipole"]).max() < 1e-3
    z, p = G[f"{name}/numbers"].astype(np.int64), G[f"{name}/positions"]
    r = X.singlepoint("gfn1", z, p, tol=1e-10, maxiter=250)
    ref = X.dipole_moment(X.make_system("gfn1", z), p, r.p).numpy()
    assert np.abs(mu - ref).max() < 1e-7


def test_dipole_gfn2_batch_vs_oracle():
    from dxtb_gb300.calculators import GFN2Calculator
    from dxtb_gb300.workloads import random_molecule
    from oracle import xtb_oracle as X

    mols = [random_molecule(7100 + i, n) for i, n in enumerate([12, 30])]
    nat = max(len(m[0]) for m in mols)
    num = torch.zeros(len(mols), nat, dtype=torch.int64)
    pos = torch.zeros(len(mols), nat, 3, dtype=torch.float64)
    for i, (z, p) in enumerate(mols):
        num[i, : len(z)] = torch.tensor(z)
        pos[i, : len(z)] = torch.tensor(p)
    c = GFN2Calculator(num, opts=OPTS)
    mu = c.dipole(pos.cuda()).cpu().numpy()
    for i, (z, p) in enumerate(mols):
        r = X.singlepoint("gfn2", z, p, tol=1e-10, maxiter=250)
        ref = X.dipole_moment(X.make_system("gfn2", z), p, r.p).numpy()
        assert np.abs(mu[i] - ref).max() < 1e-7


@pytest.mark.parametrize("name", ["H2", "LiH", "H2O", "CH4", "SiH4"])
def test_frequencies_vs_fixture(name):
    c, pos = calc("gfn1", name)
    vib = c.vibration(pos)
    vib.use_common_units()
    f = vib.freqs.cpu().numpy()
    ref = G[f"props/{name}/freqs"]
    assert f.shape == ref.shape
    assert np.all(np.abs(f - ref) <= 10.0 + 1e-3 * np.abs(ref))


@pytest.mark.parametrize("name", ["LiH", "H2O", "CH4"])
def test_ir_intensities_vs_fixture(name):
    c, pos = calc("gfn1", name)
    ir = c.ir(pos)
    ir.use_common_units()
    f, i = ir.freqs.cpu().numpy(), ir.ints.cpu().numpy()
    ref_f, ref_i = G[f"props/{name}/freqs"], G[f"props/{name}/ints"]
    assert np.all(np.abs(f - ref_f) <= 10.0 + 1e-3 * np.abs(ref_f))
    assert np.all(np.abs(i - ref_i) <= 0.1 + 1e-2 * np.abs(ref_i))
