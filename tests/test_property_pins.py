"""
Dipole moments, harmonic frequencies and IR intensities (GFN1) against the
reference's property fixtures (``test/test_properties/samples.py``, in
``tests/golden/golden.npz`` under ``props/``), on the CPU:

- the oracle's dipole moment sum_A Z_A R_A - tr(P D0) at the converged
  density, at the reference test's tolerance (``test_dipole.py``: atol 1e-3);
- ``dxtb_gb300.properties.vib_analysis`` and ``ir_ints`` applied to the
  oracle's Hessian and dipole derivative (central differences, h = 1e-3
  Bohr, of the oracle's analytic gradients and dipoles): frequencies at the
  reference test's tolerance (``test_vibration_ref.py``: 10 cm^-1 absolute,
  1e-3 relative), intensities within 1 % (the fixture's provenance is not
  stated; the reference's own IR test compares two of its routes with up to
  70 km/mol absolute for CH4).

The reference fixtures include D3 dispersion, which this path excludes; for
these molecules it moves the frequencies by far less than the tolerance.
"""

from pathlib import Path

import numpy as np
import pytest
import torch

from oracle import xtb_oracle as X

G = np.load(Path(__file__).parent / "golden" / "golden.npz")
H = 1e-3


def mol(name):
    return G[f"{name}/numbers"].astype(np.int64), G[f"{name}/positions"]


@pytest.mark.parametrize("name", ["H2", "LiH", "H2O", "CH4", "SiH4"])
def test_oracle_dipole(name):
    z, p = mol(name)
    r = X.singlepoint("gfn1", z, p, tol=1e-10, maxiter=250)
    mu = X.dipole_moment(X.make_system("gfn1", z), p, r.p).numpy()
    assert np.abs(mu - G[f"props/{name}/dipole"]).max() < 1e-3


def oracle_hessian_and_dipole_derivative(z, p0):
    sysm = X.make_system("gfn1", z)
    nat = len(z)
    hess = np.zeros((3 * nat, 3 * nat))
    dmu = np.zeros((3, 3 * nat))
    for a in range(nat):
        for x in range(3):
            gs, ms = [], []
            for sgn in (1.0, -1.0):
                p = p0.copy()
                p[a, x] += sgn * H
                r = X.singlepoint("gfn1", z, p, tol=1e-11, maxiter=250, grad=True)
                gs.append(r.extra["gradient"].numpy().ravel())
                ms.append(X.dipole_moment(sysm, p, r.p).numpy())
            hess[3 * a + x] = (gs[0] - gs[1]) / (2 * H)
            dmu[:, 3 * a + x] = (ms[0] - ms[1]) / (2 * H)
    hess = 0.5 * (hess + hess.T)
    return torch.tensor(hess).view(nat, 3, nat, 3), torch.tensor(dmu).view(3, nat, 3)


@pytest.mark.parametrize("name", ["H2", "LiH", "H2O"])
def test_frequencies_and_ir_intensities(name):
    from dxtb_gb300.properties import IRResult, ir_ints, vib_analysis

    z, p = mol(name)
    hess, dmu = oracle_hessian_and_dipole_derivative(z, p)
    vib = vib_analysis(z, torch.tensor(p), hess)
    nat = len(z)
    assert vib.modes.shape == (3 * nat, 3 * nat - (5 if nat == 2 else 6))
    ir = IRResult(vib.freqs, ir_ints(dmu, vib.modes))
    ir.use_common_units()
    f, i = ir.freqs.numpy(), ir.ints.numpy()
    ref_f, ref_i = G[f"props/{name}/freqs"], G[f"props/{name}/ints"]
    assert np.all(np.abs(f - ref_f) <= 10.0 + 1e-3 * np.abs(ref_f))
    assert np.all(np.abs(i - ref_i) <= 0.1 + 1e-2 * np.abs(ref_i))


def test_single_atom_and_units():
    """One atom: nothing to project, three zero frequencies (the fixture of
    the H atom); unit conversions and the rejected matrix-shaped Hessian."""
    from dxtb_gb300.data.masses import AU2KMMOL, AU2RCM
    from dxtb_gb300.properties import VibResult, vib_analysis

    vib = vib_analysis([1], torch.zeros(1, 3, dtype=torch.float64),
                       torch.zeros(1, 3, 1, 3, dtype=torch.float64))
    assert vib.freqs.tolist() == [0.0, 0.0, 0.0]
    r = VibResult(torch.tensor([1.0], dtype=torch.float64), torch.eye(3, dtype=torch.float64))
    assert r.to_unit("freqs", "cm^-1").item() == pytest.approx(AU2RCM)
    r.use_common_units()
    assert r.freqs.item() == pytest.approx(219474.63, rel=1e-8)
    assert AU2KMMOL == pytest.approx(1.7771e6, rel=1e-4)
    with pytest.raises(ValueError):
        vib_analysis([1, 1], torch.zeros(2, 3), torch.zeros(6, 6, dtype=torch.float64))


def test_projection_removes_rigid_motions():
    """A Hessian that is a pure translation/rotation penalty has only zero
    frequencies after the projection (non-linear and linear molecules)."""
    from dxtb_gb300.properties import _rigid_modes, vib_analysis
    from dxtb_gb300.data.masses import atomic_mass

    for name in ("H2O", "H2"):
        z, p = mol(name)
        m = torch.tensor(atomic_mass(z))
        pos = torch.tensor(p)
        rig = _rigid_modes(m, pos, len(z) == 2)
        msq = m.sqrt().repeat_interleave(3)
        # mass-weighted penalty on the rigid modes, un-mass-weighted
        hess = (msq[:, None] * (rig.T @ rig) * msq[None, :]).view(len(z), 3, len(z), 3)
        vib = vib_analysis(z, pos, hess)
        scale = torch.linalg.matrix_norm(rig.T @ rig, ord=2).item()
        assert (vib.freqs**2).max().item() < 1e-14 * scale


def test_linear_molecules_keep_3n_minus_5_modes():
    """A linear triatomic (collinear, off the coordinate axes) projects five
    rigid motions and keeps 3 nat - 5 = 4 modes; bending it gives 3."""
    from dxtb_gb300.properties import is_linear, vib_analysis

    axis = torch.tensor([1.0, 2.0, -0.5], dtype=torch.float64)
    axis = axis / axis.norm()
    lin = torch.stack([0.0 * axis, 2.2 * axis, 4.4 * axis]) + torch.tensor([0.3, -1.0, 2.0])
    assert is_linear(lin)
    bent = lin.clone()
    bent[2] += torch.tensor([0.0, 0.3, 0.0], dtype=torch.float64)
    assert not is_linear(bent)
    z = [8, 6, 8]
    for pos, nmodes in ((lin, 4), (bent, 3)):
        h = torch.eye(9, dtype=torch.float64).view(3, 3, 3, 3) * 0.5
        vib = vib_analysis(z, pos, h)
        assert vib.modes.shape == (9, nmodes)
        assert (vib.freqs > 0).all()
