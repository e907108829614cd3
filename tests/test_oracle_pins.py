"""
The CPU oracle against the fixtures of the reference's own test suite
(``tests/golden/golden.npz``, extracted by ``tests/golden/make_golden.py``).
"""

from pathlib import Path

import numpy as np
import pytest
import torch

from oracle import xtb_oracle as X

G = np.load(Path(__file__).parent / "golden" / "golden.npz")
MOLS = ["H2", "LiH", "H2O", "CH4", "SiH4", "LYS_xao"]


def mol(name):
    return G[f"{name}/numbers"].astype(np.int64), G[f"{name}/positions"]


@pytest.mark.parametrize("name", MOLS)
def test_overlap_and_h0_gfn1(name):
    """test/test_overlap/overlap.npz and test/test_hamiltonian/h0.npz (tblite
    0.3.0, stored in float32): pins the integrals, H0, the CN and the radii."""
    num, pos = mol(name)
    sysm = X.make_system("gfn1", num)
    p = torch.tensor(pos)
    s, _, _ = X.integrals(sysm, p, 1)
    cn = X.coordination_number(num, p, "exp")
    h = X.hamiltonian(sysm, p, s, cn)
    assert np.abs(s.numpy() - G[f"{name}/overlap_gfn1"]).max() < 1e-7
    assert np.abs(h.numpy() - G[f"{name}/h0_gfn1"]).max() < 2e-7


@pytest.mark.parametrize("name", ["H2", "LiH", "SiH4"])
def test_h0_gfn2_without_overlap(name):
    """test/test_hamiltonian/test_gfn2.py inline references (tblite 0.3.0):
    the GFN2 H0 built with overlap=None, i.e. the scaling matrix (self-energies
    with the GFN2 CN shift, wexp/Slater factor, shell and pair scaling, EN
    term, distance polynomial). Reference tolerance sqrt(eps) * 10."""
    num, pos = mol(name)
    sysm = X.make_system("gfn2", num)
    p = torch.tensor(pos)
    cn = X.coordination_number(num, p, "gfn")
    n = sysm.nao
    h = X.hamiltonian(sysm, p, torch.ones(n, n, dtype=torch.float64), cn)
    ref = G[f"{name}/h0scale_gfn2"]
    assert h.shape == ref.shape
    assert np.abs(h.numpy() - ref).max() < np.sqrt(np.finfo(np.float64).eps) * 10


def test_planted_radius_error_is_caught(monkeypatch):
    """A 1 % error in one atomic radius of the oracle breaks the H0 pin."""
    from dxtb_gb300.data import radii

    bad = radii.ATOMIC_RADII.copy()
    bad[8] *= 1.01
    monkeypatch.setattr(radii, "ATOMIC_RADII", bad)
    num, pos = mol("H2O")
    sysm = X.make_system("gfn1", num)
    p = torch.tensor(pos)
    s, _, _ = X.integrals(sysm, p, 1)
    h = X.hamiltonian(sysm, p, s, X.coordination_number(num, p, "exp"))
    assert np.abs(h.numpy() - G["H2O/h0_gfn1"]).max() > 1e-5


CLOSED = [2, 4, 10, 12, 18]
OPEN = [1, 6, 7, 8, 9, 16]


@pytest.mark.parametrize("method", ["gfn1", "gfn2"])
@pytest.mark.parametrize("z", CLOSED + OPEN)
def test_single_atom_scf(method, z):
    """test/test_scf/test_elements_gfn{1,2}.py reference vector (tblite):
    E_scf - TS of the free atom. Pins EV2AU, KELVIN2AU, the self-energies,
    STO-nG, ES2/ES3 on-site terms and the Fermi filling."""
    ref = G[f"atoms/{method}"][z - 1]
    r = X.singlepoint(method, [z], np.zeros((1, 3)), tol=1e-13)
    tol = 1e-9 if z in CLOSED else 2e-8
    assert abs(r.e_elec + r.e_free - ref) < tol


def test_aes2_inline_reference():
    """test/test_coulomb/test_aes2.py (LiH): AES2 energies and potentials;
    pins the GFN2 coordination number and the multipole damping."""
    for func in ("test_energy", "test_potential"):
        k = lambda n: torch.tensor(G[f"aes2_{func}/{n}"])
        num = G[f"aes2_{func}/numbers"].astype(np.int64)
        pos = k("positions")
        sysm = X.make_system("gfn2", num)
        a = X.aes2_cache(sysm, pos, X.coordination_number(num, pos, "gfn"))
        qat, qdp, qqp = k("qat"), k("qdp"), k("qqp")
        if func == "test_energy":
            vsd = torch.einsum("ijx,i->jx", a["sd"], qat)
            vdd = 0.5 * torch.einsum("ijxy,ix->jy", a["dd"], qdp)
            edp = (a["dk"][:, None] * qdp * qdp).sum(-1) + ((vsd + vdd) * qdp).sum(-1)
            vqp = torch.einsum("ijx,i->jx", a["sq"], qat)
            eqp = (a["qk"][:, None] * qqp * X.QSCALE * qqp).sum(-1) + (vqp * qqp).sum(-1)
            assert torch.allclose(edp, k("ref_eat_dp"), atol=1e-13)
            assert torch.allclose(eqp, k("ref_eat_qp"), atol=1e-13)
        else:
            vat = torch.einsum("ijx,jx->i", a["sd"], qdp) + torch.einsum("ijx,jx->i", a["sq"], qqp)
            vdp = (torch.einsum("ijx,i->jx", a["sd"], qat) + torch.einsum("ijxy,ix->jy", a["dd"], qdp)
                   + 2 * a["dk"][:, None] * qdp)
            vq = torch.einsum("ijx,i->jx", a["sq"], qat) + 2 * a["qk"][:, None] * qqp * X.QSCALE
            assert torch.allclose(vat, k("ref_vat_mo"), atol=1e-13)
            assert torch.allclose(vdp, k("ref_vat_dp"), atol=1e-13)
            assert torch.allclose(vq, k("ref_vat_qp"), atol=1e-13)


@pytest.mark.parametrize("name", ["H2", "LiH", "H2O", "CH4", "SiH4"])
def test_gfn1_autograd_forces(name):
    """test/test_scf/grad.npz '<name>_full': the reference's own autograd
    gradient of the GFN1 electronic energy (repulsion, dispersion and halogen
    excluded), stored in float32. Pins the oracle's variational gradient."""
    num, pos = mol(name)
    r = X.singlepoint("gfn1", num, pos, grad=True, exclude=("rep",), tol=1e-12)
    ref = G[f"{name}/grad_elec_gfn1"]
    assert np.abs(r.extra["gradient"].numpy() - ref).max() < 5e-8


def test_oracle_gradient_matches_finite_differences():
    """The variational gradient (incl. AES2 and repulsion) equals central
    finite differences of the converged GFN2 energy (step 1e-4 Bohr)."""
    num, pos = mol("H2O")
    r = X.singlepoint("gfn2", num, pos, grad=True, tol=1e-13)
    g = r.extra["gradient"].numpy()
    h = 1e-4
    for a, x in [(0, 2), (1, 0), (2, 2)]:
        pp, pm = pos.copy(), pos.copy()
        pp[a, x] += h
        pm[a, x] -= h
        ep = X.singlepoint("gfn2", num, pp, tol=1e-13).energy
        em = X.singlepoint("gfn2", num, pm, tol=1e-13).energy
        assert abs((ep - em) / (2 * h) - g[a, x]) < 1e-7


# ---- generalized Born / ALPB solvation (test/test_solvation/samples.py, tblite) ----


@pytest.mark.parametrize("name", ["MB16_43_01", "SiH4"])
def test_born_radii_and_psi(name):
    """OBC descreening integral and Born radii with the D3 vdW radii table."""
    from dxtb_gb300.data import radii
    from oracle import solvation_oracle as S

    z = G[f"{name}/numbers"]
    x = torch.tensor(G[f"{name}/positions"])
    born, psi = S.born_radii(x, torch.tensor(radii.lookup(radii.VDW_D3, z, "vdw")))
    assert np.abs(psi.numpy() / G[f"solv/{name}/psi"] - 1).max() < 1e-10
    assert np.abs(born.numpy() / G[f"solv/{name}/born"] - 1).max() < 1e-10


@pytest.mark.parametrize("kernel,alpb,key", [("p16", True, "energies"), ("still", False, "energies_still")])
def test_gb_atom_energies(kernel, alpb, key):
    """E_i = 1/2 q_i (A q)_i at fixed charges, eps = 78.9 (test_alpb.py:48-90)."""
    from oracle import solvation_oracle as S

    z = G["MB16_43_01/numbers"]
    x = torch.tensor(G["MB16_43_01/positions"])
    e = S.atom_energies(z, x, G["solv/MB16_43_01/charges"], epsilon=78.9, alpb=alpb, kernel=kernel)
    # the reference's own tolerance is sqrt(eps) * 10 = 1.5e-7
    assert np.abs(e.numpy() - G[f"solv/MB16_43_01/{key}"]).max() < 5e-9


def test_gfn1_alpb_solvation_energy_and_gradient():
    """GFN1 + ALPB (p16, eps 78.9) SCF: solvation energy and SCF-energy gradient
    of MB16_43_01 (test_alpb.py::test_gb_scf, test_grad.py::test_gb_scf_grad)."""
    z = G["MB16_43_01/numbers"]
    x = G["MB16_43_01/positions"]
    vac = X.singlepoint("gfn1", z, x, tol=1e-10, exclude=("rep",))
    sol = X.singlepoint("gfn1", z, x, tol=1e-10, solvation={"epsilon": 78.9}, grad=True,
                        exclude=("rep",))
    gsolv = G["solv/MB16_43_01/gsolv"].sum()
    assert abs((sol.e_elec - vac.e_elec) - gsolv) < 1e-7
    # the fixture differentiates E_scf (no -TS); the reference's tolerance is 1e-5
    assert np.abs(sol.extra["gradient"].numpy() - G["solv/MB16_43_01/gradient"]).max() < 1e-5


@pytest.mark.parametrize("method", ["gfn1", "gfn2"])
def test_anderson_loop_reaches_the_pinned_solution(method):
    """The restated full-mode loop (Anderson mixer) converges to the fixed
    point of the implicit-mode root solver, whose energies the fixtures
    above pin: to 1e-10 Eh with tight tolerances, and to the tolerance's
    order with the reference defaults (x_atol 1e-4, x_atol_max 1e-5)."""
    from dxtb_gb300.workloads import random_molecule

    num, pos = random_molecule(2104 if method == "gfn1" else 2101, 12)
    ref = X.singlepoint(method, num, pos, tol=1e-12)
    tight = X.singlepoint(method, num, pos, mixer="anderson", maxiter=200,
                          anderson={"x_atol": 1e-11, "x_atol_max": 1e-12})
    loose = X.singlepoint(method, num, pos, mixer="anderson", maxiter=100)
    assert tight.extra["converged"] and loose.extra["converged"]
    assert abs(tight.energy - ref.energy) < 1e-10
    assert abs(loose.energy - ref.energy) < 1e-6
    assert loose.iterations < tight.iterations


SCF_MOLS = ["H2", "LiH", "H2O", "CH4", "SiH4", "MB16_43_01", "LYS_xao", "AD7en+"]


@pytest.mark.parametrize("name", SCF_MOLS)
def test_gfn1_scf_energies(name):
    """test/test_scf/samples.py and samples_charged.py (tblite 0.2.1,
    repulsion and dispersion disabled; AD7en+ is a cation): the whole GFN1
    SCF of multi-atom molecules, E_scf - TS, at the reference test's
    tolerance sqrt(eps) * 10. (The GFN2 values of the same files are tblite's
    electronic energy with its self-consistent D4 part, which this path
    excludes; they are not pins here.)"""
    num, pos = mol(name)
    chrg = float(G[f"scf/{name}/charge"]) if f"scf/{name}/charge" in G.files else 0.0
    r = X.singlepoint("gfn1", num, pos, chrg=chrg, tol=1e-10, maxiter=250, exclude=("rep",))
    assert abs(r.energy - float(G[f"scf/{name}/egfn1"])) < np.sqrt(np.finfo(np.float64).eps) * 10


def test_gfn1_halogen_term_is_zero_for_accepted_elements(monkeypatch):
    """The GFN1 halogen-bond correction (components/classicals/halogen/
    hal.py): its bond strengths are nonzero only for Br, I and At, so for
    every element up to Ar the term vanishes, as in the reference's fixture
    for MB16_43_01 (test/test_classical/test_halogen/samples.py: energy and
    gradient zero), whose Cl has N and O acceptors within the cutoff. With a
    planted strength on Cl the restated term is nonzero and its autograd
    gradient matches central differences."""
    par = X.load_par("gfn1")
    strengths = {z: float(par["element"][z].get("xbond", 0.0)) for z in par["element"]}
    assert all(strengths[z] == 0.0 for z in range(1, 19))
    assert all(strengths[z] > 0.0 for z in (35, 53, 85))
    num, pos = mol("MB16_43_01")
    assert 17 in num.tolist() and {7, 8} & set(num.tolist())
    assert float(X.halogen_energy(par, num, pos)) == 0.0
    monkeypatch.setitem(par["element"][17], "xbond", 0.02)
    p = torch.tensor(pos, requires_grad=True)
    e = X.halogen_energy(par, num, p)
    assert abs(float(e.detach())) > 1e-6
    (g,) = torch.autograd.grad(e, p)
    h = 1e-5
    for a, x in [(int(np.where(num == 17)[0][0]), 0), (int(np.where(num == 8)[0][0]), 2)]:
        q = pos.copy()
        q[a, x] += h
        ep = float(X.halogen_energy(par, num, q))
        q[a, x] -= 2 * h
        em = float(X.halogen_energy(par, num, q))
        assert abs((ep - em) / (2 * h) - float(g[a, x])) < 1e-8
