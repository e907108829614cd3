"""
Parity of the CUDA path with the oracle on EVERY molecule of the benchmark
sets: the 256 GFN2 molecules of 10-60 atoms and the 64 molecules of 30-120
atoms (GFN1 and GFN2), energy and forces, against the oracle fixtures of
``golden/make_set_fixtures.py`` (tol = 1e-10, float64). Central finite
differences (h = 1e-4 Bohr) of the GPU energy check the GPU gradient on
molecules 0-3 of the 64.

Bars: |dE| <= 1e-8 Eh and max |dF| <= 1e-6 Eh/Bohr per molecule. A molecule
may only be listed in EXCLUDE with the reason written beside it, and only if
the oracle's own SCF needed more than 100 iterations there (an SCF with
several nearby solutions, where the one reached depends on rounding).
"""

from pathlib import Path

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

E_TOL = 1e-8   # Eh
F_TOL = 1e-6   # Eh/Bohr
GOLDEN = Path(__file__).parent / "golden"

# (set, method) -> {molecule index: reason}. Each listed molecule is an SCF
# whose oracle trajectory is itself not determined by the input at this
# precision: displacing one coordinate by 1e-11 Bohr changes the oracle's
# iteration count (molecule 23: 137 -> 125 / 170) or the solution it lands
# on (molecule 23 at -1e-11 Bohr: 0.043 Eh lower).
EXCLUDE: dict = {
    ("c2", "gfn2"): {},
    ("c3", "gfn1"): {
        1: "oracle 116 iterations; the GPU trajectory does not settle within 250",
        6: "oracle 105 iterations; the GPU reaches the oracle's energy (2.8e-14) and "
           "forces (1.2e-10) but does not meet the 1e-10 stopping rule within 250",
        23: "oracle 137 iterations; the GPU lands on another SCF solution (0.22 Eh)",
        37: "oracle 145 iterations; the GPU trajectory does not settle within 250",
        48: "the oracle itself does not converge within 250 iterations",
        53: "oracle 161 iterations; the GPU trajectory does not settle within 250",
    },
    ("c3", "gfn2"): {},
}


def _load(cfg):
    return dict(np.load(GOLDEN / f"sets_{cfg}.npz"))


def _batch(method, d, idx):
    from dxtb_gb300.calculators import tables
    from dxtb_gb300.engine import PackedBatch

    nat = d["nat"]
    nums = [d["numbers"][i, : nat[i]] for i in idx]
    pos = [torch.tensor(d["positions"][i, : nat[i]]) for i in idx]
    return PackedBatch(tables(method), nums, pos)


def _compare(cfg, method):
    from dxtb_gb300.engine import run

    d = _load(cfg)
    idx = list(range(len(d["nat"])))
    pb = _batch(method, d, idx)
    res = run(pb, forces=True, tol=float(d["tol"]), maxiter=int(d["maxiter"]))
    status = res.status.cpu().numpy()
    e = res.energy.cpu().numpy()
    g = res.gradient.cpu().numpy()
    de = np.abs(e - d[f"{method}/energy"])
    df = np.array([
        np.abs(g[pb.atom_off[i] : pb.atom_off[i + 1]] - d[f"{method}/gradient"][i, : d["nat"][i]]).max()
        for i in idx
    ])
    return d, status, de, df, res.iterations.cpu().numpy()


@pytest.mark.parametrize(("cfg", "method"), [("c2", "gfn2"), ("c3", "gfn1"), ("c3", "gfn2")])
def test_every_molecule_of_the_set(cfg, method):
    d, status, de, df, it = _compare(cfg, method)
    excl = EXCLUDE[(cfg, method)]
    ref_it = d[f"{method}/iterations"]
    for i, why in excl.items():
        assert ref_it[i] > 100, f"molecule {i} excluded ({why}) but the oracle converged in {ref_it[i]}"
    bad = [
        f"#{i}: status {status[i]} |dE| {de[i]:.2e} |dF| {df[i]:.2e} it {it[i]:.0f}/{ref_it[i]}"
        for i in range(len(de))
        if i not in excl and (status[i] != 0 or not de[i] <= E_TOL or not df[i] <= F_TOL)
    ]
    print(f"{cfg} {method}: max|dE| {np.max(np.delete(de, list(excl))):.2e} "
          f"max|dF| {np.max(np.delete(df, list(excl))):.2e}, excluded {sorted(excl)}")
    assert not bad, "\n".join(bad)


@pytest.mark.parametrize("method", ["gfn1", "gfn2"])
def test_finite_differences_four_molecules(method):
    """The first four molecules of the 64 outside EXCLUDE (GFN2: 0-3; GFN1:
    0, 2, 3, 4, molecule 1 being excluded): three coordinates each (first,
    middle, last atom; x, y, z), all displaced geometries in one packed
    batch."""
    from dxtb_gb300.engine import run

    d = _load("c3")
    h = 1e-4
    nat = d["nat"]
    sel = [i for i in range(len(nat)) if i not in EXCLUDE[("c3", method)]][:4]
    base = _batch(method, d, sel)
    rb = run(base, forces=True)
    assert (rb.status.cpu() == 0).all()
    g = rb.gradient.cpu().numpy()
    nums, pos, where = [], [], []
    for k, m in enumerate(sel):
        z = d["numbers"][m, : nat[m]]
        p0 = d["positions"][m, : nat[m]]
        for a, x in [(0, 0), (nat[m] // 2, 1), (nat[m] - 1, 2)]:
            for sgn in (1.0, -1.0):
                p = p0.copy()
                p[a, x] += sgn * h
                nums.append(z)
                pos.append(torch.tensor(p))
            where.append((k, a, x))
    from dxtb_gb300.calculators import tables
    from dxtb_gb300.engine import PackedBatch

    pb = PackedBatch(tables(method), nums, pos)
    r = run(pb)
    assert (r.status.cpu() == 0).all()
    e = r.energy.cpu().numpy()
    for k, (m, a, x) in enumerate(where):
        fd = (e[2 * k] - e[2 * k + 1]) / (2 * h)
        an = g[base.atom_off[m] + a, x]
        assert abs(fd - an) < F_TOL, (m, a, x, fd, an)
