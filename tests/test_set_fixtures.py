"""
The full-set oracle fixtures (``golden/sets_c2.npz``, ``golden/sets_c3.npz``)
hold exactly the benchmark molecules of the seeded generator, and the oracle
reproduces their energies and gradients (spot check on the smallest
molecules, so that the suite stays fast on the CPU).
"""

from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).parent / "golden"


@pytest.mark.parametrize(("cfg", "config"), [("c2", 2), ("c3", 3)])
def test_fixture_inputs_are_the_benchmark_molecules(cfg, config):
    from dxtb_gb300.workloads import config_molecules

    d = np.load(GOLDEN / f"sets_{cfg}.npz")
    mols = config_molecules(config)
    assert len(mols) == len(d["nat"])
    for i, (z, p) in enumerate(mols):
        n = int(d["nat"][i])
        assert n == len(z)
        assert (d["numbers"][i, :n] == z).all() and (d["numbers"][i, n:] == 0).all()
        assert np.abs(d["positions"][i, :n] - p).max() < 1e-12


@pytest.mark.parametrize(("cfg", "method"), [("c2", "gfn2"), ("c3", "gfn1")])
def test_oracle_reproduces_fixture(cfg, method):
    import torch

    from oracle import xtb_oracle as X

    torch.set_num_threads(min(4, torch.get_num_threads()))
    d = np.load(GOLDEN / f"sets_{cfg}.npz")
    i = int(np.argmin(d["nat"]))
    n = int(d["nat"][i])
    r = X.singlepoint(method, d["numbers"][i, :n], d["positions"][i, :n], grad=True,
                      tol=float(d["tol"]), maxiter=int(d["maxiter"]))
    assert abs(r.energy - d[f"{method}/energy"][i]) < 1e-9
    assert np.abs(r.extra["gradient"].numpy() - d[f"{method}/gradient"][i, :n]).max() < 1e-8
    assert r.iterations == d[f"{method}/iterations"][i]
