"""
CUDA graphs of the single point (``dxtb_graph_*``, ``engine.GraphStep``):
a replay must give the eager run's results (to the last few units of
rounding that atomic accumulation leaves), for the positions it was
captured with and for new positions of the same molecules, on a batch whose
molecules fall into the shared-SM, one-SM and cluster size classes (the
forked class streams are part of the graph). The calculator replays
the graph on repeated calls; its results equal those of the eager path.
"""

import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _batch(method="gfn2"):
    import ctypes as C

    from dxtb_gb300 import _lib
    from dxtb_gb300.calculators import tables
    from dxtb_gb300.engine import PackedBatch
    from dxtb_gb300.workloads import random_molecule

    mols = [random_molecule(8200 + i, n) for i, n in enumerate([9, 24, 45, 52, 64, 40])]
    pb = PackedBatch(tables(method), [m[0] for m in mols], [torch.tensor(m[1]) for m in mols])
    thr = (C.c_int32 * 5)()
    assert _lib.lib().dxtb_scf_get_size_classes(thr) == 0
    nao = pb.nao
    assert (nao < thr[0]).any() and (nao >= thr[1]).any()  # shared-SM and cluster classes
    return pb, mols


# The SCF kernels are deterministic; the per-molecule repulsion sums
# (index_add_) and the gradient accumulate with atomics, whose order varies
# from run to run by a few units in the last place.
ATOL = 1e-11


def _same(a, b):
    assert (a.energy - b.energy).abs().max().item() <= ATOL
    assert torch.equal(a.status, b.status)
    assert torch.equal(a.iterations, b.iterations)
    if a.gradient is not None:
        assert (a.gradient - b.gradient).abs().max().item() <= ATOL


@pytest.mark.parametrize("forces", [False, True])
def test_graph_replay_equals_eager(forces):
    from dxtb_gb300.engine import GraphStep, run

    pb, mols = _batch()
    kw = dict(tol=1e-10, maxiter=250, forces=forces)
    g = GraphStep(pb, **kw)
    ref = run(pb, **kw)
    assert (ref.status.cpu() == 0).all()
    _same(g.first, ref)
    _same(g.replay(), ref)
    # new positions: displaced and rotated copies of the molecules
    rng = np.random.default_rng(5)
    newpos = [torch.tensor(m[1] + rng.normal(scale=0.02, size=m[1].shape)) for m in mols]
    rep = g.replay(newpos)
    rep = type(rep)(**{k: (v.clone() if torch.is_tensor(v) else v) for k, v in rep.__dict__.items()})
    pb.copy_positions_(newpos)
    ref2 = run(pb, **kw)
    _same(rep, ref2)
    assert not torch.equal(ref2.energy, ref.energy)


def test_calculator_repeated_calls_replay_the_graph():
    from dxtb_gb300.calculators import GFN2Calculator

    pb, mols = _batch()
    nat = max(len(m[0]) for m in mols)
    num = torch.zeros(len(mols), nat, dtype=torch.int64)
    pos = torch.zeros(len(mols), nat, 3, dtype=torch.float64)
    for i, (z, p) in enumerate(mols):
        num[i, : len(z)] = torch.tensor(z)
        pos[i, : len(z)] = torch.tensor(p)
    opts = {"scf_mode": "implicit", "x_atol": 1e-10, "f_atol": 1e-10, "maxiter": 250,
            "guess": "sad", "exclude": ["disp", "d4sc"]}
    graph_calc = GFN2Calculator(num, opts=opts)
    os.environ["DXTB_GRAPHS"] = "0"
    try:
        eager_calc = GFN2Calculator(num, opts=opts)
        steps = [pos + 0.01 * k * torch.sin(pos) for k in range(4)]
        eager = [(eager_calc.get_energy(p.cuda()).clone(), eager_calc.get_forces(p.cuda()).clone())
                 for p in steps]
    finally:
        os.environ.pop("DXTB_GRAPHS")
    for (e_ref, f_ref), p in zip(eager, steps):
        e = graph_calc.get_energy(p.cuda())
        f = graph_calc.get_forces(p.cuda())
        assert (e - e_ref).abs().max().item() <= ATOL
        assert (f - f_ref).abs().max().item() <= ATOL
    assert set(graph_calc._graphs) == {False, True}
    assert all(g is not None for g in graph_calc._graphs.values())  # captured, not eager
