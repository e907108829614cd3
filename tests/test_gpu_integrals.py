"""
Integral wrappers (overlap / dipint / quadint) and driver classes on the CUDA
path against the oracle's restatement of the reference pair builder and the
tblite overlap fixtures.
"""

from pathlib import Path

import numpy as np
import pytest
import torch

from oracle import xtb_oracle as X

pytestmark = pytest.mark.gpu

G = np.load(Path(__file__).parent / "golden" / "golden.npz")


def _oracle(method, num, pos):
    sysm = X.make_system(method, num)
    p = torch.tensor(pos)
    s_raw = X.multipole_raw(sysm, p, X.COMP_S)[0]
    norm = X.snorm(s_raw)
    nn = norm[:, None] * norm[None, :]
    return (s_raw * nn).numpy(), (X.multipole_raw(sysm, p, X.COMP_D) * nn).numpy(), \
        (X.multipole_raw(sysm, p, X.COMP_Q9) * nn).numpy()


@pytest.mark.parametrize("method", ["gfn1", "gfn2"])
@pytest.mark.parametrize("name", ["H2O", "SiH4", "LYS_xao"])
def test_wrappers_match_oracle(method, name):
    from dxtb_gb300.integrals import dipint, overlap, quadint

    num = torch.tensor(G[f"{name}/numbers"])
    pos = torch.tensor(G[f"{name}/positions"], device="cuda")
    s, d, q = _oracle(method, num.numpy(), G[f"{name}/positions"])
    assert np.abs(overlap(num, pos, method).cpu().numpy() - s).max() < 1e-12
    assert np.abs(dipint(num, pos, method).cpu().numpy() - d).max() < 1e-12
    assert np.abs(quadint(num, pos, method).cpu().numpy() - q).max() < 1e-11
    if method == "gfn1":
        assert np.abs(overlap(num, pos, method).cpu().numpy() - G[f"{name}/overlap_gfn1"]).max() < 1e-7


def test_driver_classes_batched_padding():
    from dxtb_gb300.integrals import DipolePytorch, IntDriverPytorch, OverlapPytorch, QuadrupolePytorch

    names = ["H2O", "SiH4", "CH4"]
    nmax = max(len(G[f"{n}/numbers"]) for n in names)
    num = torch.zeros(len(names), nmax, dtype=torch.int64)
    pos = torch.zeros(len(names), nmax, 3, dtype=torch.float64)
    for i, n in enumerate(names):
        k = len(G[f"{n}/numbers"])
        num[i, :k] = torch.tensor(G[f"{n}/numbers"])
        pos[i, :k] = torch.tensor(G[f"{n}/positions"])
    drv = IntDriverPytorch(num, "gfn2", device="cuda")
    drv.setup(pos.cuda())
    S = OverlapPytorch().build(drv)
    D = DipolePytorch().build(drv)
    Q = QuadrupolePytorch().build(drv)
    for i, n in enumerate(names):
        s, d, q = _oracle("gfn2", G[f"{n}/numbers"], G[f"{n}/positions"])
        k = s.shape[0]
        assert np.abs(S[i, :k, :k].cpu().numpy() - s).max() < 1e-12
        assert np.abs(D[i, :, :k, :k].cpu().numpy() - d).max() < 1e-12
        assert np.abs(Q[i, :, :k, :k].cpu().numpy() - q).max() < 1e-11
        assert float(S[i, k:].abs().sum()) == 0.0 and float(S[i, :, k:].abs().sum()) == 0.0


@pytest.mark.parametrize("method", ["gfn1", "gfn2"])
@pytest.mark.parametrize("name", ["H2O", "SiH4"])
def test_wrapper_gradients_match_oracle_autograd(method, name):
    """The wrappers' backward (the VJP kernel) against autograd through the
    oracle's integrals, for random upstream gradients of S, D and Q."""
    from dxtb_gb300.integrals import dipint, overlap, quadint

    num = torch.tensor(G[f"{name}/numbers"])
    p0 = torch.tensor(G[f"{name}/positions"])
    sysm = X.make_system(method, num.numpy())
    gen = torch.Generator().manual_seed(7)
    for fn, comps, kind in ((overlap, X.COMP_S, 0), (dipint, X.COMP_D, 1), (quadint, X.COMP_Q9, 2)):
        pos = p0.clone().cuda().requires_grad_(True)
        m = fn(num, pos, method)
        up = torch.randn(m.shape, generator=gen, dtype=torch.float64)
        (g_gpu,) = torch.autograd.grad((m * up.cuda()).sum(), pos)
        pc = p0.clone().requires_grad_(True)
        raw = X.multipole_raw(sysm, pc, comps)
        norm = X.snorm(X.multipole_raw(sysm, pc, X.COMP_S)[0])
        ref = raw * (norm[:, None] * norm[None, :])
        if kind == 0:
            ref = ref[0]
        (g_ref,) = torch.autograd.grad((ref * up).sum(), pc)
        assert np.abs(g_gpu.cpu().numpy() - g_ref.numpy()).max() < 1e-10, fn.__name__
