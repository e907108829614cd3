"""
dxtb_scf_noalloc: the SCF entry point for callers that must not allocate
device memory (hosts that give the library a fixed pool and forbid other
allocations, plugin hosts whose allocator the C ABI cannot reach). Called
through the C ABI, its results must equal those of dxtb_scf on the same
inputs, on two calls in a row (the shared scratch array keeps the first
call's contents when the second starts). The batch holds small molecules
and one of at least 136 orbitals, so the one-SM or cluster classes, which
run on side streams forked from the caller's stream, read the scratch
header too.

This file is collected last so that a failure here never hides another test.
"""

import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

E_TOL = 1e-8  # Eh, as in the other parity tests


def test_noalloc_scf_matches_allocating_entry_point():
    from dxtb_gb300 import _lib
    from dxtb_gb300.calculators import tables
    from dxtb_gb300.data import radii
    from dxtb_gb300.engine import PackedBatch, run
    from dxtb_gb300.workloads import random_molecule

    mols = [random_molecule(5000 + i, n) for i, n in enumerate([9, 17, 26, 58])]
    pb = PackedBatch(tables("gfn2"), [m[0] for m in mols], [torch.tensor(m[1]) for m in mols])
    L = _lib.lib()
    thr = (C.c_int32 * 5)()
    assert L.dxtb_scf_get_size_classes(thr) == 0
    assert int(pb.nao.max()) >= thr[1]  # a one-SM or cluster class is in the batch
    ref = run(pb, forces=True)
    s = ref.state
    assert (ref.status.cpu() == 0).all()
    tot = pb.total
    nm, no, na = tot["mat"], tot["aos"], tot["atoms"]
    dev = pb.device
    kt = 300.0 * radii.KELVIN2AU
    for call in range(2):
        out = {k: torch.full((n,), float("nan"), dtype=torch.float64, device=dev) for k, n in
               [("P", nm), ("W", nm), ("C", nm), ("ev", no), ("occ", no), ("q", no),
                ("dp", 3 * na), ("qp", 6 * na), ("vorb", no), ("vdp", 3 * na), ("vqp", 6 * na),
                ("en", 4 * pb.nmol)]}
        status = torch.full((pb.nmol,), -1, dtype=torch.int32, device=dev)
        rc = L.dxtb_scf_noalloc(
            C.byref(pb.struct), pb.t["par_f"].data_ptr(), pb.t["par_i"].data_ptr(),
            s["S"].data_ptr(), s["H"].data_ptr(), s["D"].data_ptr(), s["Q"].data_ptr(),
            s["gamma"].data_ptr(), s["hd"].data_ptr(), s["sd"].data_ptr(), s["dd"].data_ptr(),
            s["sq"].data_ptr(), None, pb.t["n0"].data_ptr(), pb.t["nel"].data_ptr(), kt, 250,
            1e-10, pb.t["order"].data_ptr(), out["P"].data_ptr(), out["W"].data_ptr(),
            out["C"].data_ptr(), out["ev"].data_ptr(), out["occ"].data_ptr(), out["q"].data_ptr(),
            out["dp"].data_ptr(), out["qp"].data_ptr(), out["vorb"].data_ptr(),
            out["vdp"].data_ptr(), out["vqp"].data_ptr(), out["en"].data_ptr(),
            status.data_ptr(), _lib.stream_ptr())
        torch.cuda.synchronize()
        assert rc == 0
        assert (status.cpu() == 0).all()
        e_ref = s["energies"][: 4 * pb.nmol].view(-1, 4)[:, :2].sum(1)
        e_new = out["en"].view(-1, 4)[:, :2].sum(1)
        assert (e_new - e_ref).abs().max().item() < E_TOL
        assert (out["P"] - s["P"][:nm]).abs().max().item() < 1e-8
        assert (out["q"] - s["q"][:no]).abs().max().item() < 1e-8


def test_noalloc_rejects_oversized_batch():
    """A workspace beyond the fixed scratch array is refused, nothing runs."""
    from dxtb_gb300 import _lib
    from dxtb_gb300.calculators import tables
    from dxtb_gb300.engine import PackedBatch
    from dxtb_gb300.workloads import random_molecule

    # 3 n^2 doubles alone exceed 2^21 for n > 836 AOs
    num, pos = random_molecule(6000, 420)
    pb = PackedBatch(tables("gfn2"), [num], [torch.tensor(pos)])
    assert int(pb.nao[0]) > 836
    L = _lib.lib()
    dummy = torch.zeros(1, dtype=torch.float64, device=pb.device)
    p = dummy.data_ptr()
    rc = L.dxtb_scf_noalloc(C.byref(pb.struct), pb.t["par_f"].data_ptr(), pb.t["par_i"].data_ptr(),
                            p, p, p, p, p, p, p, p, p, None, p, p, 1e-3, 10, 1e-8, None,
                            p, p, p, p, p, p, p, p, p, p, p, p, p, _lib.stream_ptr())
    assert rc == 7  # DXTB_ERR_TOO_LARGE
