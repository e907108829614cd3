"""
IndexHelper maps: the oracle restatement against the reference's own golden
vectors (test/test_indexhelper/test_spread_reduce.py:34-90), and the GPU
kernel bit-exact against the oracle for single molecules and padded batches.
"""

import numpy as np
import pytest
import torch

from oracle import xtb_oracle as X

ANG = {1: [0, 0], 6: [0, 1], 14: [0, 1, 2]}


def test_oracle_maps_reference_golden_ch4():
    # test_spread_reduce.py:34-62: C H4 with H = [s, s], C = [s, p]
    ih = X.index_helper(np.array([6, 1, 1, 1, 1]), ANG)
    assert ih["unique_angular"].tolist() == [0, 0, 0, 1]
    assert ih["shells_to_atom"].tolist() == [0, 0, 1, 1, 2, 2, 3, 3, 4, 4]
    # spread_ushell_to_shell(unique_angular) golden vector
    assert ih["unique_angular"][ih["shells_to_ushell"]].tolist() == [0, 1, 0, 0, 0, 0, 0, 0, 0, 0]
    # spread_ushell_to_orbital(unique_angular) golden vector
    orb = ih["unique_angular"][ih["shells_to_ushell"]][ih["orbitals_to_shell"]]
    assert orb.tolist() == [0, 1, 1, 1, 0, 0, 0, 0, 0, 0, 0, 0]


def test_oracle_maps_reference_golden_sih2():
    # test_spread_reduce.py:65-90 (spherical part): Si H2
    ih = X.index_helper(np.array([14, 1, 1]), ANG)
    assert ih["orbitals_per_shell"].tolist() == [1, 3, 5, 1, 1, 1, 1]
    assert ih["orbital_index"].tolist() == [0, 1, 4, 9, 10, 11, 12]
    orb_atom = ih["shells_to_atom"][ih["orbitals_to_shell"]]
    assert orb_atom.tolist() == [0] * 9 + [1, 1, 2, 2]


def test_oracle_batch_padding_conventions():
    ih = X.index_helper(np.array([[6, 1, 1, 0], [1, 1, 0, 0]]), ANG)
    assert ih["shells_to_ushell"][1].tolist()[-1] == -1
    assert ih["shell_index"][1].tolist() == [0, 2, -999, -999]
    assert (ih["orbitals_to_shell"][1] == -999).sum() > 0


KEYS = ["unique_angular", "angular", "atom_to_unique", "ushells_to_unique", "ushells_per_unique",
        "shells_to_ushell", "shells_per_atom", "shell_index", "shells_to_atom",
        "orbitals_per_shell", "orbital_index", "orbitals_to_shell"]


@pytest.mark.gpu
@pytest.mark.parametrize("numbers", [
    [6, 1, 1, 1, 1],
    [14, 1, 1],
    [8, 1, 1, 16, 9, 7, 6, 6, 1],
    [[6, 1, 1, 0], [1, 1, 0, 0]],
    [[8, 1, 1, 0, 0], [16, 6, 1, 1, 9], [1, 1, 0, 0, 0]],
])
@pytest.mark.parametrize("method", ["gfn1", "gfn2"])
def test_gpu_maps_bit_exact(numbers, method):
    from dxtb_gb300.indexhelper import IndexHelper
    from dxtb_gb300.params import load_par

    ang = {z: e["angular"] for z, e in load_par(method)["element"].items()}
    num = np.array(numbers)
    ref = X.index_helper(num, ang)
    ih = IndexHelper.from_numbers_angular(torch.tensor(num, device="cuda"), ang)
    for k in KEYS:
        got = getattr(ih, k).cpu().numpy()
        assert got.shape == ref[k].shape, k
        assert np.array_equal(got, ref[k]), k


@pytest.mark.gpu
def test_gpu_spread_reduce():
    from dxtb_gb300.indexhelper import IndexHelper

    ih = IndexHelper.from_numbers_angular(torch.tensor([6, 1, 1, 1, 1], device="cuda"), ANG)
    atom = torch.tensor([6, 1, 1, 1, 1], device="cuda")
    assert ih.spread_atom_to_shell(atom).tolist() == [6, 6, 1, 1, 1, 1, 1, 1, 1, 1]
    assert ih.spread_atom_to_orbital(atom).tolist() == [6, 6, 6, 6] + [1] * 8
    assert ih.spread_uspecies_to_atom(torch.tensor([1, 6], device="cuda")).tolist() == atom.tolist()
    x = torch.arange(12, dtype=torch.float64, device="cuda")
    assert ih.reduce_orbital_to_atom(x).tolist() == [6.0, 9.0, 13.0, 17.0, 21.0]
