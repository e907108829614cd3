"""
Oracle energies and gradients for every molecule of the benchmark sets.

    python tests/golden/make_set_fixtures.py [--workers 8] [--only c2|c3]

Writes ``sets_c2.npz`` (GFN2, the 256 molecules of 10-60 atoms) and
``sets_c3.npz`` (GFN1 and GFN2, the 64 molecules of 30-120 atoms). Each file
holds the inputs exactly as computed here (zero-padded ``numbers`` and
``positions``, ``nat``), so that a run on another platform compares the same
geometry bit for bit, and per molecule and method the oracle's

- ``energy`` (Eh), ``gradient`` (dE/dR, Eh/Bohr, zero-padded),
- ``iterations`` (broyden1 iterations taken at tol = 1e-10),
- ``converged`` (False when the oracle stopped at ``maxiter``).

The oracle is the float64 CPU restatement in ``oracle/xtb_oracle.py``
(dispersion and halogen terms excluded on both sides). Workers are started
with ``spawn`` and run one molecule each with one torch thread.
"""

from __future__ import annotations

import argparse
import multiprocessing as mp
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
TOL = 1e-10
MAXITER = 250


def _one(job):
    sys.path.insert(0, str(ROOT))
    import torch

    torch.set_num_threads(1)
    from oracle import xtb_oracle as X

    method, idx, num, pos = job
    t = time.time()
    r = X.singlepoint(method, num, pos, grad=True, tol=TOL, maxiter=MAXITER)
    g = r.extra["gradient"].numpy()
    return method, idx, r.energy, g, r.iterations, time.time() - t


def _pad(mols):
    nmax = max(len(m[0]) for m in mols)
    numbers = np.zeros((len(mols), nmax), np.int64)
    positions = np.zeros((len(mols), nmax, 3))
    for i, (z, p) in enumerate(mols):
        numbers[i, : len(z)] = z
        positions[i, : len(z)] = p
    return numbers, positions, np.array([len(m[0]) for m in mols], np.int64)


def build(config: int, methods: list[str], workers: int) -> None:
    sys.path.insert(0, str(ROOT))
    from dxtb_gb300.workloads import config_molecules

    mols = config_molecules(config)
    numbers, positions, nat = _pad(mols)
    jobs = [(m, i, z, p) for m in methods for i, (z, p) in enumerate(mols)]
    # largest first so that the pool drains evenly
    jobs.sort(key=lambda j: -len(j[2]))
    out = {
        m: dict(
            energy=np.zeros(len(mols)),
            gradient=np.zeros_like(positions),
            iterations=np.zeros(len(mols), np.int64),
            seconds=np.zeros(len(mols)),
        )
        for m in methods
    }
    t0 = time.time()
    with mp.get_context("spawn").Pool(workers) as pool:
        for k, (m, i, e, g, it, sec) in enumerate(pool.imap_unordered(_one, jobs)):
            o = out[m]
            o["energy"][i] = e
            o["gradient"][i, : len(g)] = g
            o["iterations"][i] = it
            o["seconds"][i] = sec
            if (k + 1) % 16 == 0:
                print(f"c{config}: {k + 1}/{len(jobs)} in {time.time() - t0:.0f} s", flush=True)
    arrays = {"numbers": numbers, "positions": positions, "nat": nat, "tol": np.array(TOL),
              "maxiter": np.array(MAXITER)}
    for m, o in out.items():
        for k, v in o.items():
            arrays[f"{m}/{k}"] = v
        arrays[f"{m}/converged"] = o["iterations"] < MAXITER
    np.savez_compressed(HERE / f"sets_c{config}.npz", **arrays)
    print(f"wrote sets_c{config}.npz ({time.time() - t0:.0f} s)")


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--workers", type=int, default=mp.cpu_count())
    ap.add_argument("--only", choices=["c2", "c3"])
    a = ap.parse_args()
    if a.only in (None, "c2"):
        build(2, ["gfn2"], a.workers)
    if a.only in (None, "c3"):
        build(3, ["gfn1", "gfn2"], a.workers)


if __name__ == "__main__":
    main()
