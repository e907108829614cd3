"""
Oracle fixtures of six molecules of the seeded serving request stream
(200 requests, Poisson, seed 4: requests 136, 96, 48 and 166 in GFN1, 179
and 0 in GFN2, n = 486-796 orbitals) whose SCF passes through tight
two-member eigenvalue clusters (136, 96, 48, 179) or needs eigenvectors of
eigenvalues with small gaps to more than the Newton root's accuracy (0,
166), energy and gradient, SCF to 1e-10.

    python tests/golden/make_serving_fixture.py

Writes ``serving_degenerate.npz``.
"""

from __future__ import annotations

import multiprocessing as mp
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
RIDS = (136, 96, 48, 179, 0, 166)


def _one(rid):
    sys.path.insert(0, str(ROOT))
    import torch

    torch.set_num_threads(2)
    from dxtb_gb300.serving import poisson_requests
    from oracle import xtb_oracle as X

    rq = poisson_requests(200, 2000.0, 4)[rid]
    t = time.time()
    r = X.singlepoint(rq.method, rq.numbers, rq.positions, tol=1e-10, maxiter=250, grad=True)
    return rid, rq.method, rq.numbers, rq.positions, r.energy, r.extra["gradient"].numpy(), \
        r.iterations, r.extra["converged"], time.time() - t


def main() -> None:
    out = {}
    with mp.get_context("spawn").Pool(len(RIDS)) as pool:
        for rid, method, z, p, e, g, it, conv, sec in pool.imap_unordered(_one, RIDS):
            print(f"request {rid} ({method}, {len(z)} atoms): {it} iterations, converged {conv}, "
                  f"E = {e:.10f} ({sec:.0f} s)", flush=True)
            out.update({f"{rid}/method": np.array(method), f"{rid}/numbers": z, f"{rid}/positions": p,
                        f"{rid}/energy": np.array(e), f"{rid}/gradient": g, f"{rid}/iterations": np.array(it),
                        f"{rid}/converged": np.array(conv)})
    out["rids"] = np.array(RIDS)
    np.savez_compressed(HERE / "serving_degenerate.npz", **out)


if __name__ == "__main__":
    main()
