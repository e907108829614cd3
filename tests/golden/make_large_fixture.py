"""
Oracle fixture of one large molecule for the GPU parity test above n = 1000:
GFN2 + generalized Born (Still kernel, epsilon = 78.4, the solvation of the
large-system configuration) on the seeded random-walk molecule of 401 atoms
(seed 5100), and the same molecule in vacuum: energies, SCF to 1e-10. (The
oracle's gradient assembles the integrals pair by pair under autograd,
hours at this size; the GPU test checks the forces against central
differences of the GPU energy instead.)

    python tests/golden/make_large_fixture.py

Writes ``large_gb.npz`` (numbers, positions, energies, iterations).
"""

from __future__ import annotations

import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))

SEED, NAT = 5100, 400
SOLVATION = {"epsilon": 78.4, "alpb": False, "kernel": "still"}


def main() -> None:
    from dxtb_gb300.workloads import random_molecule
    from oracle import xtb_oracle as X

    z, p = random_molecule(SEED, NAT)
    t = time.time()
    r = X.singlepoint("gfn2", z, p, tol=1e-10, maxiter=250, solvation=SOLVATION)
    v = X.singlepoint("gfn2", z, p, tol=1e-10, maxiter=250)
    np.savez_compressed(
        HERE / "large_gb.npz", numbers=z, positions=p, energy=np.array(r.energy),
        iterations=np.array(r.iterations), converged=np.array(r.extra["converged"]),
        energy_vacuum=np.array(v.energy), iterations_vacuum=np.array(v.iterations),
        converged_vacuum=np.array(v.extra["converged"]), seed=np.array(SEED), nat_request=np.array(NAT),
    )
    print(f"{len(z)} atoms: GB {r.iterations} iterations, E = {r.energy:.10f}; vacuum {v.iterations} "
          f"iterations, E = {v.energy:.10f} ({time.time() - t:.0f} s)")


if __name__ == "__main__":
    main()
