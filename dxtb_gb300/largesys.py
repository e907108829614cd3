"""
Large single systems: GFN2-xTB + generalized-Born solvation (epsilon 78.4),
energy and forces, on the eight seeded synthetic molecules of 1000-2000
atoms (n = 2600-5200 orbitals). Each molecule's SCF runs on a 16-CTA
thread-block cluster; the eight run concurrently.

The solvation model is plain GB (``alpb=False``) with the Still kernel
(``GeneralizedBorn(..., kernel="still", alpb=False)``). On these dense
random-walk blobs the OBC integral saturates: tanh(...) rounds to 1 for
buried atoms, and their Born radii become infinite. The reference's P16
kernel then evaluates inf/inf = NaN. The Still kernel has the finite limit
0 for such pairs (see ``oracle/solvation_oracle.py`` for the same
expressions).

    python -m dxtb_gb300.largesys [--maxiter K] [--count N]
    python -m dxtb_gb300.largesys --atoms 310 --seed 9410 --method gfn1 --vacuum --maxiter 3

Prints one JSON line with the wall time, the SCF time per iteration,
iterations and residuals per molecule. With ``--atoms`` it runs one seeded
random-walk molecule of that many atoms instead (the profiling case of a
single large molecule on a 16-CTA cluster).
"""

from __future__ import annotations

import argparse
import json
import time

import numpy as np
import torch


def main(argv=None) -> None:
    from .calculators import tables
    from .engine import PackedBatch, run
    from .workloads import config_molecules

    p = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    p.add_argument("--maxiter", type=int, default=250)
    p.add_argument("--count", type=int, default=8)
    p.add_argument("--kernel", default="still", choices=["still", "p16"])
    p.add_argument("--atoms", type=int, default=0, help="one molecule of this many atoms")
    p.add_argument("--seed", type=int, default=0)
    p.add_argument("--method", default="gfn2", choices=["gfn1", "gfn2"])
    p.add_argument("--vacuum", action="store_true", help="no solvation")
    p.add_argument("--no-forces", action="store_true")
    a = p.parse_args(argv)
    t0 = time.time()
    if a.atoms > 0:
        from .workloads import random_molecule

        mols = [random_molecule(a.seed, a.atoms)]
    else:
        mols = config_molecules(5, count=a.count)
    t_gen = time.time() - t0
    gb = None if a.vacuum else {"epsilon": 78.4, "alpb": False, "kernel": a.kernel}
    pb = PackedBatch(tables(a.method), [m[0] for m in mols], [torch.tensor(m[1]) for m in mols])
    torch.cuda.synchronize()
    ev: dict = {}
    t = time.time()
    res = run(pb, forces=not a.no_forces, gb=gb, maxiter=a.maxiter, events=ev)
    torch.cuda.synchronize()
    wall = time.time() - t
    e4 = res.state["energies"][: 4 * pb.nmol].view(-1, 4).cpu().numpy()
    its = e4[:, 2]
    stages = {k: v[0].elapsed_time(v[1]) / 1e3 for k, v in ev.items()}
    g = res.gradient.cpu().numpy() if res.gradient is not None else np.zeros(1)
    out = {
        "workload": (f"{a.method.upper()} {'vacuum' if gb is None else 'GB'} "
                     f"{'E' if a.no_forces else 'E+F'}, one molecule of {a.atoms} atoms (seed {a.seed})"
                     if a.atoms > 0 else
                     "GFN2 + GB (Still, eps 78.4) E+F, synthetic 1000-2000-atom molecules"),
        "molecules": pb.nmol,
        "atoms": [int(v) for v in pb.nat],
        "nao": [int(v) for v in pb.nao],
        "maxiter": a.maxiter,
        "wall_s": wall,
        "stages_s": stages,
        "iterations": [int(v) for v in its],
        "status": [int(v) for v in res.status.cpu()],
        "residual": [float(v) for v in e4[:, 3]],
        "scf_s_per_iteration_max_molecule": stages["scf"] / max(1.0, float(its.max())),
        "energy": [float(v) for v in res.energy.cpu()],
        "forces_finite": bool(np.isfinite(g).all()),
        "generation_s": t_gen,
        "molecules_per_s": pb.nmol / wall,
    }
    print(json.dumps(out))


if __name__ == "__main__":
    main()
