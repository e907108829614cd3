"""
Nuclear Hessian of GFN-xTB single points as ONE packed batch.

The reference builds the Hessian by differentiating its autograd forces
again (calculators/types/autograd.py:198-329, ``hessian``: row by row with
``torch.autograd.grad`` or with ``torch.func.jacrev``), which replays the
backward graph of the SCF once per coordinate. Here the 6 nat geometries
displaced by +-h along every Cartesian coordinate are independent single
points, so they go through the batched GPU path together: one packed batch,
one launch per stage, analytic gradients from the adjoint kernels, and

    H[a, x, b, y] = (g[b, y](R + h e_ax) - g[b, y](R - h e_ax)) / (2 h),

symmetrised. With h = 1e-3 Bohr the central-difference error is O(h^2)
(~1e-7 Eh/Bohr^2) and the SCF noise at x_atol = f_atol = 1e-10 is ~1e-10 / h.
"""

from __future__ import annotations

import numpy as np
import torch

from . import engine


def hessian(tables, numbers, positions, *, h: float = 1e-3, chrg: float = 0.0, spin=None,
            etemp: float = 300.0, tol: float = 1e-10, maxiter: int = 250,
            matrix: bool = False, device=None, dipole_derivative: bool = False):
    """
    Hessian (nat, 3, nat, 3) (or (3 nat, 3 nat) with ``matrix``) of one
    molecule in Eh/Bohr^2, float64, on the GPU. ``numbers`` (nat,) and
    ``positions`` (nat, 3) in Bohr; ``tables`` is the method's parameter set
    (``calculators.tables("gfn1" | "gfn2")``). Raises RuntimeError if any
    displaced single point fails or does not converge.

    With ``dipole_derivative`` it returns ``(hessian, dmu_dr)``: the nuclear
    derivative of the dipole moment, (3, nat, 3) in e (the reference's
    ``dipole_deriv``, calculators/types/autograd.py:547-627), as central
    differences of the dipole moments of the same displaced single points
    (``dxtb_dipole_moment``, one launch for all of them).
    """
    z = np.asarray(numbers.cpu() if torch.is_tensor(numbers) else numbers, dtype=np.int64).ravel()
    z = z[z > 0]
    p0 = torch.as_tensor(positions, dtype=torch.float64).detach().reshape(-1, 3)[: len(z)].cpu()
    nat = len(z)
    disp = []
    for a in range(nat):
        for x in range(3):
            for sgn in (1.0, -1.0):
                q = p0.clone()
                q[a, x] += sgn * h
                disp.append(q)
    nd = len(disp)
    pb = engine.PackedBatch(tables, [z] * nd, disp, device, [chrg] * nd,
                            None if spin is None else [spin] * nd)
    res = engine.run(pb, etemp=etemp, maxiter=maxiter, tol=tol, forces=True,
                     scf={"mixer": "broyden1"})
    st = res.status.cpu()
    if (st != 0).any():
        from ._lib import STATUS

        raise RuntimeError(f"Hessian: displaced single points failed: "
                           f"{sorted({STATUS.get(int(c), int(c)) for c in st[st != 0]})}")
    g = res.gradient.view(nd, nat * 3)  # packed: every molecule has nat atoms
    hmat = (g[0::2] - g[1::2]) / (2.0 * h)  # row (a, x): d g / d R_ax
    hmat = 0.5 * (hmat + hmat.T)
    hout = hmat if matrix else hmat.view(nat, 3, nat, 3)
    if not dipole_derivative:
        return hout
    from .properties import dipole_moments

    mu = dipole_moments(pb, res.state["P"])  # (nd, 3)
    dmu = ((mu[0::2] - mu[1::2]) / (2.0 * h)).T  # (3, 3 nat): d mu_x / d R_(a,y)
    return hout, dmu.reshape(3, nat, 3)
