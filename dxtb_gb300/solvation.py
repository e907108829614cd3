"""
Generalized-Born / ALPB implicit solvation with the constructor of dxtb's
``GeneralizedBorn`` (``components/interactions/solvation/alpb.py:213-245``).

The object holds the model parameters. The Born radii, the interaction
matrix and the gradient come from the CUDA library (``dxtb_born_matrix``,
``dxtb_born_gradient``) when a calculator runs with
``interaction=[GeneralizedBorn(...)]``.
"""

from __future__ import annotations

import torch

from .data import radii

DEFAULT_KERNEL = "p16"
DEFAULT_ALPB = True


class GeneralizedBorn:
    """Solvation by a dielectric continuum (ALPB by default, GB with ``alpb=False``)."""

    def __init__(self, numbers, dielectric_constant, alpb: bool = DEFAULT_ALPB,
                 kernel: str = DEFAULT_KERNEL, born_scale: float = 1.0, born_offset: float = 0.0,
                 device=None, dtype=None, **kwargs):
        if kwargs.get("rvdw") is not None:
            raise NotImplementedError("custom van-der-Waals radii: the D3 table is used")
        if kernel not in ("p16", "still"):
            raise ValueError(f"unknown Born kernel {kernel!r}")
        eps = float(dielectric_constant.item() if torch.is_tensor(dielectric_constant)
                    else dielectric_constant)
        if not eps > 0.0:
            raise ValueError("dielectric constant must be positive")
        z = numbers.detach().cpu().numpy() if torch.is_tensor(numbers) else numbers
        radii.lookup(radii.VDW_D3, z, "van-der-Waals")  # raises for elements without a radius
        self.epsilon = eps
        self.alpb = bool(alpb)
        self.kernel = kernel
        self.born_scale = float(born_scale)
        self.born_offset = float(born_offset)

    def as_dict(self) -> dict:
        return {"epsilon": self.epsilon, "alpb": self.alpb, "kernel": self.kernel,
                "born_scale": self.born_scale, "born_offset": self.born_offset}
