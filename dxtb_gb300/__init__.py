"""
dxtb_gb300: GFN1/GFN2-xTB single points on one NVIDIA GB300 (sm_103a).

A drop-in for dxtb's single-point hot path: calculators with the reference's
``get_energy``/``get_forces`` interface, the integral wrappers
(overlap/dipole/quadrupole) and the IndexHelper maps, all computed by
hand-written float64 CUDA kernels behind a C ABI (include/dxtb_gb300.h).
"""

from .calculators import Calculator, GFN1Calculator, GFN2Calculator  # noqa: F401

__all__ = ["Calculator", "GFN1Calculator", "GFN2Calculator"]
