"""
Atomic masses and the spectroscopic unit constants of the vibrational
analysis.

dxtb takes them from its dependency ``tad-mctc`` 0.7.0
(``tad_mctc.data.mass.ATOMIC_MASS``, ``tad_mctc.units``), which is not part
of the dxtb source tree. The values below are the published sources those
names refer to:

``ATOMIC_MASS``
    Standard atomic weights of IUPAC (conventional values of the 2013/2015
    table), in unified atomic mass units, converted to electron masses. The
    masses enter the harmonic frequencies as 1/sqrt(m); the dxtb frequency
    fixtures (``test/test_properties/samples.py``: H2, LiH, H2O, CH4, SiH4,
    GFN1) are reproduced within their stated tolerance (10 cm^-1 absolute,
    1e-3 relative) with these values.
``AMU2AU``
    m_u / m_e (CODATA 2018).
``AU2RCM``
    Hartree in wavenumbers, E_h / (h c) in cm^-1 (CODATA 2018).
``AU2KMMOL``
    IR intensity of one atomic unit, (e^2 / m_e) per squared normal
    coordinate, in km/mol: N_A pi e^2 / (3 c^2 4 pi eps0 m_e) / 1000
    (CODATA 2018 constants).
"""

from __future__ import annotations

import math

import numpy as np

AMU2AU = 1822.888486209
AU2RCM = 219474.6313632

# CODATA 2018
_NA = 6.02214076e23
_C = 299792458.0
_E = 1.602176634e-19
_ME = 9.1093837015e-31
_EPS0 = 8.8541878128e-12
AU2KMMOL = _NA * math.pi * _E**2 / (3.0 * _C**2 * 4.0 * math.pi * _EPS0 * _ME) / 1000.0

# u, indexed by atomic number (H-Ar: the elements this path accepts)
_MASS_U = {
    1: 1.008, 2: 4.002602, 3: 6.94, 4: 9.0121831, 5: 10.81, 6: 12.011, 7: 14.007,
    8: 15.999, 9: 18.998403163, 10: 20.1797, 11: 22.98976928, 12: 24.305,
    13: 26.9815385, 14: 28.085, 15: 30.973761998, 16: 32.06, 17: 35.45, 18: 39.948,
}


def atomic_mass(numbers) -> np.ndarray:
    """Masses (electron masses) of the given atomic numbers; raises for an
    element without a listed mass."""
    z = np.asarray(numbers, dtype=np.int64).ravel()
    missing = sorted({int(v) for v in z if int(v) not in _MASS_U})
    if missing:
        raise ValueError(f"no atomic mass for elements {missing}")
    return np.array([_MASS_U[int(v)] * AMU2AU for v in z], dtype=np.float64)
