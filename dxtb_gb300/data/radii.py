"""
Element radii and unit constants used by the GFN-xTB single point.

dxtb takes these from its dependency ``tad-mctc`` 0.7.0 (``tad_mctc.data.radii``
and ``tad_mctc.units``), which is not part of the dxtb source tree. The
values below are the published tables those names refer to:

``COV_D3``
    Covalent radii of the DFT-D3 coordination number (Grimme, Antony, Ehrlich,
    Krieg, JCP 132, 154104 (2010)): the single-bond radii of Pyykkö and Atsumi
    (Chem. Eur. J. 15, 186 (2009)), metals reduced by 10 %, in Ångström and
    scaled by 4/3 when converted to Bohr.
``ATOMIC_RADII``
    Atomic radii of the distance polynomial of the GFN-xTB Hamiltonian (the
    ``atomicrad`` table of tblite), in Ångström.
``VDW_D3``
    Atomic van-der-Waals radii of DFT-D3 (used for the Born radii of the
    generalized-Born solvation model), in Ångström. H, B, N, O, F, Na, Al,
    Si and Cl are pinned by the tblite descreening integrals psi of
    MB16_43_01 and SiH4 in dxtb's ``test/test_solvation/samples.py``. A
    least-squares fit of all eight MB16_43_01 radii to its 16 psi values
    returns them at the 5-digit table values, with a relative residual of
    2e-15 (``tests/test_vdw_radii_fit.py``). C and S are the published
    table values; no fixture contains them.

Only elements whose values are either pinned by the dxtb test fixtures
(``test/test_hamiltonian/h0.npz``, computed with tblite 0.3.0) or required
by the H/C/N/O/F/S workload are listed; every other element raises, so a
missing value is never silently replaced.
"""

from __future__ import annotations

import numpy as np

# Bohr radius (CODATA 2018); enters only through the radius tables.
BOHR_ANGSTROM = 0.529177210903
AA2AU = 1.0 / BOHR_ANGSTROM
# Hartree in eV (CODATA 2010) and Boltzmann constant in Hartree/K, the values
# of tblite/mctc-lib. The single-atom SCF energies of the dxtb test suite
# (test/test_scf/test_elements_gfn{1,2}.py, tblite references) reproduce to
# 1e-15 Eh (He, Ne) with these and are off by 4.4e-8 relative with CODATA 2018.
HARTREE_EV = 27.21138505
EV2AU = 1.0 / HARTREE_EV
KELVIN2AU = 3.166808578545117e-06

# Å, indexed by atomic number
_COV_D3_AA = {
    1: 0.32, 2: 0.46, 3: 1.20, 4: 0.94, 5: 0.77, 6: 0.75, 7: 0.71, 8: 0.63,
    9: 0.64, 10: 0.67, 11: 1.40, 12: 1.25, 13: 1.13, 14: 1.04, 15: 1.10,
    16: 1.02, 17: 0.99, 18: 0.96,
}
_ATOMIC_RADII_AA = {
    1: 0.32, 2: 0.37, 3: 1.30, 4: 0.99, 5: 0.84, 6: 0.75, 7: 0.71, 8: 0.64,
    9: 0.60, 10: 0.62, 11: 1.60, 12: 1.40, 13: 1.24, 14: 1.14, 15: 1.09,
    16: 1.04, 17: 1.00, 18: 1.01,
}
_VDW_D3_AA = {
    1: 1.09155, 5: 1.60800, 6: 1.45515, 7: 1.31125, 8: 1.24085, 9: 1.14980,
    11: 1.85410, 13: 2.00530, 14: 1.89585, 16: 1.66330, 17: 1.55230,
}

MAXZ = 86


def _table(values: dict[int, float], scale: float) -> np.ndarray:
    """Dense table over Z = 0..86; NaN marks an element without a value."""
    out = np.full(MAXZ + 1, np.nan)
    for z, v in values.items():
        out[z] = v * scale
    return out


COV_D3 = _table(_COV_D3_AA, 4.0 / 3.0 * AA2AU)
"""D3 covalent radii in Bohr (4/3-scaled)."""
ATOMIC_RADII = _table(_ATOMIC_RADII_AA, AA2AU)
"""GFN-xTB atomic radii in Bohr."""
VDW_D3 = _table(_VDW_D3_AA, AA2AU)
"""D3 van-der-Waals radii in Bohr."""


def lookup(table: np.ndarray, numbers, name: str) -> np.ndarray:
    """Gather radii for ``numbers``; raise for elements without a value."""
    z = np.asarray(numbers, dtype=np.int64)
    vals = table[z]
    bad = np.isnan(vals) & (z > 0)
    if bad.any():
        raise ValueError(
            f"No {name} radius for element(s) {sorted(set(z[bad].tolist()))}"
        )
    return np.where(z > 0, vals, 0.0)
