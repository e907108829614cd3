"""
Seeded synthetic molecules for the benchmark configurations.

Heavy atoms are grown by a random walk (bond lengths uniform in
[2.6, 2.9] Bohr from a uniformly chosen existing heavy atom, uniform random
direction), each H sits 2.05 Bohr from a random heavy atom, and any placement
with a pair closer than 2.0 Bohr is rejected and redrawn. Elements
H/C/N/O/F/S are drawn with weights 0.50/0.30/0.08/0.08/0.02/0.02 and the H
count is adjusted by one so that the valence electron count is even
(neutral closed shell). Seeds are ``1000 * config + index``.
"""

from __future__ import annotations

import numpy as np

ELEMENTS = np.array([1, 6, 7, 8, 9, 16])
WEIGHTS = np.array([0.50, 0.30, 0.08, 0.08, 0.02, 0.02])
VALENCE = {1: 1, 6: 4, 7: 5, 8: 6, 9: 7, 16: 6}


def _unit(rng) -> np.ndarray:
    v = rng.normal(size=3)
    return v / np.linalg.norm(v)


def build_geometry(rng, heavy: list[int], nh: int) -> tuple[np.ndarray, np.ndarray]:
    """Place the heavy atoms by the random walk, then the hydrogens; the
    distance test against all placed atoms is one vectorised pass."""
    arr = np.empty((len(heavy) + nh, 3))
    k = 0
    for i, _ in enumerate(heavy):
        if i == 0:
            arr[0] = 0.0
            k = 1
            continue
        for _try in range(100000):
            anchor = arr[rng.integers(k)]
            p = anchor + rng.uniform(2.6, 2.9) * _unit(rng)
            dd = p - arr[:k]
            if np.sqrt(np.einsum("ij,ij->i", dd, dd)).min() >= 2.0:
                arr[k] = p
                k += 1
                break
        else:
            raise RuntimeError("could not place heavy atom")
    nheavy = k
    for _ in range(nh):
        for _try in range(100000):
            anchor = arr[rng.integers(nheavy)]
            p = anchor + 2.05 * _unit(rng)
            dd = p - arr[:k]
            if np.sqrt(np.einsum("ij,ij->i", dd, dd)).min() >= 2.0:
                arr[k] = p
                k += 1
                break
        else:
            raise RuntimeError("could not place hydrogen")
    numbers = np.array(list(heavy) + [1] * nh, dtype=np.int64)
    return numbers, arr[:k].copy()


def random_molecule(seed: int, nat: int) -> tuple[np.ndarray, np.ndarray]:
    """
    Neutral closed-shell molecule with ``nat`` (+-1) atoms of the mix. A draw
    whose hydrogens cannot all be placed (e.g. one heavy atom with eleven H)
    is redrawn with seed ``seed + 10_000_000 * k``, k = 1, 2, ...; every
    molecule that places at its own seed is unaffected by this rule.
    """
    for k in range(16):
        try:
            return _draw(seed + 10_000_000 * k, nat)
        except RuntimeError:
            continue
    raise RuntimeError(f"no placeable molecule of {nat} atoms from seed {seed}")


def _draw(seed: int, nat: int) -> tuple[np.ndarray, np.ndarray]:
    rng = np.random.default_rng(seed)
    z = rng.choice(ELEMENTS, size=nat, p=WEIGHTS)
    heavy = [int(v) for v in z if v != 1]
    if not heavy:
        heavy = [6]
    nh = nat - len(heavy)
    nel = sum(VALENCE[v] for v in heavy) + nh
    if nel % 2:
        nh = nh + 1 if nh == 0 or rng.random() < 0.5 else nh - 1
    return build_geometry(rng, heavy, max(nh, 0))


def fixed_composition(seed: int, counts: dict[int, int]) -> tuple[np.ndarray, np.ndarray]:
    """Molecule of a given composition, e.g. C8N2O2H12 = {6: 8, 7: 2, 8: 2, 1: 12}."""
    rng = np.random.default_rng(seed)
    heavy = [z for z, c in sorted(counts.items()) if z != 1 for _ in range(c)]
    rng.shuffle(heavy)
    return build_geometry(rng, [int(v) for v in heavy], counts.get(1, 0))


def config_molecules(config: int, count: int | None = None):
    """The molecule set of a benchmark configuration (1-5)."""
    if config == 1:
        return [fixed_composition(1000, {6: 8, 7: 2, 8: 2, 1: 12})]
    spec = {2: (256, 10, 60), 3: (64, 30, 120), 5: (8, 1000, 2000)}
    if config == 4:
        n = count or 200
        rng = np.random.default_rng(4000)
        sizes = np.exp(rng.uniform(np.log(8), np.log(300), size=n)).astype(int)
        return [random_molecule(4000 + i, int(s)) for i, s in enumerate(sizes)]
    n, lo, hi = spec[config]
    n = count or n
    rng = np.random.default_rng(1000 * config)
    sizes = rng.integers(lo, hi + 1, size=n)
    return [random_molecule(1000 * config + i, int(s)) for i, s in enumerate(sizes)]
