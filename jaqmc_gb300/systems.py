"""Molecular systems, Hund's-rule spins and walker initialisation (host side).

* ``unpaired_electrons`` / ``atom_spin_config`` restate the main-group rule of
  ``src/jaqmc/utils/atomic/elements.py:33-60`` and ``atom.py:68-80``.
* ``init_walkers`` restates ``initialize_electrons_gaussian``
  (``src/jaqmc/utils/atomic/initialization.py:124-163``): electrons are placed
  on their assigned nucleus — all spin-up electrons atom by atom, then all
  spin-down electrons — plus ``width * N(0, 1)`` per coordinate.
* ``balance_spins`` plays the role of ``distribute_spins`` (``:38-121``) but
  moves electrons between spin channels round-robin instead of at random, so
  that a system's assignment is deterministic.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

SYMBOLS = ["X", "H", "He", "Li", "Be", "B", "C", "N", "O", "F", "Ne",
           "Na", "Mg", "Al", "Si", "P", "S", "Cl", "Ar"]
# main-group column of each element up to Ar (element table of the reference)
_GROUP = [0, 1, 18, 1, 2, 13, 14, 15, 16, 17, 18, 1, 2, 13, 14, 15, 16, 17, 18]
_UNPAIRED_BY_GROUP = {1: 1, 2: 0, 13: 1, 14: 2, 15: 3, 16: 2, 17: 1, 18: 0}


def unpaired_electrons(z: int) -> int:
    if not 1 <= z < len(_GROUP):
        raise ValueError(f"element Z={z} is outside the supported main-group range 1..18")
    return _UNPAIRED_BY_GROUP[_GROUP[z]]


def atom_spin_config(z: int) -> tuple[int, int]:
    u = unpaired_electrons(z)
    return (z + u) // 2, (z - u) // 2


@dataclass
class Molecule:
    """Nuclear positions (bohr), charges and the electron spin split."""

    name: str
    atoms: np.ndarray            # (A, 3) float
    charges: np.ndarray          # (A,) float
    nspins: tuple[int, int]
    per_atom_spins: list = field(default_factory=list)

    @property
    def n_electrons(self) -> int:
        return sum(self.nspins)

    @property
    def n_atoms(self) -> int:
        return int(self.atoms.shape[0])


def balance_spins(zs, nspins) -> list[tuple[int, int]]:
    """Per-atom ``(n_up, n_down)`` starting from each atom's Hund configuration,
    moving electrons between channels round-robin until the totals match."""
    per = [list(atom_spin_config(z)) for z in zs]
    if sum(map(sum, per)) != sum(nspins):
        raise ValueError("electron count does not match the nuclear charges")
    cur = sum(p[0] for p in per)
    k = 0
    while cur != nspins[0]:
        up = nspins[0] > cur
        for _ in range(len(per)):
            i = k % len(per)
            k += 1
            if per[i][1 if up else 0] > 0:
                per[i][0] += 1 if up else -1
                per[i][1] += -1 if up else 1
                cur += 1 if up else -1
                break
        else:  # pragma: no cover - impossible for neutral systems
            raise ValueError("cannot balance spins")
    return [tuple(p) for p in per]


def make_molecule(name, zs, coords, nspins=None) -> Molecule:
    zs = list(zs)
    coords = np.asarray(coords, dtype=np.float64).reshape(len(zs), 3)
    if nspins is None:
        tot = sum(zs)
        nu = sum(atom_spin_config(z)[0] for z in zs)
        nspins = (nu, tot - nu)
    nspins = tuple(int(v) for v in nspins)
    return Molecule(name, coords, np.asarray(zs, dtype=np.float64), nspins,
                    balance_spins(zs, nspins))


def atom(z: int) -> Molecule:
    return make_molecule(SYMBOLS[z], [z], [[0.0, 0.0, 0.0]])


def lithium() -> Molecule:
    return make_molecule("Li", [3], [[0.0, 0.0, 0.0]], (2, 1))


def nitrogen_dimer() -> Molecule:
    return make_molecule("N2", [7, 7], [[0, 0, -1.034], [0, 0, 1.034]], (7, 7))


def methane() -> Molecule:
    d = 1.186
    h = [[d, d, d], [d, -d, -d], [-d, d, -d], [-d, -d, d]]
    return make_molecule("CH4", [6, 1, 1, 1, 1], [[0, 0, 0]] + h, (5, 5))


def benzene() -> Molecule:
    coords, zs = [], []
    for r, z in ((2.640, 6), (4.690, 1)):
        for k in range(6):
            a = k * math.pi / 3.0
            coords.append([r * math.cos(a), r * math.sin(a), 0.0])
            zs.append(z)
    return make_molecule("C6H6", zs, coords, (21, 21))


def hydrogen() -> Molecule:
    return make_molecule("H", [1], [[0.0, 0.0, 0.0]], (1, 0))


SYSTEMS = {"Li": lithium, "N2": nitrogen_dimer, "CH4": methane, "C6H6": benzene, "H": hydrogen}


def electron_centres(mol: Molecule) -> np.ndarray:
    """Starting nucleus of every electron, spin-up electrons first."""
    rows = []
    for s in range(2):
        for j, sp in enumerate(mol.per_atom_spins):
            rows += [mol.atoms[j]] * sp[s]
    return np.asarray(rows, dtype=np.float64).reshape(-1, 3)


def init_walkers(mol: Molecule, batch: int, seed: int = 1, width: float = 1.0) -> np.ndarray:
    """``(batch, n, 3)`` float32 walkers: assigned nucleus + ``width * N(0,1)``."""
    rng = np.random.default_rng(seed)
    c = electron_centres(mol)
    x = c[None] + width * rng.standard_normal((batch,) + c.shape)
    return x.astype(np.float32)
