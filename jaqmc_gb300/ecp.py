"""ECP tables and spherical quadrature rules for ``qmc_ecp_energy``.

The reference's ECPEnergy estimator (src/jaqmc/estimator/ecp/estimator.py:
33-155) takes PySCF's ECP dictionaries (``mol._ecp``: ``{symbol: [n_core,
[[l, [[[alpha, coeff], ...] for power index 0, 1, 2, ...]], ...]]}``, power
index k multiplying r^(k-2), l = -1 the local channel) and integrates the
nonlocal channels on a randomly rotated spherical rule
(src/jaqmc/estimator/ecp/quadrature.py).  This module turns both into the
device tables of the C ABI.
"""
from __future__ import annotations

import itertools
import math

import numpy as np
import torch

DEFAULT_QUADRATURE = "icosahedron_12"


def _normalised(points):
    p = np.asarray(points, np.float64)
    return p / np.linalg.norm(p, axis=1, keepdims=True)


def _cyclic(v):
    a, b, c = v
    return [(a, b, c), (c, a, b), (b, c, a)]


def _sign_variants(v):
    """Every sign pattern of the nonzero coordinates of v."""
    opts = [(x,) if x == 0 else (x, -x) for x in v]
    return [tuple(t) for t in itertools.product(*opts)]


def quadrature_rule(name: str = DEFAULT_QUADRATURE):
    """``(points (Q, 3), weights (Q,))`` of a spherical rule, weights summing
    to 1: ``icosahedron_12`` (degree 5), ``icosahedron_32`` (degree 9),
    ``octahedron_6`` / ``_18`` / ``_26`` / ``_50`` (degrees 3 / 5 / 7 / 11)."""
    kind, _, q = name.partition("_")
    q = int(q)
    phi = (1.0 + math.sqrt(5.0)) / 2.0
    if kind == "icosahedron" and q in (12, 32):
        ico = [p for base in _cyclic((0.0, 1.0, phi)) for p in _sign_variants(base)]
        if q == 12:
            return _normalised(ico), np.full(12, 1.0 / 12.0)
        # vertices of the dual dodecahedron (the icosahedron's face centres)
        dod = _sign_variants((1.0, 1.0, 1.0))
        dod += [p for base in _cyclic((0.0, phi, 1.0 / phi)) for p in _sign_variants(base)]
        pts = np.concatenate([_normalised(ico), _normalised(dod)])
        return pts, np.array([5.0 / 168.0] * 12 + [27.0 / 840.0] * 20)
    if kind == "octahedron" and q in (6, 18, 26, 50):
        groups = [[p for base in [(1.0, 0, 0), (0, 1.0, 0), (0, 0, 1.0)] for p in _sign_variants(base)]]
        groups.append([p for base in [(1.0, 1.0, 0), (1.0, 0, 1.0), (0, 1.0, 1.0)] for p in _sign_variants(base)])
        groups.append(_sign_variants((1.0, 1.0, 1.0)))
        groups.append([p for base in [(1.0, 1.0, 3.0), (1.0, 3.0, 1.0), (3.0, 1.0, 1.0)] for p in _sign_variants(base)])
        w = {6: [1 / 6], 18: [1 / 30, 1 / 15], 26: [1 / 21, 4 / 105, 27 / 840],
             50: [4 / 315, 64 / 2835, 27 / 1280, 14641 / 725760]}[q]
        pts, wts = [], []
        for g, wg in zip(groups, w):
            pts += list(_normalised(g))
            wts += [wg] * len(g)
        return np.array(pts), np.array(wts)
    raise ValueError(f"unknown quadrature {name!r}: icosahedron_12/32 or octahedron_6/18/26/50")


class ECPTables:
    """Device tables of an ECP for one molecule (the reference's ECPRadial.
    from_pyscf, estimator.py:190-265, plus the quadrature rule)."""

    def __init__(self, ecp_coefficients: dict, atom_symbols, max_core: int = 2, quadrature_id: str | None = None,
                 device=None):
        self.atom_symbols = list(atom_symbols)
        self.ecp_atoms = [i for i, s in enumerate(self.atom_symbols) if s in ecp_coefficients]
        if not self.ecp_atoms:
            raise ValueError(f"none of the atoms {self.atom_symbols} has ECP coefficients "
                             f"(given: {list(ecp_coefficients)})")
        self.n_core = {s: int(ecp_coefficients[s][0]) for s in ecp_coefficients}
        chans = [ecp_coefficients[self.atom_symbols[a]][1] for a in self.ecp_atoms]
        self.n_channels = max(max(l for l, _ in ch) for ch in chans) + 2
        self.max_terms = max(sum(len(g) for g in rad) for ch in chans for _, rad in ch)
        tab = np.zeros((len(self.ecp_atoms), self.n_channels, self.max_terms, 3), np.float32)
        for i, ch in enumerate(chans):
            for l, rad in ch:
                t = 0
                for k, group in enumerate(rad):
                    for alpha, coeff in group:
                        tab[i, l + 1, t] = (alpha, coeff, k - 2)
                        t += 1
        self.radial = tab
        self.max_core = int(max_core)
        pts, wts = quadrature_rule(quadrature_id or DEFAULT_QUADRATURE)
        self.quad = np.concatenate([pts, wts[:, None]], 1).astype(np.float32)
        self.device = device
        self._dev = None

    def effective_charges(self, charges):
        """Nuclear charges minus the electrons each ECP replaces."""
        z = np.asarray(charges, np.float64).copy()
        for a in self.ecp_atoms:
            z[a] -= self.n_core[self.atom_symbols[a]]
        return z

    def device_tables(self, device):
        if self._dev is None or self._dev["device"] != device:
            self._dev = {"device": device, "n_ecp_atoms": len(self.ecp_atoms),
                         "ecp_atoms": torch.tensor(self.ecp_atoms, dtype=torch.int32, device=device),
                         "n_channels": self.n_channels, "max_terms": self.max_terms,
                         "radial": torch.as_tensor(self.radial, device=device).contiguous(),
                         "max_core": self.max_core, "n_quad": int(self.quad.shape[0]),
                         "quad": torch.as_tensor(self.quad, device=device).contiguous()}
        return self._dev
