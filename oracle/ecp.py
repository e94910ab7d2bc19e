"""Effective-core-potential energy (oracle; test infrastructure only).

Restates the reference's ``ECPEnergy`` estimator
(``src/jaqmc/estimator/ecp/estimator.py:33-155``), its radial potentials
(``:158-275``), nearest-core selection (``:278-320``), nonlocal integral
(``src/jaqmc/estimator/ecp/nonlocal_integral.py:17-130``) and spherical
quadrature rules (``src/jaqmc/estimator/ecp/quadrature.py``), with the random
rotations supplied by the caller so that the GPU and this code integrate on
the same points:

* ``V_l(r) = sum_k c_k r^(p_k) exp(-a_k r^2)`` per channel, channel 0 the
  local part (PySCF ``l = -1``), channel ``l + 1`` the semi-local ``l``;
* local energy ``sum_{i, I} V_0(r_iI)``;
* nonlocal energy ``sum_i sum_{I nearest} sum_l V_{l+1}(r_iI) (2l + 1)
  sum_q w_q P_l(cos theta_q) psi(r_1..r_i^q..) / psi(r)``, with
  ``r_i^q = R_I + |r_i - R_I| Rot_i x_q`` and ``cos theta_q = (Rot_i x_q) .
  (r_i - R_I) / |r_i - R_I|`` (the quadrature weights sum to 1).

The ECP tables use PySCF's layout (``mol._ecp``): ``{symbol: [n_core,
[[l, [[[alpha, coeff], ...] per power index 0, 1, 2, ...]], ...]]}`` where
power index ``k`` multiplies ``r^(k - 2)``.
"""
from __future__ import annotations

import math

import numpy as np
import torch


def radial_table(ecp: dict, symbols: list, ecp_atoms: list):
    """``(alpha, coeff, power)`` arrays ``(n_ecp_atoms, n_channels, max_terms)``
    (zero-padded) from PySCF ECP dicts (estimator.py:190-265)."""
    n_ch = max(max(l for l, _ in ecp[symbols[a]][1]) + 2 for a in ecp_atoms)
    terms = [[sum(len(g) for g in rad) for _, rad in ecp[symbols[a]][1]] for a in ecp_atoms]
    T = max(max(t) for t in terms)
    al = np.zeros((len(ecp_atoms), n_ch, T))
    co = np.zeros_like(al)
    pw = np.zeros_like(al)
    for i, a in enumerate(ecp_atoms):
        for l, rad in ecp[symbols[a]][1]:
            t = 0
            for k, group in enumerate(rad):
                for alpha, coeff in group:
                    al[i, l + 1, t], co[i, l + 1, t], pw[i, l + 1, t] = alpha, coeff, k - 2
                    t += 1
    return al, co, pw


def radial(al, co, pw, r):
    """``V(r)`` for distances ``r (..., n_ecp_atoms)`` -> ``(..., n_ecp_atoms, n_channels)``."""
    r = r[..., None, None]
    return (co * r ** pw * np.exp(-al * r * r)).sum(-1)


def _signs(v):
    out = [[]]
    for x in v:
        out = [o + [s * x] for o in out for s in ((1.0, -1.0) if x != 0 else (1.0,))]
    return out


def quadrature(name: str = "icosahedron_12"):
    """Points (Q, 3) and weights (Q,) summing to 1 of the spherical rules
    (quadrature.py): icosahedron 12 / 32, octahedron 6 / 18 / 26 / 50."""
    kind, q = name.split("_")
    q = int(q)
    if kind == "icosahedron":
        t = math.atan(2.0)
        pts = [(0.0, 0.0), (math.pi, 0.0)]
        pts += [(t, 2 * math.pi * k / 5) for k in range(5)]
        pts += [(math.pi - t, 2 * math.pi * k / 5 + math.pi / 5) for k in range(5)]
        w = [1.0 / 12.0] * 12
        if q == 32:
            # face centres of the icosahedron (vertices of the dual dodecahedron)
            a = math.acos(math.sqrt((5 + 2 * math.sqrt(5)) / 15))
            b = math.acos(math.sqrt((5 - 2 * math.sqrt(5)) / 15))
            for th in (a, b):
                pts += [(th, 2 * math.pi * k / 5 + math.pi / 5) for k in range(5)]
            for th in (math.pi - b, math.pi - a):
                pts += [(th, 2 * math.pi * k / 5) for k in range(5)]
            w = [5.0 / 168.0] * 12 + [27.0 / 840.0] * 20
        elif q != 12:
            raise ValueError(f"icosahedron rules have 12 or 32 points, not {q}")
        P = np.array([[math.sin(th) * math.cos(ph), math.sin(th) * math.sin(ph), math.cos(th)] for th, ph in pts])
        return P, np.array(w)
    if kind == "octahedron":
        table = {6: [1 / 6] * 6, 18: [1 / 30] * 6 + [1 / 15] * 12,
                 26: [1 / 21] * 6 + [4 / 105] * 12 + [27 / 840] * 8,
                 50: [4 / 315] * 6 + [64 / 2835] * 12 + [27 / 1280] * 8 + [14641 / 725760] * 24}
        if q not in table:
            raise ValueError(f"octahedron rules have 6, 18, 26 or 50 points, not {q}")
        p, c, r, s = 1 / math.sqrt(2), 1 / math.sqrt(3), 1 / math.sqrt(11), 3 / math.sqrt(11)
        pts = _signs([1, 0, 0]) + _signs([0, 1, 0]) + _signs([0, 0, 1])
        pts += _signs([p, p, 0]) + _signs([p, 0, p]) + _signs([0, p, p])
        pts += _signs([c, c, c])
        pts += _signs([r, r, s]) + _signs([r, s, r]) + _signs([s, r, r])
        return np.array(pts[:q], dtype=np.float64), np.array(table[q])
    raise ValueError(f"unknown quadrature {name!r}")


def legendre(x, L: int):
    """``P_0 .. P_{L-1}`` at ``x`` (L <= 4), stacked on a new first axis."""
    out = [np.ones_like(x), x, 0.5 * (3 * x * x - 1), 0.5 * (5 * x ** 3 - 3 * x)]
    if L > 4:
        raise ValueError("at most four nonlocal channels")
    return np.stack(out[:L])


def rotation_matrices(u_phi, u_cos):
    """Rotations from two uniforms per sample (quadrature.py, Quadrature.
    sample_rotation_matrices): phi = 2 pi u1, cos theta = 1 - 2 u2."""
    phi = 2 * math.pi * np.asarray(u_phi, np.float64)
    ct = 1.0 - 2.0 * np.asarray(u_cos, np.float64)
    st = np.sqrt(np.maximum(0.0, 1.0 - ct * ct))
    sp, cp = np.sin(phi), np.cos(phi)
    m = np.stack([sp * sp + ct * cp * cp, sp * cp * (ct - 1), st * cp,
                  sp * cp * (ct - 1), cp * cp + ct * sp * sp, st * sp,
                  -st * cp, -st * sp, ct], -1)
    return m.reshape(*np.shape(phi), 3, 3)


def select_nearest_cores(values, vectors, distances, max_core: int):
    """The ``max_core`` nearest ECP atoms of every electron, nearest first
    (estimator.py:278-320): ``(values (..., max_core, C), vectors, distances)``;
    unchanged when there are no more than ``max_core`` atoms."""
    values, vectors, distances = np.asarray(values), np.asarray(vectors), np.asarray(distances)
    if distances.shape[-1] <= max_core:
        return values, vectors, distances
    order = np.argsort(distances, axis=-1, kind="stable")[..., :max_core]
    take = lambda a: np.take_along_axis(a, order[..., None], axis=-2)  # noqa: E731
    return take(values), take(vectors), np.take_along_axis(distances, order, axis=-1)


def ecp_energy(phase_logpsi, electrons, atoms, ecp_atoms, al, co, pw, rotations, quad, max_core: int = 2):
    """Per-walker ``(local, nonlocal)`` ECP energies.

    ``phase_logpsi(x (M, n, 3)) -> (sign (M,), log|psi| (M,))``;
    ``rotations (B, n, 3, 3)`` one per electron; ``quad = (points, weights)``."""
    x = np.asarray(electrons, np.float64)
    B, n, _ = x.shape
    R = np.asarray(atoms, np.float64)[ecp_atoms]
    vec = x[:, :, None, :] - R[None, None]                 # (B, n, Ae, 3)
    dist = np.linalg.norm(vec, axis=-1)                     # (B, n, Ae)
    V = radial(al, co, pw, dist)                            # (B, n, Ae, C)
    local = V[..., 0].sum((1, 2))
    n_nl = V.shape[-1] - 1
    nonlocal_ = np.zeros(B)
    if n_nl == 0:
        return local, nonlocal_
    order = np.argsort(dist, axis=-1, kind="stable")[..., :max_core]
    s0, l0 = phase_logpsi(torch.as_tensor(x))
    s0, l0 = np.asarray(s0, np.float64), np.asarray(l0, np.float64)
    pts, wts = quad
    Q = pts.shape[0]
    for i in range(n):
        rp = np.einsum("bjk,qk->bqj", rotations[:, i], pts)     # (B, Q, 3)
        for c in range(order.shape[-1]):
            a = order[:, i, c]
            Ra = R[a]                                           # (B, 3)
            r = dist[np.arange(B), i, a]
            u = vec[np.arange(B), i, a] / r[:, None]
            disp = np.repeat(x[:, None], Q, axis=1)             # (B, Q, n, 3)
            disp[:, :, i] = Ra[:, None] + r[:, None, None] * rp
            s1, l1 = phase_logpsi(torch.as_tensor(disp.reshape(B * Q, n, 3)))
            ratio = (np.asarray(s1, np.float64).reshape(B, Q) * s0[:, None]
                     * np.exp(np.asarray(l1, np.float64).reshape(B, Q) - l0[:, None]))
            cos = np.einsum("bqj,bj->bq", rp, u)
            P = legendre(cos, n_nl)                             # (L, B, Q)
            integ = np.stack([(2 * l + 1) * (P[l] * ratio * wts).sum(-1) for l in range(n_nl)], -1)
            nonlocal_ += (integ * V[np.arange(B), i, a, 1:]).sum(-1)
    return local, nonlocal_
