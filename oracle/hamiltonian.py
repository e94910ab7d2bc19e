"""Local-energy pieces (oracle; test infrastructure only).

* ``potential_energy`` — ``src/jaqmc/app/molecule/hamiltonian.py:9-22``:
  ``-sum_iI Z_I/r_iI + sum_{i<j} 1/r_ij + sum_{I<J} Z_I Z_J / R_IJ``.
* ``kinetic_from_tangents`` — ``src/jaqmc/estimator/kinetic/_common.py:61-73``:
  ``KE = -0.5 * (lap + |grad|^2)``.
* ``kinetic_bruteforce`` — the reference's ``scan`` mode
  (``src/jaqmc/estimator/kinetic/euclidean.py:84-112``): the Hessian trace by
  one reverse-over-reverse product per coordinate, here with torch autograd.
"""
from __future__ import annotations

import torch


def potential_energy(electrons, atoms, charges):
    e = torch.as_tensor(electrons)
    dtype = e.dtype
    R = torch.as_tensor(atoms).to(dtype)
    Z = torch.as_tensor(charges).to(dtype)
    B, n, _ = e.shape
    A = R.shape[0]
    r_ae = (e.unsqueeze(2) - R.reshape(1, 1, A, 3)).norm(dim=-1)
    v = -(Z / r_ae).sum((1, 2))
    if n > 1:
        iu = torch.triu_indices(n, n, 1)
        d = (e.unsqueeze(2) - e.unsqueeze(1))[:, iu[0], iu[1]].norm(dim=-1)
        v = v + (1.0 / d).sum(-1)
    if A > 1:
        iu = torch.triu_indices(A, A, 1)
        d = (R.unsqueeze(1) - R.unsqueeze(0))[iu[0], iu[1]].norm(dim=-1)
        v = v + (Z[iu[0]] * Z[iu[1]] / d).sum()
    return v


def kinetic_from_tangents(grad, lap):
    return -0.5 * lap - 0.5 * (grad * grad).sum(-1)


def kinetic_bruteforce(logpsi, electrons):
    """``-0.5 (tr H + |g|^2)`` of ``logpsi`` by autograd (float64 advised)."""
    x = torch.as_tensor(electrons).clone().requires_grad_(True)
    B, n, _ = x.shape
    lp = logpsi(x)
    (g,) = torch.autograd.grad(lp.sum(), x, create_graph=True)
    g = g.reshape(B, 3 * n)
    tr = torch.zeros(B, dtype=x.dtype)
    for d in range(3 * n):
        (h,) = torch.autograd.grad(g[:, d].sum(), x, retain_graph=True)
        tr = tr + h.reshape(B, 3 * n)[:, d]
    return (-0.5 * (tr + (g * g).sum(-1))).detach(), g.detach(), tr.detach()
