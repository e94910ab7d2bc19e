"""Kronecker-factored curvature (KFAC) optimizer over the adjoint's layer taps.

Mirrors the reference's ``KFACOptimizer`` (src/jaqmc/optimizer/kfac/kfac.py:
29-200): the same arguments and defaults (``learning_rate`` a scalar or a
schedule, default the ``Standard`` schedule 0.05 / (1 + t / 2000) of
src/jaqmc/optimizer/schedule.py:10-29; ``norm_constraint`` 1e-3,
``curvature_ema`` 0.95, ``l2_reg`` 0, ``inverse_update_period`` 1, ``damping``
1e-3) and the same ``init`` / ``update`` calls.  The reference delegates the
curvature to kfac-jax 0.0.8 (``kfac_jax.OptaxPreconditioner`` with
``estimation_mode="fisher_exact"`` on a normal predictive distribution of
log|psi| with variance 1/2); that package is not part of the reference tree,
so its published algorithm (Martens & Grosse, "Optimizing Neural Networks
with Kronecker-factored Approximate Curvature", 2015) is restated here on the
statistics this library's adjoint exports (``qmc_grad_taps``):

* Dense layers applied ``r`` times per walker (the reference's
  ``RepeatedDenseBlock``, src/jaqmc/optimizer/kfac/curvature_blocks.py:
  94-137): inputs x (with a ones column when the layer has a bias) and output
  cotangents dy = sqrt(2) d log|psi_w| / d out (the square root of the
  normal distribution's Fisher 1 / variance), averaged over all B r
  applications, A = <x x^T>, G = <dy dy^T>; the block's curvature is
  r (A (x) G).
* The envelope parameters (no dense pattern) form a diagonal block,
  F_pp = < 2 (d log|psi_w| / d theta_p)^2 > over walkers
  (curvature_blocks.py:101-121).
* Factors are exponential moving averages normalised by their accumulated
  weight: after t updates, sum_s e^(t-s) S_s / sum_s e^(t-s), e =
  ``curvature_ema`` (the first estimate is the first batch's statistics).
* Damping lambda = ``damping`` + ``l2_reg`` enters each Kronecker block as
  factored Tikhonov damping with the trace-norm pi adjustment:
  r (A (x) G) + lambda I ~= r (A + pi sqrt(lambda / r) I) (x) (G + sqrt(lambda / r) / pi I),
  pi = sqrt((tr A / dim A) / (tr G / dim G)); diagonal blocks add lambda.
* The update is u = C^-1 (-lr g) per block; with ``norm_constraint`` c it is
  scaled by min(1, sqrt(c / (u . (-lr g)))) (the reference places the
  learning rate before the preconditioner so that this bounds the Fisher
  norm of the step, kfac.py:192-198).

Parameters are the flat float32 device vector of :class:`vmc.DeviceParams`;
``update`` returns the flat update to add to them (optax.apply_updates).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Any, NamedTuple

import torch


def standard_schedule(rate: float = 0.05, delay: float = 2000.0, decay: float = 1.0):
    """``Standard`` learning-rate schedule (src/jaqmc/optimizer/schedule.py:10-29)."""
    return lambda t: rate * (1.0 / (1.0 + t / delay)) ** decay


class _Factor:
    """Exponential moving average normalised by its accumulated weight."""

    def __init__(self):
        self.raw = None
        self.weight = 0.0

    def update(self, value: torch.Tensor, ema: float):
        self.raw = value.clone() if self.raw is None else ema * self.raw + value
        self.weight = ema * self.weight + 1.0

    @property
    def value(self) -> torch.Tensor:
        return self.raw / self.weight


class KFACState(NamedTuple):
    step: int
    blocks: list  # per tap: {"A": _Factor, "G": _Factor} or {"D": _Factor}
    inverses: list  # per tap: (Ainv, Ginv) or Dinv, from the last inverse update


@dataclass
class KFACOptimizer:
    """KFAC preconditioner + learning rate (the reference's KFACOptimizer)."""

    learning_rate: Any = field(default_factory=standard_schedule)
    norm_constraint: float = 1e-3
    curvature_ema: float = 0.95
    l2_reg: float = 0.0
    inverse_update_period: int = 1
    damping: float = 1e-3
    f_log_psi: Any = None  # a vmc.FermiNetWavefunction (runtime dependency)

    # ---------------------------------------------------------------- API
    def init(self, params, *, batched_data=None, rngs=None, **extra) -> KFACState:
        """An empty curvature state (the factors start with the first update)."""
        if self.f_log_psi is None:
            raise RuntimeError("KFACOptimizer needs f_log_psi (the wavefunction) before init")
        return KFACState(0, [], [])

    def _lr(self, t: int) -> float:
        return float(self.learning_rate(t)) if callable(self.learning_rate) else float(self.learning_rate)

    def statistics(self, params, batched_data):
        """Per-tap curvature statistics of the current walkers from the GPU
        adjoint: ``[("dense", r, A, G) | ("diagonal", D)]`` and the taps."""
        wf = self.f_log_psi
        data = batched_data.data if hasattr(batched_data, "data") else batched_data
        m = wf.model(data, params)
        electrons = data["electrons"] if isinstance(data, dict) else data.electrons
        taps, _ = m.layer_taps(electrons.to(m.device, torch.float32).contiguous())
        stats = []
        for t in taps:
            dy = t["dy"].double() * math.sqrt(2.0)
            if t["kind"] == "dense":
                x = t["x"].double()
                if t["has_bias"]:
                    x = torch.cat([x, torch.ones_like(x[:, :1])], dim=1)
                rows = x.shape[0]
                stats.append(("dense", t["rows_per_walker"], x.T @ x / rows, dy.T @ dy / rows))
            else:
                stats.append(("diagonal", (dy * dy).mean(0)))
        return stats, taps

    def update(self, grads, state: KFACState, params, *, batched_data=None, rngs=None, **extra):
        """``(updates, state)``: the preconditioned, norm-constrained step for
        the flat gradient ``grads`` (the loss gradient of LossAndGrad)."""
        if not isinstance(state, KFACState):
            raise RuntimeError("KFACOptimizer.init must be called before update")
        stats, taps = self.statistics(params, batched_data)
        ema = self.curvature_ema
        blocks = state.blocks or [({"A": _Factor(), "G": _Factor()} if s[0] == "dense" else {"D": _Factor()})
                                  for s in stats]
        for blk, s in zip(blocks, stats):
            if s[0] == "dense":
                blk["A"].update(s[2], ema)
                blk["G"].update(s[3], ema)
            else:
                blk["D"].update(s[1], ema)
        lam = self.damping + self.l2_reg
        inverses = state.inverses
        if not inverses or state.step % self.inverse_update_period == 0:
            inverses = [self._inverse(blk, s, lam) for blk, s in zip(blocks, stats)]
        g = grads.to(torch.float64).reshape(-1)
        step = -self._lr(state.step) * g
        u = torch.zeros_like(step)
        for t, s, inv in zip(taps, stats, inverses):
            if s[0] == "dense":
                r = s[1]
                k0, rows_in, cols = t["kernel_offset"], t["in_cols"], t["out_cols"]
                gw = step[k0:k0 + rows_in * cols].view(rows_in, cols)
                if t["has_bias"]:
                    b0 = t["bias_offset"]
                    gw = torch.cat([gw, step[b0:b0 + cols].view(1, cols)], dim=0)
                uw = inv[0] @ gw @ inv[1] / r
                u[k0:k0 + rows_in * cols] = uw[:rows_in].reshape(-1)
                if t["has_bias"]:
                    u[b0:b0 + cols] = uw[rows_in]
            else:
                k0, cnt = t["kernel_offset"], t["out_cols"]
                u[k0:k0 + cnt] = inv * step[k0:k0 + cnt]
        if self.norm_constraint is not None:
            sq = float((u * step).sum())
            if sq > 0.0:
                u = u * min(1.0, math.sqrt(self.norm_constraint / sq))
        return u.to(grads.dtype), KFACState(state.step + 1, blocks, inverses)

    # ----------------------------------------------------------- internals
    @staticmethod
    def _inverse(blk, s, lam: float):
        if s[0] == "dense":
            r = s[1]
            A, G = blk["A"].value, blk["G"].value
            ta = float(torch.trace(A)) / A.shape[0]
            tg = float(torch.trace(G)) / G.shape[0]
            pi = math.sqrt(ta / tg) if ta > 0.0 and tg > 0.0 else 1.0
            d = math.sqrt(lam / r)
            Ai = torch.linalg.inv(A + pi * d * torch.eye(A.shape[0], dtype=A.dtype, device=A.device))
            Gi = torch.linalg.inv(G + (d / pi) * torch.eye(G.shape[0], dtype=G.dtype, device=G.device))
            return (Ai, Gi)
        return 1.0 / (blk["D"].value + lam)
