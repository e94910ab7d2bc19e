"""Walker-batch statistics (oracle; test infrastructure only).

* ``mean_reduce`` — ``src/jaqmc/estimator/base.py:27-53`` (nanmean; variance
  as ``<x^2> - <x>^2``).
* ``mad_clip`` / ``iqr_clip`` — ``src/jaqmc/utils/clip.py:11-41``.
* ``vmc_gradient`` — ``src/jaqmc/estimator/loss_grad.py:96-128``:
  ``grads = 2 (<E_c g> - <E_c><g>)`` with ``E_c`` the clipped local energy.
"""
from __future__ import annotations

import numpy as np


def mean_reduce(x):
    x = np.asarray(x, dtype=np.float64)
    m = np.nanmean(x, axis=0)
    return m, np.nanmean(x * x, axis=0) - m * m


def mad_clip(x, scale=5.0):
    x = np.asarray(x)
    med = np.nanmedian(x)
    absdev = np.nanmedian(np.abs(x - med))
    return np.clip(x, med - scale * absdev, med + scale * absdev)


def iqr_clip(x, scale=5.0):
    x = np.asarray(x)
    q1 = np.nanquantile(x, 0.25)
    q3 = np.nanquantile(x, 0.75)
    iqr = q3 - q1
    return np.clip(x, q1 - scale * iqr, q3 + scale * iqr)


def vmc_gradient(per_walker_grads, local_energy, clip="mad", scale=5.0):
    """``per_walker_grads`` ``(B, P)``; returns ``(grads (P,), loss)``."""
    e = np.asarray(local_energy, dtype=np.float64)
    ec = {"mad": mad_clip, "iqr": iqr_clip}[clip](e, scale) if clip != "none" else e
    g = np.asarray(per_walker_grads, dtype=np.float64)
    return 2.0 * ((g * ec[:, None]).mean(0) - ec.mean() * g.mean(0)), e.mean()
