"""All-electron Gaussian Metropolis-Hastings update (oracle; test infrastructure only).

Restates ``MCMCSampler._mh_update`` (``src/jaqmc/sampler/mcmc.py:96-137``)
and the width adaptation of ``MCMCSampler.step`` (``:139-199``) with the
random draws supplied by the caller, so that the same normals and uniforms can
be fed to the GPU and to this code:

* proposal ``x2 = x1 + stddev * normal``        (``gaussian_proposal``, ``:53-54``)
* ``ratio = log_prob_2 - log_prob_1`` with ``log_prob = 2 log|psi|`` (``sampler/base.py:174``)
* ``accept = ratio > log(uniform)``              (``:125-131``)
"""
from __future__ import annotations

import torch


def mh_update(logpsi, x1, lp1, normals, uniforms, stddev):
    """One update.  ``lp1`` is ``2 log|psi(x1)|``; returns ``(x, lp, accept)``."""
    x2 = x1 + normals * stddev
    lp2 = 2.0 * logpsi(x2)
    ratio = lp2 - lp1
    cond = ratio > torch.log(uniforms)
    x = torch.where(cond.reshape(-1, 1, 1), x2, x1)
    lp = torch.where(cond, lp2, lp1)
    return x, lp, cond, ratio


def mh_steps(logpsi, x, normals, uniforms, stddev):
    """``steps`` updates; ``normals`` is ``(steps, B, n, 3)``, ``uniforms`` ``(steps, B)``."""
    lp = 2.0 * logpsi(x)
    accepts = torch.zeros(x.shape[0], dtype=torch.int64)
    ratios = []
    for s in range(normals.shape[0]):
        x, lp, cond, ratio = mh_update(logpsi, x, lp, normals[s], uniforms[s], stddev)
        accepts += cond.to(torch.int64)
        ratios.append(ratio)
    return x, lp, accepts, torch.stack(ratios)


def adapt_width(stddev: float, pmoves, counter: int, pmove: float,
                adapt_frequency: int = 100, pmove_range=(0.5, 0.55)):
    """Width adaptation of ``MCMCSampler.step`` (``mcmc.py:182-197``)."""
    counter += 1
    t = counter % adapt_frequency
    pmoves = list(pmoves)
    pmoves[t] = pmove
    if t == 0:
        m = sum(pmoves) / len(pmoves)
        if m > pmove_range[1]:
            stddev = stddev * 1.1
        elif m < pmove_range[0]:
            stddev = stddev / 1.1
    return stddev, pmoves, counter
