"""Data-parallel host logic on two CPU ranks (gloo): the cross-rank energy
statistics, the all-gather clip window, the gradient weights, the sampler's
pmove (pmean over ranks) and the bench's max-over-ranks timing equal what one
process computes on all walkers."""
import os
import socket
import sys

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _energies(rank, B=64):
    rng = np.random.default_rng(100 + rank)
    e = rng.normal(-10.0, 0.5, B)
    e[rank * 3] = 40.0  # an outlier the clip window must catch
    return torch.tensor(e, dtype=torch.float64)


def _worker(rank, world, port, out):
    sys.path.insert(0, ROOT)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from jaqmc_gb300 import vmc
        import bench
        e = _energies(rank)
        m, v, c = vmc.combine_moments(float(e.mean()), float(e.var(unbiased=False)), e.numel())
        clipped = vmc.clip_observable(e, "mad", 5.0)
        clipped_iqr = vmc.clip_observable(e, "iqr", 2.0)
        w, _ = vmc.energy_gradient_weights(e, "mad", 5.0)
        gathered = vmc.gather_walkers(e)
        g = vmc.allreduce_sum(torch.full((3,), float(rank + 1), dtype=torch.float64))
        slowest = bench.max_over_ranks(10.0 + rank, torch.device("cpu"))
        # rank r accepted 10 (r + 1) of 40 (r + 1) proposals: pmove over all = 30 / 120
        pm = vmc.global_pmove(torch.tensor(10 * (rank + 1)), 40 * (rank + 1))
        out[rank] = {"m": m, "v": v, "c": c, "clipped": clipped.numpy(), "clipped_iqr": clipped_iqr.numpy(),
                     "w": w.numpy(), "gathered": gathered.numpy(), "g": g.numpy(), "slowest": slowest,
                     "pmove": float(pm)}
    finally:
        dist.destroy_process_group()


def _reference(all_e, method, scale):
    x = np.asarray(all_e)
    if method == "mad":
        med = np.median(x)
        dev = np.median(np.abs(x - med))
        return np.clip(x, med - scale * dev, med + scale * dev)
    q1, q3 = np.quantile(x, [0.25, 0.75])
    return np.clip(x, q1 - scale * (q3 - q1), q3 + scale * (q3 - q1))


def test_two_rank_reductions():
    world = 2
    out = mp.Manager().dict()
    mp.spawn(_worker, args=(world, _free_port(), out), nprocs=world, join=True)
    all_e = torch.cat([_energies(r) for r in range(world)]).numpy()
    B = all_e.size // world
    ref_mad = _reference(all_e, "mad", 5.0)
    ref_iqr = _reference(all_e, "iqr", 2.0)
    ref_w = 2.0 * (ref_mad - ref_mad.mean()) / all_e.size
    for r in range(world):
        o = out[r]
        assert o["c"] == all_e.size
        assert o["m"] == pytest.approx(all_e.mean(), rel=1e-14)
        assert o["v"] == pytest.approx(all_e.var(), rel=1e-12)
        np.testing.assert_allclose(o["clipped"], ref_mad[r * B:(r + 1) * B], rtol=0, atol=1e-12)
        np.testing.assert_allclose(o["clipped_iqr"], ref_iqr[r * B:(r + 1) * B], rtol=0, atol=1e-12)
        np.testing.assert_allclose(o["w"], ref_w[r * B:(r + 1) * B], rtol=1e-12, atol=1e-15)
        np.testing.assert_array_equal(o["gathered"], all_e)
        np.testing.assert_array_equal(o["g"], np.full(3, 3.0))
        assert o["slowest"] == 11.0
        assert o["pmove"] == pytest.approx(0.25, rel=1e-15)
    # the outliers were clipped
    assert ref_mad.max() < 0.0


def test_width_adaptation_rule():
    """x1.1 above the pmove range, /1.1 below, unchanged inside
    (src/jaqmc/sampler/mcmc.py:184-197), and the one-rank pmove."""
    from jaqmc_gb300 import vmc
    assert vmc.adapt_width(0.2, 0.6) == pytest.approx(0.22)
    assert vmc.adapt_width(0.2, 0.4) == pytest.approx(0.2 / 1.1)
    assert vmc.adapt_width(0.2, 0.52) == 0.2
    assert float(vmc.global_pmove(torch.tensor(7), 28)) == 0.25
