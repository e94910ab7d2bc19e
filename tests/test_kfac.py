"""KFAC preconditioner (host logic, CPU) on synthetic layer taps.

The reference's KFACOptimizer (src/jaqmc/optimizer/kfac/kfac.py:29-200) hands
the curvature to kfac-jax; its block algebra is restated in
jaqmc_gb300/kfac.py and checked here against dense linear algebra:
repeated-dense factors A = <x x^T>, G = 2 <dy dy^T> (curvature_blocks.py:
94-137), the factored Tikhonov damping with the pi adjustment, the diagonal
envelope block, the weight-normalised moving average and the norm
constraint.
"""
import math

import numpy as np
import pytest
import torch

from jaqmc_gb300 import kfac as K


class _FakeModel:
    device = torch.device("cpu")

    def __init__(self, taps):
        self.taps = taps

    def layer_taps(self, electrons):
        return self.taps, torch.zeros(electrons.shape[0])


class _FakeWF:
    def __init__(self, taps):
        self.m = _FakeModel(taps)

    def model(self, data, params):
        return self.m


class _Data:
    def __init__(self, B):
        self.electrons = torch.zeros(B, 2, 3)


def _taps(rng, B=6, r=3, din=4, dout=3, ndiag=5):
    x = torch.tensor(rng.normal(size=(B * r, din)), dtype=torch.float32)
    dy = torch.tensor(rng.normal(size=(B * r, dout)), dtype=torch.float32)
    dg = torch.tensor(rng.normal(size=(B, ndiag)), dtype=torch.float32)
    P = din * dout + dout + ndiag
    return [{"kind": "dense", "rows_per_walker": r, "has_bias": True, "kernel_offset": 0,
             "bias_offset": din * dout, "in_cols": din, "out_cols": dout, "x": x, "dy": dy},
            {"kind": "diagonal", "rows_per_walker": 1, "has_bias": False, "kernel_offset": din * dout + dout,
             "bias_offset": 0, "in_cols": 0, "out_cols": ndiag, "x": x[:0], "dy": dg}], P


def test_single_step_matches_dense_algebra():
    rng = np.random.default_rng(0)
    taps, P = _taps(rng)
    opt = K.KFACOptimizer(learning_rate=0.1, norm_constraint=None, damping=1e-2, f_log_psi=_FakeWF(taps))
    st = opt.init(None)
    g = torch.tensor(rng.normal(size=P))
    u, st = opt.update(g, st, None, batched_data=_Data(6))
    x = taps[0]["x"].double().numpy()
    x1 = np.concatenate([x, np.ones((x.shape[0], 1))], 1)
    dy = taps[0]["dy"].double().numpy() * math.sqrt(2)
    A = x1.T @ x1 / x1.shape[0]
    G = dy.T @ dy / dy.shape[0]
    r, lam = 3, 1e-2
    pi = math.sqrt((np.trace(A) / A.shape[0]) / (np.trace(G) / G.shape[0]))
    d = math.sqrt(lam / r)
    Ad, Gd = A + pi * d * np.eye(5), G + d / pi * np.eye(3)
    # vec(W) with W [in+1][out] row-major: the block curvature is r (Ad (x) Gd)
    C = r * np.kron(Ad, Gd)
    step = -0.1 * g.numpy()
    gw = np.concatenate([step[:12].reshape(4, 3), step[12:15].reshape(1, 3)], 0).reshape(-1)
    uw = np.linalg.solve(C, gw).reshape(5, 3)
    np.testing.assert_allclose(u[:12].numpy().reshape(4, 3), uw[:4], rtol=1e-10)
    np.testing.assert_allclose(u[12:15].numpy(), uw[4], rtol=1e-10)
    D = 2 * (taps[1]["dy"].double().numpy() ** 2).mean(0)
    np.testing.assert_allclose(u[15:].numpy(), step[15:] / (D + lam), rtol=1e-10)


def test_moving_average_is_weight_normalised():
    f = K._Factor()
    vals = [torch.tensor([1.0], dtype=torch.float64), torch.tensor([3.0], dtype=torch.float64),
            torch.tensor([5.0], dtype=torch.float64)]
    for v in vals:
        f.update(v, 0.9)
    want = (0.81 * 1 + 0.9 * 3 + 5) / (0.81 + 0.9 + 1)
    assert float(f.value) == pytest.approx(want, rel=1e-12)
    f1 = K._Factor()
    f1.update(torch.tensor([7.0]), 0.95)
    assert float(f1.value) == 7.0  # the first estimate is the first batch's


def test_norm_constraint_bounds_the_fisher_norm():
    rng = np.random.default_rng(1)
    taps, P = _taps(rng)
    g = torch.tensor(rng.normal(size=P)) * 100.0
    free = K.KFACOptimizer(learning_rate=0.1, norm_constraint=None, f_log_psi=_FakeWF(taps))
    u0, _ = free.update(g, free.init(None), None, batched_data=_Data(6))
    c = 1e-3
    con = K.KFACOptimizer(learning_rate=0.1, norm_constraint=c, f_log_psi=_FakeWF(taps))
    u1, _ = con.update(g, con.init(None), None, batched_data=_Data(6))
    sq = float((u0 * (-0.1 * g)).sum())
    assert sq > c
    np.testing.assert_allclose(u1.numpy(), u0.numpy() * math.sqrt(c / sq), rtol=1e-12)
    # the step's squared Fisher norm u^T F u = (u1 . step)^2 / sq equals c
    assert float((u1 * (-0.1 * g)).sum()) ** 2 / sq == pytest.approx(c, rel=1e-10)


def test_standard_schedule_and_inverse_period():
    lr = K.standard_schedule()
    assert lr(0) == 0.05 and lr(2000) == pytest.approx(0.025)
    rng = np.random.default_rng(2)
    taps, P = _taps(rng)
    opt = K.KFACOptimizer(learning_rate=0.1, inverse_update_period=3, f_log_psi=_FakeWF(taps))
    st = opt.init(None)
    g = torch.tensor(rng.normal(size=P))
    _, st = opt.update(g, st, None, batched_data=_Data(6))
    inv0 = st.inverses
    _, st = opt.update(g, st, None, batched_data=_Data(6))
    assert st.inverses is inv0  # kept between inverse updates
    _, st = opt.update(g, st, None, batched_data=_Data(6))
    _, st = opt.update(g, st, None, batched_data=_Data(6))  # step 3: recomputed
    assert st.inverses is not inv0
