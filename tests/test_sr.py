"""Robust SR / SPRING / MARCH (jaqmc_gb300/sr.py) against closed forms (CPU).

The reference's kernel formulation (src/jaqmc/optimizer/sr/jasr.py:222-512)
reduces, for gamma = 1 / lambda, to the textbook updates, which are checked
here in FP64 NumPy on small random score matrices:

* SR:      delta = (O^T O + lambda I)^-1 g
* SPRING:  delta = (O^T O + lambda I)^-1 (g + lambda mu delta_prev)
* robust gamma: delta = gamma g - O^T F^-1 (gamma O g - (1 - gamma lambda) F^-1 O g)

with O the centred score divided by sqrt(B); plus the constrained-norm stage
(jasr.py:707-751), MARCH 'diff' (the accumulator from update differences) and
the null-space lift leaving centred solutions unchanged.
"""
import numpy as np
import pytest
import torch

from jaqmc_gb300 import sr as SR


def _problem(B=24, P=15, seed=0):
    rng = np.random.default_rng(seed)
    S = rng.normal(size=(B, P)) * rng.uniform(0.5, 2.0, size=(1, P))
    g = rng.normal(size=P)
    return S, g


def _O(S):
    return (S - S.mean(0, keepdims=True)) / np.sqrt(S.shape[0])


def _t(x):
    return torch.as_tensor(x)


def _close(actual, ref, rel=1e-9):
    """Norm-relative agreement with the FP64 closed forms (centring, Gram and
    solves are FP64 at these sizes)."""
    a = np.asarray(actual, np.float64)
    assert np.linalg.norm(a - ref) <= rel * np.linalg.norm(ref), (np.linalg.norm(a - ref), np.linalg.norm(ref))


def test_standard_sr_and_learning_rate():
    S, g = _problem()
    lam, lr = 1e-2, 0.05
    opt = SR.RobustSR(learning_rate=lr, damping=lam)
    st = opt.init(S.shape[1])
    upd, st = opt.update(_t(g), st, _t(S).float())
    O = _O(S.astype(np.float32).astype(np.float64))
    ref = np.linalg.solve(O.T @ O + lam * np.eye(S.shape[1]), g)
    _close(upd.numpy(), -lr * ref)
    assert st.count == 1 and st.norm_count == 1


def test_spring_momentum_two_steps():
    S1, g1 = _problem(seed=1)
    S2, g2 = _problem(seed=2)
    lam, mu = 5e-3, 0.9
    opt = SR.RobustSR(learning_rate=1.0, damping=lam, spring_mu=mu)
    st = opt.init(S1.shape[1])
    d1, st = opt.precondition(_t(g1), st, _t(S1).float())
    d2, st = opt.precondition(_t(g2), st, _t(S2).float())
    I = np.eye(S1.shape[1])
    O1, O2 = _O(S1.astype(np.float32).astype(np.float64)), _O(S2.astype(np.float32).astype(np.float64))
    r1 = np.linalg.solve(O1.T @ O1 + lam * I, g1)
    r2 = np.linalg.solve(O2.T @ O2 + lam * I, g2 + lam * mu * r1)
    _close(d1.numpy(), r1)
    _close(d2.numpy(), r2)


def test_robust_gamma_formula():
    S, g = _problem(seed=3)
    lam, gamma = 1e-2, 3.0
    opt = SR.RobustSR(damping=lam, robust_gamma=gamma)
    d, _ = opt.precondition(_t(g), opt.init(S.shape[1]), _t(S).float())
    O = _O(S.astype(np.float32).astype(np.float64))
    F = O @ O.T + np.ones((O.shape[0],) * 2) / O.shape[0] + lam * np.eye(O.shape[0])  # lifted null space
    w = np.linalg.solve(F, O @ g)
    z = np.linalg.solve(F, gamma * (O @ g) - (1 - gamma * lam) * w)
    _close(d.numpy(), gamma * g - O.T @ z)


def test_constrained_norm_and_fixed():
    S, g = _problem(seed=4)
    opt = SR.RobustSR(learning_rate=10.0, damping=1e-2, max_norm=0.01)
    upd, _ = opt.update(_t(g), opt.init(S.shape[1]), _t(S).float())
    assert float(torch.linalg.norm(upd)) == pytest.approx(0.01, rel=1e-6)
    opt = SR.RobustSR(learning_rate=0.02, damping=1e-2, max_norm="fixed")
    upd, _ = opt.update(_t(g), opt.init(S.shape[1]), _t(S).float())
    assert float(torch.linalg.norm(upd)) == pytest.approx(0.02, rel=1e-6)
    with pytest.raises(ValueError):
        SR.RobustSR(max_norm="free")


def test_march_diff_accumulator():
    S, g = _problem(seed=5)
    beta = 0.9
    opt = SR.RobustSR(damping=1e-2, march_beta=beta)
    st = opt.init(S.shape[1])
    d1, st = opt.precondition(_t(g), st, _t(S).float())
    np.testing.assert_allclose(st.acc_var.numpy(), beta * 1.0 + (1 - beta) * d1.numpy() ** 2, rtol=1e-12)
    # the second step scales by 1/sqrt(acc_var): compare with SR in the scaled metric
    d2, _ = opt.precondition(_t(g), st, _t(S).float())
    s = 1.0 / np.sqrt(st.acc_var.numpy() + 1e-8)
    O = _O(S.astype(np.float32).astype(np.float64))
    Os = O * np.sqrt(s)[None, :]
    ref = s * (np.linalg.solve(Os.T @ Os + 1e-2 * np.eye(S.shape[1]), np.sqrt(s) * g) / np.sqrt(s))
    _close(d2.numpy(), ref)


def test_null_space_lift_and_gram():
    S, _ = _problem(B=10, P=40, seed=6)
    O = _O(S)
    for prec in ("f64", "f32"):
        gram = SR.gram_matrix(_t(O).float(), 1.0, block=16, precision=prec)
        np.testing.assert_allclose(gram.numpy(), O @ O.T, rtol=1e-5, atol=1e-6)
    lifted = SR.lift_null_space(gram)
    ev = np.linalg.eigvalsh(lifted.numpy())
    assert ev.min() > 0.5 / 10  # the constant direction now has eigenvalue 1


def test_required_damping_bounds_the_condition_number():
    """lam = eig_max / (kappa - 1) against the exact largest eigenvalue, and the
    argument check on kappa."""
    S, _ = _problem(B=12, P=50, seed=9)
    O = _O(S)
    gram = _t(O @ O.T)
    eig_max = np.linalg.eigvalsh(O @ O.T).max()
    lam = float(SR.estimate_required_damping(gram, 1e3, num_iters=200))
    np.testing.assert_allclose(lam, eig_max / (1e3 - 1.0), rtol=1e-4)
    with pytest.raises(ValueError):
        SR.estimate_required_damping(gram, 1.0)
