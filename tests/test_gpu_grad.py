"""GPU parameter adjoint (qmc_grad) against the oracle.

Checks, per the gradient-path configuration (CH4, FermiNet 4x(256,32), K=16):
  * per-walker d log|psi| / d theta vs torch autograd of the FP64 oracle (the
    restatement of the reference's jax.grad): norm-wise relative error per
    walker <= 1e-4 (small model) / 2e-4 (CH4), median over walkers;
  * vs FP64 central finite differences (step 1e-4) on 64 seeded parameter
    entries: relative error <= 1e-3 of each walker's gradient scale;
  * sum_w c_w d log|psi_w| equals J^T c, also when a small byte budget splits
    the batch into chunks (recomputed activations).
"""
import numpy as np
import pytest
import torch

from helpers import full_cfg, oracle_logpsi_flat, oracle_param_jacobian, setup, small_cfg
from jaqmc_gb300 import _native
from jaqmc_gb300 import systems as S

pytestmark = pytest.mark.gpu

CASES = {
    "Li-small": (S.lithium, lambda: small_cfg((2, 1), ndets=3), 6, 1e-4),
    "Li-small-nosplit": (S.lithium, lambda: small_cfg((2, 1), ndets=3, orbitals_spin_split=False), 6, 1e-4),
    "He-triplet-small": (lambda: S.make_molecule("He", [2], [[0, 0, 0]], (2, 0)), lambda: small_cfg((2, 0)), 6, 1e-4),
    "CH4-full": (S.methane, lambda: full_cfg((5, 5)), 4, 2e-4),
}


def _model(mol, cfg, flat, dev):
    m = _native.NativeFermiNet(cfg, mol.atoms, mol.charges, device=dev)
    m.set_params(torch.as_tensor(flat, device=dev))
    return m


@pytest.mark.parametrize("case", list(CASES))
def test_per_walker_jacobian_matches_autograd(case, cuda_device):
    molf, cfgf, B, tol = CASES[case]
    mol, cfg = molf(), cfgf()
    _, flat, x = setup(mol, cfg, B)
    m = _model(mol, cfg, flat, cuda_device)
    J, _, lp = m.grad(torch.as_tensor(x, device=cuda_device), per_walker=True)
    Jr, lpr = oracle_param_jacobian(flat, cfg, mol, x)
    J = J.double().cpu().numpy()
    rel = np.linalg.norm(J - Jr, axis=1) / np.linalg.norm(Jr, axis=1)
    np.testing.assert_allclose(lp.cpu().numpy(), lpr, rtol=1e-4, atol=1e-4)
    assert np.median(rel) <= tol, rel
    assert rel.max() <= 50 * tol, rel


def test_jacobian_matches_central_differences(cuda_device):
    mol = S.methane()
    cfg = full_cfg((5, 5))
    _, flat, x = setup(mol, cfg, 3)
    m = _model(mol, cfg, flat, cuda_device)
    J, _, _ = m.grad(torch.as_tensor(x, device=cuda_device), per_walker=True)
    J = J.double().cpu().numpy()
    rng = np.random.default_rng(64)
    idx = rng.choice(flat.size, 64, replace=False)
    h = 1e-4
    base = flat.astype(np.float64)
    fd = np.zeros((x.shape[0], idx.size))
    for c, p in enumerate(idx):
        up, dn = base.copy(), base.copy()
        up[p] += h
        dn[p] -= h
        fd[:, c] = (oracle_logpsi_flat(up, cfg, mol, x) - oracle_logpsi_flat(dn, cfg, mol, x)) / (2 * h)
    scale = np.abs(J).max(axis=1, keepdims=True)
    err = np.abs(J[:, idx] - fd) / scale
    assert err.max() <= 1e-3, err.max()


def test_weighted_gradient_and_budget_chunks(cuda_device):
    mol = S.lithium()
    cfg = small_cfg((2, 1), ndets=3)
    _, flat, x = setup(mol, cfg, 37)
    m = _model(mol, cfg, flat, cuda_device)
    c = torch.linspace(-1.0, 1.0, 37, dtype=torch.float64)
    xd = torch.as_tensor(x, device=cuda_device)
    J, g, _ = m.grad(xd, weights=c, per_walker=True)
    ref = (J.double().cpu() * c[:, None]).sum(0).numpy()
    np.testing.assert_allclose(g.cpu().numpy(), ref, rtol=1e-9, atol=1e-9 * np.abs(ref).max())
    # a budget that holds only a few walkers: same gradient from recomputed chunks
    one = m.lib.qmc_workspace_size(m.h, _native.OP_GRAD, 1)
    m.set_grad_budget(3 * one)
    assert m.lib.qmc_workspace_size(m.h, _native.OP_GRAD, 37) < 37 * one
    _, g2, _ = m.grad(xd, weights=c)
    np.testing.assert_allclose(g2.cpu().numpy(), g.cpu().numpy(), rtol=1e-9, atol=1e-12)
