"""Psiformer + SimpleEE Jastrow oracle against the reference's own property
tests (CPU): antisymmetry under a same-spin swap
(tests/wavefunction/molecule_wavefunction_test.py:67-82), the Jastrow formula
by hand (src/jaqmc/wavefunction/jastrow.py:48-122), and the antiparallel
electron-electron cusp d log|psi| / dr -> 1/2
(tests/wavefunction/molecule_wavefunction_test.py:538-607)."""
import numpy as np
import pytest
import torch

from jaqmc_gb300 import params as P
from oracle import psiformer as OP


def _setup(nspins, atoms, charges, seed=0, **kw):
    cfg = P.PsiformerConfig(nspins=nspins, **kw)
    tree = P.init_psiformer(cfg, len(atoms), seed=seed)
    ocfg = OP.PsiformerConfig(nspins=nspins, ndets=cfg.ndets, num_layers=cfg.num_layers, num_heads=cfg.num_heads,
                              heads_dim=cfg.heads_dim, mlp_hidden_dims=cfg.mlp_hidden_dims)
    return cfg, ocfg, tree, torch.tensor(atoms, dtype=torch.float64)


def test_same_spin_swap_antisymmetry():
    cfg, ocfg, tree, atoms = _setup((2, 1), [[0.0, 0.0, 0.0]], [3.0], ndets=2, num_layers=2, heads_dim=8,
                                    mlp_hidden_dims=[16])
    x = torch.randn(4, 3, 3, dtype=torch.float64, generator=torch.Generator().manual_seed(1))
    a = OP.evaluate(tree, ocfg, x, atoms)
    xs = x[:, [1, 0, 2]]
    b = OP.evaluate(tree, ocfg, xs, atoms)
    torch.testing.assert_close(a["logpsi"], b["logpsi"], rtol=1e-12, atol=1e-12)
    assert torch.all(a["sign_logpsi"] == -b["sign_logpsi"])


def test_jastrow_by_hand():
    cfg, ocfg, tree, atoms = _setup((2, 1), [[0.0, 0.0, 0.0]], [3.0], ndets=2, num_layers=1, heads_dim=8,
                                    mlp_hidden_dims=[16])
    tree["params"]["jastrow_layer"]["alpha_par"][:] = 0.7
    tree["params"]["jastrow_layer"]["alpha_anti"][:] = 1.3
    x = torch.tensor([[[0.1, 0.2, 0.3], [1.0, -0.5, 0.2], [-0.4, 0.6, -1.1]]], dtype=torch.float64)
    _, _, _, r = OP.features(x, atoms, (2, 1))
    r = r[0].numpy()
    ap, aa = float(np.float32(0.7)), float(np.float32(1.3))  # the parameters are float32
    want = -0.25 * ap ** 2 / (ap + r[0, 1]) - 0.5 * aa ** 2 / (aa + r[0, 2]) - 0.5 * aa ** 2 / (aa + r[1, 2])
    got = OP.jastrow(tree["params"]["jastrow_layer"], ocfg, torch.as_tensor(r)[None], torch.float64)
    assert float(got[0]) == pytest.approx(want, rel=1e-14)


@pytest.mark.parametrize("nspins,pair", [((1, 1), (0, 1)), ((2, 1), (0, 2))])
def test_antiparallel_cusp(nspins, pair):
    """Spherical average of d log|psi| / dr at r = 0.01 between an up and a down
    electron, 2 bohr from the nucleus, equals the cusp value 1/2 (+-0.1)."""
    cfg, ocfg, tree, atoms = _setup(nspins, [[0.0, 0.0, 0.0]], [3.0], ndets=4, num_layers=1, heads_dim=16,
                                    mlp_hidden_dims=[64])
    f = OP.logpsi_fn(tree, ocfg, atoms)
    g = torch.Generator().manual_seed(3)
    nsamp, dist = 200, 0.01
    d = torch.randn(nsamp, 3, dtype=torch.float64, generator=g)
    d = d / d.norm(dim=1, keepdim=True)
    center = torch.tensor([2.0, 0.0, 0.0], dtype=torch.float64)
    n = sum(nspins)
    x = torch.zeros(nsamp, n, 3, dtype=torch.float64)
    if n == 3:
        x[:, 1] = torch.tensor([-3.0, 1.0, 0.5])
    i, j = pair
    x[:, i] = center
    x[:, j] = center + dist * d
    x.requires_grad_(True)
    lp = f(x)
    grad = torch.autograd.grad(lp.sum(), x)[0]
    radial = (grad[:, j] * d).sum(1)
    assert float(radial.mean()) == pytest.approx(0.5, abs=0.1)


def test_layout_matches_tree():
    cfg = P.PsiformerConfig(nspins=(21, 21))
    leaves = P.psiformer_leaves(cfg, 12)
    tree = P.init_psiformer(cfg, 12, seed=0)
    flat = P.flatten(tree, leaves)
    back = P.unflatten(flat, leaves)
    np.testing.assert_array_equal(P.flatten(back, leaves), flat)
    assert P.count(leaves) == flat.size
