"""LapNet oracle (oracle/lapnet.py) pinned against the reference's own
property tests (restated): forward Laplacian == brute-force Hessian trace
(tests/estimator/kinetic_forward_laplacian_test.py:248-420 checks FL vs scan
for FermiNet, Psiformer and LapNet at rtol = atol = 2e-5), same-spin
antisymmetry (tests/wavefunction/molecule_wavefunction_test.py:67-82), and
the parameter layout round trip."""
import numpy as np
import pytest
import torch

from jaqmc_gb300 import params as P
from jaqmc_gb300 import systems as S
from oracle import hamiltonian as OH
from oracle import lapnet as OL

SMALL = dict(ndets=2, num_layers=2, num_heads=2, heads_dim=4)


def _ocfg(cfg):
    return OL.LapNetConfig(nspins=cfg.nspins, ndets=cfg.ndets, num_layers=cfg.num_layers, num_heads=cfg.num_heads,
                           heads_dim=cfg.heads_dim, num_local_updates=cfg.num_local_updates, envelope=cfg.envelope,
                           jastrow=cfg.jastrow, use_input_bias=cfg.use_input_bias,
                           use_backbone_bias=cfg.use_backbone_bias)


@pytest.mark.parametrize("system", ["Li", "CH4"])
@pytest.mark.parametrize("jastrow", ["simple_ee", "none"])
def test_fl_matches_bruteforce(system, jastrow):
    mol = S.SYSTEMS[system]()
    cfg = P.LapNetConfig(nspins=mol.nspins, jastrow=jastrow, **SMALL)
    tree = P.init_lapnet(cfg, mol.n_atoms, seed=3)
    x = torch.as_tensor(S.init_walkers(mol, 3, seed=2), dtype=torch.float64)
    out = OL.evaluate(tree, _ocfg(cfg), x, mol.atoms, tangents=True)
    ke = OH.kinetic_from_tangents(out["grad"], out["lap"])
    ke_ref, g_ref, _ = OH.kinetic_bruteforce(OL.logpsi_fn(tree, _ocfg(cfg), mol.atoms), x)
    np.testing.assert_allclose(out["grad"].numpy(), g_ref.numpy(), rtol=1e-9, atol=1e-9)
    np.testing.assert_allclose(ke.numpy(), ke_ref.numpy(), rtol=1e-9, atol=1e-9)


def test_same_spin_swap_flips_sign():
    mol = S.lithium()
    cfg = P.LapNetConfig(nspins=mol.nspins, **SMALL)
    tree = P.init_lapnet(cfg, mol.n_atoms, seed=1)
    x = torch.as_tensor(S.init_walkers(mol, 8, seed=4), dtype=torch.float64)
    xs = x.clone()
    xs[:, [0, 1]] = xs[:, [1, 0]]
    a = OL.evaluate(tree, _ocfg(cfg), x, mol.atoms)
    b = OL.evaluate(tree, _ocfg(cfg), xs, mol.atoms)
    assert torch.equal(a["sign_logpsi"], -b["sign_logpsi"])
    np.testing.assert_allclose(a["logpsi"].numpy(), b["logpsi"].numpy(), rtol=1e-12)


def test_layout_round_trip_and_defaults():
    mol = S.nitrogen_dimer()
    cfg = P.LapNetConfig(nspins=mol.nspins)
    leaves = P.lapnet_leaves(cfg, mol.n_atoms)
    tree = P.init_lapnet(cfg, mol.n_atoms, seed=0)
    flat = P.flatten(tree, leaves)
    back = P.unflatten(flat, leaves)
    np.testing.assert_array_equal(P.flatten(back, leaves), flat)
    names = ["/".join(p) for p, _ in leaves]
    # the last layer has no local updates of the individual stream
    assert "backbone_layer/layers_2/qk_update_layers_1/kernel" in names
    assert not any(nm.startswith("backbone_layer/layers_3/qk_update") for nm in names)
    assert ("backbone_layer", "layers_0", "qk_projection", "kernel") in [p for p, _ in leaves]
    with pytest.raises(NotImplementedError):
        P.lapnet_leaves(P.LapNetConfig(nspins=(1, 1), use_layernorm=True), 1)
