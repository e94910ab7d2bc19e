"""The diagonal and null envelopes on the GPU (src/jaqmc/wavefunction/output/
envelope.py:16-35,79-80,143-163) against the FP64 oracle on the same
parameters (pi and sigma drawn at random so that the per-dimension rates
differ), through the C ABI:

  * log|psi| and sign (FP32 and split-BF16 forms; FermiNet and Psiformer);
  * E_L on walkers burnt in from |psi|^2: median |dE_L| <= 1e-4 Ha (FP32 form)
    and max <= 3x the oracle's own FP32 max; split-BF16 form: batch mean
    within 4 standard errors (or 0.5 mHa);
  * MH accept masks with injected draws, bit-exact outside the 1e-6 band;
  * the parameter adjoint (including d/dsigma of the diagonal rates) against
    autograd of the FP64 oracle.
"""
import numpy as np
import pytest
import torch

from helpers import full_cfg, oracle_cfg, oracle_local_energy, oracle_param_jacobian, setup, small_cfg
from jaqmc_gb300 import _native
from jaqmc_gb300 import params as P
from jaqmc_gb300 import systems as S
from oracle import ferminet as OF
from oracle import mcmc as OM
from oracle import psiformer as OPS

pytestmark = pytest.mark.gpu
ENVS = ["diagonal", "null"]


def _randomise(tree, seed=5):
    rng = np.random.default_rng(seed)
    for ch in tree["params"].get("envelope_layer", {}).values():
        ch["pi"][:] = rng.uniform(0.5, 1.5, ch["pi"].shape)
        ch["sigma"][:] = rng.uniform(0.5, 1.5, ch["sigma"].shape)
    return tree


def _setup(mol, cfg, B, seed=1):
    tree = _randomise(P.init_ferminet(cfg, mol.n_atoms, seed=0))
    flat = P.flatten(tree, P.ferminet_leaves(cfg, mol.n_atoms))
    return tree, flat, S.init_walkers(mol, B, seed=seed)


def _model(mol, cfg, flat, dev, precision="fp32"):
    m = _native.NativeFermiNet(cfg, mol.atoms, mol.charges, precision=precision, device=dev)
    assert m.param_count == flat.size
    m.set_params(torch.as_tensor(flat, device=dev))
    return m


@pytest.mark.parametrize("envelope", ENVS)
@pytest.mark.parametrize("precision,tol", [("fp32", 1e-5), ("mixed", 1e-3)])
def test_forward(envelope, precision, tol, cuda_device):
    mol = S.nitrogen_dimer()
    cfg = full_cfg((7, 7), ndets=4, envelope=envelope)
    tree, flat, x = _setup(mol, cfg, 64)
    m = _model(mol, cfg, flat, cuda_device, precision)
    lp, sg, fl = m.forward(torch.as_tensor(x, device=cuda_device))
    ref = OF.evaluate(tree, oracle_cfg(cfg), torch.as_tensor(x, dtype=torch.float64), mol.atoms)
    r = ref["logpsi"].numpy()
    rel = np.abs(lp.cpu().numpy() - r) / np.maximum(1.0, np.abs(r))
    assert np.array_equal(sg.cpu().numpy(), ref["sign_logpsi"].numpy())
    assert np.median(rel) < tol and rel.max() < 20 * tol, (np.median(rel), rel.max())
    assert m.check_error() == 0


@pytest.mark.parametrize("envelope", ENVS)
def test_local_energy_equilibrated(envelope, cuda_device):
    mol = S.nitrogen_dimer()
    cfg = full_cfg((7, 7), ndets=4, envelope=envelope)
    tree, flat, x = _setup(mol, cfg, 128)
    mp = _model(mol, cfg, flat, cuda_device)
    xd = torch.as_tensor(x, device=cuda_device)
    mp.mh_steps(xd, 300, 0.15, 3, 0)
    x = xd.cpu().numpy()
    ref = np.concatenate([oracle_local_energy(tree, cfg, mol, x[i:i + 64])["e_local"].numpy() for i in (0, 64)])
    r32 = np.concatenate([oracle_local_energy(tree, cfg, mol, x[i:i + 64], dtype=torch.float32)["e_local"]
                          .double().numpy() for i in (0, 64)])
    got = mp.local_energy(xd)["e_local"].cpu().numpy()
    err, e32 = np.abs(got - ref), np.abs(r32 - ref)
    assert np.median(err) <= 1e-4, np.median(err)
    assert err.max() <= 3 * e32.max() + 1e-4, (err.max(), e32.max())
    mm = _model(mol, cfg, flat, cuda_device, "mixed")
    e = mm.local_energy(xd)["e_local"].cpu().numpy() - ref
    se = e.std(ddof=1) / np.sqrt(len(e))
    assert abs(e.mean()) <= max(5e-4, 4 * se), (e.mean(), se)
    assert mm.check_error() == 0


@pytest.mark.parametrize("envelope", ENVS)
def test_mh_accept_mask(envelope, cuda_device):
    mol = S.lithium()
    cfg = full_cfg((2, 1), ndets=4, envelope=envelope)
    tree, flat, x = _setup(mol, cfg, 64)
    m = _model(mol, cfg, flat, cuda_device)
    nz, uz = m.mh_draws(64, 3, seed=2, counter=0)
    xg = torch.as_tensor(x, device=cuda_device).clone()
    _, lpg, accg, _ = m.mh_steps(xg, 3, 0.02, 2, 0, normals=nz, uniforms=uz)
    f = OF.logpsi_fn(tree, oracle_cfg(cfg), mol.atoms)
    xo, lpo, acco, ratios = OM.mh_steps(f, torch.as_tensor(x, dtype=torch.float64), nz.cpu().double(),
                                        uz.cpu().double(), 0.02)
    keep = ~((ratios - torch.log(uz.cpu().double())).abs() < 1e-6).any(0).numpy()
    assert keep.sum() >= 62
    assert np.array_equal(accg.cpu().numpy()[keep], acco.numpy()[keep])
    np.testing.assert_allclose(lpg.cpu().numpy()[keep], lpo.numpy()[keep], rtol=1e-4, atol=1e-4)


@pytest.mark.parametrize("envelope", ENVS)
def test_adjoint(envelope, cuda_device):
    mol = S.lithium()
    cfg = small_cfg((2, 1), ndets=3, envelope=envelope)
    _, flat, x = _setup(mol, cfg, 6)
    m = _model(mol, cfg, flat, cuda_device)
    J, _, lp = m.grad(torch.as_tensor(x, device=cuda_device), per_walker=True)
    Jr, lpr = oracle_param_jacobian(flat, cfg, mol, x)
    J = J.double().cpu().numpy()
    rel = np.linalg.norm(J - Jr, axis=1) / np.linalg.norm(Jr, axis=1)
    np.testing.assert_allclose(lp.cpu().numpy(), lpr, rtol=1e-4, atol=1e-4)
    assert np.median(rel) <= 1e-4 and rel.max() <= 5e-3, rel
    if envelope == "diagonal":  # the sigma rows are there and not trivially zero
        leaves = P.ferminet_leaves(cfg, mol.n_atoms)
        sizes = [int(np.prod(s)) for _, s in leaves]
        off = sum(sizes[:-1])
        assert np.abs(Jr[:, off:]).max() > 1e-3
        np.testing.assert_allclose(J[:, off:], Jr[:, off:], rtol=1e-3, atol=1e-4 * np.abs(Jr[:, off:]).max())


@pytest.mark.parametrize("envelope", ENVS)
@pytest.mark.parametrize("precision", ["fp32", "mixed"])
def test_psiformer(envelope, precision, cuda_device):
    """Psiformer (small widths) with the other envelopes: forward and E_L."""
    mol = S.lithium()
    cfg = P.PsiformerConfig(nspins=mol.nspins, ndets=3, num_layers=2, num_heads=4, heads_dim=16,
                            mlp_hidden_dims=[64], envelope=envelope)
    tree = _randomise(P.init_psiformer(cfg, mol.n_atoms, seed=0))
    flat = P.flatten(tree, P.psiformer_leaves(cfg, mol.n_atoms))
    m = _native.NativePsiformer(cfg, mol.atoms, mol.charges, precision=precision, device=cuda_device)
    assert m.param_count == flat.size
    m.set_params(torch.as_tensor(flat, device=cuda_device))
    x = S.init_walkers(mol, 32, seed=1)
    xd = torch.as_tensor(x, device=cuda_device)
    lp, sg, _ = m.forward(xd)
    out = m.local_energy(xd)
    oc = OPS.PsiformerConfig(nspins=cfg.nspins, ndets=cfg.ndets, num_layers=cfg.num_layers,
                             num_heads=cfg.num_heads, heads_dim=cfg.heads_dim,
                             mlp_hidden_dims=list(cfg.mlp_hidden_dims), envelope=cfg.envelope,
                             orbitals_spin_split=cfg.orbitals_spin_split, jastrow=cfg.jastrow)
    ref = OPS.evaluate(tree, oc, torch.as_tensor(x, dtype=torch.float64), mol.atoms)
    fl = OPS.evaluate_fl(tree, oc, torch.as_tensor(x, dtype=torch.float64), mol.atoms)
    ke = -0.5 * (fl["lap"] + (fl["grad"] ** 2).sum(-1))
    from oracle import hamiltonian as OH
    el = (ke + OH.potential_energy(torch.as_tensor(x, dtype=torch.float64), mol.atoms, mol.charges)).numpy()
    tol = 1e-5 if precision == "fp32" else 1e-3
    r = ref["logpsi"].numpy()
    assert np.array_equal(sg.cpu().numpy(), ref["sign_logpsi"].numpy())
    assert np.median(np.abs(lp.cpu().numpy() - r) / np.maximum(1.0, np.abs(r))) < tol
    err = np.abs(out["e_local"].cpu().numpy() - el)
    assert np.median(err) < (1e-4 if precision == "fp32" else 2e-3), np.median(err)
