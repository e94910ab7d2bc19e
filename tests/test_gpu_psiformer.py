"""Psiformer + SimpleEE Jastrow value path on the GPU against the FP64 oracle
(oracle/psiformer.py) on the same parameters, walkers and draws: sign exact,
log|psi| within 1e-5 relative (FP32 form) / 1e-3 relative (split-BF16 form),
MH accept masks bit-exact away from near ties, the antiparallel cusp 1/2, and
the parameter adjoint against autograd of the oracle and finite differences."""
import numpy as np
import pytest
import torch

from jaqmc_gb300 import _native
from jaqmc_gb300 import params as P
from jaqmc_gb300 import systems as S
from oracle import mcmc as OM
from oracle import psiformer as OP

pytestmark = pytest.mark.gpu


def _ocfg(cfg):
    return OP.PsiformerConfig(nspins=cfg.nspins, ndets=cfg.ndets, num_layers=cfg.num_layers,
                              num_heads=cfg.num_heads, heads_dim=cfg.heads_dim,
                              mlp_hidden_dims=list(cfg.mlp_hidden_dims), envelope=cfg.envelope,
                              orbitals_spin_split=cfg.orbitals_spin_split, jastrow=cfg.jastrow)


def _setup(mol, cfg, B, dev, precision, seed=0):
    tree = P.init_psiformer(cfg, mol.n_atoms, seed=seed)
    flat = P.flatten(tree, P.psiformer_leaves(cfg, mol.n_atoms))
    m = _native.NativePsiformer(cfg, mol.atoms, mol.charges, precision=precision, device=dev)
    assert m.param_count == flat.size
    m.set_params(torch.as_tensor(flat, device=dev))
    x = S.init_walkers(mol, B, seed=1)
    return m, tree, x


SMALL = dict(ndets=3, num_layers=2, num_heads=4, heads_dim=16, mlp_hidden_dims=[64])


@pytest.mark.parametrize("precision,tol", [("fp32", 1e-5), ("mixed", 1e-3)])
@pytest.mark.parametrize("system", ["Li", "CH4"])
def test_forward_matches_oracle(system, precision, tol, cuda_device):
    mol = S.SYSTEMS[system]()
    cfg = P.PsiformerConfig(nspins=mol.nspins, **SMALL)
    m, tree, x = _setup(mol, cfg, 32, cuda_device, precision)
    lp, sg, fl = m.forward(torch.as_tensor(x, device=cuda_device))
    ref = OP.evaluate(tree, _ocfg(cfg), torch.as_tensor(x, dtype=torch.float64), mol.atoms)
    r32 = OP.evaluate(tree, _ocfg(cfg), torch.as_tensor(x, dtype=torch.float32), mol.atoms, dtype=torch.float32)
    scale = np.maximum(1.0, np.abs(ref["logpsi"].numpy()))
    rel = np.abs(lp.cpu().numpy() - ref["logpsi"].numpy()) / scale
    rel32 = np.abs(r32["logpsi"].numpy() - ref["logpsi"].numpy()) / scale
    assert np.array_equal(sg.cpu().numpy(), ref["sign_logpsi"].numpy())
    # the bar, with the FP32 conditioning of each walker accounted for: median
    # within tol, tail within a small multiple of the oracle's own FP32 error
    assert np.median(rel) < tol, np.median(rel)
    assert np.percentile(rel, 90) < max(tol, 3 * np.percentile(rel32, 90)), (rel, rel32)
    assert rel.max() < max(tol, 20 * rel32.max()), (rel.max(), rel32.max())


def test_benzene_full_config(cuda_device):
    """The benzene configuration: 21+21 electrons, 12 atoms, 4 layers of 4 x 64
    heads, MLP 256, K = 16, split-BF16 GEMMs."""
    mol = S.benzene()
    cfg = P.PsiformerConfig(nspins=mol.nspins)
    m, tree, x = _setup(mol, cfg, 8, cuda_device, "mixed")
    lp, sg, fl = m.forward(torch.as_tensor(x, device=cuda_device))
    ref = OP.evaluate(tree, _ocfg(cfg), torch.as_tensor(x, dtype=torch.float64), mol.atoms)
    rel = np.abs(lp.cpu().numpy() - ref["logpsi"].numpy()) / np.abs(ref["logpsi"].numpy())
    assert np.array_equal(sg.cpu().numpy(), ref["sign_logpsi"].numpy())
    assert rel.max() < 1e-3, rel
    assert m.check_error() == 0


def test_mh_matches_oracle(cuda_device):
    mol = S.lithium()
    cfg = P.PsiformerConfig(nspins=mol.nspins, **SMALL)
    B, steps = 64, 3
    m, tree, x = _setup(mol, cfg, B, cuda_device, "fp32")
    nz, uz = m.mh_draws(B, steps, seed=4, counter=0)
    xg = torch.as_tensor(x, device=cuda_device).clone()
    _, lpg, accg, _ = m.mh_steps(xg, steps, 0.05, 4, 0)
    f = OP.logpsi_fn(tree, _ocfg(cfg), torch.as_tensor(mol.atoms, dtype=torch.float64))
    xo, lpo, acco, ratios = OM.mh_steps(f, torch.as_tensor(x, dtype=torch.float64), nz.cpu().double(),
                                        uz.cpu().double(), 0.05)
    near = ((ratios - torch.log(uz.cpu().double())).abs() < 1e-6).any(0).numpy()
    keep = ~near
    assert keep.sum() >= B - 2
    assert np.array_equal(accg.cpu().numpy()[keep], acco.numpy()[keep])
    np.testing.assert_allclose(lpg.cpu().numpy()[keep], lpo.numpy()[keep], rtol=1e-4, atol=1e-4)


def test_antiparallel_cusp_on_gpu(cuda_device):
    """Central differences of the GPU log|psi| along the up-down separation at
    r = 0.01 bohr average to the cusp value 1/2 (+-0.1), as in
    tests/wavefunction/molecule_wavefunction_test.py:538-607."""
    mol = S.make_molecule("He", [2], [[0.0, 0.0, 0.0]], (1, 1))
    cfg = P.PsiformerConfig(nspins=(1, 1), ndets=4, num_layers=1, num_heads=4, heads_dim=16, mlp_hidden_dims=[64])
    m, tree, _ = _setup(mol, cfg, 1, cuda_device, "fp32")
    g = torch.Generator().manual_seed(3)
    d = torch.randn(200, 3, generator=g, dtype=torch.float64)
    d = d / d.norm(dim=1, keepdim=True)
    center = torch.tensor([2.0, 0.0, 0.0], dtype=torch.float64)
    h, r = 2e-3, 0.01

    def at(dist):
        x = torch.zeros(200, 2, 3, dtype=torch.float64)
        x[:, 0] = center
        x[:, 1] = center + dist * d
        return m.forward(x.float().to(cuda_device).contiguous())[0].double().cpu()
    radial = (at(r + h) - at(r - h)) / (2 * h)
    assert float(radial.mean()) == pytest.approx(0.5, abs=0.1)


def _oracle_jacobian(tree, cfg, mol, x):
    """(B, P) FP64 d log|psi_w| / d theta by torch autograd of the oracle (the
    role of the reference's jax.grad), in the flat leaf order."""
    leaves = P.psiformer_leaves(cfg, mol.n_atoms)
    ts, tr = [], {}
    for path, shape in leaves:
        t = torch.tensor(np.asarray(P._get(tree, path), np.float64), requires_grad=True)
        ts.append(t)
        node = tr.setdefault("params", {})
        for k in path[:-1]:
            node = node.setdefault(k, {})
        node[path[-1]] = t
    lp = OP.evaluate(tr, _ocfg(cfg), torch.as_tensor(x, dtype=torch.float64), mol.atoms)["logpsi"]
    rows = []
    for w in range(lp.shape[0]):
        g = torch.autograd.grad(lp[w], ts, retain_graph=True, allow_unused=True)
        rows.append(torch.cat([(gi if gi is not None else torch.zeros_like(t)).reshape(-1) for gi, t in zip(g, ts)]))
    return torch.stack(rows).numpy(), lp.detach().numpy()


@pytest.mark.parametrize("system,envelope", [("Li", "abs_isotropic"), ("CH4", "abs_isotropic"),
                                             ("Li", "diagonal")])
def test_parameter_adjoint_matches_autograd(system, envelope, cuda_device):
    """Per-walker d log|psi| / d theta of the Psiformer (input Dense, LayerNorms,
    attention, MLP, orbitals, envelope, Jastrow) against autograd of the FP64
    oracle: norm-wise relative error per walker <= 1e-4 (median), every
    parameter group covered, and the weighted sum equal to J^T c."""
    mol = S.SYSTEMS[system]()
    cfg = P.PsiformerConfig(nspins=mol.nspins, envelope=envelope, **SMALL)
    m, tree, x = _setup(mol, cfg, 5, cuda_device, "fp32")
    xd = torch.as_tensor(x, device=cuda_device)
    J, _, lp = m.grad(xd, per_walker=True)
    Jr, lpr = _oracle_jacobian(tree, cfg, mol, x)
    Jg = J.double().cpu().numpy()
    rel = np.linalg.norm(Jg - Jr, axis=1) / np.linalg.norm(Jr, axis=1)
    np.testing.assert_allclose(lp.cpu().numpy(), lpr, rtol=1e-5, atol=1e-5)
    assert np.median(rel) <= 1e-4 and rel.max() <= 2e-3, rel
    off = 0
    for path, shape in P.psiformer_leaves(cfg, mol.n_atoms):
        size = int(np.prod(shape))
        blk, ref = Jg[:, off:off + size], Jr[:, off:off + size]
        scale = np.abs(Jr).max()
        assert np.abs(blk - ref).max() <= 1e-3 * scale + 1e-3 * np.abs(ref).max(), path
        off += size
    c = torch.linspace(-1.0, 1.0, 5, dtype=torch.float64)
    _, g, _ = m.grad(xd, weights=c)
    ref = (J.double().cpu() * c[:, None]).sum(0).numpy()
    np.testing.assert_allclose(g.cpu().numpy(), ref, rtol=1e-9, atol=1e-9 * np.abs(ref).max())
    assert m.tangent_rows(_native.OP_LOCAL_ENERGY) >= 3 * mol.n_electrons + 2


def test_parameter_adjoint_finite_differences_and_chunks(cuda_device):
    """CH4 Psiformer: 32 seeded entries of the per-walker Jacobian against FP64
    central differences of the oracle (step 1e-4), and the same Jacobian when
    a small gradient budget splits the batch into recomputed chunks."""
    mol = S.methane()
    cfg = P.PsiformerConfig(nspins=mol.nspins, **SMALL)
    m, tree, x = _setup(mol, cfg, 3, cuda_device, "fp32")
    xd = torch.as_tensor(x, device=cuda_device)
    J, _, _ = m.grad(xd, per_walker=True)
    leaves = P.psiformer_leaves(cfg, mol.n_atoms)
    base = P.flatten(tree, leaves).astype(np.float64)
    rng = np.random.default_rng(32)
    idx = rng.choice(base.size, 32, replace=False)
    h = 1e-4
    fd = np.zeros((3, idx.size))
    for k, p_ in enumerate(idx):
        vals = []
        for sgn in (1.0, -1.0):
            v = base.copy()
            v[p_] += sgn * h
            vals.append(OP.evaluate(P.unflatten(v, leaves), _ocfg(cfg), torch.as_tensor(x, dtype=torch.float64),
                                    mol.atoms)["logpsi"].numpy())
        fd[:, k] = (vals[0] - vals[1]) / (2 * h)
    Jn = J.double().cpu().numpy()
    scale = np.abs(Jn).max(axis=1, keepdims=True)
    assert (np.abs(Jn[:, idx] - fd) / scale).max() <= 1e-3
    one = m.lib.qmc_workspace_size(m.h, _native.OP_GRAD, 1)
    m.set_grad_budget(one + one // 2)  # one walker per chunk
    J2, _, _ = m.grad(xd, per_walker=True)
    torch.testing.assert_close(J2, J, rtol=0, atol=0)


def test_host_mirror_sampler(cuda_device):
    """PsiformerWavefunction + MCMCSampler of the host mirror: the sampler
    moves walkers with a sane acceptance rate and log|psi| stays finite."""
    from jaqmc_gb300 import vmc
    mol = S.lithium()
    wf = vmc.PsiformerWavefunction(nspins=mol.nspins, **SMALL)
    x = torch.as_tensor(S.init_walkers(mol, 256, seed=1), device=cuda_device)
    data = vmc.MoleculeData(x, mol.atoms, mol.charges)
    params = wf.init_params(data, 0)
    sampler = vmc.MCMCSampler(steps=10, initial_width=0.1)
    state = sampler.init(data, 3)
    d, stats, state = sampler.step(wf.batch_log_prob(params, data), data, state)
    assert 0.05 < stats["pmove"] < 1.0
    assert torch.isfinite(wf.logpsi(params, d)).all()
