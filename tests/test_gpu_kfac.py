"""Layer taps of the adjoint (qmc_grad_taps) and KFAC training on the GPU.

* For every dense tap, sum over a walker's applications of x (x) dy (with a
  ones column for the bias) is that walker's gradient block of the layer's
  kernel and bias, i.e. the per-walker Jacobian qmc_grad returns; the diagonal
  tap is the Jacobian's envelope columns.  FermiNet, Psiformer and LapNet
  models, every parameter in exactly one block.  This pins the statistics the KFAC
  blocks are built from (src/jaqmc/optimizer/kfac/curvature_blocks.py:94-137).
* KFAC training of the hydrogen atom reaches -0.5 Ha (the reference's
  tests/hydrogen/atom_test.py:38-52 asserts this for its KFAC optimizer);
  a KFAC step of a Psiformer / LapNet is a finite descent direction.
"""
import numpy as np
import pytest
import torch

from helpers import setup, small_cfg
from jaqmc_gb300 import _native
from jaqmc_gb300 import kfac as K
from jaqmc_gb300 import systems as S
from jaqmc_gb300 import vmc

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("nspins,split", [((2, 1), True), ((2, 1), False), ((2, 0), True)])
def test_taps_rebuild_the_per_walker_jacobian(nspins, split, cuda_device):
    mol = S.make_molecule("He", [2], [[0, 0, 0]], nspins) if nspins == (2, 0) else S.lithium()
    cfg = small_cfg(nspins, ndets=3, orbitals_spin_split=split)
    _, flat, x = setup(mol, cfg, 5)
    m = _native.NativeFermiNet(cfg, mol.atoms, mol.charges, device=cuda_device)
    m.set_params(torch.as_tensor(flat, device=cuda_device))
    m.set_grad_budget(2 * m.lib.qmc_workspace_size(m.h, _native.OP_GRAD, 1))  # several chunks
    xd = torch.as_tensor(x, device=cuda_device)
    J, _, lp = m.grad(xd, per_walker=True)
    taps, lp2 = m.layer_taps(xd)
    torch.testing.assert_close(lp2, lp)
    J = J.double()
    B = x.shape[0]
    covered = torch.zeros(J.shape[1], dtype=torch.bool, device=J.device)
    for t in taps:
        r = t["rows_per_walker"]
        if t["kind"] == "dense":
            xx = t["x"].double().view(B, r, -1)
            dy = t["dy"].double().view(B, r, -1)
            blk = torch.einsum("wri,wro->wio", xx, dy).reshape(B, -1)
            k0 = t["kernel_offset"]
            torch.testing.assert_close(blk, J[:, k0:k0 + blk.shape[1]], rtol=1e-4, atol=1e-5 * float(J.abs().max()))
            covered[k0:k0 + blk.shape[1]] = True
            if t["has_bias"]:
                b0 = t["bias_offset"]
                torch.testing.assert_close(dy.sum(1), J[:, b0:b0 + t["out_cols"]], rtol=1e-4,
                                           atol=1e-5 * float(J.abs().max()))
                covered[b0:b0 + t["out_cols"]] = True
        else:
            k0 = t["kernel_offset"]
            torch.testing.assert_close(t["dy"].double(), J[:, k0:k0 + t["out_cols"]], rtol=0, atol=0)
            covered[k0:k0 + t["out_cols"]] = True
    assert bool(covered.all())  # every parameter belongs to one block


def test_kfac_training_hydrogen(cuda_device):
    mol = S.hydrogen()
    wf = vmc.FermiNetWavefunction(nspins=(1, 0), ndets=2, hidden_dims_single=[16, 16], hidden_dims_double=[4, 4])
    x = torch.as_tensor(S.init_walkers(mol, 1024, seed=1), device="cuda")
    data = vmc.MoleculeData(x, mol.atoms, mol.charges)
    params = wf.init_params(data, 0)
    sampler = vmc.MCMCSampler(steps=10, initial_width=0.3)
    state = sampler.init(data, 7)
    kin = vmc.EuclideanKinetic(f_log_psi=wf)
    tot = vmc.TotalEnergy()
    lg = vmc.LossAndGrad(f_log_psi=wf)
    opt = K.KFACOptimizer(learning_rate=K.standard_schedule(rate=0.05, delay=200), f_log_psi=wf)
    for _ in range(5):
        d, _, state = sampler.step(wf.batch_log_prob(params, data), data, state)
        data = data.merge({"electrons": d.electrons})
    ost = opt.init(params, batched_data=vmc.BatchedData(data))
    energies = []
    for it in range(150):
        d, _, state = sampler.step(wf.batch_log_prob(params, data), data, state)
        data = data.merge({"electrons": d.electrons})
        bd = vmc.BatchedData(data)
        ws = {}
        ws.update(vmc.potential_energy(params, bd, ws, None, wf=wf)[0])
        ws.update(kin.evaluate_batch_walkers(params, bd, ws, None)[0])
        ws.update(tot.evaluate_batch_walkers(params, bd, ws, None)[0])
        g = lg.gradient(params, bd, ws["total_energy"])
        energies.append(vmc.mean_reduce({"e": ws["total_energy"]})["e"])
        upd, ost = opt.update(g["grads"], ost, params, batched_data=bd)
        params.flat.add_(upd.to(params.flat.dtype))
        params.touch()
    e = float(np.mean(energies[-20:]))
    assert abs(e + 0.5) < 5e-3, energies[-20:]


def _attn_model(kind, mol, cuda_device, **kw):
    from jaqmc_gb300 import params as P
    if kind == "psiformer":
        cfg = P.PsiformerConfig(nspins=mol.nspins, ndets=3, num_layers=2, num_heads=4, heads_dim=16,
                                mlp_hidden_dims=[64], **kw)
        tree = P.init_psiformer(cfg, mol.n_atoms, seed=0)
        flat = P.flatten(tree, P.psiformer_leaves(cfg, mol.n_atoms))
        m = _native.NativePsiformer(cfg, mol.atoms, mol.charges, precision="fp32", device=cuda_device)
    else:
        cfg = P.LapNetConfig(nspins=mol.nspins, ndets=3, num_layers=2, num_heads=4, heads_dim=16, **kw)
        tree = P.init_lapnet(cfg, mol.n_atoms, seed=0)
        flat = P.flatten(tree, P.lapnet_leaves(cfg, mol.n_atoms))
        m = _native.NativeLapNet(cfg, mol.atoms, mol.charges, precision="fp32", device=cuda_device)
    m.set_params(torch.as_tensor(flat, device=cuda_device))
    return m


@pytest.mark.parametrize("kind,system,kw", [("psiformer", "Li", {}), ("psiformer", "CH4", {"envelope": "diagonal"}),
                                            ("lapnet", "Li", {}),
                                            ("lapnet", "CH4", {"use_backbone_bias": False, "use_input_bias": False})])
def test_attention_taps_rebuild_the_per_walker_jacobian(kind, system, kw, cuda_device):
    """Psiformer and LapNet taps: input projection, attention projections,
    MLP / update layers and orbitals as dense taps, the LayerNorms and the
    envelope / Jastrow tail as diagonal taps, rebuilding qmc_grad's Jacobian."""
    mol = S.SYSTEMS[system]()
    m = _attn_model(kind, mol, cuda_device, **kw)
    m.set_grad_budget(2 * m.lib.qmc_workspace_size(m.h, _native.OP_GRAD, 1))  # several chunks
    xd = torch.as_tensor(S.init_walkers(mol, 5, seed=1), device=cuda_device)
    J, _, lp = m.grad(xd, per_walker=True)
    taps, lp2 = m.layer_taps(xd)
    torch.testing.assert_close(lp2, lp)
    J = J.double()
    B = xd.shape[0]
    covered = torch.zeros(J.shape[1], dtype=torch.bool, device=J.device)
    for t in taps:
        r = t["rows_per_walker"]
        if t["kind"] == "dense":
            xx = t["x"].double().view(B, r, -1)
            dy = t["dy"].double().view(B, r, -1)
            blk = torch.einsum("wri,wro->wio", xx, dy).reshape(B, -1)
            k0 = t["kernel_offset"]
            torch.testing.assert_close(blk, J[:, k0:k0 + blk.shape[1]], rtol=1e-4, atol=1e-5 * float(J.abs().max()))
            covered[k0:k0 + blk.shape[1]] = True
            if t["has_bias"]:
                b0 = t["bias_offset"]
                torch.testing.assert_close(dy.sum(1), J[:, b0:b0 + t["out_cols"]], rtol=1e-4,
                                           atol=1e-5 * float(J.abs().max()))
                covered[b0:b0 + t["out_cols"]] = True
        else:
            k0 = t["kernel_offset"]
            torch.testing.assert_close(t["dy"].double(), J[:, k0:k0 + t["out_cols"]], rtol=0, atol=0)
            covered[k0:k0 + t["out_cols"]] = True
    assert bool(covered.all())


@pytest.mark.parametrize("kind", ["psiformer", "lapnet"])
def test_kfac_step_on_attention_models(kind, cuda_device):
    """KFAC updates of a Psiformer / LapNet wavefunction through the host
    mirror: finite, and a descent direction (u . g < 0, the preconditioner is
    positive definite)."""
    mol = S.lithium()
    small = dict(ndets=2, num_layers=1, num_heads=4, heads_dim=16, precision="fp32")
    if kind == "psiformer":
        wf = vmc.PsiformerWavefunction(nspins=mol.nspins, mlp_hidden_dims=[64], **small)
    else:
        wf = vmc.LapNetWavefunction(nspins=mol.nspins, **small)
    x = torch.as_tensor(S.init_walkers(mol, 256, seed=1), device=cuda_device)
    data = vmc.MoleculeData(x, mol.atoms, mol.charges)
    params = wf.init_params(data, 0)
    kin = vmc.EuclideanKinetic(f_log_psi=wf)
    tot = vmc.TotalEnergy()
    lg = vmc.LossAndGrad(f_log_psi=wf)
    opt = K.KFACOptimizer(learning_rate=0.02, f_log_psi=wf)
    bd = vmc.BatchedData(data)
    ost = opt.init(params, batched_data=bd)
    for _ in range(2):
        ws = {}
        ws.update(vmc.potential_energy(params, bd, ws, None, wf=wf)[0])
        ws.update(kin.evaluate_batch_walkers(params, bd, ws, None)[0])
        ws.update(tot.evaluate_batch_walkers(params, bd, ws, None)[0])
        g = lg.gradient(params, bd, ws["total_energy"])["grads"]
        upd, ost = opt.update(g, ost, params, batched_data=bd)
        assert torch.isfinite(upd).all()
        assert float((upd.double() * g.double()).sum()) < 0.0
        params.flat.add_(upd.to(params.flat.dtype))
        params.touch()
