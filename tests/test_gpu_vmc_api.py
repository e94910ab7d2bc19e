"""End-to-end use of the reference-shaped host API on the GPU.

* VMC training of the hydrogen atom with FermiNet through FermiNetWavefunction,
  MCMCSampler, the energy estimators and LossAndGrad (Adam on the flat
  parameters) reaches -0.5 Ha (tests/hydrogen/atom_test.py:38-52 asserts the
  same for its own ansatz).
* The estimator pipeline's kinetic + potential equals qmc_local_energy.
* The torch.autograd.Function and the torch.library custom op give the adjoint
  gradient.
"""
import numpy as np
import pytest
import torch

from jaqmc_gb300 import _native, torch_ops
from jaqmc_gb300 import systems as S
from jaqmc_gb300 import vmc

pytestmark = pytest.mark.gpu


def _system(mol, walkers, seed=1):
    x = torch.as_tensor(S.init_walkers(mol, walkers, seed=seed), device="cuda")
    return vmc.MoleculeData(x, mol.atoms, mol.charges)


def test_hydrogen_training_reaches_exact_energy(cuda_device):
    mol = S.hydrogen()
    wf = vmc.FermiNetWavefunction(nspins=(1, 0), ndets=2, hidden_dims_single=[16, 16], hidden_dims_double=[4, 4])
    data = _system(mol, 1024)
    params = wf.init_params(data, 0)
    sampler = vmc.MCMCSampler(steps=10, initial_width=0.3)
    state = sampler.init(data, 7)
    kin = vmc.EuclideanKinetic(f_log_psi=wf)
    tot = vmc.TotalEnergy()
    lg = vmc.LossAndGrad(f_log_psi=wf)
    opt = torch.optim.Adam([params.flat], lr=2e-2)
    for _ in range(5):  # burn-in
        d, _, state = sampler.step(wf.batch_log_prob(params, data), data, state)
        data = data.merge({"electrons": d.electrons})
    energies = []
    for it in range(400):
        d, stats, state = sampler.step(wf.batch_log_prob(params, data), data, state)
        data = data.merge({"electrons": d.electrons})
        bd = vmc.BatchedData(data)
        ws = {}
        ws.update(vmc.potential_energy(params, bd, ws, None, wf=wf)[0])
        ws.update(kin.evaluate_batch_walkers(params, bd, ws, None)[0])
        ws.update(tot.evaluate_batch_walkers(params, bd, ws, None)[0])
        g = lg.gradient(params, bd, ws["total_energy"])
        energies.append(vmc.mean_reduce({"e": ws["total_energy"]})["e"])
        opt.zero_grad()
        params.flat.grad = g["grads"].to(torch.float32)
        opt.step()
        params.touch()
    e = float(np.mean(energies[-20:]))
    assert abs(e + 0.5) < 5e-3, energies[-20:]
    assert 0.3 < stats["pmove"] < 1.0


def test_estimators_match_local_energy(cuda_device):
    mol = S.methane()
    wf = vmc.FermiNetWavefunction(nspins=mol.nspins)
    data = _system(mol, 64)
    params = wf.init_params(data, 0)
    bd = vmc.BatchedData(data)
    ws = {}
    ws.update(vmc.potential_energy(params, bd, ws, None, wf=wf)[0])
    ws.update(vmc.EuclideanKinetic(f_log_psi=wf).evaluate_batch_walkers(params, bd, ws, None)[0])
    ws.update(vmc.TotalEnergy().evaluate_batch_walkers(params, bd, ws, None)[0])
    m = wf.model(data, params)
    ref = m.local_energy(data.electrons)
    torch.testing.assert_close(ws["total_energy"], ref["e_local"])
    red = vmc.mean_reduce({"total_energy": ws["total_energy"]})
    assert set(red) == {"total_energy", "total_energy_var"}


def test_autograd_function_and_custom_op(cuda_device):
    mol = S.lithium()
    wf = vmc.FermiNetWavefunction(nspins=mol.nspins, ndets=3, hidden_dims_single=[8, 8], hidden_dims_double=[4, 4])
    data = _system(mol, 16)
    params = wf.init_params(data, 0)
    m = wf.model(data, params)
    w = torch.linspace(-1, 1, 16, device="cuda")
    flat = params.flat.clone().requires_grad_(True)
    lp = torch_ops.ferminet_logpsi(flat, data.electrons, m)
    (lp * w).sum().backward()
    _, g, _ = m.grad(data.electrons, weights=w.double())
    torch.testing.assert_close(flat.grad, g.float(), rtol=1e-5, atol=1e-6)
    h = torch_ops.register(m)
    flat2 = params.flat.clone().requires_grad_(True)
    lp2 = torch.ops.qmc_gb300.ferminet_logpsi(flat2, data.electrons, h)
    torch.testing.assert_close(lp2, lp.detach())
    (lp2 * w).sum().backward()
    torch.testing.assert_close(flat2.grad, flat.grad)


def test_evaluation_stage_exact_hydrogen(cuda_device, tmp_path):
    """Evaluation stage (sampling + energy estimators, no optimiser) on the
    exact hydrogen ground state psi ~ exp(-r): every local energy is -1/2, so
    the digest has E = -0.5 Ha with zero variance and the virial split
    <T> = -<V>/2 = 0.5 Ha (to sampling noise)."""
    import os

    import sys
    sys.path.insert(0, os.path.dirname(__file__))
    from helpers import hydrogenic_tree
    from jaqmc_gb300 import params as P

    mol = S.hydrogen()
    wf = vmc.FermiNetWavefunction(nspins=(1, 0), ndets=2, hidden_dims_single=[16, 16], hidden_dims_double=[4, 4])
    data = _system(mol, 2048)
    tree = hydrogenic_tree(wf.config, 1, sigma=1.0)
    params = vmc.DeviceParams(tree, P.ferminet_leaves(wf.config, 1), data.electrons.device)
    sampler = vmc.MCMCSampler(steps=10, initial_width=0.5)
    stage = vmc.EvaluationStage(wf, sampler, vmc.energy_pipeline(wf), iterations=20, burn_in=20,
                                save_dir=str(tmp_path), prefix="h")
    digest, stacked, *_ = stage.run(params, data, sampler.init(data, 11))
    assert set(stacked) >= {"total_energy", "total_energy_var", "energy:kinetic", "energy:potential"}
    assert stacked["total_energy"].shape == (20,)
    assert abs(float(digest["total_energy"]) + 0.5) < 1e-4
    assert float(digest["total_energy_var"]) < 1e-6
    assert abs(float(digest["energy:kinetic"]) - 0.5) < 0.03
    assert abs(float(digest["energy:potential"]) + 1.0) < 0.03
    assert os.path.exists(os.path.join(tmp_path, "h_digest.npz"))


def test_sr_on_adjoint_scores_matches_closed_form(cuda_device):
    """Robust SR (standard form) on the adjoint's per-walker scores equals
    (O^T O + lambda I)^-1 g solved in FP64 on the device."""
    from jaqmc_gb300 import sr as SR

    mol = S.lithium()
    wf = vmc.FermiNetWavefunction(nspins=mol.nspins, ndets=2, hidden_dims_single=[16, 16], hidden_dims_double=[4, 4])
    data = _system(mol, 96)
    params = wf.init_params(data, 0)
    bd = vmc.BatchedData(data)
    ws = {}
    ws.update(vmc.potential_energy(params, bd, ws, None, wf=wf)[0])
    ws.update(vmc.EuclideanKinetic(f_log_psi=wf).evaluate_batch_walkers(params, bd, ws, None)[0])
    ws.update(vmc.TotalEnergy().evaluate_batch_walkers(params, bd, ws, None)[0])
    st = vmc.LossAndGrad(f_log_psi=wf, per_walker=True).gradient(params, bd, ws["total_energy"])
    g, score = st["grads"], st["grad_logpsi"]
    lam = 1e-2
    opt = SR.RobustSR(learning_rate=1.0, damping=lam)
    delta, _ = opt.precondition(g, opt.init(g.numel(), g.device), score)
    O = score.double()
    O = (O - O.mean(0, keepdim=True)) / O.shape[0] ** 0.5
    ref = torch.linalg.solve(O.T @ O + lam * torch.eye(O.shape[1], dtype=O.dtype, device=O.device), g.double())
    assert float(torch.linalg.norm(delta - ref)) <= 1e-8 * float(torch.linalg.norm(ref))


def test_hydrogen_training_with_sr(cuda_device):
    """VMC on the hydrogen atom with robust SR over the adjoint's scores
    reaches -0.5 Ha."""
    from jaqmc_gb300 import sr as SR

    mol = S.hydrogen()
    wf = vmc.FermiNetWavefunction(nspins=(1, 0), ndets=2, hidden_dims_single=[16, 16], hidden_dims_double=[4, 4])
    data = _system(mol, 512)
    params = wf.init_params(data, 0)
    sampler = vmc.MCMCSampler(steps=10, initial_width=0.3)
    state = sampler.init(data, 7)
    kin, tot = vmc.EuclideanKinetic(f_log_psi=wf), vmc.TotalEnergy()
    lg = vmc.LossAndGrad(f_log_psi=wf, per_walker=True)
    opt = SR.RobustSR(learning_rate=0.1, max_norm=0.1, damping=1e-3)
    ostate = opt.init(params.flat.numel(), params.flat.device)
    for _ in range(5):
        d, _, state = sampler.step(wf.batch_log_prob(params, data), data, state)
        data = data.merge({"electrons": d.electrons})
    energies = []
    for it in range(300):
        d, _, state = sampler.step(wf.batch_log_prob(params, data), data, state)
        data = data.merge({"electrons": d.electrons})
        bd = vmc.BatchedData(data)
        ws = {}
        ws.update(vmc.potential_energy(params, bd, ws, None, wf=wf)[0])
        ws.update(kin.evaluate_batch_walkers(params, bd, ws, None)[0])
        ws.update(tot.evaluate_batch_walkers(params, bd, ws, None)[0])
        st = lg.gradient(params, bd, ws["total_energy"])
        energies.append(vmc.mean_reduce({"e": ws["total_energy"]})["e"])
        upd, ostate = opt.update(st["grads"], ostate, st["grad_logpsi"])
        with torch.no_grad():
            params.flat += upd.to(torch.float32)
        params.touch()
    e = float(np.mean(energies[-20:]))
    assert abs(e + 0.5) < 5e-3, energies[-20:]


def test_resume_from_checkpoint_continues_the_run(cuda_device, tmp_path):
    """A run checkpointed after 3 of 6 sampler + energy steps and resumed from
    the file (parameters, walkers, sampler state through
    load_reference_checkpoint) reproduces the uninterrupted run's walkers and
    energies bit for bit (src/jaqmc/utils/checkpoint.py:26-274 is the layout;
    src/jaqmc/workflow/stage/base.py:122-190 resumes at saved step + 1)."""
    mol = S.lithium()
    wf = vmc.FermiNetWavefunction(nspins=mol.nspins)
    data = _system(mol, 256)
    params = wf.init_params(data, 0)
    sampler = vmc.MCMCSampler(steps=10, initial_width=0.2, adapt_frequency=1000)
    kin = vmc.EuclideanKinetic(f_log_psi=wf)

    def step(params, data, state):
        d, _, state = sampler.step(wf.batch_log_prob(params, data), data, state)
        data = data.merge({"electrons": d.electrons})
        bd = vmc.BatchedData(data)
        ws = vmc.potential_energy(params, bd, {}, None, wf=wf)[0]
        ws.update(kin.evaluate_batch_walkers(params, bd, ws, None)[0])
        return data, state, (ws["energy:kinetic"] + ws["energy:potential"]).cpu().numpy()

    state = sampler.init(data, 5)
    ref = []
    for it in range(6):
        data, state, e = step(params, data, state)
        ref.append((data.electrons.cpu().numpy().copy(), e))
        if it == 2:
            path = tmp_path / "ckpt_000002.npz"
            vmc.save_checkpoint(path, 2, params, data, state)
    r = vmc.load_reference_checkpoint(path, wf, mol.n_atoms)
    assert r["step"] == 3
    data2 = vmc.MoleculeData(torch.as_tensor(r["electrons"], device="cuda"), mol.atoms, mol.charges)
    state2 = r["sampler_state"]
    for it in range(3, 6):
        data2, state2, e = step(r["params"], data2, state2)
        np.testing.assert_array_equal(data2.electrons.cpu().numpy(), ref[it][0])
        np.testing.assert_array_equal(e, ref[it][1])


def test_request_graph_matches_eager_calls(cuda_device):
    """RequestGraph (MH with a device counter + local energy + mean/variance,
    captured once and replayed) gives bitwise the results of the same eager
    calls from the same walkers and counter."""
    from jaqmc_gb300 import _native
    from jaqmc_gb300 import params as P
    from jaqmc_gb300 import systems as S
    mol = S.lithium()
    cfg = P.FermiNetConfig(nspins=mol.nspins, ndets=4, hidden_dims_single=[32, 32], hidden_dims_double=[8, 8])
    tree = P.init_ferminet(cfg, mol.n_atoms, seed=0)
    flat = torch.as_tensor(P.flatten(tree, P.ferminet_leaves(cfg, mol.n_atoms)), device=cuda_device)
    m = _native.NativeFermiNet(cfg, mol.atoms, mol.charges, precision="fp32", device=cuda_device)
    m.set_params(flat)
    x0 = torch.as_tensor(S.init_walkers(mol, 64, seed=1), device=cuda_device)
    xg = x0.clone()
    rg = _native.RequestGraph(m, xg, 5, 0.05, 3, counter=7)  # one eager request, then capture
    outs = [rg.run().clone() for _ in range(3)]
    torch.cuda.synchronize()
    xe = x0.clone()
    for k in range(4):
        m.mh_steps(xe, 5, 0.05, 3, 7 + 5 * k)
        mv = _native.reduce_mean_var(m.local_energy(xe)["e_local"])
        if k:
            assert torch.equal(mv, outs[k - 1]), k
    assert torch.equal(xe, xg)
    assert int(rg.counter.item()) == 7 + 20
