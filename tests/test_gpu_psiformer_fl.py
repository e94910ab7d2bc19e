"""Psiformer + SimpleEE Jastrow forward-Laplacian local energy on the GPU
against the FP64 forward-Laplacian oracle (oracle/psiformer.py evaluate_fl,
itself pinned against autograd) on the same parameters and walkers.

Bars: per-walker E_L within 1e-4 Ha for the bulk of the walkers, with the
tails held to a small multiple of the oracle's own FP32 error (a walker near a
node amplifies any FP32 rounding), the batch-mean E_L within 0.5 mHa,
log|psi| within 1e-4 and the potential within 1e-5 relative.  The split-BF16
form carries the GEMM operands to ~2^-16 relative, so its per-walker bar is
wider and its batch mean must show no bias beyond four standard errors."""
import json
import os

import numpy as np
import pytest
import torch

from jaqmc_gb300 import _native
from jaqmc_gb300 import params as P
from jaqmc_gb300 import systems as S
from oracle import hamiltonian as OH
from oracle import psiformer as OP

pytestmark = pytest.mark.gpu

STATS = os.environ.get("QMC_PARITY_STATS")


def _record(name, stats):
    if not STATS:
        return
    os.makedirs(os.path.dirname(os.path.abspath(STATS)), exist_ok=True)
    with open(STATS, "a") as f:
        f.write(json.dumps({"case": name, **stats}) + "\n")


def _ocfg(cfg):
    return OP.PsiformerConfig(nspins=cfg.nspins, ndets=cfg.ndets, num_layers=cfg.num_layers,
                              num_heads=cfg.num_heads, heads_dim=cfg.heads_dim,
                              mlp_hidden_dims=list(cfg.mlp_hidden_dims), envelope=cfg.envelope,
                              orbitals_spin_split=cfg.orbitals_spin_split, jastrow=cfg.jastrow)


def _setup(mol, cfg, B, dev, precision, seed=0):
    tree = P.init_psiformer(cfg, mol.n_atoms, seed=seed)
    flat = P.flatten(tree, P.psiformer_leaves(cfg, mol.n_atoms))
    m = _native.NativePsiformer(cfg, mol.atoms, mol.charges, precision=precision, device=dev)
    m.set_params(torch.as_tensor(flat, device=dev))
    x = S.init_walkers(mol, B, seed=1)
    return m, tree, x


def _oracle(tree, cfg, mol, x, dtype):
    xt = torch.as_tensor(x, dtype=dtype)
    r = OP.evaluate_fl(tree, _ocfg(cfg), xt, mol.atoms, dtype=dtype)
    ke = OH.kinetic_from_tangents(r["grad"], r["lap"])
    pe = OH.potential_energy(xt, mol.atoms, mol.charges)
    return {"e_local": (ke + pe).double().numpy(), "kinetic": ke.double().numpy(),
            "potential": pe.double().numpy(), "logpsi": r["logpsi"].double().numpy()}


SMALL = dict(ndets=3, num_layers=2, num_heads=4, heads_dim=16, mlp_hidden_dims=[64])


@pytest.mark.parametrize("precision", ["fp32", "mixed"])
@pytest.mark.parametrize("system", ["Li", "CH4"])
def test_local_energy_matches_oracle(system, precision, cuda_device):
    mol = S.SYSTEMS[system]()
    cfg = P.PsiformerConfig(nspins=mol.nspins, **SMALL)
    B = 32
    m, tree, x = _setup(mol, cfg, B, cuda_device, precision)
    out = m.local_energy(torch.as_tensor(x, device=cuda_device))
    assert m.check_error() == 0
    r64 = _oracle(tree, cfg, mol, x, torch.float64)
    r32 = _oracle(tree, cfg, mol, x, torch.float32)
    ref = r64["e_local"]
    got = out["e_local"].cpu().double().numpy()
    err = np.abs(got - ref)
    e32 = np.abs(r32["e_local"] - ref)
    se = (got - ref).std(ddof=1) / np.sqrt(B)
    _record(f"psiformer_local_energy/{system}/{precision}",
            {"max_abs": float(err.max()), "median_abs": float(np.median(err)),
             "frac_within_1e-4": float((err <= 1e-4).mean()), "mean_err": float(got.mean() - ref.mean()),
             "oracle32_max_abs": float(e32.max()), "oracle32_median_abs": float(np.median(e32)), "n": B})
    assert np.isfinite(got).all()
    assert (out["flags"].cpu().numpy() & _native.FLAG_NONFINITE).sum() == 0
    np.testing.assert_allclose(out["potential"].cpu().numpy(), r64["potential"], rtol=1e-5, atol=1e-5)
    if precision == "fp32":
        assert np.median(err) <= 3 * np.median(e32) + 1e-4, (np.median(err), np.median(e32))
        assert np.quantile(err, 0.9) <= 3 * np.quantile(e32, 0.9) + 1e-4
        assert err.max() <= 20 * e32.max() + 1e-3, (err.max(), e32.max())
        assert abs(got.mean() - ref.mean()) <= 3 * e32.mean() + 5e-4
        np.testing.assert_allclose(out["logpsi"].cpu().numpy(), r64["logpsi"], rtol=1e-4, atol=1e-4)
    else:
        assert np.median(err) <= 3 * np.median(e32) + 2e-3, (np.median(err), np.median(e32))
        assert abs(got.mean() - ref.mean()) <= max(5e-4, 4 * se), (got.mean() - ref.mean(), se)
        np.testing.assert_allclose(out["logpsi"].cpu().numpy(), r64["logpsi"], rtol=1e-3, atol=1e-3)


@pytest.mark.parametrize("precision", ["fp32", "mixed"])
def test_chunked_equals_whole(precision, cuda_device):
    """Walkers run in chunks under the energy budget; every per-walker result
    is bit-identical to the single-chunk call."""
    mol = S.methane()
    cfg = P.PsiformerConfig(nspins=mol.nspins, **SMALL)
    B = 20
    m, _, x = _setup(mol, cfg, B, cuda_device, precision)
    xd = torch.as_tensor(x, device=cuda_device)
    whole = m.local_energy(xd)
    one = m.workspace(_native.OP_LOCAL_ENERGY, 1)[1]
    m.set_energy_budget(3 * one)
    assert m.workspace(_native.OP_LOCAL_ENERGY, B)[1] <= 3 * one
    parts = m.local_energy(xd)
    for k in ("e_local", "kinetic", "potential", "logpsi"):
        assert torch.equal(whole[k], parts[k]), k


def test_benzene_full_config(cuda_device):
    """The benzene configuration (21+21 electrons, 12 atoms, 4 layers of 4 x 64
    heads, MLP 256, K = 16; T = 128 tangents per electron) on 16 walkers
    burnt in from |psi|^2, both forms against the FP64 oracle.

    FP32 form: per-walker |dE_L| median within 3x the FP32 oracle's own
    median (+ 0.1 mHa) and maximum within 3x its maximum (+ 1 mHa); batch mean
    within four paired standard errors (+ 0.1 mHa).
    Split-BF16 form: its error is the rounding of the GEMM and attention
    operands to hi + lo bf16 (about 2^-17 relative), which the kinetic energy
    amplifies to mHa per walker on this system.  The oracle with that operand
    rounding emulated (oracle/lap.py split_bf16_gemms) states the size to
    expect: the
    per-walker median within 3x the emulation's (+ 1 mHa), the maximum within
    5x (+ 10 mHa), and the batch mean unbiased: within max(0.5 mHa, 4 paired
    standard errors) of FP64."""
    from oracle import lap
    mol = S.benzene()
    cfg = P.PsiformerConfig(nspins=mol.nspins)
    B = 16
    tree = P.init_psiformer(cfg, mol.n_atoms, seed=0)
    flat = torch.as_tensor(P.flatten(tree, P.psiformer_leaves(cfg, mol.n_atoms)), device=cuda_device)
    models = {}
    for precision in ("mixed", "fp32"):
        m = _native.NativePsiformer(cfg, mol.atoms, mol.charges, precision=precision, device=cuda_device)
        m.set_params(flat)
        models[precision] = m
    xd = torch.as_tensor(S.init_walkers(mol, 256, seed=1), device=cuda_device)
    models["mixed"].mh_steps(xd, 200, 0.15, 1000, 0)
    xd = xd[:B].contiguous()
    x = xd.cpu().numpy()
    r64 = _oracle(tree, cfg, mol, x, torch.float64)
    r32 = _oracle(tree, cfg, mol, x, torch.float32)
    K0 = 4 * mol.n_atoms + 1
    with lap.split_bf16_gemms(lambda W: W.shape[0] != K0, attention=True):
        remu = _oracle(tree, cfg, mol, x, torch.float64)
    ref = r64["e_local"]
    e32 = np.abs(r32["e_local"] - ref)
    eemu = np.abs(remu["e_local"] - ref)
    for precision, m in models.items():
        out = m.local_energy(xd)
        assert m.check_error() == 0
        got = out["e_local"].cpu().double().numpy()
        d = got - ref
        err = np.abs(d)
        se = d.std(ddof=1) / np.sqrt(B)
        _record(f"psiformer_local_energy/C6H6/{precision}",
                {"max_abs": float(err.max()), "median_abs": float(np.median(err)), "mean_err": float(d.mean()),
                 "paired_se": float(se), "oracle32_median_abs": float(np.median(e32)),
                 "oracle32_max_abs": float(e32.max()), "emulated_median_abs": float(np.median(eemu)),
                 "emulated_max_abs": float(eemu.max()), "n": B})
        assert np.isfinite(got).all()
        np.testing.assert_allclose(out["logpsi"].cpu().numpy(), r64["logpsi"], rtol=1e-4 if precision == "fp32"
                                   else 1e-3)
        if precision == "fp32":
            assert np.median(err) <= 3 * np.median(e32) + 1e-4, (np.median(err), np.median(e32))
            assert err.max() <= 3 * e32.max() + 1e-3, (err.max(), e32.max())
            assert abs(d.mean()) <= 4 * se + 1e-4, (d.mean(), se)
        else:
            assert np.median(err) <= 3 * np.median(eemu) + 1e-3, (np.median(err), np.median(eemu))
            assert err.max() <= 5 * eemu.max() + 1e-2, (err.max(), eemu.max())
            assert abs(d.mean()) <= max(5e-4, 4 * se), (d.mean(), se)


def test_host_mirror_evaluation_stage(cuda_device, tmp_path):
    """PsiformerWavefunction through the host mirror's evaluation stage
    (sampling + kinetic / potential / total energy estimators): finite
    per-step energies, E = <T> + <V>, and the kinetic estimator equal to the
    library's local energy on the stage's final walkers."""
    from jaqmc_gb300 import vmc
    mol = S.lithium()
    wf = vmc.PsiformerWavefunction(nspins=mol.nspins, **SMALL)
    x = torch.as_tensor(S.init_walkers(mol, 256, seed=1), device=cuda_device)
    data = vmc.MoleculeData(x, mol.atoms, mol.charges)
    params = wf.init_params(data, 0)
    sampler = vmc.MCMCSampler(steps=5, initial_width=0.1)
    stage = vmc.EvaluationStage(wf, sampler, vmc.energy_pipeline(wf), iterations=4, burn_in=5,
                                save_dir=str(tmp_path), prefix="psi")
    digest, stacked, data_out, *_ = stage.run(params, data, sampler.init(data, 5))
    for k in ("total_energy", "energy:kinetic", "energy:potential"):
        assert np.isfinite(np.asarray(stacked[k])).all(), k
    assert abs(float(digest["total_energy"]) - float(digest["energy:kinetic"])
               - float(digest["energy:potential"])) < 1e-3 * max(1.0, abs(float(digest["total_energy"])))
    m = wf.model(data_out, params)
    out = m.local_energy(data_out.electrons.contiguous())
    ke = vmc.EuclideanKinetic(f_log_psi=wf).evaluate_batch_walkers(params, vmc.BatchedData(data_out), {}, None)[0]
    assert torch.equal(ke["energy:kinetic"], out["kinetic"])
