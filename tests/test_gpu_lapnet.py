"""LapNet + SimpleEE Jastrow on the GPU against the FP64 oracle
(oracle/lapnet.py, itself pinned against the brute-force Hessian trace) on the
same parameters, walkers and draws.

Bars, as for the Psiformer: sign exact; log|psi| within 1e-5 relative (FP32
form) / 1e-3 (split-BF16 form) with tails held to a small multiple of the
oracle's own FP32 error; per-walker E_L within 1e-4 Ha for the bulk of the
walkers (FP32 form), batch mean without bias beyond four standard errors
(split-BF16 form); potential within 1e-5 relative; MH accept masks
bit-exact away from near ties (|log ratio - log u| < 1e-6); the FP32
parameter adjoint against autograd of the FP64 oracle and central
differences."""
import json
import os

import numpy as np
import pytest
import torch

from jaqmc_gb300 import _native
from jaqmc_gb300 import params as P
from jaqmc_gb300 import systems as S
from oracle import hamiltonian as OH
from oracle import lapnet as OL
from oracle import mcmc as OM

pytestmark = pytest.mark.gpu

STATS = os.environ.get("QMC_PARITY_STATS")
SMALL = dict(ndets=3, num_layers=2, num_heads=4, heads_dim=16)


def _record(name, stats):
    if not STATS:
        return
    os.makedirs(os.path.dirname(os.path.abspath(STATS)), exist_ok=True)
    with open(STATS, "a") as f:
        f.write(json.dumps({"case": name, **stats}) + "\n")


def _ocfg(cfg):
    return OL.LapNetConfig(nspins=cfg.nspins, ndets=cfg.ndets, num_layers=cfg.num_layers, num_heads=cfg.num_heads,
                           heads_dim=cfg.heads_dim, num_local_updates=cfg.num_local_updates, envelope=cfg.envelope,
                           jastrow=cfg.jastrow, use_input_bias=cfg.use_input_bias,
                           use_backbone_bias=cfg.use_backbone_bias)


def _setup(mol, cfg, B, dev, precision, seed=0):
    tree = P.init_lapnet(cfg, mol.n_atoms, seed=seed)
    flat = P.flatten(tree, P.lapnet_leaves(cfg, mol.n_atoms))
    m = _native.NativeLapNet(cfg, mol.atoms, mol.charges, precision=precision, device=dev)
    assert m.param_count == flat.size
    m.set_params(torch.as_tensor(flat, device=dev))
    x = S.init_walkers(mol, B, seed=1)
    return m, tree, x


def _oracle(tree, cfg, mol, x, dtype, tangents=True):
    xt = torch.as_tensor(x, dtype=dtype)
    r = OL.evaluate(tree, _ocfg(cfg), xt, mol.atoms, dtype=dtype, tangents=tangents)
    out = {"logpsi": r["logpsi"].double().numpy(), "sign": r["sign_logpsi"].numpy()}
    if tangents:
        ke = OH.kinetic_from_tangents(r["grad"], r["lap"])
        pe = OH.potential_energy(xt, mol.atoms, mol.charges)
        out.update(e_local=(ke + pe).double().numpy(), potential=pe.double().numpy())
    return out


def _check_logpsi(lp, ref, r32, tol):
    scale = np.maximum(1.0, np.abs(ref))
    rel = np.abs(lp - ref) / scale
    rel32 = np.abs(r32 - ref) / scale
    assert np.median(rel) < tol, np.median(rel)
    assert np.percentile(rel, 90) < max(tol, 3 * np.percentile(rel32, 90)), (rel, rel32)
    assert rel.max() < max(tol, 20 * rel32.max()), (rel.max(), rel32.max())


@pytest.mark.parametrize("precision,tol", [("fp32", 1e-5), ("mixed", 1e-3)])
@pytest.mark.parametrize("system", ["Li", "CH4"])
def test_forward_matches_oracle(system, precision, tol, cuda_device):
    mol = S.SYSTEMS[system]()
    cfg = P.LapNetConfig(nspins=mol.nspins, **SMALL)
    m, tree, x = _setup(mol, cfg, 32, cuda_device, precision)
    lp, sg, _ = m.forward(torch.as_tensor(x, device=cuda_device))
    ref = _oracle(tree, cfg, mol, x, torch.float64, tangents=False)
    r32 = _oracle(tree, cfg, mol, x, torch.float32, tangents=False)
    assert np.array_equal(sg.cpu().numpy(), ref["sign"])
    _check_logpsi(lp.cpu().double().numpy(), ref["logpsi"], r32["logpsi"], tol)


@pytest.mark.parametrize("precision", ["fp32", "mixed"])
@pytest.mark.parametrize("system", ["Li", "CH4"])
def test_local_energy_matches_oracle(system, precision, cuda_device):
    mol = S.SYSTEMS[system]()
    cfg = P.LapNetConfig(nspins=mol.nspins, **SMALL)
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
    _record(f"lapnet_local_energy/{system}/{precision}",
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
        np.testing.assert_allclose(out["logpsi"].cpu().numpy(), r64["logpsi"], rtol=1e-4, atol=1e-4)
    else:
        assert np.median(err) <= 3 * np.median(e32) + 2e-3, (np.median(err), np.median(e32))
        assert abs(got.mean() - ref.mean()) <= max(5e-4, 4 * se), (got.mean() - ref.mean(), se)
        np.testing.assert_allclose(out["logpsi"].cpu().numpy(), r64["logpsi"], rtol=1e-3, atol=1e-3)


def test_without_biases_and_one_local_update(cuda_device):
    """use_input_bias = use_backbone_bias = False, one local update per layer,
    three layers, the isotropic envelope and no Jastrow: value and E_L."""
    mol = S.methane()
    cfg = P.LapNetConfig(nspins=mol.nspins, ndets=2, num_layers=3, num_heads=2, heads_dim=32, num_local_updates=1,
                         use_input_bias=False, use_backbone_bias=False, envelope="isotropic", jastrow="none")
    B = 16
    m, tree, x = _setup(mol, cfg, B, cuda_device, "fp32")
    xd = torch.as_tensor(x, device=cuda_device)
    lp, sg, _ = m.forward(xd)
    out = m.local_energy(xd)
    r64 = _oracle(tree, cfg, mol, x, torch.float64)
    r32 = _oracle(tree, cfg, mol, x, torch.float32)
    assert np.array_equal(sg.cpu().numpy(), r64["sign"])
    _check_logpsi(lp.cpu().double().numpy(), r64["logpsi"], r32["logpsi"], 1e-5)
    err = np.abs(out["e_local"].cpu().double().numpy() - r64["e_local"])
    e32 = np.abs(r32["e_local"] - r64["e_local"])
    assert np.median(err) <= 3 * np.median(e32) + 1e-4, (np.median(err), np.median(e32))


def test_default_config_nitrogen(cuda_device):
    """The reference defaults (4 layers, 4 heads x 64, K = 16, two local
    updates, biases on) on N2, both forms: log|psi| and E_L."""
    mol = S.nitrogen_dimer()
    cfg = P.LapNetConfig(nspins=mol.nspins)
    B = 4
    r64 = None
    for precision, tol in (("fp32", 2e-3), ("mixed", 2e-2)):
        m, tree, x = _setup(mol, cfg, B, cuda_device, precision)
        xd = torch.as_tensor(x, device=cuda_device)
        lp, sg, _ = m.forward(xd)
        out = m.local_energy(xd)
        assert m.check_error() == 0
        if r64 is None:
            r64 = _oracle(tree, cfg, mol, x, torch.float64)
        assert np.array_equal(sg.cpu().numpy(), r64["sign"])
        np.testing.assert_allclose(lp.cpu().numpy(), r64["logpsi"], rtol=1e-3)
        got = out["e_local"].cpu().double().numpy()
        err = np.abs(got - r64["e_local"]) / np.maximum(1.0, np.abs(r64["e_local"]))
        _record(f"lapnet_local_energy/N2-default/{precision}", {"rel_max": float(err.max()), "n": B})
        assert np.isfinite(got).all()
        assert err.max() < tol, (got, r64["e_local"])


def test_mh_matches_oracle(cuda_device):
    mol = S.lithium()
    cfg = P.LapNetConfig(nspins=mol.nspins, **SMALL)
    B, steps = 64, 3
    m, tree, x = _setup(mol, cfg, B, cuda_device, "fp32")
    nz, uz = m.mh_draws(B, steps, seed=4, counter=0)
    xg = torch.as_tensor(x, device=cuda_device).clone()
    _, lpg, accg, _ = m.mh_steps(xg, steps, 0.05, 4, 0)
    f = OL.logpsi_fn(tree, _ocfg(cfg), torch.as_tensor(mol.atoms, dtype=torch.float64))
    xo, lpo, acco, ratios = OM.mh_steps(f, torch.as_tensor(x, dtype=torch.float64), nz.cpu().double(),
                                        uz.cpu().double(), 0.05)
    near = ((ratios - torch.log(uz.cpu().double())).abs() < 1e-6).any(0).numpy()
    keep = ~near
    assert keep.sum() >= B - 2
    assert np.array_equal(accg.cpu().numpy()[keep], acco.numpy()[keep])
    np.testing.assert_allclose(lpg.cpu().numpy()[keep], lpo.numpy()[keep], rtol=1e-4, atol=1e-4)


def _oracle_jacobian(tree, cfg, mol, x):
    """(B, P) FP64 d log|psi_w| / d theta by torch autograd of the oracle (the
    role of the reference's jax.grad), in the flat leaf order."""
    leaves = P.lapnet_leaves(cfg, mol.n_atoms)
    ts, tr = [], {}
    for path, shape in leaves:
        t = torch.tensor(np.asarray(P._get(tree, path), np.float64), requires_grad=True)
        ts.append(t)
        node = tr.setdefault("params", {})
        for k in path[:-1]:
            node = node.setdefault(k, {})
        node[path[-1]] = t
    lp = OL.evaluate(tr, _ocfg(cfg), torch.as_tensor(x, dtype=torch.float64), mol.atoms)["logpsi"]
    rows = []
    for w in range(lp.shape[0]):
        g = torch.autograd.grad(lp[w], ts, retain_graph=True, allow_unused=True)
        rows.append(torch.cat([(gi if gi is not None else torch.zeros_like(t)).reshape(-1) for gi, t in zip(g, ts)]))
    return torch.stack(rows).numpy(), lp.detach().numpy()


@pytest.mark.parametrize("case", ["Li", "CH4", "CH4-nobias-1update", "Li-diagonal-3layers"])
def test_parameter_adjoint_matches_autograd(case, cuda_device):
    """Per-walker d log|psi| / d theta of LapNet (input projection, query/key,
    value, output and value-update projections, local updates of the
    individual stream, orbitals, envelope, Jastrow) against autograd of the
    FP64 oracle: norm-wise relative error per walker <= 1e-4 (median), every
    parameter leaf covered, and the weighted sum equal to J^T c."""
    system = case.split("-")[0]
    mol = S.SYSTEMS[system]()
    kw = dict(SMALL)
    if "nobias" in case:
        kw.update(use_input_bias=False, use_backbone_bias=False, num_local_updates=1, jastrow="none")
    if "diagonal" in case:
        kw.update(envelope="diagonal", num_layers=3)
    cfg = P.LapNetConfig(nspins=mol.nspins, **kw)
    m, tree, x = _setup(mol, cfg, 5, cuda_device, "fp32")
    xd = torch.as_tensor(x, device=cuda_device)
    J, _, lp = m.grad(xd, per_walker=True)
    Jr, lpr = _oracle_jacobian(tree, cfg, mol, x)
    Jg = J.double().cpu().numpy()
    rel = np.linalg.norm(Jg - Jr, axis=1) / np.linalg.norm(Jr, axis=1)
    _record(f"lapnet_adjoint/{case}", {"rel_median": float(np.median(rel)), "rel_max": float(rel.max())})
    # log|psi| to the forward parity bar: 1e-5 relative, or the FP32
    # oracle's own error on a badly conditioned walker
    r32 = _oracle(tree, cfg, mol, x, torch.float32, tangents=False)["logpsi"]
    _check_logpsi(lp.cpu().double().numpy(), lpr, r32, 1e-5)
    assert np.median(rel) <= 1e-4 and rel.max() <= 2e-3, rel
    off = 0
    scale = np.abs(Jr).max()
    for path, shape in P.lapnet_leaves(cfg, mol.n_atoms):
        size = int(np.prod(shape))
        blk, ref = Jg[:, off:off + size], Jr[:, off:off + size]
        assert np.abs(blk - ref).max() <= 1e-3 * scale + 1e-3 * np.abs(ref).max(), path
        off += size
    c = torch.linspace(-1.0, 1.0, 5, dtype=torch.float64)
    _, g, _ = m.grad(xd, weights=c)
    ref = (J.double().cpu() * c[:, None]).sum(0).numpy()
    np.testing.assert_allclose(g.cpu().numpy(), ref, rtol=1e-9, atol=1e-9 * np.abs(ref).max())


def test_parameter_adjoint_finite_differences_and_chunks(cuda_device):
    """CH4 LapNet: 32 seeded entries of the per-walker Jacobian against FP64
    central differences of the oracle (step 1e-4), and the same Jacobian when
    a small gradient budget splits the batch into recomputed chunks."""
    mol = S.methane()
    cfg = P.LapNetConfig(nspins=mol.nspins, **SMALL)
    m, tree, x = _setup(mol, cfg, 3, cuda_device, "fp32")
    xd = torch.as_tensor(x, device=cuda_device)
    J, _, _ = m.grad(xd, per_walker=True)
    leaves = P.lapnet_leaves(cfg, mol.n_atoms)
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
            vals.append(OL.evaluate(P.unflatten(v, leaves), _ocfg(cfg), torch.as_tensor(x, dtype=torch.float64),
                                    mol.atoms)["logpsi"].numpy())
        fd[:, k] = (vals[0] - vals[1]) / (2 * h)
    Jn = J.double().cpu().numpy()
    scale = np.abs(Jn).max(axis=1, keepdims=True)
    assert (np.abs(Jn[:, idx] - fd) / scale).max() <= 1e-3
    one = m.lib.qmc_workspace_size(m.h, _native.OP_GRAD, 1)
    m.set_grad_budget(one + one // 2)  # one walker per chunk
    J2, _, _ = m.grad(xd, per_walker=True)
    torch.testing.assert_close(J2, J, rtol=0, atol=0)


def test_host_mirror_evaluation_stage(cuda_device, tmp_path):
    """LapNetWavefunction through the host mirror's evaluation stage: finite
    per-step energies, E = <T> + <V>, and the kinetic estimator equal to the
    library's local energy on the stage's final walkers."""
    from jaqmc_gb300 import vmc
    mol = S.lithium()
    wf = vmc.LapNetWavefunction(nspins=mol.nspins, **SMALL)
    x = torch.as_tensor(S.init_walkers(mol, 256, seed=1), device=cuda_device)
    data = vmc.MoleculeData(x, mol.atoms, mol.charges)
    params = wf.init_params(data, 0)
    sampler = vmc.MCMCSampler(steps=5, initial_width=0.1)
    stage = vmc.EvaluationStage(wf, sampler, vmc.energy_pipeline(wf), iterations=4, burn_in=5,
                                save_dir=str(tmp_path), prefix="lapnet")
    digest, stacked, data_out, *_ = stage.run(params, data, sampler.init(data, 5))
    for k in ("total_energy", "energy:kinetic", "energy:potential"):
        assert np.isfinite(np.asarray(stacked[k])).all(), k
    assert abs(float(digest["total_energy"]) - float(digest["energy:kinetic"])
               - float(digest["energy:potential"])) < 1e-3 * max(1.0, abs(float(digest["total_energy"])))
    m = wf.model(data_out, params)
    out = m.local_energy(data_out.electrons.contiguous())
    ke = vmc.EuclideanKinetic(f_log_psi=wf).evaluate_batch_walkers(params, vmc.BatchedData(data_out), {}, None)[0]
    assert torch.equal(ke["energy:kinetic"], out["kinetic"])
