"""The FP32 CUDA path against the committed golden fixtures
(tests/golden/*.npz: seeded walkers, FP64 oracle values and the oracle's own
FP32 values), through the C ABI.  Bars as in the live-oracle tests: sign
exact; log|psi| and E_L per walker within 1e-5 relative / 1e-4 Ha at the
median, tails within a small multiple of the FP32 oracle's own error; the
potential within 1e-5 relative; the benzene configuration within 2e-3
relative (E_L) and 1e-3 (log|psi|)."""
import glob
import json
import os
import sys

import numpy as np
import pytest
import torch

from jaqmc_gb300 import _native

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden as G  # noqa: E402

pytestmark = pytest.mark.gpu

FIXTURES = sorted(glob.glob(os.path.join(HERE, "golden", "*.npz")))
MH = [f for f in FIXTURES if os.path.basename(f).startswith("mh_")]
GRAD = [f for f in FIXTURES if os.path.basename(f).startswith("grad_")]
VALUE = [f for f in FIXTURES if f not in MH and f not in GRAD]
MODELS = {"ferminet": _native.NativeFermiNet, "psiformer": _native.NativePsiformer, "lapnet": _native.NativeLapNet}


@pytest.mark.parametrize("path", GRAD, ids=lambda p: os.path.basename(p)[:-4])
def test_grad_matches_fixture(path, cuda_device):
    """The adjoint's per-walker d log|psi| / d theta against the FP64 oracle's
    on the fixture's 64 entries (error <= 1e-3 of each walker's largest
    component) and along its 8 seeded unit directions (RMS error <= 2e-2 of
    the oracle's |J| / sqrt(P): the live test's worst-walker bar of 1e-2 on
    the whole vector, with room for the scatter of an 8-direction estimate)."""
    z = np.load(path)
    meta = json.loads(str(z["meta"]))
    case, B, seed, entries, projections = G.GRAD_CASES[meta["case"]]
    mol, cfg, _, flat, _ = G.build(case)
    assert G.params_sha(flat) == meta["params_sha256"]
    m = _native.NativeFermiNet(cfg, mol.atoms, mol.charges, device=cuda_device)
    m.set_params(torch.as_tensor(flat, device=cuda_device))
    J, _, lp = m.grad(torch.as_tensor(z["walkers"], device=cuda_device), per_walker=True)
    assert m.check_error() == 0
    J = J.double().cpu().numpy()
    idx, R = G.grad_probes(flat.size, seed, entries, projections)
    assert np.array_equal(idx, z["entries"])
    scale = np.abs(J).max(axis=1, keepdims=True)
    assert (np.abs(J[:, idx] - z["jacobian_entries"]) / scale).max() <= 1e-3
    rms = np.sqrt(((J @ R - z["projections"]) ** 2).mean(axis=1))
    assert (rms / (z["jacobian_norm"] / np.sqrt(flat.size))).max() <= 2e-2
    np.testing.assert_allclose(lp.cpu().numpy(), z["logpsi"], rtol=1e-4, atol=1e-4)


@pytest.mark.parametrize("path", MH, ids=lambda p: os.path.basename(p)[:-4])
def test_mh_matches_fixture(path, cuda_device):
    """The fixture's Philox draws injected into qmc_mh_steps: accept counts
    bit-exact on the walkers with no near tie (|ratio - log u| < 1e-6 at any
    step, excluded and counted), positions within 1e-5, 2 log|psi| within 1e-4."""
    z = np.load(path)
    meta = json.loads(str(z["meta"]))
    mol, cfg, _, flat, _ = G.build(meta["model_case"])
    assert G.params_sha(flat) == meta["params_sha256"]
    m = MODELS[meta["model"]](cfg, mol.atoms, mol.charges, precision="fp32", device=cuda_device)
    m.set_params(torch.as_tensor(flat, device=cuda_device))
    xg = torch.as_tensor(z["walkers"], device=cuda_device).clone()
    nz = torch.as_tensor(z["normals"], device=cuda_device)
    uz = torch.as_tensor(z["uniforms"], device=cuda_device)
    _, lpg, accg, _ = m.mh_steps(xg, meta["steps"], meta["stddev"], meta["seed"], 0, normals=nz, uniforms=uz)
    assert m.check_error() == 0
    near = (np.abs(z["ratios"] - np.log(z["uniforms"].astype(np.float64))) < 1e-6).any(0)
    keep = ~near
    assert keep.sum() >= meta["walkers"] - 2
    assert np.array_equal(accg.cpu().numpy()[keep], z["accepts"][keep])
    np.testing.assert_allclose(xg.cpu().numpy()[keep], z["x_final"][keep], atol=1e-5)
    np.testing.assert_allclose(lpg.cpu().numpy()[keep], z["log_prob"][keep], rtol=1e-4, atol=1e-4)


@pytest.mark.parametrize("path", VALUE, ids=lambda p: os.path.basename(p)[:-4])
def test_fp32_path_matches_fixture(path, cuda_device):
    z = np.load(path)
    meta = json.loads(str(z["meta"]))
    mol, cfg, _, flat, _ = G.build(meta["case"])
    assert G.params_sha(flat) == meta["params_sha256"]
    m = MODELS[meta["model"]](cfg, mol.atoms, mol.charges, precision="fp32", device=cuda_device)
    m.set_params(torch.as_tensor(flat, device=cuda_device))
    x = torch.as_tensor(z["walkers"], device=cuda_device)
    lp, sg, _ = m.forward(x)
    out = m.local_energy(x)
    assert m.check_error() == 0
    assert np.array_equal(sg.cpu().numpy(), z["sign"])
    ref = z["logpsi"]
    err = np.abs(lp.cpu().double().numpy() - ref)
    e32 = np.abs(z["logpsi_fp32"] - ref)
    el = out["e_local"].cpu().double().numpy()
    eerr = np.abs(el - z["e_local"])
    ee32 = np.abs(z["e_local_fp32"] - z["e_local"])
    np.testing.assert_allclose(out["potential"].cpu().numpy(), z["potential"], rtol=1e-5, atol=1e-5)
    if meta["system"] == "C6H6":
        assert (eerr / np.abs(z["e_local"])).max() < 2e-3
        np.testing.assert_allclose(lp.cpu().numpy(), ref, rtol=1e-3)
        return
    tol = 1e-5 * np.maximum(1.0, np.abs(ref)).max()
    assert np.median(err) <= 3 * np.median(e32) + tol
    assert err.max() <= 20 * e32.max() + 10 * tol
    assert np.median(eerr) <= 3 * np.median(ee32) + 1e-4
    assert np.quantile(eerr, 0.9) <= 3 * np.quantile(ee32, 0.9) + 1e-4
    assert eerr.max() <= 20 * ee32.max() + 1e-3
    assert abs(el.mean() - z["e_local"].mean()) <= 3 * ee32.mean() + 5e-4
