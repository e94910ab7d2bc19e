"""The golden fixtures (tests/golden/*.npz, written by tests/golden/make_golden.py)
on the CPU: the seeded parameters, walkers and Philox draws regenerate bit for
bit, and the FP64 oracle reproduces the stored log|psi|, sign, local energies
and MH updates."""
import glob
import json
import os
import sys

import numpy as np
import pytest
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden as G  # noqa: E402

FIXTURES = sorted(glob.glob(os.path.join(HERE, "golden", "*.npz")))
MH = [f for f in FIXTURES if os.path.basename(f).startswith("mh_")]
GRAD = [f for f in FIXTURES if os.path.basename(f).startswith("grad_")]
VALUE = [f for f in FIXTURES if f not in MH and f not in GRAD]


def test_every_case_has_a_fixture():
    grad_models = {c[0] for c in G.GRAD_CASES.values()}
    want = [c for c in G.CASES if c not in grad_models] + list(G.MH_CASES) + list(G.GRAD_CASES)
    assert sorted(os.path.basename(f)[:-4] for f in FIXTURES) == sorted(want)


@pytest.mark.parametrize("path", GRAD, ids=lambda p: os.path.basename(p)[:-4])
def test_oracle_reproduces_grad_fixture(path):
    z = np.load(path)
    meta = json.loads(str(z["meta"]))
    flat, x, v = G.oracle_grad(meta["case"])
    assert G.params_sha(flat) == meta["params_sha256"]
    assert np.array_equal(x.astype(np.float32), z["walkers"])
    assert np.array_equal(v["entries"], z["entries"])
    np.testing.assert_allclose(v["jacobian_entries"], z["jacobian_entries"], rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(v["projections"], z["projections"], rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(v["jacobian_norm"], z["jacobian_norm"], rtol=1e-10)
    np.testing.assert_allclose(v["logpsi"], z["logpsi"], rtol=1e-11)


@pytest.mark.parametrize("path", MH, ids=lambda p: os.path.basename(p)[:-4])
def test_oracle_reproduces_mh_fixture(path):
    z = np.load(path)
    meta = json.loads(str(z["meta"]))
    mol, cfg, tree, flat, x, normals, uniforms = G.build_mh(meta["case"])
    assert G.params_sha(flat) == meta["params_sha256"]
    assert np.array_equal(x.astype(np.float32), z["walkers"])
    assert np.array_equal(normals, z["normals"]) and np.array_equal(uniforms, z["uniforms"])
    v = G.oracle_mh(meta["case"], mol, cfg, tree, x, normals, uniforms)
    assert np.array_equal(v["accepts"], z["accepts"])
    np.testing.assert_allclose(v["x_final"], z["x_final"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(v["log_prob"], z["log_prob"], rtol=1e-11, atol=1e-10)


@pytest.mark.parametrize("path", VALUE, ids=lambda p: os.path.basename(p)[:-4])
def test_oracle_reproduces_fixture(path):
    z = np.load(path)
    meta = json.loads(str(z["meta"]))
    mol, cfg, tree, flat, x = G.build(meta["case"])
    assert G.params_sha(flat) == meta["params_sha256"]
    assert np.array_equal(x.astype(np.float32), z["walkers"])
    v = G.oracle_values(meta["case"], mol, cfg, tree, x, torch.float64)
    assert np.array_equal(v["sign"], z["sign"])
    np.testing.assert_allclose(v["logpsi"], z["logpsi"], rtol=1e-11, atol=1e-10)
    np.testing.assert_allclose(v["potential"], z["potential"], rtol=1e-12, atol=1e-10)
    np.testing.assert_allclose(v["e_local"], z["e_local"], rtol=1e-9, atol=1e-8)
