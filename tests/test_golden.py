"""The golden fixtures (tests/golden/*.npz, written by tests/golden/make_golden.py)
on the CPU: the seeded parameters and walkers regenerate bit for bit, and the
FP64 oracle reproduces the stored log|psi|, sign and local energies."""
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


def test_every_case_has_a_fixture():
    assert sorted(os.path.basename(f)[:-4] for f in FIXTURES) == sorted(G.CASES)


@pytest.mark.parametrize("path", FIXTURES, ids=lambda p: os.path.basename(p)[:-4])
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
