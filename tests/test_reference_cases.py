"""The reference's own known-answer tests, restated on the oracle and on the
library's host-side tables: the numbers below are those the reference
asserts, so these pin the restatement to the reference's expectations.

* ECP radial potentials in PySCF's layout, the local channel at index 0 and
  semi-local l at l + 1, powers r^(k - 2) (tests/estimator/ecp/
  ecp_potential_test.py);
* nearest-core selection (same file, TestSelectNearestCores);
* the nonlocal integral's Legendre indexing on a constant wavefunction: only
  the s channel contributes, V_s itself (tests/estimator/ecp/
  ecp_nonlocal_test.py);
* the SimpleEE Jastrow's cusp derivatives, 1/4 for parallel and 1/2 for
  antiparallel spins (tests/wavefunction/jastrow_test.py)."""
import math

import numpy as np
import pytest
import torch

from jaqmc_gb300 import ecp as E
from oracle import ecp as OE
from oracle import lap
from oracle import psiformer as OP


def _ecp(channels):
    """One element "X" from channels of (power_idx, alpha, c) terms, the first
    the local channel (PySCF l = -1)."""
    out = []
    for l_idx, terms in enumerate(channels):
        radial = [[] for _ in range(max((t[0] for t in terms), default=-1) + 1)]
        for k, alpha, c in terms:
            radial[k].append([alpha, c])
        out.append([l_idx - 1, radial])
    return {"X": [len(channels), out]}


def _values(ecp, electrons, atoms, symbols):
    ecp_atoms = [i for i, s in enumerate(symbols) if s in ecp]
    al, co, pw = OE.radial_table(ecp, symbols, ecp_atoms)
    R = np.asarray(atoms, np.float64)[ecp_atoms]
    vec = np.asarray(electrons, np.float64)[:, None, :] - R[None]
    d = np.linalg.norm(vec, axis=-1)
    return ecp_atoms, OE.radial(al, co, pw, d), vec, d


def test_single_channel():
    ecp = _ecp([[(2, 2.0, 3.0)]])
    idx, V, vec, d = _values(ecp, [[1.0, 0.0, 0.0]], [[0.0, 0.0, 0.0]], ["X"])
    assert V.shape == (1, 1, 1) and vec.shape == (1, 1, 3) and d.shape == (1, 1)
    np.testing.assert_allclose(V[0, 0, 0], 3.0 * math.exp(-2.0), atol=1e-6)
    np.testing.assert_allclose(d[0, 0], 1.0, atol=1e-6)
    np.testing.assert_allclose(vec[0, 0], [1.0, 0.0, 0.0], atol=1e-6)


def test_two_channels():
    ecp = _ecp([[(2, 2.0, 3.0)], [(2, 1.0, 1.5)]])
    _, V, _, _ = _values(ecp, [[2.0, 0.0, 0.0]], [[0.0, 0.0, 0.0]], ["X"])
    assert V.shape == (1, 1, 2)
    np.testing.assert_allclose(V[0, 0, 0], 3.0 * math.exp(-8.0), atol=1e-6)
    np.testing.assert_allclose(V[0, 0, 1], 1.5 * math.exp(-4.0), atol=1e-6)


def test_multiple_terms_and_electrons():
    ecp = _ecp([[(2, 1.0, 2.0), (2, 3.0, 5.0)]])
    _, V, _, _ = _values(ecp, [[1.0, 0.0, 0.0]], [[0.0, 0.0, 0.0]], ["X"])
    np.testing.assert_allclose(V[0, 0, 0], 2.0 * math.exp(-1.0) + 5.0 * math.exp(-3.0), atol=1e-6)
    ecp = _ecp([[(2, 1.0, 1.0)]])
    _, V, _, d = _values(ecp, [[1.0, 0.0, 0.0], [0.0, 3.0, 0.0]], [[0.0, 0.0, 0.0]], ["X"])
    assert V.shape == (2, 1, 1)
    np.testing.assert_allclose(d[:, 0], [1.0, 3.0], atol=1e-6)
    np.testing.assert_allclose(V[:, 0, 0], [math.exp(-1.0), math.exp(-9.0)], atol=1e-6)


def test_only_ecp_atoms_enter():
    ecp = _ecp([[(2, 1.0, 1.0)]])
    idx, V, _, d = _values(ecp, [[1.0, 0.0, 0.0]], [[0.0, 0.0, 0.0], [5.0, 0.0, 0.0]], ["X", "H"])
    assert idx == [0] and V.shape == (1, 1, 1)
    np.testing.assert_allclose(d[0, 0], 1.0, atol=1e-6)
    t = E.ECPTables(ecp, ["X", "H"], max_core=1)
    assert list(t.ecp_atoms) == [0]


def test_nearest_core_selection():
    V = np.array([[[1.0], [2.0]]])
    sv, _, sd = OE.select_nearest_cores(V, np.ones((1, 2, 3)), np.array([[1.0, 2.0]]), max_core=5)
    np.testing.assert_array_equal(sv, V)
    np.testing.assert_array_equal(sd, [[1.0, 2.0]])
    V = np.array([[[10.0], [20.0], [30.0]], [[40.0], [50.0], [60.0]]])
    d = np.array([[1.0, 3.0, 2.0], [3.0, 1.0, 2.0]])
    sv, _, sd = OE.select_nearest_cores(V, np.zeros((2, 3, 3)), d, max_core=2)
    assert sv.shape == (2, 2, 1) and sd.shape == (2, 2)
    np.testing.assert_allclose(sd, [[1.0, 2.0], [1.0, 2.0]])
    np.testing.assert_allclose(sv[..., 0], [[10.0, 30.0], [50.0, 60.0]])
    sv, _, sd = OE.select_nearest_cores(np.array([[[1.0], [2.0], [3.0]]]), np.zeros((1, 3, 3)),
                                        np.array([[5.0, 1.0, 3.0]]), max_core=1)
    np.testing.assert_allclose(sd[0, 0], 1.0)
    np.testing.assert_allclose(sv[0, 0, 0], 2.0)


def test_pyscf_channel_mapping():
    mock = {"X": [2, [[-1, [[], [[3.0, 7.0]]]], [0, [[], [], [[1.0, 5.0]]]]]]}
    al, co, pw = OE.radial_table(mock, ["X"], [0])
    assert (al[0, 0, 0], co[0, 0, 0], pw[0, 0, 0]) == (3.0, 7.0, -1.0)
    assert (al[0, 1, 0], co[0, 1, 0], pw[0, 1, 0]) == (1.0, 5.0, 0.0)
    t = E.ECPTables(mock, ["X"], max_core=1)
    np.testing.assert_array_equal(t.radial[0, 0, 0], [3.0, 7.0, -1.0])
    np.testing.assert_array_equal(t.radial[0, 1, 0], [1.0, 5.0, 0.0])


@pytest.mark.parametrize("channel,want", [(1, 2.5), (2, 0.0)])
def test_nonlocal_legendre_indexing_constant_wavefunction(channel, want):
    """psi constant: only the s channel (index 1) contributes, V_s."""
    vals = [[(2, 0.0, 0.0)], [(2, 0.0, 0.0)], [(2, 0.0, 0.0)], [(2, 0.0, 0.0)]]
    vals[channel] = [(2, 0.0, 2.5 if channel == 1 else 5.0)]
    ecp = _ecp(vals)
    al, co, pw = OE.radial_table(ecp, ["X"], [0])

    def constant(x):
        return torch.ones(x.shape[0], dtype=torch.float64), torch.zeros(x.shape[0], dtype=torch.float64)
    rng = np.random.default_rng(42)
    rot = OE.rotation_matrices(rng.random((1, 1)), rng.random((1, 1)))
    _, nonlocal_ = OE.ecp_energy(constant, np.array([[[1.0, 0.0, 0.0]]]), np.zeros((1, 3)), [0], al, co, pw, rot,
                                 OE.quadrature("octahedron_26"), max_core=1)
    np.testing.assert_allclose(nonlocal_[0], want, atol=1e-5)


@pytest.mark.parametrize("same,want", [(True, 0.25), (False, 0.5)])
def test_jastrow_cusp_derivative(same, want):
    """dJ/dr at r -> 0 of the pair term: 1/4 (parallel), 1/2 (antiparallel)."""
    nspins = (2, 0) if same else (1, 1)
    cfg = OP.PsiformerConfig(nspins=nspins)
    p = {"alpha_par": np.array([1.0]), "alpha_anti": np.array([1.0])}
    h = 1e-6
    vals = []
    for r in (0.0, h):
        x = torch.tensor([[[0.0, 0.0, 0.0], [r, 0.0, 0.0]]], dtype=torch.float64)
        vals.append(float(OP.jastrow_lt(p, cfg, lap.seed(x, with_tangents=False), torch.float64).x[0]))
    np.testing.assert_allclose((vals[1] - vals[0]) / h, want, atol=1e-3)
