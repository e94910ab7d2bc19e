"""ECP estimator pieces on the CPU: the spherical quadrature rules of the
package and of the oracle integrate polynomials exactly to their design
degree (src/jaqmc/estimator/ecp/quadrature.py), the PySCF-layout radial
tables (src/jaqmc/estimator/ecp/estimator.py:190-275), and the oracle's
nonlocal integral on a wavefunction whose moved electron is spherically
symmetric about the ECP atom (every ratio is 1: the s channel integrates to
V_s(r), the others to 0)."""
import math

import numpy as np
import pytest
import torch

from jaqmc_gb300 import ecp as E
from oracle import ecp as OE

RULES = [("icosahedron_12", 5), ("icosahedron_32", 9), ("octahedron_6", 3), ("octahedron_18", 5),
         ("octahedron_26", 7), ("octahedron_50", 11)]

# a made-up ECP in PySCF's layout: local channel (l = -1) and s, p channels
TOY_ECP = {"Li": [2, [[-1, [[], [[1.5, -2.0]], [[0.7, 0.3], [2.0, 1.1]]]],
                      [0, [[], [], [[1.2, 3.0], [0.4, -0.5]]]],
                      [1, [[], [[0.9, 0.8]], [[1.6, -1.2]]]]]]}


def _dfact(k):
    return 1 if k <= 0 else k * _dfact(k - 2)


def _sphere_mean(a, b, c):
    if a % 2 or b % 2 or c % 2:
        return 0.0
    return _dfact(a - 1) * _dfact(b - 1) * _dfact(c - 1) / _dfact(a + b + c + 1)


@pytest.mark.parametrize("name,deg", RULES)
def test_rules_exact_to_their_degree(name, deg):
    for P, w in (E.quadrature_rule(name), OE.quadrature(name)):
        assert np.allclose(np.linalg.norm(P, axis=1), 1.0) and abs(w.sum() - 1.0) < 1e-14
        for a in range(deg + 1):
            for b in range(deg + 1 - a):
                for c in range(deg + 1 - a - b):
                    v = (w * P[:, 0] ** a * P[:, 1] ** b * P[:, 2] ** c).sum()
                    assert abs(v - _sphere_mean(a, b, c)) < 1e-13, (name, a, b, c)


def test_radial_tables_match_the_oracle():
    t = E.ECPTables(TOY_ECP, ["Li"], max_core=1)
    al, co, pw = OE.radial_table(TOY_ECP, ["Li"], [0])
    # the device table is float32
    np.testing.assert_array_equal(t.radial[..., 0], al.astype(np.float32))
    np.testing.assert_array_equal(t.radial[..., 1], co.astype(np.float32))
    np.testing.assert_array_equal(t.radial[..., 2], pw.astype(np.float32))
    r = np.linspace(0.1, 3.0, 7)
    V = OE.radial(al, co, pw, r[:, None])
    # channel 0 by hand: -2 r^-1 e^{-1.5 r^2} + 0.3 e^{-0.7 r^2} + 1.1 e^{-2 r^2}
    want = -2.0 / r * np.exp(-1.5 * r * r) + 0.3 * np.exp(-0.7 * r * r) + 1.1 * np.exp(-2.0 * r * r)
    np.testing.assert_allclose(V[:, 0, 0], want, rtol=1e-12)
    assert t.n_channels == 3 and t.effective_charges([3.0])[0] == 1.0


def test_rotations_are_proper():
    rng = np.random.default_rng(0)
    R = OE.rotation_matrices(rng.random(50), rng.random(50))
    np.testing.assert_allclose(R @ np.swapaxes(R, -1, -2), np.broadcast_to(np.eye(3), R.shape), atol=1e-12)
    np.testing.assert_allclose(np.linalg.det(R), 1.0, atol=1e-12)


def test_nonlocal_integral_of_a_symmetric_factor():
    """psi = prod_i exp(-|r_i - R|): moving one electron on its sphere about R
    leaves psi unchanged, so sum_l V_l (2l+1) <P_l> = V_s(r) exactly."""
    R0 = np.zeros((1, 3))

    def phase_logpsi(x):
        lp = -torch.linalg.norm(x - torch.as_tensor(R0), dim=-1).sum(-1)
        return torch.ones_like(lp), lp

    rng = np.random.default_rng(3)
    x = rng.normal(size=(4, 3, 3))
    rot = OE.rotation_matrices(rng.random((4, 3)), rng.random((4, 3)))
    al, co, pw = OE.radial_table(TOY_ECP, ["Li"], [0])
    loc, nl = OE.ecp_energy(phase_logpsi, x, R0, [0], al, co, pw, rot, OE.quadrature("icosahedron_12"), 1)
    r = np.linalg.norm(x, axis=-1)
    V = OE.radial(al, co, pw, r[..., None])[..., 0, :]
    np.testing.assert_allclose(loc, V[..., 0].sum(-1), rtol=1e-12)
    np.testing.assert_allclose(nl, V[..., 1].sum(-1), rtol=1e-10, atol=1e-12)
