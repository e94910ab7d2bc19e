"""Pins the CPU oracle against the reference's own known-answer and property
tests (restated; the reference itself cannot be imported without JAX).

* FL == brute-force Hessian trace on FermiNet —
  tests/estimator/kinetic_forward_laplacian_test.py:248-293 (rtol = atol = 2e-5)
* analytic harmonic kinetic energy — same file :41-79 (rtol 1e-5, atol 1e-6)
* slogdet FL rule vs brute force — tests/laplacian/primitives/slogdet_test.py:28-173
* antisymmetry — tests/wavefunction/molecule_wavefunction_test.py:52-121
* exact hydrogen-like energies — tests/hydrogen/atom_test.py:38-52 (-0.5 Ha)
* clip / gradient algebra — tests/estimator/loss_grad_test.py:23-77
* Philox4x32-10 published known-answer vectors
"""
import numpy as np
import pytest
import torch

from helpers import hydrogenic_tree, oracle_cfg, oracle_local_energy, small_cfg
from jaqmc_gb300 import params as P
from jaqmc_gb300 import systems as S
from oracle import ferminet as OF
from oracle import hamiltonian as OH
from oracle import lap
from oracle import philox as OP
from oracle import stats as OS

TWO_ELECTRONS = np.array([[0.7, -0.2, 0.3], [-0.4, 0.5, -0.6]])
HE = np.array([[0.0, 0.0, 0.0]])


@pytest.mark.parametrize("split", [False, True])
@pytest.mark.parametrize("dtype,tol", [(torch.float32, 2e-5), (torch.float64, 1e-10)])
def test_fl_matches_bruteforce_two_electron_fixture(split, dtype, tol):
    cfg = small_cfg((1, 1), orbitals_spin_split=split)
    tree = P.init_ferminet(cfg, 1, seed=123)
    oc = oracle_cfg(cfg)
    x = torch.as_tensor(TWO_ELECTRONS[None], dtype=dtype)
    out = OF.evaluate(tree, oc, x, HE, dtype=dtype, tangents=True)
    ke = OH.kinetic_from_tangents(out["grad"], out["lap"])
    ke_ref, _, _ = OH.kinetic_bruteforce(OF.logpsi_fn(tree, oc, HE), x.double())
    assert torch.isfinite(ke).all()
    np.testing.assert_allclose(ke.double().numpy(), ke_ref.numpy(), rtol=tol, atol=tol)


@pytest.mark.parametrize("nspins,A", [((2, 1), 1), ((3, 2), 2), ((2, 0), 1), ((0, 2), 1), ((1, 0), 1)])
def test_fl_matches_bruteforce_spins(nspins, A):
    cfg = small_cfg(nspins, ndets=3)
    tree = P.init_ferminet(cfg, A, seed=7)
    oc = oracle_cfg(cfg)
    atoms = np.array([[0.0, 0.0, 0.0], [0.3, -0.2, 1.4]])[:A]
    x = torch.randn(4, cfg.n, 3, dtype=torch.float64, generator=torch.Generator().manual_seed(3))
    out = OF.evaluate(tree, oc, x, atoms, tangents=True)
    ke = OH.kinetic_from_tangents(out["grad"], out["lap"])
    ke_ref, g_ref, _ = OH.kinetic_bruteforce(OF.logpsi_fn(tree, oc, atoms), x)
    np.testing.assert_allclose(out["grad"].numpy(), g_ref.numpy(), rtol=1e-9, atol=1e-9)
    np.testing.assert_allclose(ke.numpy(), ke_ref.numpy(), rtol=1e-9, atol=1e-9)


@pytest.mark.parametrize("n_particles,n_dims,coeff",
                         [(1, 1, 0.5), (3, 3, 0.5), (2, 3, 0.3), (5, 3, 0.3), (3, 2, 0.3), (10, 1, 0.3),
                          (20, 3, 0.2)])
def test_harmonic_kinetic_energy(n_particles, n_dims, coeff):
    g = torch.Generator().manual_seed(42 + n_particles * 10 + n_dims)
    x = torch.randn(1, n_particles, n_dims, dtype=torch.float32, generator=g)
    X = lap.seed(x)
    lp = (X * X).sum(-1).sum(-1).scale(-coeff)
    ke = OH.kinetic_from_tangents(lp.J, lp.L)
    exact = coeff * n_particles * n_dims - 2 * coeff ** 2 * float((x.double() ** 2).sum())
    np.testing.assert_allclose(float(ke[0]), exact, rtol=1e-5, atol=1e-6)


def test_slogdet_rule_matches_bruteforce():
    g = torch.Generator().manual_seed(0)
    W1 = torch.randn(6, 16, dtype=torch.float64, generator=g)
    W2 = torch.randn(6, 16, dtype=torch.float64, generator=g)

    def mat(X):  # (B, 2, 3) -> (B, 2, 4, 4) smooth matrix function
        flat = X.reshape(X.shape[0], 6)
        return torch.stack([torch.tanh(flat @ W1), torch.sin(flat @ W2)], 1).reshape(-1, 2, 4, 4)

    x = torch.randn(3, 2, 3, dtype=torch.float64, generator=g)
    X = lap.seed(x)
    flat = X.reshape(6)
    A = lap.stack([lap.tanh(lap.linear(flat, W1)), lap.linear(flat, W2)], 1)
    # sin via the generic elementwise rule
    s = A[1]
    s = lap.unary(s, torch.sin(s.x), torch.cos(s.x), -torch.sin(s.x))
    A = lap.stack([A[0], s], 1).reshape(2, 4, 4)
    _, ld = lap.slogdet(A)

    def f(xx):
        return torch.linalg.slogdet(mat(xx))[1].sum(-1)

    _, g_ref, tr_ref = OH.kinetic_bruteforce(f, x)
    np.testing.assert_allclose(ld.J.sum(-1).numpy(), g_ref.numpy(), rtol=1e-10, atol=1e-10)
    np.testing.assert_allclose(ld.L.sum(-1).numpy(), tr_ref.numpy(), rtol=1e-9, atol=1e-9)


def test_antisymmetry_same_spin_swap():
    cfg = P.FermiNetConfig(nspins=(2, 0))
    tree = P.init_ferminet(cfg, 1, seed=42)
    x = torch.randn(1, 2, 3, dtype=torch.float64, generator=torch.Generator().manual_seed(42))
    a = OF.evaluate(tree, oracle_cfg(cfg), x, HE)
    b = OF.evaluate(tree, oracle_cfg(cfg), x.flip(1), HE)
    assert float(a["sign_logpsi"][0]) == -float(b["sign_logpsi"][0])
    assert float(a["logpsi"][0]) == pytest.approx(float(b["logpsi"][0]), rel=5e-4)


def test_opposite_spin_swap_changes_value():
    cfg = P.FermiNetConfig(nspins=(1, 1))
    tree = P.init_ferminet(cfg, 1, seed=42)
    x = torch.randn(1, 2, 3, dtype=torch.float64, generator=torch.Generator().manual_seed(42))
    a = OF.evaluate(tree, oracle_cfg(cfg), x, HE)
    b = OF.evaluate(tree, oracle_cfg(cfg), x.flip(1), HE)
    pa = a["sign_logpsi"] * torch.exp(a["logpsi"])
    pb = b["sign_logpsi"] * torch.exp(b["logpsi"])
    assert not torch.allclose(pa, pb, rtol=1e-3)


def test_hydrogen_atom_exact_energy():
    """psi = c exp(-r) is the H ground state: E_L = -0.5 for every walker."""
    mol = S.hydrogen()
    cfg = small_cfg((1, 0), ndets=2)
    tree = hydrogenic_tree(cfg, 1, sigma=1.0)
    x = S.init_walkers(mol, 64, seed=5)
    out = oracle_local_energy(tree, cfg, mol, x)
    np.testing.assert_allclose(out["e_local"].numpy(), -0.5, atol=1e-10)


def test_hydrogenic_helium_exact_energy():
    """Product of two 1s orbitals (exponent 2): E_L = -4 + 1/r12."""
    mol = S.make_molecule("He", [2], [[0, 0, 0]], (1, 1))
    cfg = small_cfg((1, 1), ndets=2)
    tree = hydrogenic_tree(cfg, 1, sigma=2.0)
    orb = tree["params"]["orbital_layer"]["SplitChannelDense_0"]
    orb["DenseGeneral_0"]["kernel"][:] = 0.0
    orb["DenseGeneral_0"]["kernel"][:, :, 0] = 0.5
    orb["DenseGeneral_1"]["kernel"][:] = 0.0
    orb["DenseGeneral_1"]["kernel"][:, :, 1] = 0.5
    x = S.init_walkers(mol, 64, seed=6)
    out = oracle_local_energy(tree, cfg, mol, x)
    r12 = np.linalg.norm(x[:, 0] - x[:, 1], axis=-1)
    np.testing.assert_allclose(out["e_local"].numpy(), -4.0 + 1.0 / r12, rtol=1e-6, atol=1e-6)


def test_potential_energy_by_hand():
    e = np.array([[[0.0, 0.0, 1.0], [0.0, 2.0, 0.0]]])
    R = np.array([[0.0, 0.0, 0.0], [3.0, 0.0, 0.0]])
    Z = np.array([2.0, 1.0])
    v = float(OH.potential_energy(torch.as_tensor(e), R, Z)[0])
    ee = 1 / np.sqrt(5.0)
    en = -(2 / 1 + 1 / np.sqrt(10) + 2 / 2 + 1 / np.sqrt(13))
    nn = 2 * 1 / 3.0
    assert v == pytest.approx(ee + en + nn, rel=1e-12)


def test_clip_and_gradient_algebra():
    x = np.array([0.0, 1.0, 2.0, 100.0])
    q1, q3 = np.nanquantile(x, 0.25), np.nanquantile(x, 0.75)
    np.testing.assert_allclose(OS.iqr_clip(x, 1.0), np.clip(x, q1 - (q3 - q1), q3 + (q3 - q1)))
    med = np.median(x)
    dev = np.median(np.abs(x - med))
    clipped = np.clip(x, med - dev, med + dev)
    np.testing.assert_allclose(OS.mad_clip(x, 1.0), clipped)
    g = np.array([[1.0], [2.0], [3.0], [4.0]])
    grads, loss = OS.vmc_gradient(g, x, clip="mad", scale=1.0)
    assert loss == pytest.approx(x.mean())
    np.testing.assert_allclose(grads, 2 * ((g[:, 0] * clipped).mean() - clipped.mean() * g[:, 0].mean()))
    m, v = OS.mean_reduce(np.array([1.0, np.nan, 3.0]))
    assert m == pytest.approx(2.0) and v == pytest.approx(1.0)


def test_philox_known_answers():
    cases = [((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
             ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
             ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
              (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1))]
    for c, k, want in cases:
        got = OP.philox4x32_10(np.array(c, np.uint32), np.array(k, np.uint32))
        assert tuple(int(v) for v in got) == want


def test_mh_draws_statistics():
    z, u = OP.mh_draws(seed=2, step=0, batch=4096, n=5)
    assert abs(z.mean()) < 0.02 and abs(z.std() - 1) < 0.02
    assert 0 < u.min() and u.max() < 1 and abs(u.mean() - 0.5) < 0.02


def _random_envelopes(tree, rng):
    for ch in tree["params"].get("envelope_layer", {}).values():
        ch["pi"][:] = rng.uniform(0.5, 1.5, ch["pi"].shape)
        ch["sigma"][:] = rng.uniform(0.4, 1.6, ch["sigma"].shape)


@pytest.mark.parametrize("envelope", ["diagonal", "null"])
@pytest.mark.parametrize("nspins,A", [((2, 1), 1), ((3, 2), 2)])
def test_fl_matches_bruteforce_other_envelopes(envelope, nspins, A):
    """The diagonal (per-dimension decay, src/jaqmc/wavefunction/output/
    envelope.py:143-163) and null (:79-80,110-112) envelopes through the
    forward Laplacian: gradient and kinetic energy equal the brute-force
    Hessian trace."""
    cfg = small_cfg(nspins, ndets=3, envelope=envelope)
    tree = P.init_ferminet(cfg, A, seed=7)
    _random_envelopes(tree, np.random.default_rng(5))
    oc = oracle_cfg(cfg)
    atoms = np.array([[0.0, 0.0, 0.0], [0.3, -0.2, 1.4]])[:A]
    x = torch.randn(4, cfg.n, 3, dtype=torch.float64, generator=torch.Generator().manual_seed(3))
    out = OF.evaluate(tree, oc, x, atoms, tangents=True)
    ke = OH.kinetic_from_tangents(out["grad"], out["lap"])
    ke_ref, g_ref, _ = OH.kinetic_bruteforce(OF.logpsi_fn(tree, oc, atoms), x)
    np.testing.assert_allclose(out["grad"].numpy(), g_ref.numpy(), rtol=1e-9, atol=1e-9)
    np.testing.assert_allclose(ke.numpy(), ke_ref.numpy(), rtol=1e-9, atol=1e-9)


def test_diagonal_envelope_with_equal_rates_is_abs_isotropic():
    """sigma_c = s for the three dimensions gives ||s (r - R)|| = |s| r: the
    diagonal envelope equals the abs_isotropic one with sigma = s."""
    mol = S.methane()
    cd = small_cfg(mol.nspins, ndets=2, envelope="diagonal")
    ci = small_cfg(mol.nspins, ndets=2, envelope="abs_isotropic")
    td = P.init_ferminet(cd, mol.n_atoms, seed=1)
    ti = P.init_ferminet(ci, mol.n_atoms, seed=1)
    rng = np.random.default_rng(2)
    for nm, ch in ti["params"]["envelope_layer"].items():
        ch["pi"][:] = rng.uniform(0.5, 1.5, ch["pi"].shape)
        ch["sigma"][:] = rng.uniform(-1.5, 1.5, ch["sigma"].shape)
        td["params"]["envelope_layer"][nm]["pi"][:] = ch["pi"]
        td["params"]["envelope_layer"][nm]["sigma"][:] = ch["sigma"][:, :, None, :]
    x = torch.as_tensor(S.init_walkers(mol, 6, seed=3), dtype=torch.float64)
    a = OF.evaluate(td, oracle_cfg(cd), x, mol.atoms, tangents=True)
    b = OF.evaluate(ti, oracle_cfg(ci), x, mol.atoms, tangents=True)
    for k in ("logpsi", "grad", "lap"):
        np.testing.assert_allclose(a[k].numpy(), b[k].numpy(), rtol=1e-12, atol=1e-12)
    assert [s for _, s in P.ferminet_leaves(cd, mol.n_atoms)][-1] == (mol.n_electrons, mol.n_atoms, 3, 2)
