"""ECP energy on the GPU (qmc_ecp_energy) against the oracle
(oracle/ecp.py, restating src/jaqmc/estimator/ecp/estimator.py:33-155 and
nonlocal_integral.py:17-130) on the same parameters, walkers and injected
rotations, with the FP64 FermiNet oracle as the wavefunction: local part
within 1e-5 relative; nonlocal part within 1e-4 Ha + 1e-4 relative per
walker (the ratios psi'/psi come from FP32 forward passes).  Also: Philox
rotations are reproducible per (seed, counter) and the host estimator
returns local + nonlocal as energy:ecp."""
import numpy as np
import pytest
import torch

from helpers import oracle_cfg, setup, small_cfg
from jaqmc_gb300 import _native
from jaqmc_gb300 import ecp as E
from jaqmc_gb300 import systems as S
from jaqmc_gb300 import vmc
from oracle import ecp as OE
from oracle import ferminet as OF

pytestmark = pytest.mark.gpu

TOY = {"Li": [2, [[-1, [[], [[1.5, -2.0]], [[0.7, 0.3], [2.0, 1.1]]]],
                  [0, [[], [], [[1.2, 3.0], [0.4, -0.5]]]],
                  [1, [[], [[0.9, 0.8]], [[1.6, -1.2]]]]]],
       "H": [0, [[-1, [[], [], [[1.0, -0.4]]]], [0, [[], [], [[0.8, 0.6]]]]]]}


def _case(name):
    if name == "Li":
        mol, symbols, max_core = S.lithium(), ["Li"], 1
    else:  # LiH: both atoms carry an ECP, one nearest core per electron
        mol = S.make_molecule("LiH", [3, 1], [[0, 0, 0], [0, 0, 3.0]], (2, 2))
        symbols, max_core = ["Li", "H"], 1
    return mol, symbols, max_core


@pytest.mark.parametrize("name,quad", [("Li", "icosahedron_12"), ("LiH", "octahedron_18")])
def test_ecp_energy_matches_oracle(name, quad, cuda_device):
    mol, symbols, max_core = _case(name)
    cfg = small_cfg(mol.nspins, ndets=2, hidden_dims_single=[16, 16])
    tree, flat, x = setup(mol, cfg, 12)
    m = _native.NativeFermiNet(cfg, mol.atoms, mol.charges, device=cuda_device)
    m.set_params(torch.as_tensor(flat, device=cuda_device))
    tabs = E.ECPTables(TOY, symbols, max_core=max_core, quadrature_id=quad)
    rng = np.random.default_rng(5)
    rot = OE.rotation_matrices(rng.random((12, mol.n_electrons)), rng.random((12, mol.n_electrons)))
    loc, nl = m.ecp_energy(torch.as_tensor(x, device=cuda_device), tabs.device_tables(cuda_device),
                           rotations=torch.as_tensor(rot.reshape(12, mol.n_electrons, 9)))
    oc = oracle_cfg(cfg)

    def phase_logpsi(xx):
        out = OF.evaluate(tree, oc, xx.to(torch.float64), mol.atoms)
        return out["sign_logpsi"].numpy(), out["logpsi"].numpy()

    al, co, pw = OE.radial_table(TOY, symbols, tabs.ecp_atoms)
    pts, wts = tabs.quad[:, :3].astype(np.float64), tabs.quad[:, 3].astype(np.float64)
    rloc, rnl = OE.ecp_energy(phase_logpsi, x, mol.atoms, tabs.ecp_atoms, al, co, pw, rot, (pts, wts), max_core)
    np.testing.assert_allclose(loc.cpu().numpy(), rloc, rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(nl.cpu().numpy(), rnl, rtol=1e-4, atol=1e-4)
    assert np.abs(rnl).max() > 1e-2  # the nonlocal part is not trivially small here


def test_philox_rotations_and_estimator(cuda_device):
    mol, symbols, max_core = _case("Li")
    wf = vmc.FermiNetWavefunction(nspins=mol.nspins, ndets=2, hidden_dims_single=[8, 8], hidden_dims_double=[4, 4])
    x = torch.as_tensor(S.init_walkers(mol, 64, seed=2), device="cuda")
    data = vmc.MoleculeData(x, mol.atoms, mol.charges)
    params = wf.init_params(data, 0)
    m = wf.model(data, params)
    tabs = E.ECPTables(TOY, symbols, max_core=max_core).device_tables(m.device)
    a = m.ecp_energy(x, tabs, seed=9, counter=4)
    b = m.ecp_energy(x, tabs, seed=9, counter=4)
    c = m.ecp_energy(x, tabs, seed=9, counter=5)
    assert torch.equal(a[0], b[0]) and torch.equal(a[1], b[1])
    assert torch.equal(a[0], c[0]) and not torch.equal(a[1], c[1])  # only the rotations changed
    est = vmc.ECPEnergy(max_core=max_core, phase_logpsi=wf, ecp_coefficients=TOY, atom_symbols=symbols)
    st = est.init(data, 9)
    out, st = est.evaluate_batch_walkers(params, vmc.BatchedData(data), {}, st)
    assert st["calls"] == 1
    assert torch.isfinite(out["energy:ecp"]).all() and out["energy:ecp"].shape == (64,)
