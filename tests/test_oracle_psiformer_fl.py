"""Forward-Laplacian Psiformer oracle (oracle/psiformer.py evaluate_fl)
against autograd: log|psi| equals the value oracle, and the kinetic energy
from the propagated gradient and Laplacian equals the brute-force autograd
Hessian trace (FP64, small configurations; CPU)."""
import sys
import os

import torch

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
from jaqmc_gb300 import params as P  # noqa: E402
from jaqmc_gb300 import systems as S  # noqa: E402
from oracle import hamiltonian as OH  # noqa: E402
from oracle import psiformer as OP  # noqa: E402


def test_fl_matches_autograd():
    for mol in (S.lithium(), S.atom(4)):
        kw = dict(nspins=mol.nspins, ndets=2, num_layers=2, num_heads=2, heads_dim=4, mlp_hidden_dims=[8])
        tree = P.init_psiformer(P.PsiformerConfig(**kw), mol.n_atoms, seed=3)
        cfg = OP.PsiformerConfig(**kw)
        x = torch.as_tensor(S.init_walkers(mol, 3, seed=2), dtype=torch.float64)
        fl = OP.evaluate_fl(tree, cfg, x, mol.atoms)
        ref = OP.evaluate(tree, cfg, x, mol.atoms)["logpsi"]
        assert torch.allclose(fl["logpsi"], ref, atol=1e-12)
        ke, g, _ = OH.kinetic_bruteforce(OP.logpsi_fn(tree, cfg, mol.atoms), x)
        assert torch.allclose(fl["grad"], g, atol=1e-10, rtol=1e-10)
        assert torch.allclose(OH.kinetic_from_tangents(fl["grad"], fl["lap"]), ke, atol=1e-9, rtol=1e-10)
