"""Shared set-up for the parity tests: systems, parameters and oracle calls."""
from __future__ import annotations

import numpy as np
import torch

from jaqmc_gb300 import params as P
from jaqmc_gb300 import systems as S
from oracle import ferminet as OF
from oracle import hamiltonian as OH


def oracle_cfg(cfg: P.FermiNetConfig) -> OF.FermiNetConfig:
    return OF.FermiNetConfig(nspins=tuple(cfg.nspins), ndets=cfg.ndets,
                             hidden_dims_single=list(cfg.hidden_dims_single),
                             hidden_dims_double=list(cfg.hidden_dims_double),
                             use_last_layer=cfg.use_last_layer, envelope=cfg.envelope,
                             orbitals_spin_split=cfg.orbitals_spin_split)


def small_cfg(nspins, **kw) -> P.FermiNetConfig:
    base = dict(nspins=tuple(nspins), ndets=2, hidden_dims_single=[8, 8], hidden_dims_double=[4, 4])
    base.update(kw)
    return P.FermiNetConfig(**base)


def full_cfg(nspins, **kw) -> P.FermiNetConfig:
    base = dict(nspins=tuple(nspins))
    base.update(kw)
    return P.FermiNetConfig(**base)


def setup(mol: S.Molecule, cfg: P.FermiNetConfig, batch: int, seed_params=0, seed_walkers=1, width=1.0):
    tree = P.init_ferminet(cfg, mol.n_atoms, seed=seed_params)
    leaves = P.ferminet_leaves(cfg, mol.n_atoms)
    flat = P.flatten(tree, leaves)
    x = S.init_walkers(mol, batch, seed=seed_walkers, width=width)
    return tree, flat, x


def oracle_forward(tree, cfg, mol, x, dtype=torch.float64, tangents=False):
    return OF.evaluate(tree, oracle_cfg(cfg), torch.as_tensor(x, dtype=dtype), mol.atoms,
                       dtype=dtype, tangents=tangents)


def oracle_local_energy(tree, cfg, mol, x, dtype=torch.float64):
    out = oracle_forward(tree, cfg, mol, x, dtype=dtype, tangents=True)
    ke = OH.kinetic_from_tangents(out["grad"], out["lap"])
    pe = OH.potential_energy(torch.as_tensor(x, dtype=dtype), mol.atoms, mol.charges)
    return {"e_local": ke + pe, "kinetic": ke, "potential": pe, "logpsi": out["logpsi"],
            "sign": out["sign_logpsi"]}


def hydrogenic_tree(cfg: P.FermiNetConfig, n_atoms: int, sigma: float, seed=0):
    """Parameters for which every orbital equals c * exp(-sigma r) up to a
    constant: all stream kernels zero with a constant bias, and the envelope
    sigma set to ``sigma``.  For one electron, psi = c exp(-sigma r) exactly."""
    tree = P.init_ferminet(cfg, n_atoms, seed=seed)
    bb = tree["params"]["backbone_layer"]
    for k, v in bb.items():
        v["kernel"][:] = 0.0
        v["bias"][:] = 0.3
    for leaf in tree["params"]["envelope_layer"].values():
        leaf["sigma"][:] = sigma
        leaf["pi"][:] = 1.0
    return tree
