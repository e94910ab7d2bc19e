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


def oracle_param_jacobian(flat, cfg, mol, x):
    """(B, P) float64 d log|psi_w| / d theta by torch autograd on the oracle
    (the role of the reference's jax.grad), in the flat leaf order."""
    leaves = P.ferminet_leaves(cfg, mol.n_atoms)
    ts = []
    tree = {}
    off = 0
    for path, shape in leaves:
        size = int(np.prod(shape))
        t = torch.tensor(np.asarray(flat[off:off + size], np.float64).reshape(shape), requires_grad=True)
        off += size
        ts.append(t)
        node = tree.setdefault("params", {})
        for k in path[:-1]:
            node = node.setdefault(k, {})
        node[path[-1]] = t
    out = OF.evaluate(tree, oracle_cfg(cfg), torch.as_tensor(x, dtype=torch.float64), mol.atoms,
                      dtype=torch.float64)
    lp = out["logpsi"]
    rows = []
    for w in range(lp.shape[0]):
        g = torch.autograd.grad(lp[w], ts, retain_graph=True, allow_unused=True)
        rows.append(torch.cat([(gi if gi is not None else torch.zeros_like(t)).reshape(-1)
                               for gi, t in zip(g, ts)]))
    return torch.stack(rows).numpy(), lp.detach().numpy()


def oracle_logpsi_flat(flat, cfg, mol, x):
    tree = P.unflatten(np.asarray(flat, np.float64), P.ferminet_leaves(cfg, mol.n_atoms))
    return OF.evaluate(tree, oracle_cfg(cfg), torch.as_tensor(x, dtype=torch.float64), mol.atoms,
                       dtype=torch.float64)["logpsi"].numpy()
