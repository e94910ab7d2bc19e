"""Generate the golden fixtures of the parity tests: seeded walkers and the
FP64 oracle's log|psi|, sign and local energy (with its kinetic and potential
parts), plus the oracle's own FP32 results, which set the per-walker FP32
conditioning bars; and MH fixtures: walkers, Philox4x32-10 draws (the
oracle's restatement, injected on both sides) and the FP64 oracle's accept
counts, final walkers, log-probabilities and acceptance ratios; and a
gradient fixture: the FP64 oracle's per-walker d log|psi| / d theta (torch
autograd, the role of the reference's jax.grad) on 64 seeded parameter
entries and projected on 8 seeded random unit vectors.  Parameters
are not stored: they are regenerated from their seed by
``jaqmc_gb300.params`` and checked against the stored SHA-256 of the flat
float32 vector.

    python tests/golden/make_golden.py          # writes tests/golden/*.npz

The reference (JAX/Flax) cannot run in this environment and its own tests hold
no numeric vectors for these paths, so the values come from the oracle under
``oracle/``, which is pinned by the property tests in ``tests/test_oracle*.py``.
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from jaqmc_gb300 import params as P  # noqa: E402
from jaqmc_gb300 import systems as S  # noqa: E402
from oracle import ferminet as OF  # noqa: E402
from oracle import hamiltonian as OH  # noqa: E402
from oracle import mcmc as OM  # noqa: E402
from oracle import philox as OX  # noqa: E402
from oracle import lapnet as OL  # noqa: E402
from oracle import psiformer as OP  # noqa: E402

PSI_SMALL = dict(ndets=3, num_layers=2, num_heads=4, heads_dim=16, mlp_hidden_dims=[64])
LAP_SMALL = dict(ndets=3, num_layers=2, num_heads=4, heads_dim=16)

# name: (model, system, config keyword arguments, walkers); params seed 0, walkers seed 1
CASES = {
    "ferminet_li_full": ("ferminet", "Li", {}, 48),
    "ferminet_n2_full": ("ferminet", "N2", {}, 32),
    "psiformer_li_small": ("psiformer", "Li", PSI_SMALL, 32),
    "psiformer_ch4_small": ("psiformer", "CH4", PSI_SMALL, 32),
    "psiformer_c6h6_full": ("psiformer", "C6H6", {}, 2),
    "lapnet_li_small": ("lapnet", "Li", LAP_SMALL, 32),
    "lapnet_ch4_small": ("lapnet", "CH4", LAP_SMALL, 32),
}


# MH fixtures: name -> (case whose model and system they use, walkers, steps, stddev, seed)
MH_CASES = {
    "mh_ferminet_li_full": ("ferminet_li_full", 64, 3, 0.02, 2),
    "mh_ferminet_n2_full": ("ferminet_n2_full", 64, 3, 0.02, 2),
    "mh_psiformer_li_small": ("psiformer_li_small", 64, 3, 0.05, 4),
    "mh_lapnet_li_small": ("lapnet_li_small", 64, 3, 0.05, 4),
}


# gradient fixtures: name -> (case, walkers, seed of the entries and projections, entries, projections)
GRAD_CASES = {
    "grad_ferminet_ch4_full": ("ferminet_ch4_full", 4, 64, 64, 8),
}
CASES["ferminet_ch4_full"] = ("ferminet", "CH4", {}, 4)


def grad_probes(P_, seed, entries, projections):
    """Seeded parameter entries and unit projection vectors (P, projections)."""
    rng = np.random.default_rng(seed)
    idx = np.sort(rng.choice(P_, entries, replace=False))
    R = rng.standard_normal((P_, projections))
    return idx, R / np.linalg.norm(R, axis=0)


def build(case):
    """(mol, cfg, tree, flat, walkers) of a case, from its seeds."""
    model, system, kw, B = CASES[case]
    mol = S.SYSTEMS[system]()
    if model == "ferminet":
        cfg = P.FermiNetConfig(nspins=mol.nspins, **kw)
        tree = P.init_ferminet(cfg, mol.n_atoms, seed=0)
        flat = P.flatten(tree, P.ferminet_leaves(cfg, mol.n_atoms))
    elif model == "lapnet":
        cfg = P.LapNetConfig(nspins=mol.nspins, **kw)
        tree = P.init_lapnet(cfg, mol.n_atoms, seed=0)
        flat = P.flatten(tree, P.lapnet_leaves(cfg, mol.n_atoms))
    else:
        cfg = P.PsiformerConfig(nspins=mol.nspins, **kw)
        tree = P.init_psiformer(cfg, mol.n_atoms, seed=0)
        flat = P.flatten(tree, P.psiformer_leaves(cfg, mol.n_atoms))
    x = S.init_walkers(mol, B, seed=1)
    return mol, cfg, tree, np.asarray(flat, np.float32), x


def params_sha(flat) -> str:
    return hashlib.sha256(np.ascontiguousarray(flat, np.float32).tobytes()).hexdigest()


def oracle_values(case, mol, cfg, tree, x, dtype):
    """log|psi|, sign, E_L, kinetic and potential energy from the oracle."""
    model = CASES[case][0]
    xt = torch.as_tensor(x, dtype=dtype)
    if model == "ferminet":
        oc = OF.FermiNetConfig(nspins=tuple(cfg.nspins), ndets=cfg.ndets,
                               hidden_dims_single=list(cfg.hidden_dims_single),
                               hidden_dims_double=list(cfg.hidden_dims_double), use_last_layer=cfg.use_last_layer,
                               envelope=cfg.envelope, orbitals_spin_split=cfg.orbitals_spin_split)
        r = OF.evaluate(tree, oc, xt, mol.atoms, dtype=dtype, tangents=True)
        sign = r["sign_logpsi"]
    elif model == "lapnet":
        r = OL.evaluate(tree, lapnet_config(cfg), xt, mol.atoms, dtype=dtype, tangents=True)
        sign = r["sign_logpsi"]
    else:
        oc = OP.PsiformerConfig(nspins=tuple(cfg.nspins), ndets=cfg.ndets, num_layers=cfg.num_layers,
                                num_heads=cfg.num_heads, heads_dim=cfg.heads_dim,
                                mlp_hidden_dims=list(cfg.mlp_hidden_dims), envelope=cfg.envelope,
                                orbitals_spin_split=cfg.orbitals_spin_split, jastrow=cfg.jastrow)
        r = OP.evaluate_fl(tree, oc, xt, mol.atoms, dtype=dtype)
        sign = r["sign"]
    ke = OH.kinetic_from_tangents(r["grad"], r["lap"])
    pe = OH.potential_energy(xt, mol.atoms, mol.charges)
    f = lambda t: t.detach().double().numpy()  # noqa: E731
    return {"logpsi": f(r["logpsi"]), "sign": f(sign), "e_local": f(ke + pe), "kinetic": f(ke), "potential": f(pe)}


def lapnet_config(cfg):
    return OL.LapNetConfig(nspins=tuple(cfg.nspins), ndets=cfg.ndets, num_layers=cfg.num_layers,
                           num_heads=cfg.num_heads, heads_dim=cfg.heads_dim, num_local_updates=cfg.num_local_updates,
                           envelope=cfg.envelope, jastrow=cfg.jastrow, use_input_bias=cfg.use_input_bias,
                           use_backbone_bias=cfg.use_backbone_bias)


def logpsi_fn(case, mol, cfg, tree):
    """FP64 oracle log|psi| of a case's model, as a function of the walkers."""
    if CASES[case][0] == "ferminet":
        oc = OF.FermiNetConfig(nspins=tuple(cfg.nspins), ndets=cfg.ndets,
                               hidden_dims_single=list(cfg.hidden_dims_single),
                               hidden_dims_double=list(cfg.hidden_dims_double), use_last_layer=cfg.use_last_layer,
                               envelope=cfg.envelope, orbitals_spin_split=cfg.orbitals_spin_split)
        return OF.logpsi_fn(tree, oc, mol.atoms)
    if CASES[case][0] == "lapnet":
        return OL.logpsi_fn(tree, lapnet_config(cfg), torch.as_tensor(mol.atoms, dtype=torch.float64))
    oc = OP.PsiformerConfig(nspins=tuple(cfg.nspins), ndets=cfg.ndets, num_layers=cfg.num_layers,
                            num_heads=cfg.num_heads, heads_dim=cfg.heads_dim, mlp_hidden_dims=list(cfg.mlp_hidden_dims),
                            envelope=cfg.envelope, orbitals_spin_split=cfg.orbitals_spin_split, jastrow=cfg.jastrow)
    return OP.logpsi_fn(tree, oc, torch.as_tensor(mol.atoms, dtype=torch.float64))


def build_mh(name):
    """(mol, cfg, tree, flat, walkers, normals, uniforms) of an MH fixture."""
    case, B, steps, _, seed = MH_CASES[name]
    mol, cfg, tree, flat, _ = build(case)
    x = S.init_walkers(mol, B, seed=1)
    draws = [OX.mh_draws(seed, s, B, mol.n_electrons) for s in range(steps)]
    normals = np.stack([d[0] for d in draws]).astype(np.float32)
    uniforms = np.stack([d[1] for d in draws]).astype(np.float32)
    return mol, cfg, tree, flat, x, normals, uniforms


def oracle_mh(name, mol, cfg, tree, x, normals, uniforms):
    case, _, _, stddev, _ = MH_CASES[name]
    f = logpsi_fn(case, mol, cfg, tree)
    xo, lpo, acc, ratios = OM.mh_steps(f, torch.as_tensor(x, dtype=torch.float64),
                                       torch.as_tensor(normals, dtype=torch.float64),
                                       torch.as_tensor(uniforms, dtype=torch.float64), stddev)
    return {"x_final": xo.numpy(), "log_prob": lpo.numpy(), "accepts": acc.numpy(), "ratios": ratios.numpy()}


def oracle_grad(name):
    """(flat, walkers, meta-free values) of a gradient fixture."""
    sys.path.insert(0, os.path.dirname(HERE))
    from helpers import oracle_param_jacobian
    case, B, seed, entries, projections = GRAD_CASES[name]
    mol, cfg, _, flat, _ = build(case)
    x = S.init_walkers(mol, B, seed=1)
    J, lp = oracle_param_jacobian(flat, cfg, mol, x)
    idx, R = grad_probes(flat.size, seed, entries, projections)
    return flat, x, {"entries": idx, "jacobian_entries": J[:, idx], "projections": J @ R,
                     "jacobian_norm": np.linalg.norm(J, axis=1), "logpsi": lp}


def main():
    torch.set_num_threads(os.cpu_count() or 1)
    for name in GRAD_CASES:
        flat, x, v = oracle_grad(name)
        case, B, seed, entries, projections = GRAD_CASES[name]
        meta = {"case": name, "model_case": case, "walkers": B, "seed": seed, "params_sha256": params_sha(flat)}
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), meta=json.dumps(meta), walkers=x.astype(np.float32),
                            **v)
        print(name, "|J| per walker", v["jacobian_norm"])
    for name in MH_CASES:
        mol, cfg, tree, flat, x, normals, uniforms = build_mh(name)
        v = oracle_mh(name, mol, cfg, tree, x, normals, uniforms)
        case, B, steps, stddev, seed = MH_CASES[name]
        meta = {"case": name, "model_case": case, "model": CASES[case][0], "walkers": B, "steps": steps,
                "stddev": stddev, "seed": seed, "params_sha256": params_sha(flat)}
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), meta=json.dumps(meta), walkers=x.astype(np.float32),
                            normals=normals, uniforms=uniforms, **v)
        print(name, "accepts", int(v["accepts"].sum()))
    for case in CASES:
        if case in (c[0] for c in GRAD_CASES.values()):
            continue  # a model for the gradient fixture only
        mol, cfg, tree, flat, x = build(case)
        v64 = oracle_values(case, mol, cfg, tree, x, torch.float64)
        v32 = oracle_values(case, mol, cfg, tree, x, torch.float32)
        meta = {"case": case, "model": CASES[case][0], "system": CASES[case][1], "config": CASES[case][2],
                "walkers": CASES[case][3], "params_seed": 0, "walkers_seed": 1, "params_sha256": params_sha(flat)}
        np.savez_compressed(os.path.join(HERE, f"{case}.npz"), meta=json.dumps(meta), walkers=x.astype(np.float32),
                            **v64, **{f"{k}_fp32": v for k, v in v32.items()})
        print(case, "E_L mean", float(v64["e_local"].mean()))


if __name__ == "__main__":
    main()
