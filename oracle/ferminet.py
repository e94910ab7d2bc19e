"""FermiNet log|psi| with optional forward-Laplacian tangents (oracle).

Test infrastructure only.  Restates, for a batch of walkers:

* ``MoleculeFeatures`` — ``src/jaqmc/wavefunction/input/atomic.py:46-79`` with
  ``pair_displacements_within/between`` — ``src/jaqmc/geometry/obc.py:7-88``
  (diagonal shifted by the identity before the norm, then masked, ``:41-47``);
* ``FermiLayers`` — ``src/jaqmc/wavefunction/backbone/ferminet.py:30-90``
  (aggregation order ``[h1, <h1>_up, <h1>_dn, <h2>_up, <h2>_dn]`` ``:82-90``,
  residual ``(x+y)/sqrt(2)`` ``:60-63``, last layer skips the two-electron
  update ``:41-48``);
* ``OrbitalProjection`` — ``src/jaqmc/wavefunction/output/orbital.py:24-31,60-78``;
* ``Envelope`` (isotropic / abs_isotropic / diagonal / null) —
  ``src/jaqmc/wavefunction/output/envelope.py:98-163``;
* ``LogDet`` — ``src/jaqmc/wavefunction/output/logdet.py:53-80``;
* composition — ``src/jaqmc/app/molecule/wavefunction/ferminet.py:76-96``.

Parameters use the Flax tree of the reference (``Dense_k/kernel`` in creation
order, ``SplitChannelDense_0/DenseGeneral_s/kernel``, ``_env_up/pi`` ...), as
plain arrays; the same tree is produced by ``jaqmc_gb300`` for the GPU side.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import torch

from . import lap
from .lap import LT


@dataclass
class FermiNetConfig:
    nspins: tuple
    ndets: int = 16
    hidden_dims_single: list = field(default_factory=lambda: [256] * 4)
    hidden_dims_double: list = field(default_factory=lambda: [32] * 4)
    use_last_layer: bool = False
    envelope: str = "abs_isotropic"  # or "isotropic", "diagonal", "null"
    orbitals_spin_split: bool = True


def _t(a, dtype):
    return torch.as_tensor(a).to(dtype)


def split_channels(h: LT, nspins, axis: int = 1):
    """``split_nonempty_channels`` (``src/jaqmc/utils/array.py:23-47``) on a
    batched axis."""
    nu, nd = nspins
    if (nu > 0) + (nd > 0) <= 1:
        return [h]
    idx_u = (slice(None),) * (axis - 1) + (slice(0, nu),)
    idx_d = (slice(None),) * (axis - 1) + (slice(nu, nu + nd),)
    return [h[idx_u], h[idx_d]]


def features(x: LT, atoms: torch.Tensor):
    """ae ``(B,n,4A)``, ee ``(B,n,n,4)``, r_ae ``(B,n,A)``, ae_vec ``(B,n,A,3)``."""
    B, n, _ = x.shape
    A = atoms.shape[0]
    ae_vec = x.unsqueeze(2) - atoms.reshape(1, 1, A, 3)
    r_ae = lap.norm_last(ae_vec)
    ee_vec = x.unsqueeze(2) - x.unsqueeze(1)
    eye = torch.eye(n, dtype=x.x.dtype)
    r_ee = lap.norm_last(ee_vec + eye.reshape(1, n, n, 1).expand(1, n, n, 3)).scale(1.0 - eye)
    ae = lap.concat([r_ae.unsqueeze(-1), ae_vec], -1).reshape(n, 4 * A)
    ee = lap.concat([r_ee.unsqueeze(-1), ee_vec], -1)
    return ae, ee, r_ae, ae_vec


def aggregate(h1: LT, h2: LT, nspins):
    n = h1.shape[1]
    parts = [h1]
    for ha in split_channels(h1, nspins, 1):
        parts.append(ha.mean(1).unsqueeze(1).expand_as_value((n, h1.shape[-1])))
    for ha in split_channels(h2, nspins, 1):
        parts.append(ha.mean(1))
    return lap.concat(parts, -1)


def residual(x: LT, y: LT) -> LT:
    if tuple(x.shape) == tuple(y.shape):
        return (x + y).scale(1.0 / (2.0 ** 0.5))
    return y


def backbone(p, cfg: FermiNetConfig, ae: LT, ee: LT, dtype):
    layers = list(zip(cfg.hidden_dims_single, cfg.hidden_dims_double))
    h1, h2 = ae, ee
    k = 0
    for li, _ in enumerate(layers):
        d = p[f"Dense_{k}"]
        k += 1
        h1n = lap.tanh(lap.linear(aggregate(h1, h2, cfg.nspins), _t(d["kernel"], dtype), _t(d["bias"], dtype)))
        h1_next = residual(h1, h1n)
        if li < len(layers) - 1 or cfg.use_last_layer:
            d2 = p[f"Dense_{k}"]
            k += 1
            h2 = residual(h2, lap.tanh(lap.linear(h2, _t(d2["kernel"], dtype), _t(d2["bias"], dtype))))
        h1 = h1_next
    if cfg.use_last_layer:
        h1 = aggregate(h1, h2, cfg.nspins)
    return h1


def orbital_projection(p, cfg: FermiNetConfig, h1: LT, dtype) -> LT:
    nu, nd = cfg.nspins
    n = nu + nd
    K = cfg.ndets
    active = [s for s in cfg.nspins if s > 0]
    if cfg.orbitals_spin_split and len(active) > 1:
        outs = []
        for s, hs in enumerate(split_channels(h1, cfg.nspins, 1)):
            W = _t(p["SplitChannelDense_0"][f"DenseGeneral_{s}"]["kernel"], dtype)
            b = p["SplitChannelDense_0"][f"DenseGeneral_{s}"].get("bias")
            ns = hs.shape[1]
            o = lap.linear(hs, W.reshape(W.shape[0], K * n), None if b is None else _t(b, dtype).reshape(K * n))
            outs.append(o.reshape(ns, K, n))
        orb = lap.concat(outs, 1)
    else:
        W = _t(p["DenseGeneral_0"]["kernel"], dtype)
        b = p["DenseGeneral_0"].get("bias")
        orb = lap.linear(h1, W.reshape(W.shape[0], K * n), None if b is None else _t(b, dtype).reshape(K * n))
        orb = orb.reshape(n, K, n)
    return orb.permute(2, 1, 3)  # (B, K, n, n)


def isotropic_envelope(pe, r_ae: LT, is_abs: bool, dtype) -> LT:
    """``_IsotropicEnvelope`` (``envelope.py:123-140``): ``(B, K, n_s, n_orb)``."""
    pi = _t(pe["pi"], dtype)        # (n_orb, A, K)
    sigma = _t(pe["sigma"], dtype)  # (n_orb, A, K)
    B, ns, A = r_ae.shape
    n_orb, _, K = pi.shape
    r = r_ae.reshape(ns, 1, A, 1).expand_as_value((ns, n_orb, A, K))
    sr = r.scale(sigma)
    expo = -lap.absval(sr) if is_abs else -sr
    env = lap.exp(expo).scale(pi).sum(3)   # (B, ns, n_orb, K)
    return env.permute(3, 1, 2)


def diagonal_envelope(pe, ae_vec: LT, dtype) -> LT:
    """``_DiagonalEnvelope`` (``envelope.py:143-163``): per-dimension decay
    rates, ``sum_I pi exp(-|| sigma_I (.) (r_i - R_I) ||)`` ->
    ``(B, K, n_s, n_orb)``.  ``sigma`` has shape ``(n_orb, A, 3, K)``."""
    pi = _t(pe["pi"], dtype)        # (n_orb, A, K)
    sigma = _t(pe["sigma"], dtype)  # (n_orb, A, 3, K)
    B, ns, A, _ = ae_vec.shape
    n_orb, _, _, K = sigma.shape
    v = ae_vec.reshape(ns, 1, A, 3, 1).expand_as_value((ns, n_orb, A, 3, K))
    sv = v.scale(sigma)
    dist = lap.sqrt((sv * sv).sum(4))            # (B, ns, n_orb, A, K)
    env = lap.exp(-dist).scale(pi).sum(3)        # (B, ns, n_orb, K)
    return env.permute(3, 1, 2)


def _one_envelope(pe, cfg, r_ae: LT, ae_vec: LT, dtype) -> LT:
    if cfg.envelope == "diagonal":
        return diagonal_envelope(pe, ae_vec, dtype)
    return isotropic_envelope(pe, r_ae, cfg.envelope == "abs_isotropic", dtype)


def envelope(p, cfg: FermiNetConfig, r_ae: LT, dtype, ae_vec: LT | None = None) -> LT | None:
    """``Envelope.__call__`` (``envelope.py:98-120``); ``None`` for the null
    envelope (the orbitals are used as they are)."""
    if cfg.envelope == "null":
        return None
    if cfg.envelope not in ("isotropic", "abs_isotropic", "diagonal"):
        raise NotImplementedError(cfg.envelope)
    nu, nd = cfg.nspins
    if cfg.orbitals_spin_split and nu > 0 and nd > 0:
        e_u = _one_envelope(p["_env_up"], cfg, r_ae[:nu], None if ae_vec is None else ae_vec[:nu], dtype)
        e_d = _one_envelope(p["_env_down"], cfg, r_ae[nu:], None if ae_vec is None else ae_vec[nu:], dtype)
        return lap.concat([e_u, e_d], 2)
    return _one_envelope(p["_env"], cfg, r_ae, ae_vec, dtype)


def orbitals(params, cfg: FermiNetConfig, x: LT, atoms, dtype) -> LT:
    p = params["params"]
    ae, ee, r_ae, ae_vec = features(x, atoms)
    h1 = backbone(p["backbone_layer"], cfg, ae, ee, dtype)
    orb = orbital_projection(p["orbital_layer"], cfg, h1, dtype)
    env = envelope(p.get("envelope_layer", {}), cfg, r_ae, dtype, ae_vec)
    return orb if env is None else orb * env


def evaluate(params, cfg: FermiNetConfig, electrons, atoms, *, dtype=torch.float64,
             tangents: bool = False):
    """Batched ``FermiNetWavefunction.evaluate``.

    Returns a dict with ``logpsi`` / ``sign_logpsi`` / ``sign_logdets`` /
    ``abs_logdets`` (as the reference's ``RealLogDetOutput``) and, when
    ``tangents`` is set, ``grad`` ``(B, 3n)`` and ``lap`` ``(B,)`` of log|psi|.
    """
    electrons = _t(electrons, dtype)
    atoms = _t(atoms, dtype)
    x = lap.seed(electrons, with_tangents=tangents)
    A = orbitals(params, cfg, x, atoms, dtype)
    sign, ld = lap.slogdet(A)
    s, lp = lap.signed_logsumexp(sign, ld, -1)
    out = {"logpsi": lp.x, "sign_logpsi": s, "sign_logdets": sign, "abs_logdets": ld.x,
           "orbitals": A.x}
    if tangents:
        out["grad"] = lp.J
        out["lap"] = lp.L
    return out


def logpsi_fn(params, cfg, atoms, dtype=torch.float64):
    """A plain ``electrons (B,n,3) -> logpsi (B,)`` closure (autograd-friendly)."""
    def f(electrons):
        x = lap.seed(electrons, with_tangents=False)
        A = orbitals(params, cfg, x, _t(atoms, dtype), dtype)
        sign, ld = lap.slogdet(A)
        return lap.signed_logsumexp(sign, ld, -1)[1].x
    return f
