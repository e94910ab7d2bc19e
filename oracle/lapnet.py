"""LapNet log|psi| with optional forward-Laplacian tangents (oracle; test
infrastructure only).

Restates ``LapNetWavefunction`` (``src/jaqmc/app/molecule/wavefunction/
lapnet.py:27-140``) with its backbone (``src/jaqmc/wavefunction/backbone/
lapnet/_backbone.py:15-250``) and attention (``_attention.py:17-29``):

* features: the log-rescaled ae features of ``MoleculeFeatures`` plus a +-1
  spin column (``_backbone.py`` ``individual_stream_block``);
* individual stream hs = input Dense of the features; the dense stream starts
  as hd = hs;
* per layer: (q, k) = split(Dense_qk(hs)); hs <- hs + tanh(Dense_u(hs)) for
  each of ``num_local_updates`` local updates (none in the last layer);
  v = Dense_v(hd); o = softmax(q k^T / sqrt(Dh)) v per head;
  r = hd + Dense_out(o); hd <- r + tanh(Dense_update(r));
* orbitals (spin split) x envelope, log-sum-exp of determinants, plus the
  SimpleEE Jastrow.

The same code carries the forward-Laplacian tangents (value, Jacobian over
the 3n coordinates, Laplacian) through ``oracle/lap.py``; the reference's
sparse Local1 rule for the attention (``_attention.py:144-280``) is an
efficient evaluation of the same derivatives, so the dense rules give the
same numbers.  LayerNorm (``use_layernorm``) is not restated.
"""
from __future__ import annotations

from dataclasses import dataclass

import torch

from . import ferminet as OF
from . import lap
from .psiformer import _bilinear, features_lt, jastrow_lt


@dataclass
class LapNetConfig:
    nspins: tuple
    ndets: int = 16
    num_layers: int = 4
    num_heads: int = 4
    heads_dim: int = 64
    num_local_updates: int = 2
    envelope: str = "abs_isotropic"
    jastrow: str = "simple_ee"
    use_input_bias: bool = True
    use_backbone_bias: bool = True
    orbitals_spin_split: bool = True  # the reference fixes it (lapnet.py:103-108)


def _t(a, dtype):
    return torch.as_tensor(a).to(dtype)


def _dense(p, x, dtype):
    b = p.get("bias")
    return lap.linear(x, _t(p["kernel"], dtype), None if b is None else _t(b, dtype))


def backbone(p, cfg: LapNetConfig, ae, dtype):
    """Dense stream hd after ``num_layers`` LapNet blocks."""
    H, Dh = cfg.num_heads, cfg.heads_dim
    D = H * Dh
    n = ae.shape[1]
    hs = _dense(p["input_projection"], ae, dtype)
    hd = hs
    for l in range(cfg.num_layers):
        q = p[f"layers_{l}"]
        qk = _dense(q["qk_projection"], hs, dtype)
        Q = qk[(slice(None), slice(0, D))].reshape(n, H, Dh).scale(1.0 / Dh ** 0.5)
        K = qk[(slice(None), slice(D, 2 * D))].reshape(n, H, Dh)
        for j in range(cfg.num_local_updates if l < cfg.num_layers - 1 else 0):
            hs = hs + lap.tanh(_dense(q[f"qk_update_layers_{j}"], hs, dtype))
        V = _dense(q["value_projection"], hd, dtype).reshape(n, H, Dh)
        s = _bilinear(Q, K, "bqhd,bkhd->bhqk")
        e = lap.exp(s - s.x.max(-1, keepdim=True).values)
        w = e * lap.reciprocal(e.sum(-1)).unsqueeze(-1)
        o = _bilinear(w, V, "bhqk,bkhd->bqhd", split_value=True).reshape(n, D)
        r = hd + _dense(q["output_projection"], o, dtype)
        hd = r + lap.tanh(_dense(q["value_update"], r, dtype))
    return hd


def evaluate(params, cfg: LapNetConfig, electrons, atoms, *, dtype=torch.float64, tangents: bool = False):
    """Batched ``LapNetWavefunction.evaluate``: ``logpsi``, ``sign_logpsi`` and,
    with ``tangents``, ``grad`` (B, 3n) and ``lap`` (B,) of log|psi|."""
    p = params["params"]
    e = _t(electrons, dtype)
    R = _t(atoms, dtype)
    xl = lap.seed(e, with_tangents=tangents)
    ae, r_ae = features_lt(xl, R, cfg.nspins)
    h = backbone(p["backbone_layer"], cfg, ae, dtype)
    orb = OF.orbital_projection(p["orbital_layer"], cfg, h, dtype)
    env = OF.envelope(p.get("envelope_layer", {}), cfg, r_ae, dtype, xl.unsqueeze(2) - R.reshape(-1, 3))
    sign, ld = lap.slogdet(orb if env is None else orb * env)
    s, lp = lap.signed_logsumexp(sign, ld, -1)
    if cfg.jastrow == "simple_ee":
        lp = lp + jastrow_lt(p["jastrow_layer"], cfg, xl, dtype)
    out = {"logpsi": lp.x, "sign_logpsi": s}
    if tangents:
        out["grad"] = lp.J.reshape(e.shape[0], -1)
        out["lap"] = lp.L
    return out


def logpsi_fn(params, cfg, atoms, dtype=torch.float64):
    def f(electrons):
        return evaluate(params, cfg, electrons, atoms, dtype=dtype)["logpsi"]
    return f
