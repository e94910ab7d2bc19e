"""Psiformer + SimpleEE Jastrow log|psi| (oracle, value and autograd gradient).

Test infrastructure only.  Restates, for a batch of walkers:

* ``MoleculeFeatures(rescale=True)`` — ``src/jaqmc/wavefunction/input/atomic.py:46-79``:
  per atom ``[log(1+r), vec * log(1+r) / r]``;
* ``PsiformerBackbone`` — ``src/jaqmc/wavefunction/backbone/psiformer.py:160-187``:
  spin column (+1 up, -1 down) appended, ``Dense`` to the attention width,
  ``num_layers`` Pre-LN ``PsiformerLayer`` blocks (``:61-99``): LayerNorm
  (eps 1e-5, variance E[x^2] - E[x]^2 as Flax computes it), multi-head
  dot-product attention with biased query / key / value projections, queries
  scaled by 1/sqrt(head_dim), softmax over keys, biased output projection over
  (heads, head_dim), residual; LayerNorm, ``tanh(Dense)`` for each MLP width
  and a final ``tanh(Dense)`` back to the attention width, residual;
* ``OrbitalProjection``, ``Envelope``, ``LogDet`` as for FermiNet
  (``oracle/ferminet.py``);
* ``SimpleEEJastrow`` — ``src/jaqmc/wavefunction/jastrow.py:48-122``:
  ``sum_{i<j, same spin} -1/4 a_par^2 / (a_par + r) + sum_{i up, j down}
  -1/2 a_anti^2 / (a_anti + r)``, added to log|psi|
  (``src/jaqmc/app/molecule/wavefunction/psiformer.py:149-156``).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import torch

from . import ferminet as OF
from . import lap


@dataclass
class PsiformerConfig:
    nspins: tuple
    ndets: int = 16
    num_layers: int = 4
    num_heads: int = 4
    heads_dim: int = 64
    mlp_hidden_dims: list = field(default_factory=lambda: [256])
    envelope: str = "abs_isotropic"
    orbitals_spin_split: bool = True
    jastrow: str = "simple_ee"


def _t(a, dtype):
    return torch.as_tensor(a).to(dtype)


def features(electrons: torch.Tensor, atoms: torch.Tensor, nspins):
    """Rescaled ae features with the spin column ``(B, n, 4A + 1)``, r_ae and
    the e-e distance matrix (diagonal zero)."""
    B, n, _ = electrons.shape
    ae_vec = electrons[:, :, None, :] - atoms[None, None, :, :]
    r_ae = torch.linalg.norm(ae_vec, dim=-1)
    log_r = torch.log1p(r_ae)[..., None]
    ae = torch.cat([log_r, ae_vec * log_r / r_ae[..., None]], dim=-1).reshape(B, n, -1)
    spins = torch.cat([torch.ones(nspins[0]), -torch.ones(nspins[1])]).to(electrons.dtype)
    ae = torch.cat([ae, spins.expand(B, n)[..., None]], dim=-1)
    ee_vec = electrons[:, :, None, :] - electrons[:, None, :, :]
    eye = torch.eye(n, dtype=electrons.dtype)
    r_ee = torch.linalg.norm(ee_vec + eye[..., None], dim=-1) * (1.0 - eye)
    return ae, r_ae, ae_vec, r_ee


def layer_norm(x, scale, bias, eps=1e-5):
    mean = x.mean(-1, keepdim=True)
    var = torch.clamp((x * x).mean(-1, keepdim=True) - mean * mean, min=0.0)
    return (x - mean) * torch.rsqrt(var + eps) * scale + bias


def attention(p, x, cfg: PsiformerConfig, dtype):
    H, Dh = cfg.num_heads, cfg.heads_dim

    def proj(name):
        W = _t(p[name]["kernel"], dtype)   # (D, H, Dh)
        b = _t(p[name]["bias"], dtype)     # (H, Dh)
        return torch.einsum("bnd,dhk->bnhk", x, W) + b
    q = proj("query") / (Dh ** 0.5)
    k = proj("key")
    v = proj("value")
    w = torch.softmax(torch.einsum("bqhd,bkhd->bhqk", q, k), dim=-1)
    o = torch.einsum("bhqk,bkhd->bqhd", w, v)
    Wo = _t(p["out"]["kernel"], dtype)     # (H, Dh, D)
    return torch.einsum("bqhd,hde->bqe", o, Wo) + _t(p["out"]["bias"], dtype)


def dense(p, x, dtype):
    return x @ _t(p["kernel"], dtype) + _t(p["bias"], dtype)


def backbone(p, cfg: PsiformerConfig, ae, dtype):
    x = dense(p["Dense_0"], ae, dtype)
    for l in range(cfg.num_layers):
        q = p[f"PsiformerLayer_{l}"]
        xin = layer_norm(x, _t(q["LayerNorm_0"]["scale"], dtype), _t(q["LayerNorm_0"]["bias"], dtype))
        x = x + attention(q["MultiHeadDotProductAttention_0"], xin, cfg, dtype)
        h = layer_norm(x, _t(q["LayerNorm_1"]["scale"], dtype), _t(q["LayerNorm_1"]["bias"], dtype))
        for k in range(len(cfg.mlp_hidden_dims) + 1):
            h = torch.tanh(dense(q[f"Dense_{k}"], h, dtype))
        x = x + h
    return x


def jastrow(p, cfg: PsiformerConfig, r_ee, dtype):
    """``(B,)`` SimpleEE Jastrow of the e-e distance matrices."""
    nu, nd = cfg.nspins
    n = nu + nd
    a_par = _t(p["alpha_par"], dtype)[0]
    a_anti = _t(p["alpha_anti"], dtype)[0]
    i, j = torch.triu_indices(n, n, 1)
    same = (i < nu) == (j < nu)
    r = r_ee[:, i, j]
    f_par = -(0.25 * a_par ** 2) / (a_par + r)
    f_anti = -(0.5 * a_anti ** 2) / (a_anti + r)
    return torch.where(same, f_par, f_anti).sum(-1)


def evaluate(params, cfg: PsiformerConfig, electrons, atoms, *, dtype=torch.float64):
    """Batched ``PsiformerWavefunction.evaluate``: ``logpsi``, ``sign_logpsi``,
    ``sign_logdets``, ``abs_logdets`` and the Jastrow term."""
    p = params["params"]
    electrons = _t(electrons, dtype)
    atoms = _t(atoms, dtype)
    ae, r_ae, ae_vec, r_ee = features(electrons, atoms, cfg.nspins)
    h = backbone(p["backbone_layer"], cfg, ae, dtype)
    h_lt = lap.const(h, 0)
    orb = OF.orbital_projection(p["orbital_layer"], cfg, h_lt, dtype)
    env = OF.envelope(p.get("envelope_layer", {}), cfg, lap.const(r_ae, 0), dtype, lap.const(ae_vec, 0))
    A = orb if env is None else orb * env
    sign, ld = lap.slogdet(A)
    s, lp = lap.signed_logsumexp(sign, ld, -1)
    J = jastrow(p["jastrow_layer"], cfg, r_ee, dtype) if cfg.jastrow == "simple_ee" else torch.zeros_like(lp.x)
    return {"logpsi": lp.x + J, "sign_logpsi": s, "sign_logdets": sign, "abs_logdets": ld.x, "jastrow": J,
            "orbitals": A.x}


def logpsi_fn(params, cfg, atoms, dtype=torch.float64):
    """``electrons (B,n,3) -> logpsi (B,)`` (autograd-friendly)."""
    def f(electrons):
        return evaluate(params, cfg, electrons, atoms, dtype=dtype)["logpsi"]
    return f


# ---------------------------------------------------------------- forward Laplacian
# The same network carried through the forward-Laplacian tangent algebra of
# ``oracle/lap.py`` (value, Jacobian over the 3n coordinates, Laplacian),
# composing the reference interpreter's rules: linear maps, the elementwise
# rule, and the product rule for the bilinear attention terms
# (``src/jaqmc/laplacian/primitives/arithmetic.py:385``,
# ``dot_general.py:713``, ``elementwise.py:42-72``).
def _bilinear(a, b, eq: str, split_value: bool = False):
    """``einsum(eq, a, b)`` of two tangent carriers (walker axis first in
    every operand): J by the product rule, L = L_a b + a L_b + 2 sum_d J_a J_b.

    Inside ``lap.split_bf16_gemms(..., attention=True)`` every product of
    the tangent terms (and of the values too with ``split_value``) takes its
    operands split into hi + lo bf16 with the lo x lo product dropped, as the
    library's warp-MMA forward-Laplacian attention forms them."""
    from .lap import LT
    lhs, out = eq.split("->")
    ea, eb = lhs.split(",")
    ja, jb, jo = ea[0] + "z" + ea[1:], eb[0] + "z" + eb[1:], out[0] + "z" + out[1:]
    if lap.split_attention():
        def mul(e, u, v):
            uh, ul = lap._split_bf16(u)
            vh, vl = lap._split_bf16(v)
            return (torch.einsum(e, uh, vh) + torch.einsum(e, uh, vl) + torch.einsum(e, ul, vh)).to(u.dtype)
        x = mul(eq, a.x, b.x) if split_value else torch.einsum(eq, a.x, b.x)
    else:
        def mul(e, u, v):
            return torch.einsum(e, u, v)
        x = torch.einsum(eq, a.x, b.x)
    J = mul(f"{ja},{eb}->{jo}", a.J, b.x) + mul(f"{ea},{jb}->{jo}", a.x, b.J)
    L = mul(eq, a.L, b.x) + mul(eq, a.x, b.L) + 2.0 * mul(f"{ja},{jb}->{out}", a.J, b.J)
    return LT(x, J, L)


def features_lt(xl, atoms: torch.Tensor, nspins):
    """Tangent form of :func:`features`: ``(ae (B, n, 4A+1), r_ae (B, n, A))``."""
    B, n, _ = xl.shape
    A = atoms.shape[0]
    ae = xl.unsqueeze(2) - atoms.reshape(A, 3)
    r = lap.norm_last(ae)
    lr = lap.log1p(r)
    vec = ae * (lr * lap.reciprocal(r)).unsqueeze(-1)
    f = lap.concat([lr.unsqueeze(-1), vec], -1).reshape(n, 4 * A)
    spins = torch.cat([torch.ones(nspins[0]), -torch.ones(nspins[1])]).to(xl.x.dtype)
    return lap.concat([f, lap.const(spins.expand(B, n)[..., None].clone(), xl.D)], -1), r


def layer_norm_lt(a, scale, bias, eps=1e-5):
    m = a.mean(-1).unsqueeze(-1)
    var = (a * a).mean(-1).unsqueeze(-1) - m * m
    inv = lap.reciprocal(lap.sqrt(var + eps))
    return ((a - m) * inv).scale(scale) + bias


def attention_lt(p, x, cfg: PsiformerConfig, dtype):
    H, Dh = cfg.num_heads, cfg.heads_dim
    n = x.shape[1]

    def proj(name):
        W = _t(p[name]["kernel"], dtype)
        b = _t(p[name]["bias"], dtype)
        return lap.linear(x, W.reshape(W.shape[0], H * Dh), b.reshape(H * Dh)).reshape(n, H, Dh)
    q = proj("query").scale(1.0 / Dh ** 0.5)
    k = proj("key")
    v = proj("value")
    s = _bilinear(q, k, "bqhd,bkhd->bhqk")
    e = lap.exp(s - s.x.max(-1, keepdim=True).values)
    w = e * lap.reciprocal(e.sum(-1)).unsqueeze(-1)
    o = _bilinear(w, v, "bhqk,bkhd->bqhd", split_value=True).reshape(n, H * Dh)
    Wo = _t(p["out"]["kernel"], dtype)
    return lap.linear(o, Wo.reshape(H * Dh, Wo.shape[-1]), _t(p["out"]["bias"], dtype))


def backbone_lt(p, cfg: PsiformerConfig, ae, dtype):
    x = lap.linear(ae, _t(p["Dense_0"]["kernel"], dtype), _t(p["Dense_0"]["bias"], dtype))
    for l in range(cfg.num_layers):
        q = p[f"PsiformerLayer_{l}"]
        xin = layer_norm_lt(x, _t(q["LayerNorm_0"]["scale"], dtype), _t(q["LayerNorm_0"]["bias"], dtype))
        x = x + attention_lt(q["MultiHeadDotProductAttention_0"], xin, cfg, dtype)
        h = layer_norm_lt(x, _t(q["LayerNorm_1"]["scale"], dtype), _t(q["LayerNorm_1"]["bias"], dtype))
        for k in range(len(cfg.mlp_hidden_dims) + 1):
            h = lap.tanh(lap.linear(h, _t(q[f"Dense_{k}"]["kernel"], dtype), _t(q[f"Dense_{k}"]["bias"], dtype)))
        x = x + h
    return x


def jastrow_lt(p, cfg: PsiformerConfig, xl, dtype):
    nu, nd = cfg.nspins
    n = nu + nd
    if n < 2:
        return lap.const(xl.x.new_zeros(xl.shape[0]), xl.D)
    a_par = _t(p["alpha_par"], dtype)[0]
    a_anti = _t(p["alpha_anti"], dtype)[0]
    i, j = torch.triu_indices(n, n, 1)
    diff = (xl.unsqueeze(2) - xl.unsqueeze(1))[(i, j)]
    r = lap.norm_last(diff)
    same = ((i < nu) == (j < nu)).to(dtype)
    f_par = lap.reciprocal(r + a_par).scale(-0.25 * a_par ** 2)
    f_anti = lap.reciprocal(r + a_anti).scale(-0.5 * a_anti ** 2)
    return (f_par.scale(same) + f_anti.scale(1.0 - same)).sum(-1)


def evaluate_fl(params, cfg: PsiformerConfig, electrons, atoms, *, dtype=torch.float64):
    """Forward-Laplacian ``log|psi|``: ``{"logpsi", "grad" (B, 3n), "lap" (B,),
    "sign"}`` of the Psiformer + SimpleEE Jastrow."""
    p = params["params"]
    e = _t(electrons, dtype)
    R = _t(atoms, dtype)
    xl = lap.seed(e)
    ae, r_ae = features_lt(xl, R, cfg.nspins)
    h = backbone_lt(p["backbone_layer"], cfg, ae, dtype)
    orb = OF.orbital_projection(p["orbital_layer"], cfg, h, dtype)
    env = OF.envelope(p.get("envelope_layer", {}), cfg, r_ae, dtype, xl.unsqueeze(2) - R.reshape(-1, 3))
    sign, ld = lap.slogdet(orb if env is None else orb * env)
    s, lp = lap.signed_logsumexp(sign, ld, -1)
    if cfg.jastrow == "simple_ee":
        lp = lp + jastrow_lt(p["jastrow_layer"], cfg, xl, dtype)
    B = e.shape[0]
    return {"logpsi": lp.x, "grad": lp.J.reshape(B, -1), "lap": lp.L, "sign": s}
