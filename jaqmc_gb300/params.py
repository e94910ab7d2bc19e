"""Wavefunction hyper-parameters, parameter trees and the flat device layout.

Parameter trees mirror the Flax trees of the reference so that a reference
checkpoint's ``params`` can be loaded leaf by leaf:

* FermiNet — ``src/jaqmc/app/molecule/wavefunction/ferminet.py:44-76``:
  ``backbone_layer/Dense_k`` (single and two-electron Dense layers in creation
  order, ``src/jaqmc/wavefunction/backbone/ferminet.py:37-63``),
  ``orbital_layer/SplitChannelDense_0/DenseGeneral_s`` or
  ``orbital_layer/DenseGeneral_0`` (``src/jaqmc/wavefunction/output/orbital.py:60-78``),
  ``envelope_layer/_env_up|_env_down|_env`` with ``pi`` and ``sigma``
  (``src/jaqmc/wavefunction/output/envelope.py:65-95,123-163``; ``sigma`` has a
  per-dimension axis for the diagonal envelope, and the null envelope has no
  parameters).

Initialisation is fan-in scaled ``N(0, 1/fan_in)`` for kernels, zero biases,
and ones for the envelope ``pi`` / ``sigma`` (their reference initialisers).

``flatten`` orders the leaves for the C ABI (``include/qmc.h``): per layer the
single-stream kernel and bias, then the two-electron kernel and bias when that
layer updates the two-electron stream; then the orbital kernels (and biases)
per spin channel; then ``pi`` and ``sigma`` per envelope channel.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass
class FermiNetConfig:
    """Hyper-parameters of ``FermiNetWavefunction`` (same names and defaults)."""

    nspins: tuple = (1, 1)
    ndets: int = 16
    hidden_dims_single: list = field(default_factory=lambda: [256] * 4)
    hidden_dims_double: list = field(default_factory=lambda: [32] * 4)
    use_last_layer: bool = False
    envelope: str = "abs_isotropic"
    orbitals_spin_split: bool = True
    full_det: bool = True

    @property
    def n(self) -> int:
        return int(sum(self.nspins))

    @property
    def channels(self) -> int:
        """Number of non-empty spin channels (aggregation width multiplier)."""
        return int(sum(1 for s in self.nspins if s > 0))

    @property
    def split(self) -> bool:
        """Whether orbitals/envelopes are per spin channel."""
        return bool(self.orbitals_spin_split and self.nspins[0] > 0 and self.nspins[1] > 0)

    def layer_dims(self, n_atoms: int):
        """``[(d1_in, d2_in, d1_out, d2_out, updates_two_electron)]`` per layer."""
        out = []
        d1, d2 = 4 * n_atoms, 4
        L = len(self.hidden_dims_single)
        for l, (s, dd) in enumerate(zip(self.hidden_dims_single, self.hidden_dims_double)):
            upd = l < L - 1 or self.use_last_layer
            out.append((d1, d2, s, dd, upd))
            d1 = s
            if upd:
                d2 = dd
        return out


def _dense(rng, fan_in, fan_out, bias=True):
    d = {"kernel": (rng.standard_normal((fan_in, fan_out)) / np.sqrt(fan_in)).astype(np.float32)}
    if bias:
        d["bias"] = np.zeros((fan_out,), np.float32)
    return d


def init_ferminet(cfg: FermiNetConfig, n_atoms: int, seed: int = 0):
    """A Flax-shaped parameter tree (numpy float32) for ``cfg``."""
    rng = np.random.default_rng(seed)
    n, K, C = cfg.n, cfg.ndets, cfg.channels
    bb, k = {}, 0
    for (d1, d2, s, dd, upd) in cfg.layer_dims(n_atoms):
        bb[f"Dense_{k}"] = _dense(rng, d1 + C * d1 + C * d2, s)
        k += 1
        if upd:
            bb[f"Dense_{k}"] = _dense(rng, d2, dd)
            k += 1
    d_last = cfg.hidden_dims_single[-1]
    if cfg.use_last_layer:
        d_last = d_last + C * d_last + C * cfg.hidden_dims_double[-1]

    def dg():
        return {"kernel": (rng.standard_normal((d_last, K, n)) / np.sqrt(d_last)).astype(np.float32)}

    if cfg.split:
        orb = {"SplitChannelDense_0": {"DenseGeneral_0": dg(), "DenseGeneral_1": dg()}}
    else:
        orb = {"DenseGeneral_0": dg()}

    def env():
        return {"pi": np.ones((n, n_atoms, K), np.float32),
                "sigma": np.ones(envelope_sigma_shape(cfg.envelope, n, n_atoms, K), np.float32)}

    tree = {"backbone_layer": bb, "orbital_layer": orb}
    if cfg.envelope != "null":
        tree["envelope_layer"] = {"_env_up": env(), "_env_down": env()} if cfg.split else {"_env": env()}
    return {"params": tree}


ENVELOPES = ("isotropic", "abs_isotropic", "diagonal", "null")


def envelope_sigma_shape(envelope: str, n: int, n_atoms: int, K: int):
    """Shape of an envelope channel's ``sigma``: ``(n_orb, A, K)`` for the
    isotropic envelopes, ``(n_orb, A, 3, K)`` for the diagonal one
    (src/jaqmc/wavefunction/output/envelope.py:131-134,153-156)."""
    if envelope not in ENVELOPES:
        raise ValueError(f"unknown envelope {envelope!r}: one of {ENVELOPES}")
    return (n, n_atoms, 3, K) if envelope == "diagonal" else (n, n_atoms, K)


def envelope_leaves(envelope: str, split: bool, n: int, n_atoms: int, K: int):
    """``pi`` and ``sigma`` per envelope channel; none for the null envelope
    (src/jaqmc/wavefunction/output/envelope.py:58-96)."""
    if envelope == "null":
        return []
    out = []
    for nm in (["_env_up", "_env_down"] if split else ["_env"]):
        out.append((("envelope_layer", nm, "pi"), (n, n_atoms, K)))
        out.append((("envelope_layer", nm, "sigma"), envelope_sigma_shape(envelope, n, n_atoms, K)))
    return out


def ferminet_leaves(cfg: FermiNetConfig, n_atoms: int):
    """``[(path, shape)]`` in C-ABI order."""
    n, K, C = cfg.n, cfg.ndets, cfg.channels
    out, k = [], 0
    for (d1, d2, s, dd, upd) in cfg.layer_dims(n_atoms):
        out.append((("backbone_layer", f"Dense_{k}", "kernel"), (d1 + C * d1 + C * d2, s)))
        out.append((("backbone_layer", f"Dense_{k}", "bias"), (s,)))
        k += 1
        if upd:
            out.append((("backbone_layer", f"Dense_{k}", "kernel"), (d2, dd)))
            out.append((("backbone_layer", f"Dense_{k}", "bias"), (dd,)))
            k += 1
    if cfg.use_last_layer:
        raise NotImplementedError("use_last_layer=True is not supported by the GPU path")
    d_last = cfg.hidden_dims_single[-1]
    if cfg.split:
        for s in range(2):
            out.append((("orbital_layer", "SplitChannelDense_0", f"DenseGeneral_{s}", "kernel"), (d_last, K, n)))
    else:
        out.append((("orbital_layer", "DenseGeneral_0", "kernel"), (d_last, K, n)))
    out += envelope_leaves(cfg.envelope, cfg.split, n, n_atoms, K)
    return out


def _get(tree, path):
    t = tree["params"]
    for p in path:
        t = t[p]
    return t


def _set(tree, path, value):
    t = tree.setdefault("params", {})
    for p in path[:-1]:
        t = t.setdefault(p, {})
    t[path[-1]] = value


def flatten(tree, leaves) -> np.ndarray:
    parts = []
    for path, shape in leaves:
        a = np.asarray(_get(tree, path), dtype=np.float32)
        if tuple(a.shape) != tuple(shape):
            raise ValueError(f"{'/'.join(path)}: expected shape {shape}, got {a.shape}")
        parts.append(a.reshape(-1))
    return np.concatenate(parts) if parts else np.zeros((0,), np.float32)


def unflatten(flat, leaves):
    tree, off = {}, 0
    flat = np.asarray(flat)
    for path, shape in leaves:
        size = int(np.prod(shape))
        _set(tree, path, flat[off:off + size].reshape(shape).copy())
        off += size
    if off != flat.size:
        raise ValueError(f"flat parameter vector has {flat.size} entries, layout needs {off}")
    return tree


def count(leaves) -> int:
    return int(sum(int(np.prod(s)) for _, s in leaves))


# ------------------------------------------------------------------ Psiformer
@dataclass
class PsiformerConfig:
    """Hyper-parameters of ``PsiformerWavefunction``
    (src/jaqmc/app/molecule/wavefunction/psiformer.py:38-94): same names and
    defaults; Pre-LN layers, biases on, abs_isotropic envelope, SimpleEE
    Jastrow, log-rescaled input features."""

    nspins: tuple = (1, 1)
    ndets: int = 16
    num_layers: int = 4
    num_heads: int = 4
    heads_dim: int = 64
    mlp_hidden_dims: list = field(default_factory=lambda: [256])
    envelope: str = "abs_isotropic"
    orbitals_spin_split: bool = True
    jastrow: str = "simple_ee"
    jastrow_alpha_init: float = 1.0
    rescale: bool = True
    full_det: bool = True

    @property
    def n(self) -> int:
        return int(sum(self.nspins))

    @property
    def dim(self) -> int:
        return self.num_heads * self.heads_dim

    @property
    def split(self) -> bool:
        return bool(self.orbitals_spin_split and self.nspins[0] > 0 and self.nspins[1] > 0)


def psiformer_leaves(cfg: PsiformerConfig, n_atoms: int):
    """``[(path, shape)]`` in C-ABI order (the network's order)."""
    n, K, D, H, Dh = cfg.n, cfg.ndets, cfg.dim, cfg.num_heads, cfg.heads_dim
    out = [(("backbone_layer", "Dense_0", "kernel"), (4 * n_atoms + 1, D)),
           (("backbone_layer", "Dense_0", "bias"), (D,))]
    for l in range(cfg.num_layers):
        base = ("backbone_layer", f"PsiformerLayer_{l}")
        out.append((base + ("LayerNorm_0", "scale"), (D,)))
        out.append((base + ("LayerNorm_0", "bias"), (D,)))
        mha = base + ("MultiHeadDotProductAttention_0",)
        for nm in ("query", "key", "value"):
            out.append((mha + (nm, "kernel"), (D, H, Dh)))
            out.append((mha + (nm, "bias"), (H, Dh)))
        out.append((mha + ("out", "kernel"), (H, Dh, D)))
        out.append((mha + ("out", "bias"), (D,)))
        out.append((base + ("LayerNorm_1", "scale"), (D,)))
        out.append((base + ("LayerNorm_1", "bias"), (D,)))
        dims = list(cfg.mlp_hidden_dims) + [D]
        din = D
        for k, dout in enumerate(dims):
            out.append((base + (f"Dense_{k}", "kernel"), (din, dout)))
            out.append((base + (f"Dense_{k}", "bias"), (dout,)))
            din = dout
    if cfg.split:
        for s in range(2):
            out.append((("orbital_layer", "SplitChannelDense_0", f"DenseGeneral_{s}", "kernel"), (D, K, n)))
    else:
        out.append((("orbital_layer", "DenseGeneral_0", "kernel"), (D, K, n)))
    out += envelope_leaves(cfg.envelope, cfg.split, n, n_atoms, K)
    if cfg.jastrow == "simple_ee":
        out.append((("jastrow_layer", "alpha_par"), (1,)))
        out.append((("jastrow_layer", "alpha_anti"), (1,)))
    return out


def init_psiformer(cfg: PsiformerConfig, n_atoms: int, seed: int = 0):
    """A Flax-shaped parameter tree: fan-in-scaled N(0, 1/fan_in) kernels, zero
    biases, LayerNorm scale 1 / bias 0, envelope pi = sigma = 1, Jastrow alphas
    at ``jastrow_alpha_init``."""
    rng = np.random.default_rng(seed)
    tree = {}
    for path, shape in psiformer_leaves(cfg, n_atoms):
        name = path[-1]
        if name == "kernel":
            if path[-2] == "out":
                fan_in = shape[0] * shape[1]
            else:
                fan_in = shape[0]
            v = (rng.standard_normal(shape) / np.sqrt(fan_in)).astype(np.float32)
        elif name == "scale" or name in ("pi", "sigma"):
            v = np.ones(shape, np.float32)
        elif name in ("alpha_par", "alpha_anti"):
            v = np.full(shape, cfg.jastrow_alpha_init, np.float32)
        else:
            v = np.zeros(shape, np.float32)
        _set(tree, path, v)
    return tree


# ------------------------------------------------------------------ LapNet
@dataclass
class LapNetConfig:
    """Hyper-parameters of ``LapNetWavefunction``
    (src/jaqmc/app/molecule/wavefunction/lapnet.py:27-75): same names and
    defaults (no LayerNorm, biases on, two local updates of the individual
    stream, abs_isotropic envelope, spin-split orbitals, SimpleEE Jastrow,
    log-rescaled input features)."""

    nspins: tuple = (1, 1)
    ndets: int = 16
    num_layers: int = 4
    num_heads: int = 4
    heads_dim: int = 64
    use_layernorm: bool = False
    jastrow: str = "simple_ee"
    use_input_bias: bool = True
    use_backbone_bias: bool = True
    num_local_updates: int = 2
    envelope: str = "abs_isotropic"
    use_orbital_bias: bool = False
    rescale: bool = True
    jastrow_alpha_init: float = 1.0
    full_det: bool = True
    orbitals_spin_split: bool = True

    @property
    def n(self) -> int:
        return int(sum(self.nspins))

    @property
    def dim(self) -> int:
        return self.num_heads * self.heads_dim

    @property
    def split(self) -> bool:
        return bool(self.nspins[0] > 0 and self.nspins[1] > 0)


def lapnet_leaves(cfg: LapNetConfig, n_atoms: int):
    """``[(path, shape)]`` in C-ABI order: the input projection, per layer the
    query/key, value, output and value-update projections and the local
    updates of the individual stream (``src/jaqmc/wavefunction/backbone/
    lapnet/_backbone.py:39-66``), orbitals, envelope, Jastrow."""
    if cfg.use_layernorm:
        raise NotImplementedError("LapNet with use_layernorm=True is not supported")
    n, K, D = cfg.n, cfg.ndets, cfg.dim
    bb = ("backbone_layer",)
    out = [(bb + ("input_projection", "kernel"), (4 * n_atoms + 1, D))]
    if cfg.use_input_bias:
        out.append((bb + ("input_projection", "bias"), (D,)))

    def dense(base, name, din, dout):
        out.append((base + (name, "kernel"), (din, dout)))
        if cfg.use_backbone_bias:
            out.append((base + (name, "bias"), (dout,)))
    for l in range(cfg.num_layers):
        base = bb + (f"layers_{l}",)
        dense(base, "qk_projection", D, 2 * D)
        dense(base, "value_projection", D, D)
        dense(base, "output_projection", D, D)
        dense(base, "value_update", D, D)
        for j in range(cfg.num_local_updates if l < cfg.num_layers - 1 else 0):
            dense(base, f"qk_update_layers_{j}", D, D)
    if cfg.split:
        for s in range(2):
            out.append((("orbital_layer", "SplitChannelDense_0", f"DenseGeneral_{s}", "kernel"), (D, K, n)))
    else:
        out.append((("orbital_layer", "DenseGeneral_0", "kernel"), (D, K, n)))
    out += envelope_leaves(cfg.envelope, cfg.split, n, n_atoms, K)
    if cfg.jastrow == "simple_ee":
        out.append((("jastrow_layer", "alpha_par"), (1,)))
        out.append((("jastrow_layer", "alpha_anti"), (1,)))
    return out


def init_lapnet(cfg: LapNetConfig, n_atoms: int, seed: int = 0):
    """A Flax-shaped parameter tree: fan-in-scaled N(0, 1/fan_in) kernels,
    backbone biases N(0, 1) (the reference's bias initialiser,
    _backbone.py:42-66), envelope ones, Jastrow alphas at jastrow_alpha_init."""
    rng = np.random.default_rng(seed)
    tree = {}
    for path, shape in lapnet_leaves(cfg, n_atoms):
        name = path[-1]
        if name == "kernel":
            v = (rng.standard_normal(shape) / np.sqrt(shape[0])).astype(np.float32)
        elif name == "bias":
            v = rng.standard_normal(shape).astype(np.float32)
        elif name in ("pi", "sigma"):
            v = np.ones(shape, np.float32)
        else:
            v = np.full(shape, cfg.jastrow_alpha_init, np.float32)
        _set(tree, path, v)
    return tree
