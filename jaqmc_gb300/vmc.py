"""Host-side mirror of the reference's wavefunction / sampler / estimator
protocols, backed by the GB300 library (``libqmc.so``).

Each class keeps the reference's name, fields, method signatures and stats
keys so that a workflow written against the reference drops onto this
implementation:

* :class:`MoleculeData`, :class:`BatchedData` — ``src/jaqmc/app/molecule/data.py:13-28``,
  ``src/jaqmc/data.py`` (electrons batched on axis 0).
* :class:`FermiNetWavefunction` — ``src/jaqmc/app/molecule/wavefunction/ferminet.py:21-137``
  (``init_params``, ``evaluate``, ``logpsi``, ``phase_logpsi``); evaluation is
  batched (the reference's callers ``vmap`` a single-walker function).
* :class:`MCMCSampler` — ``src/jaqmc/sampler/mcmc.py:58-199`` (``init``, ``step``,
  width adaptation, ``pmove``).
* :class:`EuclideanKinetic`, :func:`potential_energy`, :class:`TotalEnergy`,
  :class:`LossAndGrad`, :func:`mean_reduce` — ``src/jaqmc/estimator/kinetic/euclidean.py:29-135``,
  ``src/jaqmc/app/molecule/hamiltonian.py:9-22``, ``src/jaqmc/estimator/total_energy.py:16-70``,
  ``src/jaqmc/estimator/loss_grad.py:25-128``, ``src/jaqmc/estimator/base.py:27-53``.

Everything numerical runs on the GPU through the C ABI; there is no CPU path.
"""
from __future__ import annotations

import dataclasses
from dataclasses import dataclass, field
from typing import Any, NamedTuple

import numpy as np
import torch
import torch.distributed

from . import _native
from . import params as P


# ----------------------------------------------------------------- data
@dataclass
class MoleculeData:
    electrons: Any  # (n, 3) or (B, n, 3)
    atoms: Any      # (A, 3)
    charges: Any    # (A,)

    def merge(self, other: dict) -> "MoleculeData":
        return dataclasses.replace(self, **other)

    def subset(self, keys):
        return {k: getattr(self, k) for k in keys}

    def __getitem__(self, key):
        return getattr(self, key)


@dataclass
class BatchedData:
    data: MoleculeData
    fields_with_batch: list = field(default_factory=lambda: ["electrons"])

    @property
    def batch_size(self) -> int:
        return int(self.data.electrons.shape[0])


def _device_electrons(e, device) -> torch.Tensor:
    t = torch.as_tensor(e)
    if t.dim() == 2:
        t = t.unsqueeze(0)
    return t.to(device=device, dtype=torch.float32).contiguous()


# ----------------------------------------------------------------- wavefunction
class DeviceParams:
    """A parameter tree plus its flat float32 copy on the device (the layout of
    ``qmc_model_set_params``).  Optimisers may update ``flat`` in place; call
    :meth:`touch` afterwards so the model reloads it."""

    def __init__(self, tree, leaves, device):
        self.leaves = leaves
        self.flat = torch.as_tensor(P.flatten(tree, leaves), device=device)
        self.version = 0

    def touch(self):
        self.version += 1

    def tree(self):
        return P.unflatten(self.flat.detach().cpu().numpy(), self.leaves)


@dataclass
class FermiNetWavefunction:
    """FermiNet ansatz (same hyper-parameters and defaults as the reference)
    evaluated by the GB300 library.  ``precision`` selects the plain FP32 or the
    split-BF16 tensor-core form."""

    nspins: tuple = (1, 1)
    ndets: int = 16
    hidden_dims_single: list = field(default_factory=lambda: [256] * 4)
    hidden_dims_double: list = field(default_factory=lambda: [32] * 4)
    use_last_layer: bool = False
    envelope: str = "abs_isotropic"
    orbitals_spin_split: bool = True
    full_det: bool = True
    precision: str = "fp32"
    device: Any = None

    def __post_init__(self):
        self._models = {}
        self._loaded = {}

    @property
    def config(self) -> P.FermiNetConfig:
        return P.FermiNetConfig(nspins=tuple(self.nspins), ndets=self.ndets,
                                hidden_dims_single=list(self.hidden_dims_single),
                                hidden_dims_double=list(self.hidden_dims_double),
                                use_last_layer=self.use_last_layer, envelope=self.envelope,
                                orbitals_spin_split=self.orbitals_spin_split)

    def _dev(self):
        dev = torch.device(self.device or "cuda")
        return dev if dev.index is not None else torch.device("cuda", torch.cuda.current_device())

    # -- protocol ------------------------------------------------------
    def init_params(self, data: MoleculeData, rngs=0) -> DeviceParams:
        seed = int(rngs) if np.isscalar(rngs) else int(np.asarray(rngs).ravel()[0])
        atoms = np.asarray(data.atoms, np.float64).reshape(-1, 3)
        tree = P.init_ferminet(self.config, atoms.shape[0], seed=seed)
        return DeviceParams(tree, P.ferminet_leaves(self.config, atoms.shape[0]), self._dev())

    def model(self, data: MoleculeData, params: DeviceParams) -> _native.NativeFermiNet:
        atoms = np.asarray(torch.as_tensor(data.atoms).cpu(), np.float32).reshape(-1, 3)
        charges = np.asarray(torch.as_tensor(data.charges).cpu(), np.float32).reshape(-1)
        key = (atoms.tobytes(), charges.tobytes(), self.precision)
        m = self._models.get(key)
        if m is None:
            m = _native.NativeFermiNet(self.config, atoms, charges, precision=self.precision,
                                       device=self._dev())
            self._models[key] = m
        stamp = (id(params), params.version)
        if self._loaded.get(key) != stamp:
            m.set_params(params.flat)
            self._loaded[key] = stamp
        return m

    def evaluate(self, params: DeviceParams, data: MoleculeData) -> dict:
        m = self.model(data, params)
        lp, sg, fl = m.forward(_device_electrons(data.electrons, self._dev()))
        return {"logpsi": lp, "sign_logpsi": sg, "flags": fl}

    def logpsi(self, params, data):
        return self.evaluate(params, data)["logpsi"]

    def phase_logpsi(self, params, data):
        out = self.evaluate(params, data)
        return out["sign_logpsi"], out["logpsi"]

    def orbitals(self, params, data):
        raise NotImplementedError("orbital matrices are internal to the GPU path (pretraining is out of scope)")

    def batch_log_prob(self, params: DeviceParams, data: MoleculeData) -> "BoundLogProb":
        """The ``2 log|psi|`` callable that :class:`MCMCSampler` runs on the GPU."""
        return BoundLogProb(self, params, data)


@dataclass
class PsiformerWavefunction(FermiNetWavefunction):
    """Psiformer ansatz with the SimpleEE Jastrow (hyper-parameters and
    defaults of ``src/jaqmc/app/molecule/wavefunction/psiformer.py:38-94``),
    evaluated by the GB300 library: log|psi| and the MH sampler.  Its local
    energy is not provided by the library (value path only)."""

    num_layers: int = 4
    num_heads: int = 4
    heads_dim: int = 64
    mlp_hidden_dims: list = field(default_factory=lambda: [256])
    jastrow: str = "simple_ee"
    jastrow_alpha_init: float = 1.0
    precision: str = "mixed"

    @property
    def config(self) -> P.PsiformerConfig:
        return P.PsiformerConfig(nspins=tuple(self.nspins), ndets=self.ndets, num_layers=self.num_layers,
                                 num_heads=self.num_heads, heads_dim=self.heads_dim,
                                 mlp_hidden_dims=list(self.mlp_hidden_dims), envelope=self.envelope,
                                 orbitals_spin_split=self.orbitals_spin_split, jastrow=self.jastrow,
                                 jastrow_alpha_init=self.jastrow_alpha_init)

    def init_params(self, data: MoleculeData, rngs=0) -> DeviceParams:
        seed = int(rngs) if np.isscalar(rngs) else int(np.asarray(rngs).ravel()[0])
        A = np.asarray(data.atoms, np.float64).reshape(-1, 3).shape[0]
        tree = P.init_psiformer(self.config, A, seed=seed)
        return DeviceParams(tree, P.psiformer_leaves(self.config, A), self._dev())

    def model(self, data: MoleculeData, params: DeviceParams) -> _native.NativePsiformer:
        atoms = np.asarray(torch.as_tensor(data.atoms).cpu(), np.float32).reshape(-1, 3)
        charges = np.asarray(torch.as_tensor(data.charges).cpu(), np.float32).reshape(-1)
        key = (atoms.tobytes(), charges.tobytes(), self.precision)
        m = self._models.get(key)
        if m is None:
            m = _native.NativePsiformer(self.config, atoms, charges, precision=self.precision, device=self._dev())
            self._models[key] = m
        stamp = (id(params), params.version)
        if self._loaded.get(key) != stamp:
            m.set_params(params.flat)
            self._loaded[key] = stamp
        return m


@dataclass
class BoundLogProb:
    """``x -> 2 log|psi(x)|`` bound to a wavefunction, parameters and system."""

    wf: FermiNetWavefunction
    params: DeviceParams
    data: MoleculeData

    def __call__(self, electrons):
        return 2.0 * self.wf.logpsi(self.params, self.data.merge({"electrons": electrons}))


# ----------------------------------------------------------------- sampler
class MCMCState(NamedTuple):
    stddev: float
    pmoves: np.ndarray
    counter: int
    rng_counter: int
    seed: int


@dataclass
class MCMCSampler:
    """All-electron Gaussian Metropolis-Hastings sampler (Philox draws on the GPU)."""

    steps: int = 10
    initial_width: float = 0.1
    adapt_frequency: int = 100
    pmove_range: tuple = (0.5, 0.55)

    def init(self, data, rngs=0) -> MCMCState:
        seed = int(rngs) if np.isscalar(rngs) else int(np.asarray(rngs).ravel()[0])
        return MCMCState(float(self.initial_width), np.zeros(self.adapt_frequency), 0, 0, seed)

    def step(self, batch_log_prob: BoundLogProb, data, state: MCMCState, rngs=None):
        if not isinstance(batch_log_prob, BoundLogProb):
            raise TypeError("MCMCSampler.step needs the BoundLogProb of a GB300 wavefunction "
                            "(FermiNetWavefunction.batch_log_prob)")
        if self.steps == 0:
            return data, {"pmove": 0.0}, state
        wf, params, system = batch_log_prob.wf, batch_log_prob.params, batch_log_prob.data
        electrons = data["electrons"] if isinstance(data, dict) else data.electrons
        x = _device_electrons(electrons, wf._dev()).clone()
        m = wf.model(system, params)
        accepts = torch.zeros(x.shape[0], dtype=torch.int32, device=x.device)
        m.mh_steps(x, self.steps, state.stddev, state.seed, state.rng_counter, accepts=accepts)
        pmove = float(accepts.sum().item()) / (self.steps * x.shape[0])
        # width adaptation (src/jaqmc/sampler/mcmc.py:182-197)
        counter = state.counter + 1
        t = counter % self.adapt_frequency
        pmoves = state.pmoves.copy()
        pmoves[t] = pmove
        stddev = state.stddev
        if t == 0:
            mean = float(np.mean(pmoves))
            if mean > self.pmove_range[1]:
                stddev = stddev * 1.1
            elif mean < self.pmove_range[0]:
                stddev = stddev / 1.1
        new_state = MCMCState(stddev, pmoves, counter, state.rng_counter + self.steps, state.seed)
        new_data = {"electrons": x} if isinstance(data, dict) else data.merge({"electrons": x})
        return new_data, {"pmove": pmove}, new_state


# ------------------------------------------------------- data-parallel ranks
# Walkers are sharded across ranks (one GPU each) with no data-path
# collective; the reference's per-step exchanges are host-side reductions of a
# few numbers: the pmean of the energy statistics (src/jaqmc/estimator/base.py:
# 43-48), the all-gather of the clip window (src/jaqmc/utils/clip.py:21,38)
# and the pmean of the gradient.  They run over torch.distributed when a
# process group with more than one rank is initialised, and are identities
# otherwise.
def _ranks(group=None) -> int:
    d = torch.distributed
    return d.get_world_size(group) if d.is_available() and d.is_initialized() else 1


def combine_moments(mean: float, var: float, count: int, group=None):
    """Global (mean, variance, count) from each rank's FP64 batch moments,
    weighting ranks by their walker counts."""
    if _ranks(group) == 1:
        return mean, var, count
    t = torch.tensor([count * mean, count * (var + mean * mean), float(count)], dtype=torch.float64,
                     device=_collective_device(group))
    torch.distributed.all_reduce(t, group=group)
    n = float(t[2])
    m = float(t[0]) / n
    return m, float(t[1]) / n - m * m, int(n)


def _collective_device(group=None):
    backend = torch.distributed.get_backend(group)
    return torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else torch.device("cpu")


def gather_walkers(x: torch.Tensor, group=None) -> torch.Tensor:
    """All ranks' per-walker values concatenated in rank order (equal batch
    sizes per rank, as the reference's all_gather assumes)."""
    if _ranks(group) == 1:
        return x
    dev = _collective_device(group)
    xl = x.detach().to(dev)
    parts = [torch.empty_like(xl) for _ in range(_ranks(group))]
    torch.distributed.all_gather(parts, xl, group=group)
    return torch.cat(parts).to(x.device)


def allreduce_sum(x: torch.Tensor, group=None) -> torch.Tensor:
    if _ranks(group) == 1:
        return x
    dev = _collective_device(group)
    t = x.detach().to(dev).clone()
    torch.distributed.all_reduce(t, group=group)
    return t.to(x.device)


# ----------------------------------------------------------------- estimators
def mean_reduce(walker_stats: dict, include_variance: bool = True, group=None) -> dict:
    """FP64 walker-batch mean and variance on the GPU (NaNs skipped), combined
    across ranks."""
    out = {}
    for k, v in walker_stats.items():
        x = torch.as_tensor(v).reshape(-1)
        mv = _native.reduce_mean_var(x).cpu().numpy()
        count = int(torch.isfinite(x).sum()) if _ranks(group) > 1 else x.numel()
        m, var, _ = combine_moments(float(mv[0]), float(mv[1]), count, group)
        out[k] = m
        if include_variance:
            out[f"{k}_var"] = var
    return out


class _EnergyCache:
    """Local energies of the last (params, walkers) evaluated, shared by the
    kinetic and potential estimators so one GPU pass serves both."""

    def __init__(self):
        self.key = None
        self.value = None

    def get(self, wf, params, data):
        e = data.electrons
        key = (id(wf), id(params), params.version, id(e), getattr(e, "_version", None))
        if self.key != key:
            m = wf.model(data, params)
            self.value = m.local_energy(_device_electrons(e, wf._dev()))
            self.key = key
        return self.value


_energy_cache = _EnergyCache()


@dataclass
class EuclideanKinetic:
    """Forward-Laplacian kinetic energy ``-1/2 (lap log|psi| + |grad log|psi||^2)``."""

    f_log_psi: Any = None  # the FermiNetWavefunction
    data_field: str = "electrons"

    def init(self, data, rngs=None):
        return None

    def evaluate_batch_walkers(self, params, batched_data: BatchedData, prev_walker_stats, state, rngs=None):
        out = _energy_cache.get(self.f_log_psi, params, batched_data.data)
        return {"energy:kinetic": out["kinetic"]}, state

    def reduce(self, walker_stats):
        return mean_reduce(walker_stats)


def potential_energy(params, batched_data: BatchedData, prev_walker_stats, state, rngs=None, wf=None):
    """Coulomb potential per walker (computed in the same GPU pass as E_L)."""
    out = _energy_cache.get(wf, params, batched_data.data)
    return {"energy:potential": out["potential"]}, state


@dataclass
class TotalEnergy:
    output_name: str = "total_energy"
    components: list | None = None

    def evaluate_batch_walkers(self, params, batched_data, prev_walker_stats, state, rngs=None):
        keys = self.components or [k for k in prev_walker_stats if k.startswith("energy:")]
        total = None
        for k in keys:
            total = prev_walker_stats[k] if total is None else total + prev_walker_stats[k]
        return {self.output_name: total}, state

    def reduce(self, walker_stats):
        return mean_reduce(walker_stats)


def clip_observable(x: torch.Tensor, method: str = "mad", scale: float = 5.0, group=None) -> torch.Tensor:
    """MAD / IQR clipping window over all ranks' walkers (``src/jaqmc/utils/clip.py:11-68``):
    medians and quartiles as ``nanmedian`` / ``nanquantile`` (the two middle
    values averaged for an even count)."""
    if method == "none":
        return x
    if method not in ("mad", "iqr"):
        raise ValueError(f"Unknown clip method {method!r}.")
    allx = gather_walkers(x, group).double()
    if method == "mad":
        med = torch.nanquantile(allx, 0.5)
        dev = torch.nanquantile((allx - med).abs(), 0.5)
        lo, hi = med - scale * dev, med + scale * dev
    else:
        q = torch.nanquantile(allx, torch.tensor([0.25, 0.75], dtype=torch.float64, device=allx.device))
        iqr = q[1] - q[0]
        lo, hi = q[0] - scale * iqr, q[1] + scale * iqr
    return x.clamp(lo.to(x.dtype).item(), hi.to(x.dtype).item())


def energy_gradient_weights(loss: torch.Tensor, clip_method: str = "mad", clip_scale: float = 5.0, group=None):
    """c_w = 2 (E_c,w - <E_c>) / B_total with the clipped local energies of all
    ranks (``src/jaqmc/estimator/loss_grad.py:96-128``); the gradient is then
    sum_w c_w d log|psi_w| / d theta summed over ranks."""
    ec = clip_observable(loss.double(), clip_method, clip_scale, group)
    tot = allreduce_sum(torch.stack([ec.sum(), torch.tensor(float(ec.numel()), dtype=torch.float64,
                                                             device=ec.device)]), group)
    mean, B = tot[0] / tot[1], tot[1]
    return 2.0 * (ec - mean) / B, ec


@dataclass
class LossAndGrad:
    """VMC energy gradient ``2 (<E_c g> - <E_c><g>)`` through the GPU adjoint;
    the per-walker gradients are contracted on the device instead of being
    materialised (``per_walker=True`` keeps them, e.g. for SR)."""

    loss_key: str = "total_energy"
    clip_method: str = "mad"
    clip_scale: float = 5.0
    f_log_psi: Any = None
    per_walker: bool = False

    def evaluate_batch_walkers(self, params, batched_data, prev_walker_stats, state, rngs=None):
        return {"loss": prev_walker_stats[self.loss_key]}, state

    def gradient(self, params, batched_data: BatchedData, loss: torch.Tensor, group=None):
        wf = self.f_log_psi
        loss = torch.as_tensor(loss).to(wf._dev()).double()
        weights, ec = energy_gradient_weights(loss, self.clip_method, self.clip_scale, group)
        m = wf.model(batched_data.data, params)
        J, g, _ = m.grad(_device_electrons(batched_data.data.electrons, wf._dev()), weights=weights,
                         per_walker=self.per_walker)
        g = allreduce_sum(g, group)
        stats = {"loss": float(loss.mean()), "clipped_loss": float(ec.mean()), "grads": g}
        if J is not None:
            stats["grad_logpsi"] = J
        return stats
