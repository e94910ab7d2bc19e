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
* :class:`EstimatorPipeline`, :class:`EvaluationStage` — ``src/jaqmc/estimator/base.py:287-427``,
  ``src/jaqmc/workflow/stage/evaluation.py:150-272`` (sampling and estimation
  without an optimiser, per-step statistics and the digest).
* :func:`load_reference_checkpoint`, :func:`save_checkpoint` —
  ``src/jaqmc/utils/checkpoint.py:26-274`` (the stage state's ``.npz`` key layout).

Everything numerical runs on the GPU through the C ABI; there is no CPU path.
"""
from __future__ import annotations

import dataclasses
import functools
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
    evaluated by the GB300 library: log|psi|, the MH sampler, the
    forward-Laplacian local energy (the same estimators as FermiNet) and the
    FP32 parameter adjoint (at most 64 electrons, head width <= 64)."""

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
class LapNetWavefunction(FermiNetWavefunction):
    """LapNet ansatz with the SimpleEE Jastrow (hyper-parameters and defaults
    of ``src/jaqmc/app/molecule/wavefunction/lapnet.py:27-75``), evaluated by
    the GB300 library: log|psi|, the MH sampler, the forward-Laplacian local
    energy, the ECP estimator and the FP32 parameter adjoint (``LossAndGrad``;
    at most 64 electrons, head width <= 64).  ``use_layernorm`` is not
    built."""

    num_layers: int = 4
    num_heads: int = 4
    heads_dim: int = 64
    use_layernorm: bool = False
    jastrow: str = "simple_ee"
    use_input_bias: bool = True
    use_backbone_bias: bool = True
    num_local_updates: int = 2
    jastrow_alpha_init: float = 1.0
    precision: str = "mixed"

    @property
    def config(self) -> P.LapNetConfig:
        return P.LapNetConfig(nspins=tuple(self.nspins), ndets=self.ndets, num_layers=self.num_layers,
                              num_heads=self.num_heads, heads_dim=self.heads_dim, use_layernorm=self.use_layernorm,
                              jastrow=self.jastrow, use_input_bias=self.use_input_bias,
                              use_backbone_bias=self.use_backbone_bias, num_local_updates=self.num_local_updates,
                              envelope=self.envelope, jastrow_alpha_init=self.jastrow_alpha_init,
                              orbitals_spin_split=self.orbitals_spin_split)

    def init_params(self, data: MoleculeData, rngs=0) -> DeviceParams:
        seed = int(rngs) if np.isscalar(rngs) else int(np.asarray(rngs).ravel()[0])
        A = np.asarray(data.atoms, np.float64).reshape(-1, 3).shape[0]
        tree = P.init_lapnet(self.config, A, seed=seed)
        return DeviceParams(tree, P.lapnet_leaves(self.config, A), self._dev())

    def model(self, data: MoleculeData, params: DeviceParams) -> _native.NativeLapNet:
        atoms = np.asarray(torch.as_tensor(data.atoms).cpu(), np.float32).reshape(-1, 3)
        charges = np.asarray(torch.as_tensor(data.charges).cpu(), np.float32).reshape(-1)
        key = (atoms.tobytes(), charges.tobytes(), self.precision)
        m = self._models.get(key)
        if m is None:
            m = _native.NativeLapNet(self.config, atoms, charges, precision=self.precision, device=self._dev())
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
    pmoves: np.ndarray  # or a float64 device tensor once the sampler has stepped
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
        # pmove over all ranks' walkers (pmean, src/jaqmc/sampler/mcmc.py:180),
        # kept on the device: no host synchronisation between adaptations
        pmove = global_pmove(accepts.sum(), self.steps * x.shape[0])
        # width adaptation (src/jaqmc/sampler/mcmc.py:182-197)
        counter = state.counter + 1
        t = counter % self.adapt_frequency
        pmoves = torch.as_tensor(state.pmoves, dtype=torch.float64).to(x.device).clone()
        pmoves[t] = pmove
        stddev = state.stddev
        if t == 0:
            stddev = adapt_width(stddev, float(pmoves.mean()), self.pmove_range)
        new_state = MCMCState(stddev, pmoves, counter, state.rng_counter + self.steps, state.seed)
        new_data = {"electrons": x} if isinstance(data, dict) else data.merge({"electrons": x})
        return new_data, {"pmove": pmove}, new_state


def adapt_width(stddev: float, mean_pmove: float, pmove_range=(0.5, 0.55)) -> float:
    """Widen the proposal by 1.1 when the mean acceptance over the last
    adaptation window is above the range, narrow it by 1.1 when below
    (src/jaqmc/sampler/mcmc.py:184-197)."""
    if mean_pmove > pmove_range[1]:
        return stddev * 1.1
    if mean_pmove < pmove_range[0]:
        return stddev / 1.1
    return stddev


def global_pmove(accepted: torch.Tensor, proposals: int, group=None) -> torch.Tensor:
    """Fraction of accepted proposals over every rank's walkers, the pmean of
    pmove (src/jaqmc/sampler/mcmc.py:180).  ``accepted`` is this rank's count
    as a 0-d tensor and ``proposals`` this rank's number of proposals; the
    result is a float64 0-d tensor on ``accepted``'s device.  On one rank it
    is computed on the device without a host synchronisation; with several
    ranks the counts are summed (ranks weighted by their proposals)."""
    acc = accepted.to(torch.float64)
    if _ranks(group) == 1:
        return acc / float(proposals)
    t = allreduce_sum(torch.stack([acc, torch.zeros_like(acc) + float(proposals)]), group)
    return t[0] / t[1]


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
class ECPEnergy:
    """Effective-core-potential energy ``energy:ecp`` (the reference's
    ECPEnergy, src/jaqmc/estimator/ecp/estimator.py:33-155): the local channel
    plus the nonlocal channels integrated on a randomly rotated spherical rule
    around the ``max_core`` nearest ECP atoms of each electron, every
    displaced configuration evaluated by the GPU forward pass
    (``qmc_ecp_energy``).  ``ecp_coefficients`` are PySCF ECP dictionaries,
    ``atom_symbols`` the molecule's element symbols; the rotations come from
    Philox draws keyed by ``rngs`` and the call count (state)."""

    max_core: int = 2
    quadrature_id: str | None = None
    phase_logpsi: Any = None  # the wavefunction
    ecp_coefficients: dict = field(default_factory=dict)
    atom_symbols: list = field(default_factory=list)

    def init(self, data, rngs=None):
        from . import ecp as _ecp
        self._tables = _ecp.ECPTables(self.ecp_coefficients, self.atom_symbols, self.max_core, self.quadrature_id)
        seed = 0 if rngs is None else (int(rngs) if np.isscalar(rngs) else int(np.asarray(rngs).ravel()[0]))
        return {"seed": seed, "calls": 0}

    def evaluate_batch_walkers(self, params, batched_data: BatchedData, prev_walker_stats, state, rngs=None):
        if state is None:
            state = self.init(batched_data.data, rngs)
        wf = self.phase_logpsi
        m = wf.model(batched_data.data, params)
        x = _device_electrons(batched_data.data.electrons, wf._dev())
        loc, nl = m.ecp_energy(x, self._tables.device_tables(m.device), seed=state["seed"],
                               counter=state["calls"])
        return {"energy:ecp": loc + nl}, {**state, "calls": state["calls"] + 1}

    def reduce(self, walker_stats):
        return mean_reduce(walker_stats)


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


# ------------------------------------------------------------ evaluation
class EstimatorPipeline:
    """Ordered estimators (``src/jaqmc/estimator/base.py:287-427``).

    Each estimator sees the walker statistics of the ones before it (the
    kinetic and potential parts feed :class:`TotalEnergy`).  An estimator is an
    object with ``evaluate_batch_walkers`` and optionally ``init``, ``reduce``,
    ``finalize_stats`` and ``finalize_state``, or a plain function
    ``f(params, batched_data, prev_walker_stats, state, rngs) -> (stats, state)``
    (reduced by :func:`mean_reduce`, averaged over steps).
    """

    def __init__(self, estimators: dict, group=None):
        self.estimators = dict(estimators)
        self.group = group
        self._reduce_keys: dict[str, frozenset] = {}

    def init(self, data, rngs=None) -> dict:
        return {name: (est.init(data, rngs) if hasattr(est, "init") else None)
                for name, est in self.estimators.items()}

    def evaluate(self, params, batched_data, state: dict, rngs=None):
        """``(step_stats, state)``: every estimator's ``reduce`` output merged."""
        walker_stats, step_stats, state = {}, {}, dict(state)
        for name, est in self.estimators.items():
            f = est.evaluate_batch_walkers if hasattr(est, "evaluate_batch_walkers") else est
            parts, state[name] = f(params, batched_data, walker_stats, state.get(name), rngs)
            walker_stats.update(parts)
            reduced = est.reduce(parts) if hasattr(est, "reduce") else mean_reduce(parts, group=self.group)
            self._reduce_keys[name] = frozenset(reduced)
            step_stats.update(reduced)
        return step_stats, state

    def finalize_stats(self, batched_stats: dict, state: dict) -> dict:
        """Per-step statistics (leading step axis) -> final values; by default
        the NaN-skipping mean over steps."""
        if not self._reduce_keys:
            raise RuntimeError("finalize_stats() called before evaluate(); key ownership is unknown.")
        out = {}
        for name, est in self.estimators.items():
            own = {k: np.asarray(batched_stats[k]) for k in self._reduce_keys.get(name, ()) if k in batched_stats}
            if hasattr(est, "finalize_stats"):
                out.update(est.finalize_stats(own, state.get(name)))
            else:
                out.update({k: np.nanmean(v, axis=0) for k, v in own.items()})
        return out

    def digest(self, batched_stats: dict, state: dict, *, n_steps: int) -> dict:
        """:meth:`finalize_stats` merged with each estimator's ``finalize_state``."""
        result = self.finalize_stats(batched_stats, state) if batched_stats else {}
        for name, est in self.estimators.items():
            if hasattr(est, "finalize_state"):
                result.update(est.finalize_state(state.get(name), n_steps=n_steps))
        return result


def energy_pipeline(wf, group=None) -> EstimatorPipeline:
    """The molecule workflow's energy estimators: potential, kinetic, total."""
    return EstimatorPipeline({
        "potential": functools.partial(potential_energy, wf=wf),
        "kinetic": EuclideanKinetic(f_log_psi=wf),
        "total_energy": TotalEnergy(),
    }, group=group)


@dataclass
class EvaluationStage:
    """Evaluation work stage: sampling and estimation without parameter
    updates (``src/jaqmc/workflow/stage/evaluation.py:150-272``).

    ``burn_in`` sampler steps, then per iteration one sampler step and the
    estimator pipeline; the per-step statistics are kept (and written to
    ``[prefix_]stats.npz`` when ``save_dir`` is set, the reference's HDF5 file
    in NumPy form) and the digest (:meth:`EstimatorPipeline.digest`) goes to
    ``[prefix_]digest.npz``.  With ``digest_step_interval`` > 0 a preview of
    the running digest is passed to ``log`` every that many steps.
    """

    wf: Any
    sampler: MCMCSampler
    pipeline: EstimatorPipeline
    iterations: int = 10
    burn_in: int = 0
    digest_step_interval: int = 0
    save_dir: str | None = None
    prefix: str = ""
    log: Any = None

    def run(self, params, data, sampler_state, estimator_state=None, rngs=None):
        """Returns ``(digest, stacked_stats, data, sampler_state, estimator_state)``."""
        est_state = estimator_state if estimator_state is not None else self.pipeline.init(data, rngs)

        def sample(data, sampler_state):
            d, _, sampler_state = self.sampler.step(self.wf.batch_log_prob(params, data), data, sampler_state)
            return data.merge({"electrons": d.electrons if hasattr(d, "electrons") else d["electrons"]}), sampler_state

        for _ in range(self.burn_in):
            data, sampler_state = sample(data, sampler_state)
        history: dict[str, list] = {}
        for step in range(self.iterations):
            data, sampler_state = sample(data, sampler_state)
            step_stats, est_state = self.pipeline.evaluate(params, BatchedData(data), est_state, rngs)
            for k, v in step_stats.items():
                history.setdefault(k, []).append(float(v))
            last = step + 1 == self.iterations
            if self.log and ((self.digest_step_interval and (step + 1) % self.digest_step_interval == 0) or last):
                self.log(step, self.pipeline.finalize_stats(history, est_state))
        stacked = {k: np.asarray(v) for k, v in history.items()}
        digest = self.pipeline.digest(stacked, est_state, n_steps=self.iterations)
        if self.save_dir is not None:
            import os
            os.makedirs(self.save_dir, exist_ok=True)
            pre = f"{self.prefix}_" if self.prefix else ""
            np.savez(os.path.join(self.save_dir, f"{pre}stats.npz"), **stacked)
            if digest:
                np.savez(os.path.join(self.save_dir, f"{pre}digest.npz"), **digest)
        return digest, stacked, data, sampler_state, est_state


# ------------------------------------------------------------ checkpoints
# The reference's NumPyCheckpointManager (src/jaqmc/utils/checkpoint.py:26-274)
# writes a work stage's state pytree as one .npz: every leaf under its
# slash-joined key path plus ``step``.  For the sampling stages the state is
# (params, batched_data, sampler_state, estimator_state[, opt_state]), so the
# wavefunction parameters sit at ``params/params/<module path>`` (the Flax
# variables dict), the walkers at ``batched_data/data/electrons`` and the MCMC
# state at ``sampler_state/stddev`` and ``sampler_state/pmoves``.
_CKPT_PARAMS = "params/params/"
_CKPT_ELECTRONS = "batched_data/data/electrons"
# this library's sampler counters (the Philox stream position and seed, the
# adaptation counter), kept apart from the reference's keys, which a
# reference restore reads by its own state's paths and so ignores these
_CKPT_OWN = "qmc_gb300/"


def _param_leaves(wf, n_atoms: int):
    if isinstance(wf, PsiformerWavefunction):
        return P.psiformer_leaves(wf.config, n_atoms)
    return P.ferminet_leaves(wf.config, n_atoms)


def load_reference_checkpoint(path, wf, n_atoms: int, device=None) -> dict:
    """Restore a reference checkpoint into this library's objects.

    Returns ``{"step", "params", "electrons", "sampler_state"}``: ``step`` is
    the run's initial step (saved step + 1, as the reference's
    ``restore_from_file`` returns), ``params`` a :class:`DeviceParams` in the
    layout of ``wf`` (shapes checked leaf by leaf), ``electrons`` the saved
    walkers (or None) and ``sampler_state`` an :class:`MCMCState` with the
    saved proposal width and acceptance history (or None); a file written by
    :func:`save_checkpoint` also restores the Philox stream position, seed and
    adaptation counter, so that a resumed run draws what the uninterrupted run
    would have drawn.
    """
    leaves = _param_leaves(wf, n_atoms)
    with np.load(path, allow_pickle=False) as f:
        tree: dict = {}
        for p, shape in leaves:
            key = _CKPT_PARAMS + "/".join(p)
            if key not in f.files:
                raise KeyError(f"checkpoint {path} has no parameter {key}")
            a = np.asarray(f[key], np.float32)
            if tuple(a.shape) != tuple(shape):
                raise ValueError(f"{key}: checkpoint shape {a.shape}, model expects {tuple(shape)}")
            P._set(tree, p, a)
        electrons = np.asarray(f[_CKPT_ELECTRONS], np.float32) if _CKPT_ELECTRONS in f.files else None
        sstate = None
        if "sampler_state/stddev" in f.files:
            pm = np.asarray(f["sampler_state/pmoves"], np.float64) if "sampler_state/pmoves" in f.files else None

            def own(name):
                k = _CKPT_OWN + name
                return int(np.asarray(f[k]).item()) if k in f.files else 0
            sstate = MCMCState(float(np.asarray(f["sampler_state/stddev"])), pm, own("sampler_counter"),
                               own("sampler_rng_counter"), own("sampler_seed"))
        step = int(np.asarray(f["step"]).item()) + 1 if "step" in f.files else 0
    dev = device if device is not None else (wf._dev() if torch.cuda.is_available() else torch.device("cpu"))
    return {"step": step, "params": DeviceParams(tree, leaves, dev), "electrons": electrons,
            "sampler_state": sstate}


def save_checkpoint(path, step: int, params: DeviceParams, data=None, sampler_state: MCMCState | None = None):
    """Write ``params`` (and optionally the walkers and the MCMC state) with
    the reference's key layout (compressed .npz, as its ``save``).  The file
    holds no optimiser or estimator state."""
    tree = params.tree()
    arrays = {"step": np.asarray(step)}
    for p, _ in params.leaves:
        arrays[_CKPT_PARAMS + "/".join(p)] = np.asarray(P._get(tree, p))
    if data is not None:
        e = data["electrons"] if isinstance(data, dict) else data.electrons
        arrays[_CKPT_ELECTRONS] = np.asarray(torch.as_tensor(e).detach().cpu(), np.float32)
    if sampler_state is not None:
        arrays["sampler_state/stddev"] = np.asarray(sampler_state.stddev, np.float32)
        pm = sampler_state.pmoves
        pm = pm.detach().cpu().numpy() if isinstance(pm, torch.Tensor) else np.asarray(pm)
        arrays["sampler_state/pmoves"] = pm.astype(np.float32)
        arrays[_CKPT_OWN + "sampler_counter"] = np.asarray(sampler_state.counter, np.int64)
        arrays[_CKPT_OWN + "sampler_rng_counter"] = np.asarray(sampler_state.rng_counter, np.uint64)
        arrays[_CKPT_OWN + "sampler_seed"] = np.asarray(sampler_state.seed, np.uint64)
    with open(path, "wb") as f:
        np.savez_compressed(f, allow_pickle=False, **arrays)
