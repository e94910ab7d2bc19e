"""JAX front end over the XLA FFI handlers in ``xla/qmc_xla_ffi.cc`` — UNTESTED.

Neither the development container nor the GPU image has jax/jaxlib, so this
module is written to the documented ``jax.ffi`` API and has never run.  It
provides ``MoleculeWavefunction``-compatible batched callables:

* :func:`logpsi` — ``jax.ffi.ffi_call("qmc_forward", ...)`` with
  ``vmap_method="broadcast_all"`` so that the reference's ``jax.vmap`` over
  walkers maps onto one batched call;
* :func:`local_energy` and :func:`mh_steps` — the estimator and sampler paths.

Known limits: the reference's forward-Laplacian interpreter and KFAC's jaxpr
pattern matcher cannot see inside a custom call, so the kinetic energy must
come from :func:`local_energy` (selected with
``estimators.energy.kinetic.module=``) and KFAC needs explicit layer
statistics; SR or Adam work with the adjoint gradients.
"""
from __future__ import annotations

import ctypes
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
XLA_LIB = HERE / "libqmc_xla.so"


def build() -> Path:
    """Compile the FFI handlers against jaxlib's headers (needs jax)."""
    import jax  # noqa: F401  (fails where jax is absent)

    inc = jax.ffi.include_dir()
    cmd = ["g++", "-O2", "-std=c++17", "-shared", "-fPIC", f"-I{inc}", f"-I{HERE.parent / 'include'}",
           "-I/usr/local/cuda/include", str(HERE / "xla" / "qmc_xla_ffi.cc"), "-o", str(XLA_LIB),
           f"-L{HERE}", "-lqmc", "-Wl,-rpath," + str(HERE)]
    subprocess.run(cmd, check=True)
    return XLA_LIB


def register():
    import jax

    lib = ctypes.cdll.LoadLibrary(str(XLA_LIB))
    for name, sym in (("qmc_forward", "QmcForward"), ("qmc_local_energy", "QmcLocalEnergy"),
                      ("qmc_mh_steps", "QmcMhSteps")):
        jax.ffi.register_ffi_target(name, jax.ffi.pycapsule(getattr(lib, sym)), platform="CUDA")


def _ws(model, op, B):
    ws, nb = model.workspace(op, B)
    return dict(model=int(model.h.value), workspace=int(ws.data_ptr()), workspace_bytes=int(ws.numel()))


def logpsi(model, params, electrons):
    """Batched log|psi| and sign of ``(B, n, 3)`` float32 electrons; ``params``
    is the flat float32 parameter vector (reference leaf order)."""
    import jax
    import jax.numpy as jnp

    B = electrons.shape[0]
    out = (jax.ShapeDtypeStruct((B,), jnp.float32), jax.ShapeDtypeStruct((B,), jnp.float32))
    call = jax.ffi.ffi_call("qmc_forward", out, vmap_method="broadcast_all")
    return call(params, electrons, **_ws(model, 0, B))


def local_energy(model, params, electrons):
    """(E_L, kinetic, potential) per walker."""
    import jax
    import jax.numpy as jnp

    B = electrons.shape[0]
    shp = jax.ShapeDtypeStruct((B,), jnp.float32)
    call = jax.ffi.ffi_call("qmc_local_energy", (shp, shp, shp), vmap_method="broadcast_all")
    return call(params, electrons, **_ws(model, 1, B))


def mh_steps(model, params, electrons, counter, steps, stddev, seed):
    """``steps`` MH updates; ``counter`` is a uint64[1] device array threaded
    through calls like a PRNG key.  Returns (electrons, log_prob, accepts,
    counter)."""
    import jax
    import jax.numpy as jnp

    B = electrons.shape[0]
    out = (jax.ShapeDtypeStruct(electrons.shape, jnp.float32), jax.ShapeDtypeStruct((B,), jnp.float32),
           jax.ShapeDtypeStruct((B,), jnp.uint32), jax.ShapeDtypeStruct((1,), jnp.uint64))
    call = jax.ffi.ffi_call("qmc_mh_steps", out, vmap_method="broadcast_all")
    return call(params, electrons, counter, steps=int(steps), stddev=float(stddev), seed=int(seed),
                **_ws(model, 2, B))


class FermiNetWavefunction:
    """``MoleculeWavefunction``-shaped front end (``src/jaqmc/app/molecule/
    wavefunction/ferminet.py:21-135``) whose log|psi| is one batched custom
    call.  ``init_params`` returns the flat parameter vector; ``logpsi`` is
    written for the reference's ``jax.vmap`` over walkers (broadcast_all).
    UNTESTED."""

    full_det = True

    def __init__(self, nspins=(1, 1), ndets=16, hidden_dims_single=(256,) * 4, hidden_dims_double=(32,) * 4,
                 envelope="abs_isotropic", orbitals_spin_split=True, precision="fp32"):
        from . import params as P
        self.cfg = P.FermiNetConfig(nspins=tuple(nspins), ndets=ndets, hidden_dims_single=list(hidden_dims_single),
                                    hidden_dims_double=list(hidden_dims_double), envelope=envelope,
                                    orbitals_spin_split=orbitals_spin_split)
        self.precision = precision
        self._models = {}

    def model(self, data):
        import numpy as np

        from . import _native
        key = (np.asarray(data.atoms).tobytes(), np.asarray(data.charges).tobytes())
        if key not in self._models:
            self._models[key] = _native.NativeFermiNet(self.cfg, np.asarray(data.atoms), np.asarray(data.charges),
                                                       precision=self.precision)
        return self._models[key]

    def init_params(self, data, rngs):
        import jax.numpy as jnp
        import numpy as np

        from . import params as P
        A = np.asarray(data.atoms).reshape(-1, 3).shape[0]
        seed = int(np.asarray(rngs).ravel()[-1]) if rngs is not None else 0
        return jnp.asarray(P.flatten(P.init_ferminet(self.cfg, A, seed=seed), P.ferminet_leaves(self.cfg, A)))

    def phase_logpsi(self, params, data):
        lp, sign = logpsi(self.model(data), params, data.electrons)
        return sign, lp

    def logpsi(self, params, data):
        return logpsi(self.model(data), params, data.electrons)[0]


class PsiformerWavefunction(FermiNetWavefunction):
    """``PsiformerWavefunction``-shaped front end (``src/jaqmc/app/molecule/
    wavefunction/psiformer.py:38-146``) over the same three custom calls: the
    library's Psiformer handle serves log|psi|, MH steps and the
    forward-Laplacian local energy.  UNTESTED."""

    def __init__(self, nspins=(1, 1), ndets=16, num_layers=4, num_heads=4, heads_dim=64, mlp_hidden_dims=(256,),
                 envelope="abs_isotropic", orbitals_spin_split=True, jastrow="simple_ee", precision="mixed"):
        from . import params as P
        self.cfg = P.PsiformerConfig(nspins=tuple(nspins), ndets=ndets, num_layers=num_layers, num_heads=num_heads,
                                     heads_dim=heads_dim, mlp_hidden_dims=list(mlp_hidden_dims), envelope=envelope,
                                     orbitals_spin_split=orbitals_spin_split, jastrow=jastrow)
        self.precision = precision
        self._models = {}

    def model(self, data):
        import numpy as np

        from . import _native
        key = (np.asarray(data.atoms).tobytes(), np.asarray(data.charges).tobytes())
        if key not in self._models:
            self._models[key] = _native.NativePsiformer(self.cfg, np.asarray(data.atoms), np.asarray(data.charges),
                                                        precision=self.precision)
        return self._models[key]

    def init_params(self, data, rngs):
        import jax.numpy as jnp
        import numpy as np

        from . import params as P
        A = np.asarray(data.atoms).reshape(-1, 3).shape[0]
        seed = int(np.asarray(rngs).ravel()[-1]) if rngs is not None else 0
        return jnp.asarray(P.flatten(P.init_psiformer(self.cfg, A, seed=seed), P.psiformer_leaves(self.cfg, A)))


class LapNetWavefunction(FermiNetWavefunction):
    """``LapNetWavefunction``-shaped front end (``src/jaqmc/app/molecule/
    wavefunction/lapnet.py:27-140``) over the same custom calls on the
    library's LapNet handle.  UNTESTED."""

    def __init__(self, nspins=(1, 1), ndets=16, num_layers=4, num_heads=4, heads_dim=64, use_layernorm=False,
                 jastrow="simple_ee", use_input_bias=True, use_backbone_bias=True, num_local_updates=2,
                 envelope="abs_isotropic", precision="mixed"):
        from . import params as P
        self.cfg = P.LapNetConfig(nspins=tuple(nspins), ndets=ndets, num_layers=num_layers, num_heads=num_heads,
                                  heads_dim=heads_dim, use_layernorm=use_layernorm, jastrow=jastrow,
                                  use_input_bias=use_input_bias, use_backbone_bias=use_backbone_bias,
                                  num_local_updates=num_local_updates, envelope=envelope)
        self.precision = precision
        self._models = {}

    def model(self, data):
        import numpy as np

        from . import _native
        key = (np.asarray(data.atoms).tobytes(), np.asarray(data.charges).tobytes())
        if key not in self._models:
            self._models[key] = _native.NativeLapNet(self.cfg, np.asarray(data.atoms), np.asarray(data.charges),
                                                     precision=self.precision)
        return self._models[key]

    def init_params(self, data, rngs):
        import jax.numpy as jnp
        import numpy as np

        from . import params as P
        A = np.asarray(data.atoms).reshape(-1, 3).shape[0]
        seed = int(np.asarray(rngs).ravel()[-1]) if rngs is not None else 0
        return jnp.asarray(P.flatten(P.init_lapnet(self.cfg, A, seed=seed), P.lapnet_leaves(self.cfg, A)))


class EuclideanKinetic:
    """``estimators.energy.kinetic`` replacement: kinetic energy from the
    library's fused forward Laplacian (``evaluate_batch_walkers`` protocol of
    ``src/jaqmc/estimator/base.py:126-152``).  UNTESTED."""

    def __init__(self, f_log_psi=None, wf: FermiNetWavefunction | None = None):
        self.wf = wf or getattr(f_log_psi, "__self__", None)

    def init(self, data, rngs):
        return None

    def evaluate_batch_walkers(self, params, batched_data, prev_walker_stats, state, rngs=None):
        data = batched_data.data
        _, ke, _ = local_energy(self.wf.model(data), params, data.electrons)
        return {"energy:kinetic": ke}, state


class MCMCSampler:
    """``sampler`` replacement with the ``init`` / ``step`` protocol of
    ``src/jaqmc/sampler/base.py:28-76``: all-electron Gaussian MH with the
    Philox index in the sampler state.  UNTESTED."""

    def __init__(self, steps=10, initial_width=0.02, seed=0, wf: FermiNetWavefunction | None = None):
        self.steps, self.width, self.seed, self.wf = steps, initial_width, seed, wf

    def init(self, data, rngs):
        import jax.numpy as jnp
        return {"stddev": self.width, "counter": jnp.zeros((1,), jnp.uint64)}

    def step(self, batch_log_prob, data, state, rngs=None):
        params = batch_log_prob.params
        x, _, acc, ctr = mh_steps(self.wf.model(data), params, data.electrons, state["counter"], self.steps,
                                  state["stddev"], self.seed)
        pmove = acc.sum() / (self.steps * acc.shape[0])
        return data.merge({"electrons": x}), {"pmove": pmove}, {**state, "counter": ctr}
