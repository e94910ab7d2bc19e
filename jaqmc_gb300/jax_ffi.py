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


def logpsi(model, electrons):
    """Batched log|psi| of ``(B, n, 3)`` float32 electrons for a
    ``jaqmc_gb300._native.NativeFermiNet`` model."""
    import jax
    import jax.numpy as jnp

    B = electrons.shape[0]
    ws, nb = model.workspace(0, B)
    out = (jax.ShapeDtypeStruct((B,), jnp.float32), jax.ShapeDtypeStruct((B,), jnp.float32))
    call = jax.ffi.ffi_call("qmc_forward", out, vmap_method="broadcast_all")
    lp, sign = call(electrons, model=int(model.h.value), workspace=int(ws.data_ptr()),
                    workspace_bytes=int(ws.numel()))
    return lp


def local_energy(model, electrons):
    import jax
    import jax.numpy as jnp

    B = electrons.shape[0]
    ws, nb = model.workspace(1, B)
    shp = jax.ShapeDtypeStruct((B,), jnp.float32)
    call = jax.ffi.ffi_call("qmc_local_energy", (shp, shp, shp), vmap_method="broadcast_all")
    return call(electrons, model=int(model.h.value), workspace=int(ws.data_ptr()), workspace_bytes=int(ws.numel()))


def mh_steps(model, electrons, steps, stddev, seed, counter):
    import jax
    import jax.numpy as jnp

    B = electrons.shape[0]
    ws, nb = model.workspace(2, B)
    out = (jax.ShapeDtypeStruct(electrons.shape, jnp.float32), jax.ShapeDtypeStruct((B,), jnp.float32),
           jax.ShapeDtypeStruct((B,), jnp.uint32))
    call = jax.ffi.ffi_call("qmc_mh_steps", out, vmap_method="broadcast_all")
    return call(electrons, model=int(model.h.value), workspace=int(ws.data_ptr()),
                workspace_bytes=int(ws.numel()), steps=int(steps), stddev=float(stddev), seed=int(seed),
                counter=int(counter))
