"""PyTorch wrappers of the GB300 library.

* :class:`FermiNetLogPsi` — ``torch.autograd.Function``: forward is
  ``qmc_forward`` (log|psi| per walker), backward contracts the incoming
  per-walker cotangent with the hand-written parameter adjoint
  (``qmc_grad(weights = dL/dlog|psi|)``), i.e. the reference's
  ``jax.value_and_grad`` of ``LossAndGrad`` (``src/jaqmc/estimator/loss_grad.py:79-83``)
  composed with the loss.
* ``torch.ops.qmc_gb300.ferminet_logpsi`` — the same as a ``torch.library``
  custom op with a registered autograd formula, for use under ``torch.compile``
  graphs that call into the library (the op itself always runs the CUDA path).

Gradients with respect to electron positions are not provided (the local
energy has its own forward-Laplacian entry point).
"""
from __future__ import annotations

import itertools

import torch

from . import _native

_registry: dict[int, _native.NativeFermiNet] = {}
_ids = itertools.count(1)


def register(model: _native.NativeFermiNet) -> int:
    """Handle of ``model`` for the custom op."""
    h = next(_ids)
    _registry[h] = model
    return h


class FermiNetLogPsi(torch.autograd.Function):
    @staticmethod
    def forward(ctx, flat_params, electrons, model):
        model.set_params(flat_params.detach())
        lp, _, _ = model.forward(electrons)
        ctx.model = model
        ctx.save_for_backward(electrons)
        return lp

    @staticmethod
    def backward(ctx, grad_lp):
        (electrons,) = ctx.saved_tensors
        _, g, _ = ctx.model.grad(electrons, weights=grad_lp.detach().double())
        return g.to(torch.float32), None, None


def ferminet_logpsi(flat_params: torch.Tensor, electrons: torch.Tensor, model) -> torch.Tensor:
    return FermiNetLogPsi.apply(flat_params, electrons, model)


@torch.library.custom_op("qmc_gb300::ferminet_logpsi", mutates_args=())
def _logpsi_op(flat_params: torch.Tensor, electrons: torch.Tensor, handle: int) -> torch.Tensor:
    m = _registry[handle]
    m.set_params(flat_params)
    return m.forward(electrons.contiguous())[0]


@_logpsi_op.register_fake
def _(flat_params, electrons, handle):
    return electrons.new_empty(electrons.shape[0])


def _setup_context(ctx, inputs, output):
    ctx.save_for_backward(inputs[1])
    ctx.handle = inputs[2]


def _backward(ctx, grad):
    (electrons,) = ctx.saved_tensors
    _, g, _ = _registry[ctx.handle].grad(electrons.contiguous(), weights=grad.detach().double())
    return g.to(torch.float32), None, None


torch.library.register_autograd("qmc_gb300::ferminet_logpsi", _backward, setup_context=_setup_context)
