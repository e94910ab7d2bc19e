"""The allocation-free forward entry point (qmc_forward_noalloc).

Callers that may not allocate device memory while they run use this variant;
its scratch is a fixed 64 MiB device array inside the library.  Both model
families (FermiNet and Psiformer) go through it.  Checked here
through the C ABI against qmc_forward (the entry point with a caller
workspace): two calls in a row must both agree, and an oversized batch must be
refused up front.  This file is collected last on purpose.
"""
import numpy as np
import pytest
import torch

from helpers import full_cfg, setup
from jaqmc_gb300 import _native
from jaqmc_gb300 import systems as S

pytestmark = pytest.mark.gpu


def _reference_forward(m, x):
    lp, sg, fl = m.forward(x)
    return lp.cpu().numpy(), sg.cpu().numpy(), fl.cpu().numpy()


@pytest.mark.parametrize("precision", ["fp32", "mixed"])
def test_noalloc_forward_matches_workspace_forward(precision, cuda_device):
    mol = S.nitrogen_dimer()
    cfg = full_cfg((7, 7))
    _, flat, _ = setup(mol, cfg, 1)
    m = _native.NativeFermiNet(cfg, mol.atoms, mol.charges, precision=precision, device=cuda_device)
    m.set_params(torch.as_tensor(flat, device=cuda_device))
    lib = _native.load()
    stream = _native.stream_handle()
    for seed, B in ((1, 256), (2, 300)):  # two calls in a row, different batches
        x = torch.as_tensor(S.init_walkers(mol, B, seed=seed), device=cuda_device)
        want_lp, want_sg, want_fl = _reference_forward(m, x)
        lp = torch.full((B,), float("nan"), device=cuda_device)
        sg = torch.zeros(B, device=cuda_device)
        fl = torch.full((B,), 255, dtype=torch.uint8, device=cuda_device)
        _native.check(lib.qmc_forward_noalloc(m.h, B, x.data_ptr(), lp.data_ptr(), sg.data_ptr(),
                                              fl.data_ptr(), stream))
        torch.cuda.synchronize()
        np.testing.assert_allclose(lp.cpu().numpy(), want_lp, rtol=1e-6, atol=1e-6)
        assert np.array_equal(sg.cpu().numpy(), want_sg)
        assert np.array_equal(fl.cpu().numpy(), want_fl)


def _noalloc(m, x, with_outputs=True):
    lib = _native.load()
    B = x.shape[0]
    lp = torch.full((B,), float("nan"), device=x.device)
    sg = torch.zeros(B, device=x.device) if with_outputs else None
    fl = torch.full((B,), 255, dtype=torch.uint8, device=x.device) if with_outputs else None
    _native.check(lib.qmc_forward_noalloc(m.h, B, x.data_ptr(), lp.data_ptr(), _native.ptr(sg), _native.ptr(fl),
                                          _native.stream_handle()))
    torch.cuda.synchronize()
    return lp, sg, fl


def test_noalloc_largest_batch_and_optional_outputs(cuda_device):
    """The largest batch whose workspace fits the 64 MiB array is accepted and
    matches qmc_forward; sign and flags may be NULL on an accepted call."""
    mol = S.nitrogen_dimer()
    cfg = full_cfg((7, 7))
    _, flat, _ = setup(mol, cfg, 1)
    m = _native.NativeFermiNet(cfg, mol.atoms, mol.charges, device=cuda_device)
    m.set_params(torch.as_tensor(flat, device=cuda_device))
    lo, hi = 1, 8192
    while lo < hi:  # largest B with workspace <= 64 MiB
        mid = (lo + hi + 1) // 2
        if m.lib.qmc_workspace_size(m.h, _native.OP_FORWARD, mid) <= 64 << 20:
            lo = mid
        else:
            hi = mid - 1
    B = lo
    assert m.lib.qmc_workspace_size(m.h, _native.OP_FORWARD, B + 1) > 64 << 20
    x = torch.as_tensor(S.init_walkers(mol, B, seed=4), device=cuda_device)
    want_lp, want_sg, want_fl = _reference_forward(m, x)
    lp, sg, fl = _noalloc(m, x)
    np.testing.assert_allclose(lp.cpu().numpy(), want_lp, rtol=1e-6, atol=1e-6)
    assert np.array_equal(sg.cpu().numpy(), want_sg) and np.array_equal(fl.cpu().numpy(), want_fl)
    lp2, _, _ = _noalloc(m, x[:B // 2].contiguous(), with_outputs=False)
    np.testing.assert_allclose(lp2.cpu().numpy(), want_lp[:B // 2], rtol=1e-6, atol=1e-6)


@pytest.mark.parametrize("precision", ["fp32", "mixed"])
def test_noalloc_psiformer_matches_workspace_forward(precision, cuda_device):
    """Psiformer models (lithium, small widths) through the same entry point."""
    from jaqmc_gb300 import params as P
    mol = S.lithium()
    cfg = P.PsiformerConfig(nspins=mol.nspins, ndets=3, num_layers=2, num_heads=4, heads_dim=16,
                            mlp_hidden_dims=[64])
    tree = P.init_psiformer(cfg, mol.n_atoms, seed=0)
    flat = P.flatten(tree, P.psiformer_leaves(cfg, mol.n_atoms))
    m = _native.NativePsiformer(cfg, mol.atoms, mol.charges, precision=precision, device=cuda_device)
    m.set_params(torch.as_tensor(flat, device=cuda_device))
    for seed, B in ((1, 64), (2, 96)):
        x = torch.as_tensor(S.init_walkers(mol, B, seed=seed), device=cuda_device)
        want_lp, want_sg, want_fl = _reference_forward(m, x)
        lp, sg, fl = _noalloc(m, x)
        np.testing.assert_allclose(lp.cpu().numpy(), want_lp, rtol=1e-6, atol=1e-6)
        assert np.array_equal(sg.cpu().numpy(), want_sg) and np.array_equal(fl.cpu().numpy(), want_fl)


def test_noalloc_argument_errors_before_size(cuda_device):
    """A model without parameters is refused for that reason, not for size."""
    mol = S.nitrogen_dimer()
    cfg = full_cfg((7, 7))
    m = _native.NativeFermiNet(cfg, mol.atoms, mol.charges, device=cuda_device)
    B = 4096
    x = torch.zeros((B, mol.n_electrons, 3), device=cuda_device)
    lp = torch.empty(B, device=cuda_device)
    lib = _native.load()
    st = lib.qmc_forward_noalloc(m.h, B, x.data_ptr(), lp.data_ptr(), None, None, _native.stream_handle())
    assert st == 1 and b"parameters not set" in lib.qmc_last_error()


def test_noalloc_rejects_batches_beyond_the_array(cuda_device):
    mol = S.nitrogen_dimer()
    cfg = full_cfg((7, 7))
    _, flat, _ = setup(mol, cfg, 1)
    m = _native.NativeFermiNet(cfg, mol.atoms, mol.charges, device=cuda_device)
    m.set_params(torch.as_tensor(flat, device=cuda_device))
    B = 4096
    assert m.lib.qmc_workspace_size(m.h, _native.OP_FORWARD, B) > 64 << 20
    x = torch.as_tensor(S.init_walkers(mol, B, seed=1), device=cuda_device)
    lp = torch.empty(B, device=cuda_device)
    lib = _native.load()
    st = lib.qmc_forward_noalloc(m.h, B, x.data_ptr(), lp.data_ptr(), None, None, _native.stream_handle())
    assert st == 6
    assert b"built-in array" in lib.qmc_last_error()
