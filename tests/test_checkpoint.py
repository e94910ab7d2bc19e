"""Checkpoint interop with the reference's .npz layout (host logic, CPU).

A file laid out as the reference's NumPyCheckpointManager writes a sampling
stage state (src/jaqmc/utils/checkpoint.py:26-274: leaves under slash-joined
key paths, ``step``; parameters at ``params/params/<module path>``, walkers
at ``batched_data/data/electrons``, MCMC state at ``sampler_state/*``) loads
into the library's flat parameter layout, round-trips through
:func:`vmc.save_checkpoint`, and rejects shape mismatches.
"""
import numpy as np
import pytest
import torch

from jaqmc_gb300 import params as P
from jaqmc_gb300 import vmc


def _reference_style_npz(path, tree, leaves, electrons, step):
    arrays = {"step": np.asarray(step), "batched_data/data/electrons": electrons,
              "batched_data/data/atoms": np.zeros((2, 3), np.float32),
              "sampler_state/stddev": np.asarray(0.123, np.float32),
              "sampler_state/pmoves": np.linspace(0.4, 0.6, 100).astype(np.float32),
              "opt_state/0/count": np.asarray(7)}
    for p, _ in leaves:
        arrays["params/params/" + "/".join(p)] = P._get(tree, p)
    np.savez_compressed(path, allow_pickle=False, **arrays)


@pytest.mark.parametrize("kind", ["ferminet", "psiformer"])
def test_load_reference_layout_and_round_trip(tmp_path, kind):
    if kind == "ferminet":
        wf = vmc.FermiNetWavefunction(nspins=(2, 1), ndets=3, hidden_dims_single=[8, 8], hidden_dims_double=[4, 4])
        tree = P.init_ferminet(wf.config, 2, seed=4)
        leaves = P.ferminet_leaves(wf.config, 2)
    else:
        wf = vmc.PsiformerWavefunction(nspins=(2, 1), ndets=2, num_layers=1, num_heads=2, heads_dim=4,
                                       mlp_hidden_dims=[8])
        tree = P.init_psiformer(wf.config, 2, seed=4)
        leaves = P.psiformer_leaves(wf.config, 2)
    x = np.random.default_rng(0).normal(size=(5, 3, 3)).astype(np.float32)
    src = tmp_path / "ckpt_000041.npz"
    _reference_style_npz(src, tree, leaves, x, 41)
    r = vmc.load_reference_checkpoint(src, wf, 2, device=torch.device("cpu"))
    assert r["step"] == 42
    np.testing.assert_array_equal(r["params"].flat.numpy(), P.flatten(tree, leaves))
    np.testing.assert_array_equal(r["electrons"], x)
    assert r["sampler_state"].stddev == pytest.approx(0.123)
    assert r["sampler_state"].pmoves.shape == (100,)
    out = tmp_path / "mine.npz"
    vmc.save_checkpoint(out, 41, r["params"], {"electrons": torch.as_tensor(x)}, r["sampler_state"])
    r2 = vmc.load_reference_checkpoint(out, wf, 2, device=torch.device("cpu"))
    np.testing.assert_array_equal(r2["params"].flat.numpy(), r["params"].flat.numpy())
    np.testing.assert_array_equal(r2["electrons"], x)
    assert r2["step"] == 42


def test_shape_mismatch_is_an_error(tmp_path):
    wf = vmc.FermiNetWavefunction(nspins=(2, 1), ndets=3, hidden_dims_single=[8, 8], hidden_dims_double=[4, 4])
    other = vmc.FermiNetWavefunction(nspins=(2, 1), ndets=4, hidden_dims_single=[8, 8], hidden_dims_double=[4, 4])
    tree = P.init_ferminet(other.config, 2, seed=1)
    src = tmp_path / "c.npz"
    _reference_style_npz(src, tree, P.ferminet_leaves(other.config, 2), np.zeros((1, 3, 3), np.float32), 0)
    with pytest.raises(ValueError):
        vmc.load_reference_checkpoint(src, wf, 2, device=torch.device("cpu"))
