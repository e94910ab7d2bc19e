"""The algorithmic work counts behind bench.py's rooflines (CPU): the
Psiformer forward and request FLOPs of the benzene configuration, and the
attention tangent count, against the hand counts of the layer shapes."""
import os
import sys

import pytest

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402
from jaqmc_gb300 import params as P  # noqa: E402
from jaqmc_gb300 import systems as S  # noqa: E402


def test_psiformer_benzene_counts():
    mol = S.benzene()
    cfg = P.PsiformerConfig(nspins=mol.nspins)
    n, A, D = mol.n_electrons, mol.n_atoms, 256
    # per electron row: input layer (4A+1) x D, per layer QKV 3 D^2 + out D^2 +
    # MLP D*256 + 256*D, orbitals D x K n; per walker: 2 n^2 D per layer of
    # attention (scores and mixing); 2 FLOP per multiply-add
    per_row = (4 * A + 1) * D + 4 * (3 * D * D + D * D + D * 256 + 256 * D) + D * 16 * n
    want = 2 * (n * per_row + 4 * 2 * n * n * D)
    got = bench.psiformer_forward_flops(cfg, n, A)
    assert got == want
    assert got == pytest.approx(154.9e6, rel=1e-3)
    pk = {"bf16_tflops_sustained": 1729.0}
    rl = bench.psiformer_request_roofline(cfg, n, A, 4096, 10, 1000.0, "mixed", pk, "measured")
    assert rl["algorithmic_tflop_per_request"] == pytest.approx(87.5, rel=1e-3)
    assert rl["achieved"] == pytest.approx(rl["algorithmic_tflop_per_request"], rel=1e-12)  # 1 s per request
    att = bench.psiformer_attention_fl_roofline(cfg, n, 4096, 1000.0)
    assert att["algorithmic_flop_per_request"] == 2 * 18 * n ** 3 * 64 * 4 * 4 * 4096
    assert bench.psiformer_attention_fl_roofline(cfg, n, 4096, 0.0) is None


def test_ferminet_counts():
    """Dense FLOPs per FermiNet forward at widths 4 x (256, 32), K = 16 (Li,
    CH4, N2), and the N2 request count (20 MH steps + 3n + 2 tangents)."""
    want = {"Li": 3.977472e6, "CH4": 14.38208e6, "N2": 20.579328e6}
    for name, v in want.items():
        mol = S.SYSTEMS[name]()
        cfg = P.FermiNetConfig(nspins=mol.nspins)
        assert bench.ferminet_forward_flops(cfg, mol.n_atoms) == pytest.approx(v, rel=1e-9)
    mol = S.nitrogen_dimer()
    cfg = P.FermiNetConfig(nspins=mol.nspins)
    # N2 by hand: layer 0 input 3*8 + 2*4, layers 1-3 input 3*256 + 2*32,
    # pair layers 4->32->32->32, orbitals 256 -> 16 x 14
    n = 14
    hand = 2 * (n * 32 * 256 + 3 * n * 832 * 256 + n * n * (4 * 32 + 32 * 32 + 32 * 32) + n * 256 * 16 * n)
    assert bench.ferminet_forward_flops(cfg, 2) == hand
    rl = bench.ferminet_request_roofline(cfg, 2, 4096, 20, 1000.0, "mixed", {"bf16_tflops_sustained": 1.0}, "x")
    assert rl["algorithmic_tflop_per_request"] == pytest.approx(hand * 64 * 4096 / 1e12, rel=1e-12)
