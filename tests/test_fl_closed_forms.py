"""The closed-form tangent rules that the Psiformer forward-Laplacian kernels
(jaqmc_gb300/csrc/psiformer_fl.cu) evaluate, restated in FP64 exactly as the
kernels compute them, against the oracle's composed rules (oracle/lap.py,
oracle/psiformer.py), itself pinned against autograd.  CPU only: this pins the
algebra of each kernel on its own; the GPU tests pin the kernels end to end."""
import os
import sys

import torch

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
from jaqmc_gb300 import systems as S  # noqa: E402
from oracle import lap  # noqa: E402
from oracle import psiformer as OP  # noqa: E402

F64 = torch.float64


def _random_lt(gen, B, Z, *shape, scale=1.0):
    x = scale * torch.randn(B, *shape, generator=gen, dtype=F64)
    J = torch.randn(B, Z, *shape, generator=gen, dtype=F64)
    L = torch.randn(B, *shape, generator=gen, dtype=F64)
    return lap.LT(x, J, L)


def test_layer_norm_closed_form():
    """k_psi_group_fl: LayerNorm of one electron's rows with the centred
    variance, J r = -r^3 mean(u J v), and the column sums C = sum_d J v J r -
    sum_d J mu J r."""
    g = torch.Generator().manual_seed(0)
    B, Z, D = 3, 11, 40
    a = _random_lt(g, B, Z, D, scale=2.0)
    a.x = a.x + 0.7  # a nonzero mean
    s = torch.randn(D, generator=g, dtype=F64)
    b = torch.randn(D, generator=g, dtype=F64)
    ref = OP.layer_norm_lt(a, s, b)
    eps = 1e-5
    mu = a.x.mean(-1, keepdim=True)
    u = a.x - mu
    var = (u * u).mean(-1, keepdim=True)
    r = (var + eps) ** -0.5
    dmu = a.J.mean(-1, keepdim=True)                           # (B, Z, 1)
    dv = 2.0 * (u[:, None] * a.J).mean(-1, keepdim=True)       # (B, Z, 1)
    dr = -0.5 * r[:, None] ** 3 * dv
    Lmu = a.L.mean(-1, keepdim=True)
    Q = (a.J * a.J).sum((1, 2))[:, None]
    Lv = 2.0 * (u * a.L).mean(-1, keepdim=True) + 2.0 * (Q / D - (dmu * dmu).sum(1))
    Lr = -0.5 * r ** 3 * Lv + 0.75 * r ** 5 * (dv * dv).sum(1)
    C = (a.J * dr).sum(1) - (dmu * dr).sum(1)
    y0 = s * u * r + b
    yJ = s * ((a.J - dmu) * r[:, None] + u[:, None] * dr)
    yL = s * ((a.L - Lmu) * r + u * Lr + 2.0 * C)
    assert torch.allclose(y0, ref.x, atol=1e-12)
    assert torch.allclose(yJ, ref.J, atol=1e-11)
    assert torch.allclose(yL, ref.L, atol=1e-10)


def test_tanh_closed_form():
    """k_psi_group_fl with act: h = tanh(z + b), J h = h' J z,
    L h = h' L z + h'' sum_d (J_d z)^2."""
    g = torch.Generator().manual_seed(1)
    z = _random_lt(g, 2, 7, 16)
    b = torch.randn(16, generator=g, dtype=F64)
    ref = lap.tanh(z + b)
    h = torch.tanh(z.x + b)
    h1 = 1 - h * h
    assert torch.allclose(h1[:, None] * z.J, ref.J, atol=1e-13)
    assert torch.allclose(h1 * z.L - 2 * h * h1 * (z.J * z.J).sum(1), ref.L, atol=1e-12)


def test_attention_closed_form():
    """k_psi_attention_fl: J S, b = J S - sum_k a J S, J a = a b,
    L a = a (sum_d b^2 - sum_k a sum_d b^2 + L S - sum_k a L S),
    J o = J a v0 + a J v, L o = L a v0 + a L v + 2 sum_d J a J v, with the
    queries already scaled."""
    g = torch.Generator().manual_seed(2)
    B, Z, n, Dh = 2, 9, 6, 8
    q = _random_lt(g, B, Z, n, Dh, scale=0.5)
    k = _random_lt(g, B, Z, n, Dh, scale=0.5)
    v = _random_lt(g, B, Z, n, Dh)
    S_ = OP._bilinear(q, k, "bqd,bkd->bqk")
    e = lap.exp(S_ - S_.x.max(-1, keepdim=True).values)
    w = e * lap.reciprocal(e.sum(-1)).unsqueeze(-1)
    ref = OP._bilinear(w, v, "bqk,bkd->bqd")
    a = torch.softmax(q.x @ k.x.transpose(-1, -2), -1)                                  # (B, n, n)
    dS = torch.einsum("bzqd,bkd->bzqk", q.J, k.x) + torch.einsum("bqd,bzkd->bzqk", q.x, k.J)
    XS = torch.einsum("bzqd,bzkd->bqk", q.J, k.J)
    bb = dS - (a[:, None] * dS).sum(-1, keepdim=True)
    da = a[:, None] * bb
    Bq = (bb * bb).sum(1)
    LS = q.L @ k.x.transpose(-1, -2) + q.x @ k.L.transpose(-1, -2) + 2 * XS
    La = a * (Bq - (a * Bq).sum(-1, keepdim=True) + LS - (a * LS).sum(-1, keepdim=True))
    oJ = torch.einsum("bzqk,bkd->bzqd", da, v.x) + torch.einsum("bqk,bzkd->bzqd", a, v.J)
    oL = La @ v.x + a @ v.L + 2 * torch.einsum("bzqk,bzkd->bqd", da, v.J)
    assert torch.allclose(a @ v.x, ref.x, atol=1e-12)
    assert torch.allclose(oJ, ref.J, atol=1e-11)
    assert torch.allclose(oL, ref.L, atol=1e-10)


def test_feature_and_jastrow_closed_forms():
    """k_psi_features_fl: the rescaled features' Jacobian (own electron only)
    and Laplacian, and the SimpleEE Jastrow's gradient and Laplacian."""
    mol = S.methane()
    x = torch.as_tensor(S.init_walkers(mol, 3, seed=4), dtype=torch.float64)
    atoms = torch.as_tensor(mol.atoms, dtype=torch.float64)
    xl = lap.seed(x)
    ae, _ = OP.features_lt(xl, atoms, mol.nspins)
    B, n, A = x.shape[0], x.shape[1], atoms.shape[0]
    d = x[:, :, None, :] - atoms                                    # (B, n, A, 3)
    r = d.norm(dim=-1)
    l = torch.log1p(r)
    ip, ir = 1 / (1 + r), 1 / r
    gg = l * ir
    a0 = ip * ir
    b0 = (ip - gg) * ir * ir
    lapl = -ip * ip + 2 * ip * ir
    lapv = (-ip * ip + 2 * ip * ir - 2 * gg * ir) * ir
    Lf = torch.cat([lapl[..., None], d * lapv[..., None]], -1).reshape(B, n, 4 * A)
    assert torch.allclose(Lf, ae.L[..., :4 * A], atol=1e-10)
    assert ae.J[..., 4 * A:].abs().max() == 0                         # the spin column is constant
    J = ae.J[..., :4 * A].reshape(B, n, 3, n, A, 4)                  # direction (e, c) -> feature (i, I, q)
    for e_ in range(n):
        for c in range(3):
            got = J[:, e_, c, e_]                                   # own electron
            want = torch.cat([(d[:, e_, :, c] * a0[:, e_])[..., None],
                              torch.eye(3, dtype=F64)[c] * gg[:, e_, :, None]
                              + d[:, e_] * (d[:, e_, :, c] * b0[:, e_])[..., None]], -1)
            assert torch.allclose(got, want, atol=1e-11)
            others = torch.cat([J[:, e_, c, :e_], J[:, e_, c, e_ + 1:]], 1)
            assert others.abs().max() == 0
    cfg = OP.PsiformerConfig(nspins=mol.nspins)
    tree = {"alpha_par": torch.tensor([0.8], dtype=F64), "alpha_anti": torch.tensor([1.3], dtype=F64)}
    jl = OP.jastrow_lt(tree, cfg, xl, torch.float64)
    nu = mol.nspins[0]
    grad = torch.zeros(B, n, 3, dtype=F64)
    Lj = torch.zeros(B, dtype=F64)
    for i in range(n):
        for j in range(n):
            if i == j:
                continue
            same = (i < nu) == (j < nu)
            al, cf = (0.8, 0.25) if same else (1.3, 0.5)
            dij = x[:, i] - x[:, j]
            rij = dij.norm(dim=-1)
            ia = 1 / (al + rij)
            grad[:, i] += (cf * al * al * ia * ia / rij)[:, None] * dij
            if j > i:
                Lj += 2 * (-2 * cf * al * al * ia ** 3 + 2 * cf * al * al * ia * ia / rij)
    assert torch.allclose(grad.reshape(B, -1), jl.J, atol=1e-12)
    assert torch.allclose(Lj, jl.L, atol=1e-11)
