"""Robust stochastic reconfiguration (SR, SPRING, MARCH) over the library's
per-walker score matrix.

Restates the reference's optimizer ``robust_sr``
(``src/jaqmc/optimizer/sr/jasr.py:67-206``), built as ``scale_by_fisher_inverse``
(``:222-512``) -> ``scale_by_constrained_norm`` (``:707-751``) -> ``scale(-1)``,
with the Gram helpers ``calc_gram_matrix`` (``:514-568``), ``lift_null_space``
(``:641-665``), ``estimate_required_damping`` (``:667-705``) and
``normalize_masked`` (``:813-839``).  The kernel (B x B) form:

    O  = (score - mean) / sqrt(B)          score: d log|psi_w| / d theta, B x P
    F  = O diag(s) O^T (null space lifted) + lambda I
    u_g = O (s g),  u_p = O p,  w = F^-1 u_g
    z  = F^-1 (gamma u_g + u_p - (1 - gamma lambda) w)
    delta = gamma s g + p - s O^T z        p = mu delta_prev (SPRING), s = MARCH scale

then ``update = -delta * min(lr, C / |delta|)``.  The score comes from the GPU
adjoint (``LossAndGrad(per_walker=True)`` -> ``grad_logpsi``).  Everything
runs on the device in torch.  The Gram matrix (rows scaled by their max
magnitude as the reference does) is FP64 like the reference's mixed-precision
default while its 2 B^2 P FLOPs stay affordable at GB300's low FP64 rate
(``gram_precision="auto"``, limit ``f64_flop_limit``); beyond that it is FP32
products over 1024-column blocks (no TF32) summed in FP64.  The B x B
Cholesky solves and the matrix-vector products O v and O^T z are FP64 (for
gamma = 1 / lambda the update is a difference of two terms ~gamma times
larger than itself).
"""
from __future__ import annotations

from typing import Callable, NamedTuple

import torch


def _schedule(value, default=None) -> Callable[[int], float] | None:
    """Scalar or schedule -> ``step -> value`` (``ensure_schedule``, jasr.py:787-811)."""
    if callable(value):
        return value
    if value is None:
        return None if default is None else (lambda _: default)
    return lambda _: value


class RobustSRState(NamedTuple):
    count: int                 # preconditioner steps (FisherInverseState.counter)
    prev_delta: torch.Tensor   # (P,) previous preconditioned direction
    acc_var: torch.Tensor      # (P,) MARCH accumulator (ones when unused)
    norm_count: int            # constrained-norm schedule step


def normalize_masked(x: torch.Tensor, mask: torch.Tensor, mode: str = "mean") -> torch.Tensor:
    """``x / norm`` on the masked entries, norm = their sum or mean (1 if <= 0)."""
    s = torch.where(mask, x, torch.zeros_like(x)).sum()
    if mode == "sum":
        norm = s
    elif mode == "mean":
        cnt = mask.to(x.dtype).sum()
        norm = s / cnt if cnt > 0 else torch.ones((), dtype=x.dtype, device=x.device)
    else:
        raise ValueError(f"normalisation mode must be 'sum' or 'mean' (got {mode!r})")
    norm = norm if norm > 0 else torch.ones((), dtype=x.dtype, device=x.device)
    return torch.where(mask, x / norm, x)


def gram_matrix(score: torch.Tensor, scale, block: int = 1024, precision: str = "f64") -> torch.Tensor:
    """FP64 ``(O diag(s) O^T)`` of an already centred score matrix (used by
    the tests and callers holding O): see :func:`_centred_gram`."""
    B, P = score.shape
    zero = torch.zeros(P, dtype=torch.float64, device=score.device)
    sc = scale if torch.is_tensor(scale) else torch.full((P,), float(scale), dtype=torch.float64,
                                                         device=score.device)
    return _centred_gram(score, zero, torch.ones(B, dtype=torch.float64, device=score.device), 1.0, sc,
                         block, precision)


def _blocks(P: int, block: int):
    return [(c0, min(P, c0 + block)) for c0 in range(0, P, block)]


def _centred_block(S, mean, rescale, inv_sqrt_b, c0, c1) -> torch.Tensor:
    """FP64 column block ``(rescale * S - mean) / sqrt(B)`` of the centred
    score (centring in FP64, so columns with a large mean keep their spread)."""
    return (S[:, c0:c1].double() * rescale[:, None] - mean[c0:c1]) * inv_sqrt_b


def _centred_gram(S, mean, rescale, inv_sqrt_b, scale, block: int, precision: str) -> torch.Tensor:
    """FP64 ``O diag(scale) O^T`` for O = centred score: rows normalised by
    their max |entry| (clipped at 1e-4; the reference's calc_gram_matrix),
    products in FP64 (``"f64"``) or in FP32 over ``block``-column pieces summed
    in FP64 (``"f32"``), row scales put back, symmetrised."""
    B, P = S.shape
    big = _blocks(P, 16384)
    rf = torch.zeros(B, dtype=torch.float64, device=S.device)
    for c0, c1 in big:
        ob = _centred_block(S, mean, rescale, inv_sqrt_b, c0, c1) * torch.sqrt(scale[c0:c1])
        rf = torch.maximum(rf, ob.abs().amax(dim=1))
    rf = rf.clamp(min=1e-4)
    gram = torch.zeros((B, B), dtype=torch.float64, device=S.device)
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    try:
        for c0, c1 in big:
            ob = _centred_block(S, mean, rescale, inv_sqrt_b, c0, c1) * torch.sqrt(scale[c0:c1]) / rf[:, None]
            if precision == "f64":
                gram += ob @ ob.T
            else:
                obf = ob.float()
                for d0 in range(0, c1 - c0, block):
                    piece = obf[:, d0:d0 + block]
                    gram += (piece @ piece.T).double()
    finally:
        torch.backends.cuda.matmul.allow_tf32 = prev
    gram = gram * (rf[:, None] * rf[None, :])
    return (gram + gram.T) / 2


def lift_null_space(gram: torch.Tensor) -> torch.Tensor:
    """Project the Gram matrix onto the complement of the constant walker
    vector u = 1/sqrt(B) (centre every row and column: P G P with
    P = I - u u^T), then give that direction unit weight again with u u^T.

    Centred scores make the solution blind to u, so lifting it keeps the
    matrix invertible without changing the update (real scores, one device)."""
    B = gram.shape[0]
    row = gram.mean(dim=1, keepdim=True)
    col = gram.mean(dim=0, keepdim=True)
    centred = gram - row - col + row.mean()
    return centred + 1.0 / B


def estimate_required_damping(gram: torch.Tensor, target_cond_num: float, num_iters: int = 10) -> torch.Tensor:
    """Smallest damping lam >= 0 with (eig_max + lam) / lam <= target_cond_num,
    taking the smallest eigenvalue of the (positive semi-definite) Gram
    matrix as 0.  eig_max is the Rayleigh quotient after ``num_iters``
    multiplications, started from the square roots of the diagonal scaled by
    1 + 0.5 frac(i phi) (phi the golden ratio): the diagonal weights the
    walkers with large scores, and the deterministic scatter keeps a
    component along every eigenvector, which a centred Gram matrix's own
    rows or diagonal can lack."""
    if not target_cond_num > 1.0:
        raise ValueError(f"the target condition number has to exceed 1 (got {target_cond_num})")
    B = gram.shape[0]
    idx = torch.arange(B, dtype=gram.dtype, device=gram.device)
    scatter = 1.0 + 0.5 * torch.frac(idx * 0.6180339887498949)
    v = torch.sqrt(torch.clamp(torch.diagonal(gram), min=0.0)) * scatter + 1e-30
    v = v / torch.linalg.norm(v)
    for _ in range(num_iters):
        w = gram @ v
        nrm = torch.linalg.norm(w)
        if not float(nrm) > 0.0:
            break
        v = w / nrm
    return torch.clamp(torch.dot(v, gram @ v) / (target_cond_num - 1.0), min=0.0)


class RobustSR:
    """The reference's ``robust_sr`` with the same arguments and defaults
    (``robust_gamma=None`` is standard SR, gamma = 1 / damping)."""

    def __init__(self, learning_rate=1e-2, max_norm=None, damping=1e-3, max_cond_num=None, robust_gamma=None,
                 spring_mu=None, march_beta=None, march_mode: str = "diff", eps: float = 1e-8,
                 score_norm_clip=None, gram_precision: str = "auto", gram_block: int = 1024,
                 f64_flop_limit: float = 2e11):
        if isinstance(robust_gamma, str) and robust_gamma != "sqrt":
            raise ValueError(f"unsupported robust_gamma {robust_gamma!r}: give None, a number, a schedule or 'sqrt'")
        if isinstance(max_norm, str) and max_norm != "fixed":
            raise ValueError(f"unsupported max_norm {max_norm!r}: give None, a number, a schedule or 'fixed'")
        if march_mode not in ("diff", "var"):
            raise ValueError("march_mode must be 'diff' or 'var'")
        self.robust_gamma = robust_gamma
        self.get_damping = _schedule(damping, 0.0)
        self.get_mu = _schedule(spring_mu, 0.0)
        self.get_beta = _schedule(march_beta, 0.0)
        self.spring = spring_mu is not None
        self.march = march_beta is not None
        self.march_mode = march_mode
        self.max_cond_num = max_cond_num
        self.eps = eps
        self.score_norm_clip = score_norm_clip
        if gram_precision not in ("auto", "f64", "f32"):
            raise ValueError("gram_precision must be 'auto', 'f64' or 'f32'")
        self.gram_precision = gram_precision
        self.gram_block = gram_block
        self.f64_flop_limit = f64_flop_limit  # 'auto': FP64 Gram up to this many FLOPs
        if isinstance(max_norm, str):  # 'fixed': the update norm is the learning rate
            self.get_lr, self.get_norm = _schedule(1e8), _schedule(learning_rate)
        else:
            self.get_lr, self.get_norm = _schedule(learning_rate), _schedule(max_norm)

    def init(self, n_params: int, device=None) -> RobustSRState:
        z = torch.zeros(n_params, dtype=torch.float64, device=device)
        return RobustSRState(0, z, torch.ones_like(z), 0)

    def _gamma(self, step: int, lam: float) -> float:
        g = self.robust_gamma
        if callable(g):
            gamma = float(g(step))
        elif g is None:
            gamma = 1.0 / max(lam, self.eps)
        elif g == "sqrt":
            gamma = max(lam, self.eps) ** -0.5
        else:
            gamma = float(g)
        b1, b2 = 1.0, 1.0 / max(lam, self.eps)
        return min(max(gamma, min(b1, b2)), max(b1, b2))

    def precondition(self, grads: torch.Tensor, state: RobustSRState, score: torch.Tensor):
        """``scale_by_fisher_inverse``: ``(delta, state)`` for the flat
        gradient ``grads`` (P,) and the raw score matrix ``score`` (B, P)."""
        count, prev_delta, acc_var, norm_count = state
        g = grads.to(torch.float64)
        S = score.to(torch.float32)
        B, P = S.shape
        dev = S.device
        big = _blocks(P, 16384)
        if self.score_norm_clip is not None:
            rescale = torch.clamp(self.score_norm_clip / S.abs().mean(dim=1).double(), min=0.0, max=1.0)
        else:
            rescale = torch.ones(B, dtype=torch.float64, device=dev)
        mean = torch.cat([(S[:, c0:c1].double() * rescale[:, None]).mean(dim=0) for c0, c1 in big])
        isb = B ** -0.5
        blk = lambda c0, c1: _centred_block(S, mean, rescale, isb, c0, c1)  # noqa: E731
        p = self.get_mu(count) * prev_delta if self.spring else torch.zeros_like(g)
        beta = self.get_beta(count)
        if self.march and self.march_mode == "var":
            sv = torch.cat([(blk(c0, c1) ** 2).sum(dim=0) for c0, c1 in big])
            mask = sv > self.eps
            sv = normalize_masked(sv, mask, "mean")
            acc_var = torch.where(mask, beta * acc_var + (1.0 - beta) * sv, acc_var)
        scale = torch.rsqrt(acc_var + self.eps) if self.march else torch.ones_like(g)
        sg = scale * g
        u_g = torch.zeros(B, dtype=torch.float64, device=dev)
        u_p = torch.zeros(B, dtype=torch.float64, device=dev)
        for c0, c1 in big:
            ob = blk(c0, c1)
            u_g += ob @ sg[c0:c1]
            if self.spring:
                u_p += ob @ p[c0:c1]
        prec = self.gram_precision
        if prec == "auto":
            prec = "f64" if 2.0 * B * B * P <= self.f64_flop_limit else "f32"
        gram = _centred_gram(S, mean, rescale, isb, scale, self.gram_block, prec)
        gram = lift_null_space(gram)
        lam = float(self.get_damping(count))
        if self.max_cond_num is not None:
            lam = max(lam, float(estimate_required_damping(gram, self.max_cond_num)))
        gamma = self._gamma(count, lam)
        F = gram + lam * torch.eye(B, dtype=gram.dtype, device=dev)
        L = torch.linalg.cholesky(F)
        w = torch.cholesky_solve(u_g[:, None], L)[:, 0]
        z = torch.cholesky_solve((gamma * u_g + u_p - (1.0 - gamma * lam) * w)[:, None], L)[:, 0]
        otz = torch.cat([blk(c0, c1).T @ z for c0, c1 in big])
        delta = gamma * sg + p - scale * otz
        if self.march and self.march_mode == "diff":
            acc_var = beta * acc_var + (1.0 - beta) * (delta - prev_delta) ** 2
        return delta, RobustSRState(count + 1, delta, acc_var, norm_count)

    def update(self, grads: torch.Tensor, state: RobustSRState, score: torch.Tensor):
        """Full ``robust_sr`` step: ``(updates, state)`` with
        ``updates = -delta * min(lr, C / (|delta| + eps))`` (add to the flat
        parameters)."""
        delta, state = self.precondition(grads, state, score)
        lr = self.get_lr(state.norm_count) if self.get_lr is not None else 1.0
        if self.get_norm is None:
            eff = lr
        else:
            eff = min(lr, self.get_norm(state.norm_count) / (float(torch.linalg.norm(delta)) + self.eps))
        return -eff * delta, state._replace(norm_count=state.norm_count + 1)
