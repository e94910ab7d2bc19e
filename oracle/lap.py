"""Forward-Laplacian tangent algebra (oracle; test infrastructure only).

A :class:`LT` carries, for a batch of walkers,

* ``x``  — the value, shape ``(B, *s)``;
* ``J``  — the Jacobian w.r.t. the ``D`` flattened electron coordinates,
           shape ``(B, D, *s)``;
* ``L``  — the Laplacian (sum over the ``D`` coordinates of the second
           derivative), shape ``(B, *s)``.

The propagation rules restate the dense rules of the reference's vendored
forward-Laplacian interpreter:

* linear maps (dot_general, add, concat, mean, reshape, transpose) act on
  ``x``, ``J`` and ``L`` alike — ``src/jaqmc/laplacian/primitives/dot_general.py:713``,
  ``src/jaqmc/laplacian/primitives/reductions.py:25``;
* unary elementwise ``f``: ``J' = f'(x) J``, ``L' = f'(x) L + f''(x) sum_d J_d^2``
  — ``src/jaqmc/laplacian/primitives/elementwise.py:42-72``;
* products: ``L(ab) = L(a) b + 2 sum_d J_d(a) J_d(b) + a L(b)``
  — ``src/jaqmc/laplacian/primitives/arithmetic.py:385``;
* ``slogdet``: ``J = tr(A^-1 J_A)``, ``L = tr(A^-1 L_A) - sum_d tr(A^-1 J_d A^-1 J_d)``
  — ``src/jaqmc/laplacian/primitives/slogdet.py:25-72``.

With ``D == 0`` the same code is a plain forward pass (the tangent tensors are
empty), which lets the model code in this package serve both purposes.

:func:`split_bf16_gemms` makes ``linear`` round its operands the way the
library's split-BF16 tensor-core GEMMs do, so that the oracle can state what
that precision form should give (its operand rounding, nothing else).
"""
from __future__ import annotations

from contextlib import contextmanager

import torch


class LT:
    __slots__ = ("x", "J", "L")

    def __init__(self, x: torch.Tensor, J: torch.Tensor, L: torch.Tensor):
        self.x, self.J, self.L = x, J, L

    # ---- shape helpers -------------------------------------------------
    @property
    def D(self) -> int:
        return self.J.shape[1]

    @property
    def shape(self):
        return self.x.shape

    def _jax(self, axis: int) -> int:
        """Translate a value axis (>= 1, or negative) to the Jacobian axis."""
        if axis < 0:
            return axis
        if axis == 0:
            raise ValueError("axis 0 is the walker axis")
        return axis + 1

    # ---- linear structural ops ----------------------------------------
    def __getitem__(self, idx):
        """Index the non-walker axes: ``lt[idx]`` applies ``x[:, idx]``."""
        if not isinstance(idx, tuple):
            idx = (idx,)
        return LT(self.x[(slice(None),) + idx],
                  self.J[(slice(None), slice(None)) + idx],
                  self.L[(slice(None),) + idx])

    def reshape(self, *shape):
        B, D = self.x.shape[0], self.J.shape[1]
        return LT(self.x.reshape(B, *shape), self.J.reshape(B, D, *shape),
                  self.L.reshape(B, *shape))

    def permute(self, *dims):
        """Permute non-walker axes; ``dims`` index them from 1."""
        return LT(self.x.permute(0, *dims), self.J.permute(0, 1, *[d + 1 for d in dims]),
                  self.L.permute(0, *dims))

    def unsqueeze(self, axis: int):
        return LT(self.x.unsqueeze(axis), self.J.unsqueeze(self._jax(axis)),
                  self.L.unsqueeze(axis))

    def expand_as_value(self, shape):
        """Broadcast non-walker axes to ``shape`` (which excludes the walker axis)."""
        B, D = self.x.shape[0], self.J.shape[1]
        return LT(self.x.expand(B, *shape), self.J.expand(B, D, *shape),
                  self.L.expand(B, *shape))

    def sum(self, axis: int):
        return LT(self.x.sum(axis), self.J.sum(self._jax(axis)), self.L.sum(axis))

    def mean(self, axis: int):
        return LT(self.x.mean(axis), self.J.mean(self._jax(axis)), self.L.mean(axis))

    # ---- arithmetic ----------------------------------------------------
    def __add__(self, o):
        if isinstance(o, LT):
            return LT(self.x + o.x, self.J + o.J, self.L + o.L)
        return self._expand_to(self.x + o)

    __radd__ = __add__

    def __sub__(self, o):
        if isinstance(o, LT):
            return LT(self.x - o.x, self.J - o.J, self.L - o.L)
        return self._expand_to(self.x - o)

    def __neg__(self):
        return LT(-self.x, -self.J, -self.L)

    def _expand_to(self, x: torch.Tensor) -> "LT":
        """Broadcast ``J`` and ``L`` to the (possibly larger) value ``x``."""
        B, D = x.shape[0], self.J.shape[1]
        return LT(x, self.J.expand(B, D, *x.shape[1:]), self.L.expand(*x.shape))

    def scale(self, c):
        """Multiply by a tangent-free factor ``c``.

        ``c`` is a scalar, a tensor shaped like the value (walker axis
        included), or a tensor that broadcasts against the non-walker axes.
        """
        if torch.is_tensor(c) and c.dim() > 0:
            x = self.x * c
            cj = c.unsqueeze(1) if c.dim() == self.x.dim() else c
            B, D = x.shape[0], self.J.shape[1]
            return LT(x, (self.J * cj).expand(B, D, *x.shape[1:]), (self.L * c).expand(*x.shape))
        return LT(self.x * c, self.J * c, self.L * c)

    def __mul__(self, o):
        if not isinstance(o, LT):
            return self.scale(o)
        x = self.x * o.x
        ax, bx = self.x.unsqueeze(1), o.x.unsqueeze(1)
        J = self.J * bx + ax * o.J
        L = self.L * o.x + o.L * self.x + 2.0 * (self.J * o.J).sum(1)
        return LT(x, J, L)

    __rmul__ = __mul__


def const(x: torch.Tensor, D: int) -> LT:
    """A tangent-free quantity (zero Jacobian and Laplacian)."""
    B = x.shape[0]
    return LT(x, x.new_zeros((B, D) + tuple(x.shape[1:])), torch.zeros_like(x))


def seed(electrons: torch.Tensor, with_tangents: bool = True) -> LT:
    """Seed the flattened electron coordinates: ``J = I_{3n}``, ``L = 0``.

    Restates ``make_laplacian_input`` (``src/jaqmc/laplacian/seed.py:75-121``)
    in its dense form.
    """
    B, n, d = electrons.shape
    D = n * d if with_tangents else 0
    J = electrons.new_zeros((B, D, n, d))
    if with_tangents:
        eye = torch.eye(D, dtype=electrons.dtype).reshape(D, n, d)
        J = J + eye.unsqueeze(0)
    return LT(electrons, J, torch.zeros_like(electrons))


def concat(parts, axis: int) -> LT:
    ja = axis if axis < 0 else axis + 1
    return LT(torch.cat([p.x for p in parts], axis), torch.cat([p.J for p in parts], ja),
              torch.cat([p.L for p in parts], axis))


def stack(parts, axis: int) -> LT:
    ja = axis if axis < 0 else axis + 1
    return LT(torch.stack([p.x for p in parts], axis), torch.stack([p.J for p in parts], ja),
              torch.stack([p.L for p in parts], axis))


_SPLIT_SELECT = None  # predicate on W: emulate the split-BF16 product for this GEMM
_SPLIT_ATTENTION = False  # emulate the split-BF16 attention products too


def split_attention() -> bool:
    return _SPLIT_ATTENTION


def _split_bf16(a: torch.Tensor):
    """FP32 value of ``a`` as hi + lo bf16 (both round-to-nearest-even)."""
    a = a.to(torch.float32).to(torch.float64)
    hi = a.to(torch.bfloat16).to(torch.float64)
    lo = (a - hi).to(torch.bfloat16).to(torch.float64)
    return hi, lo


def _split_matmul(a: torch.Tensor, W: torch.Tensor) -> torch.Tensor:
    ah, al = _split_bf16(a)
    wh, wl = _split_bf16(W)
    return (ah @ wh + ah @ wl + al @ wh).to(a.dtype)


@contextmanager
def split_bf16_gemms(select=lambda W: True, attention: bool = False):
    """Within the block, ``linear`` with a weight ``W`` for which
    ``select(W)`` holds rounds both operands to FP32, splits each into a high
    and a low bf16 part and forms ``hi_a hi_W + hi_a lo_W + lo_a hi_W`` (the
    low x low product dropped) in the oracle's dtype: the product of the
    library's split-BF16 tensor-core GEMMs up to their FP32 accumulation.
    The value, Jacobian and Laplacian rows are rounded alike, as they are on
    the GPU.  With ``attention`` the forward-Laplacian attention products of
    the Psiformer / LapNet oracles are split the same way (all but the value
    scores, which the library forms in FP32)."""
    global _SPLIT_SELECT, _SPLIT_ATTENTION
    prev, prev_att = _SPLIT_SELECT, _SPLIT_ATTENTION
    _SPLIT_SELECT = select
    _SPLIT_ATTENTION = bool(attention)
    try:
        yield
    finally:
        _SPLIT_SELECT, _SPLIT_ATTENTION = prev, prev_att


def linear(a: LT, W: torch.Tensor, b: torch.Tensor | None = None) -> LT:
    """``a @ W + b`` over the last axis (dot_general rule)."""
    if _SPLIT_SELECT is not None and _SPLIT_SELECT(W):
        x = _split_matmul(a.x, W)
        if b is not None:
            x = x + b
        return LT(x, _split_matmul(a.J, W), _split_matmul(a.L, W))
    x = a.x @ W
    if b is not None:
        x = x + b
    return LT(x, a.J @ W, a.L @ W)


def unary(a: LT, y: torch.Tensor, d1: torch.Tensor, d2: torch.Tensor) -> LT:
    """Generic elementwise rule given value ``y=f(x)``, ``f'(x)``, ``f''(x)``."""
    J = a.J * d1.unsqueeze(1)
    L = d1 * a.L + d2 * (a.J * a.J).sum(1)
    return LT(y, J, L)


def tanh(a: LT) -> LT:
    y = torch.tanh(a.x)
    d1 = 1.0 - y * y
    return unary(a, y, d1, -2.0 * y * d1)


def exp(a: LT) -> LT:
    y = torch.exp(a.x)
    return unary(a, y, y, y)


def log(a: LT) -> LT:
    inv = 1.0 / a.x
    return unary(a, torch.log(a.x), inv, -inv * inv)


def log1p(a: LT) -> LT:
    inv = 1.0 / (1.0 + a.x)
    return unary(a, torch.log1p(a.x), inv, -inv * inv)


def sqrt(a: LT) -> LT:
    y = torch.sqrt(a.x)
    d1 = 0.5 / y
    return unary(a, y, d1, -0.5 * d1 / a.x)


def reciprocal(a: LT) -> LT:
    inv = 1.0 / a.x
    return unary(a, inv, -inv * inv, 2.0 * inv * inv * inv)


def absval(a: LT) -> LT:
    """``|x|`` away from zero: multiplication by the sign mask
    (``src/jaqmc/laplacian/primitives/elementwise.py:118-126``)."""
    s = torch.where(a.x >= 0, torch.ones_like(a.x), -torch.ones_like(a.x))
    return unary(a, a.x.abs(), s, torch.zeros_like(a.x))


def norm_last(a: LT) -> LT:
    """Euclidean norm over the last axis."""
    return sqrt((a * a).sum(-1))


def slogdet(a: LT):
    """``(sign, log|det|)`` over the last two axes with the slogdet FL rule
    (``src/jaqmc/laplacian/primitives/slogdet.py:25-72``)."""
    A = a.x
    sign, ld = torch.linalg.slogdet(A)
    if a.D == 0:
        return sign, LT(ld, A.new_zeros((A.shape[0], 0) + tuple(ld.shape[1:])), torch.zeros_like(ld))
    Ainv = torch.linalg.inv(A)
    # M_d = A^-1 J_d  -> (B, D, ..., n, n)
    M = Ainv.unsqueeze(1) @ a.J
    J = M.diagonal(dim1=-2, dim2=-1).sum(-1)
    tL = (Ainv @ a.L).diagonal(dim1=-2, dim2=-1).sum(-1)
    hess = -(M * M.transpose(-1, -2)).sum((1, -1, -2))
    return sign, LT(ld, J, tL + hess)


def signed_logsumexp(sign: torch.Tensor, ld: LT, axis: int = -1):
    """``log|sum_k s_k exp(ld_k)|`` and its sign, with the max shift of
    ``src/jaqmc/wavefunction/output/logdet.py:65-77``.

    Tangents follow from composing the exp / sum / log rules:
    ``J = sum_k w_k J_k`` and ``L = sum_k w_k (L_k + sum_d J_kd^2) - sum_d J_d^2``
    with ``w_k = s_k exp(ld_k) / psi``.
    """
    m = ld.x.max(axis, keepdim=True).values
    e = sign * torch.exp(ld.x - m)
    S = e.sum(axis)
    val = torch.log(S.abs()) + m.squeeze(axis)
    s = torch.sign(S)
    w = e / S.unsqueeze(axis)
    if ld.D == 0:
        return s, LT(val, ld.J.sum(ld._jax(axis)), ld.L.sum(axis))
    ja = ld._jax(axis)
    J = (ld.J * w.unsqueeze(1)).sum(ja)
    L = (w * (ld.L + (ld.J * ld.J).sum(1))).sum(axis) - (J * J).sum(1)
    return s, LT(val, J, L)
