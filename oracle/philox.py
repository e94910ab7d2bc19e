"""Philox4x32-10 and the MH draw layout (oracle; test infrastructure only).

Integer-exact numpy restatement of the counter-based generator of Salmon,
Moraes, Dror & Shaw (SC'11) used by the GPU sampler, plus the mapping from
words to the open-interval uniforms the sampler consumes.  The reference
samples with jax.random (threefry); parity runs therefore inject the same
draws into both sides (``src/jaqmc/sampler/mcmc.py:125-131`` consumes them).
"""
from __future__ import annotations

import numpy as np

M0, M1 = np.uint64(0xD2511F53), np.uint64(0xCD9E8D57)
W0, W1 = np.uint32(0x9E3779B9), np.uint32(0xBB67AE85)
MASK = np.uint64(0xFFFFFFFF)


def philox4x32_10(ctr, key):
    """``ctr``: uint32 array (..., 4); ``key``: uint32 array (..., 2)."""
    c = [np.asarray(ctr, dtype=np.uint32)[..., i].astype(np.uint64) for i in range(4)]
    k0 = np.asarray(key, dtype=np.uint32)[..., 0].copy()
    k1 = np.asarray(key, dtype=np.uint32)[..., 1].copy()
    with np.errstate(over="ignore"):
        for _ in range(10):
            p0 = M0 * c[0]
            p1 = M1 * c[2]
            hi0, lo0 = p0 >> np.uint64(32), p0 & MASK
            hi1, lo1 = p1 >> np.uint64(32), p1 & MASK
            c = [hi1 ^ c[1] ^ k0.astype(np.uint64), lo1, hi0 ^ c[3] ^ k1.astype(np.uint64), lo0]
            k0 = (k0 + W0).astype(np.uint32)
            k1 = (k1 + W1).astype(np.uint32)
    return np.stack([x.astype(np.uint32) for x in c], -1)


def u01(words):
    """``((x >> 8) + 0.5) * 2^-24`` as float32 (exact)."""
    w = np.asarray(words, dtype=np.uint32)
    return ((w >> np.uint32(8)).astype(np.float32) + np.float32(0.5)) * np.float32(1.0 / 16777216.0)


def mh_words(seed: int, step: int, batch: int, n: int):
    """Words for one MH update: ``(batch, nb + 1, 4)`` with counter
    ``(block, walker, step_lo, step_hi)`` and key ``(seed_lo, seed_hi)``."""
    nb = (3 * n + 3) // 4
    b = np.arange(nb + 1, dtype=np.uint32)
    w = np.arange(batch, dtype=np.uint32)
    ctr = np.zeros((batch, nb + 1, 4), np.uint32)
    ctr[..., 0] = b[None, :]
    ctr[..., 1] = w[:, None]
    ctr[..., 2] = np.uint32(step & 0xFFFFFFFF)
    ctr[..., 3] = np.uint32((step >> 32) & 0xFFFFFFFF)
    key = np.zeros((batch, nb + 1, 2), np.uint32)
    key[..., 0] = np.uint32(seed & 0xFFFFFFFF)
    key[..., 1] = np.uint32((seed >> 32) & 0xFFFFFFFF)
    return philox4x32_10(ctr, key)


def mh_draws(seed: int, step: int, batch: int, n: int):
    """Normals ``(batch, n, 3)`` (Box-Muller on word pairs, float64) and the
    accept uniforms ``(batch,)`` (float32, bit-exact with the GPU)."""
    words = mh_words(seed, step, batch, n)
    nb = (3 * n + 3) // 4
    wn = words[:, :nb, :].reshape(batch, nb * 4)
    u = u01(wn).astype(np.float64)
    u1, u2 = u[:, 0::2], u[:, 1::2]
    rad = np.sqrt(-2.0 * np.log(u1))
    z = np.stack([rad * np.cos(2 * np.pi * u2), rad * np.sin(2 * np.pi * u2)], -1).reshape(batch, -1)
    return z[:, :3 * n].reshape(batch, n, 3), u01(words[:, nb, 0])
