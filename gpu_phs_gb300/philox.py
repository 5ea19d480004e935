"""Philox4x32-10 counter-based generator (Salmon et al., SC'11) in numpy.

Defines the random-number stream x the benchmarks and tests use, identically on
the host (here) and on the device (phs_philox_fill in the CUDA library):

    element e of the flat array x[n_events * n_x] takes block = e >> 1,
    counter = (block & 0xffffffff, block >> 32, 0, 0), key = (seed_lo, seed_hi);
    the 4 output words r0..r3 give two doubles
        u0 = ((r0 << 32 | r1) >> 11) * 2**-53,  u1 = ((r2 << 32 | r3) >> 11) * 2**-53
    and element e takes u_(e & 1).  Every value lies in [0, 1).
"""
from __future__ import annotations

import numpy as np

M0 = np.uint64(0xD2511F53)
M1 = np.uint64(0xCD9E8D57)
W0 = np.uint32(0x9E3779B9)
W1 = np.uint32(0xBB67AE85)
_MASK32 = np.uint64(0xFFFFFFFF)


def philox4x32_10(ctr: np.ndarray, key: np.ndarray) -> np.ndarray:
    """ctr: uint32 [..., 4]; key: uint32 [..., 2] (broadcast).  Returns uint32 [..., 4]."""
    c0, c1, c2, c3 = (ctr[..., i].astype(np.uint64) for i in range(4))
    k0 = np.broadcast_to(key[..., 0], c0.shape).astype(np.uint32)
    k1 = np.broadcast_to(key[..., 1], c0.shape).astype(np.uint32)
    for r in range(10):
        p0 = M0 * c0
        p1 = M1 * c2
        hi0, lo0 = p0 >> np.uint64(32), p0 & _MASK32
        hi1, lo1 = p1 >> np.uint64(32), p1 & _MASK32
        c0, c1, c2, c3 = (hi1 ^ c1 ^ k0.astype(np.uint64), lo1,
                          hi0 ^ c3 ^ k1.astype(np.uint64), lo0)
        if r < 9:
            k0 = k0 + W0
            k1 = k1 + W1
    return np.stack([c0, c1, c2, c3], axis=-1).astype(np.uint32)


def uniform_x(seed: int, n_events: int, n_x: int, first_event: int = 0) -> np.ndarray:
    """x[n_events, n_x] float64 in [0,1): events first_event .. first_event+n_events-1
    of the stream for ``seed``."""
    e0 = first_event * n_x
    n = n_events * n_x
    if n == 0:
        return np.zeros((n_events, n_x), np.float64)
    b_lo, b_hi = e0 >> 1, (e0 + n - 1) >> 1
    blocks = np.arange(b_lo, b_hi + 1, dtype=np.uint64)
    ctr = np.zeros((blocks.size, 4), np.uint32)
    ctr[:, 0] = (blocks & _MASK32).astype(np.uint32)
    ctr[:, 1] = (blocks >> np.uint64(32)).astype(np.uint32)
    key = np.array([seed & 0xFFFFFFFF, (seed >> 32) & 0xFFFFFFFF], np.uint32)
    r = philox4x32_10(ctr, key).astype(np.uint64)
    u = np.empty((blocks.size, 2), np.float64)
    u[:, 0] = ((r[:, 0] << np.uint64(32) | r[:, 1]) >> np.uint64(11)).astype(np.float64)
    u[:, 1] = ((r[:, 2] << np.uint64(32) | r[:, 3]) >> np.uint64(11)).astype(np.float64)
    u *= 2.0 ** -53
    flat = u.reshape(-1)[e0 - 2 * b_lo: e0 - 2 * b_lo + n]
    return flat.reshape(n_events, n_x).copy()
