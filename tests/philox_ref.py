"""Philox4x32-10 counter-based generator (Salmon, Moraes, Dror, Shaw,
"Parallel random numbers: as easy as 1, 2, 3", SC'11) restated in numpy, and
the Box-Muller noise the GPU's STOCH kick draws from it.  Test helper."""
import math

import numpy as np

M32 = 0xFFFFFFFF

M32 = 0xFFFFFFFF


def philox4x32_10(ctr, key):
    """Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) on uint64 numpy arrays
    holding 32-bit words; the same generator the STOCH kick uses on the GPU."""
    c0, c1, c2, c3 = [np.asarray(c, dtype=np.uint64) for c in ctr]
    k0, k1 = np.uint64(key[0]), np.uint64(key[1])
    for _ in range(10):
        p0 = np.uint64(0xD2511F53) * c0
        p1 = np.uint64(0xCD9E8D57) * c2
        hi0, lo0 = p0 >> np.uint64(32), p0 & np.uint64(M32)
        hi1, lo1 = p1 >> np.uint64(32), p1 & np.uint64(M32)
        c0, c1, c2, c3 = (hi1 ^ c1 ^ k0) & np.uint64(M32), lo1, (hi0 ^ c3 ^ k1) & np.uint64(M32), lo0
        k0 = (k0 + np.uint64(0x9E3779B9)) & np.uint64(M32)
        k1 = (k1 + np.uint64(0xBB67AE85)) & np.uint64(M32)
    return c0, c1, c2, c3


def stoch_noise(seed, step, n):
    """(n, 3) standard normals of particle i at `step`: Box-Muller on two Philox
    blocks with counter (i, step lo, step hi, 0|1), key = seed."""
    i = np.arange(n, dtype=np.uint64)
    key = (seed & M32, (seed >> 32) & M32)
    lo, hi = step & M32, (step >> 32) & M32
    r0 = philox4x32_10((i, np.full(n, lo), np.full(n, hi), np.zeros(n)), key)
    r1 = philox4x32_10((i, np.full(n, lo), np.full(n, hi), np.ones(n)), key)
    s = 2.0 ** -32
    u1, u2 = (r0[0].astype(np.float64) + 0.5) * s, (r0[1].astype(np.float64) + 0.5) * s
    u3, u4 = (r1[0].astype(np.float64) + 0.5) * s, (r1[1].astype(np.float64) + 0.5) * s
    ra, rb = np.sqrt(-2.0 * np.log(u1)), np.sqrt(-2.0 * np.log(u3))
    return np.stack([ra * np.cos(2 * math.pi * u2), ra * np.sin(2 * math.pi * u2), rb * np.cos(2 * math.pi * u4)], 1)


