"""Philox4x32-10 (Salmon, Moraes, Dror & Shaw, "Parallel random numbers: as
easy as 1, 2, 3", SC 2011) restated for checking the library's per-trajectory
QJMC uniform streams.  Test infrastructure only.

The reference draws its QJMC uniforms from Julia's global RNG with rand()
(src/algorithms/mps/qjmc.jl:64,97,99); the library's seeded ensembles give
trajectory t the stream below instead (parity runs pass explicit draws)."""

import numpy as np

M0, M1 = 0xD2511F53, 0xCD9E8D57
W0, W1 = 0x9E3779B9, 0xBB67AE85
MASK = 0xFFFFFFFF


def philox4x32_10(counter, key):
    """Ten rounds on a 4x32-bit counter with a 2x32-bit key; returns 4 words."""
    c0, c1, c2, c3 = [int(x) & MASK for x in counter]
    k0, k1 = [int(x) & MASK for x in key]
    for _ in range(10):
        p0, p1 = M0 * c0, M1 * c2
        hi0, lo0 = p0 >> 32, p0 & MASK
        hi1, lo1 = p1 >> 32, p1 & MASK
        c0, c1, c2, c3 = (hi1 ^ c1 ^ k0) & MASK, lo1, (hi0 ^ c3 ^ k1) & MASK, lo0
        k0, k1 = (k0 + W0) & MASK, (k1 + W1) & MASK
    return c0, c1, c2, c3


def trajectory_uniforms(seed, traj, n):
    """Draw k of trajectory ``traj``: the top 53 bits of 64-bit word k % 2 of
    philox4x32_10(counter=(k//2 low, traj, k//2 high, 0), key=(seed low,
    seed high)), scaled to [0, 1)."""
    out = np.zeros(int(n))
    key = (seed & MASK, (seed >> 32) & MASK)
    for k in range(0, int(n), 2):
        b = k // 2
        c = philox4x32_10((b & MASK, traj, (b >> 32) & MASK, 0), key)
        w0, w1 = (c[1] << 32) | c[0], (c[3] << 32) | c[2]
        out[k] = (w0 >> 11) / 9007199254740992.0
        if k + 1 < n:
            out[k + 1] = (w1 >> 11) / 9007199254740992.0
    return out
