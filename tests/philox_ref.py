"""A numpy restatement of Philox4x32-10 (Salmon, Moraes, Dror and Shaw,
SC'11) and of the small-mean Poisson inversion of xpsi_gb300/csrc/synth.cu,
used by the tests as the checker of the GPU draws."""
import math

import numpy as np

M0, M1, W0, W1 = 0xD2511F53, 0xCD9E8D57, 0x9E3779B9, 0xBB67AE85


def philox4x32_10(c, k):
    x, y, z, w = c
    k0, k1 = k
    for _ in range(10):
        p0 = M0 * x
        p1 = M1 * z
        x, y, z, w = ((p1 >> 32) ^ y ^ k0) & 0xffffffff, p1 & 0xffffffff, \
            ((p0 >> 32) ^ w ^ k1) & 0xffffffff, p0 & 0xffffffff
        k0 = (k0 + W0) & 0xffffffff
        k1 = (k1 + W1) & 0xffffffff
    return [x, y, z, w]


def first_uniform(seed, elem):
    """The first uniform double the GPU stream of element `elem` yields."""
    r = philox4x32_10([elem & 0xffffffff, (elem >> 32) & 0xffffffff, 0, 0x5eed5eed],
                      [seed & 0xffffffff, (seed >> 32) & 0xffffffff])
    return float(((r[0] >> 5) << 26) | (r[1] >> 6)) * 2.0 ** -53


def poisson_small(mu, u):
    """Inversion by sequential search, as the GPU does for mu < 10."""
    p = math.exp(-mu)
    F = p
    k = 0
    while u > F and k < 1000:
        k += 1
        p *= mu / k
        F += p
    return k
