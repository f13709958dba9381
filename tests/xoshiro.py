"""Independent numpy implementation of the generator contract, used to
check the engine's streams: xoshiro256+ (Blackman & Vigna), SplitMix64
seeding, jump() by 2^128 with the published jump polynomial, and the
53-bit uniform.  Written from the published algorithm descriptions,
separately from dust2_gb300/csrc/dust2gpu/random.hpp."""

import numpy as np

M64 = (1 << 64) - 1
JUMP = (0x180EC6D33CFD0ABA, 0xD5A61266F0C9392C, 0xA9582618E03FC9AA,
        0x39ABDC4529B1661C)


def splitmix64(x):
    x = (x + 0x9E3779B97F4A7C15) & M64
    z = x
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M64
    return x, z ^ (z >> 31)


def seed_state(seed):
    s = []
    x = seed & M64
    for _ in range(4):
        x, z = splitmix64(x)
        s.append(z)
    return s


def rotl(x, k):
    return ((x << k) | (x >> (64 - k))) & M64


def next_(s):
    result = (s[0] + s[3]) & M64
    t = (s[1] << 17) & M64
    s[2] ^= s[0]
    s[3] ^= s[1]
    s[1] ^= s[2]
    s[0] ^= s[3]
    s[2] ^= t
    s[3] = rotl(s[3], 45)
    return result


def jump(s):
    acc = [0, 0, 0, 0]
    for word in JUMP:
        for b in range(64):
            if word & (1 << b):
                for i in range(4):
                    acc[i] ^= s[i]
            next_(s)
    s[:] = acc


def random_real(s):
    return (next_(s) >> 11) * 2.0 ** -53


def streams(seed, n):
    """Words of the first n streams of an integer seed (uint64 array)."""
    s = seed_state(seed)
    out = np.empty(4 * n, dtype=np.uint64)
    for k in range(n):
        if k > 0:
            jump(s)
        out[4 * k:4 * k + 4] = s
    return out
