"""CPU ORACLE (test infrastructure only): the device samplers' generator and value maps restated in Python,
so the GPU draws can be checked value for value.

Philox4x32 with 10 rounds (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3",
SC 2011), pinned by the published known-answer vectors in tests/test_sampler.py.  The value maps follow the
library's samplers: uniform residue = (64 random bits) mod q (the reference's `rng.gen::<u64>() % q`,
src/rns/keys.rs:87-99); ternary = the first of the four 32-bit words below 2^32 - 1, mod 3, mapped
0 -> 0, 1 -> 1, 2 -> -1 (keys.rs:123-147).
"""
from __future__ import annotations

from typing import List

MASK = 0xFFFFFFFF


def philox4x32_10(counter: List[int], key: List[int]) -> List[int]:
    c = [x & MASK for x in counter]
    k0, k1 = key[0] & MASK, key[1] & MASK
    for _ in range(10):
        p0 = 0xD2511F53 * c[0]
        p1 = 0xCD9E8D57 * c[2]
        c = [(p1 >> 32) ^ c[1] ^ k0, p1 & MASK, (p0 >> 32) ^ c[3] ^ k1, p0 & MASK]
        k0 = (k0 + 0x9E3779B9) & MASK
        k1 = (k1 + 0xBB67AE85) & MASK
    return c


def draw(seed: int, stream_id: int, index: int) -> List[int]:
    return philox4x32_10([index & MASK, index >> 32, stream_id & MASK, (stream_id >> 32) & MASK],
                         [seed & MASK, (seed >> 32) & MASK])


def uniform_residue(seed: int, stream_id: int, index: int, q: int) -> int:
    r = draw(seed, stream_id, index)
    return ((r[1] << 32) | r[0]) % q


def ternary_value(seed: int, stream_id: int, index: int) -> int:
    v = 0
    for w in reversed(draw(seed, stream_id, index)):
        if w != MASK:
            v = w % 3
    return {0: 0, 1: 1, 2: -1}[v]
