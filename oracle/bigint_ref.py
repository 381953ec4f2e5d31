"""CPU ORACLE (test infrastructure only): an independent big-integer restatement.

Where `oracle.c` follows the reference's Garner / base-2^30 digit machinery step
by step, this module states the same maps through exact Python integers:

* decomposition (`decompose_poly_rns_with_levels`, src/rns/keyswitching.rs:196-236):
  CRT-reconstruct X in [0, Q), centre it (X > floor(Q/2) -> X - Q), split it
  into balanced base-2^30 digits in [-2^29, 2^29), keep `levels` digits (the
  final carry is dropped as in the release build, keyswitching.rs:434-454);
* centred basis conversion (`convert_centered_residues_to_target`,
  keyswitching.rs:365-379) used by ModUp and ModDown;
* rescale (`rescale_poly_rns`, src/rns/ops.rs:135-186).

It is slow (pure Python) and only used on small cases to cross-check the C
oracle and the GPU path.
"""
from __future__ import annotations

import math
from typing import List, Sequence

import numpy as np


def crt(moduli: Sequence[int], residues: Sequence[int]) -> int:
    Q = math.prod(moduli)
    x = 0
    for q, r in zip(moduli, residues):
        part = Q // q
        x += int(r) * part * pow(part % q, -1, q)
    return x % Q


def centred(x: int, modulus: int) -> int:
    return x if x <= (modulus >> 1) else x - modulus


def balanced_digits(value: int, levels: int, bits: int = 30) -> List[int]:
    base = 1 << bits
    half = base >> 1
    out = []
    for _ in range(levels):
        d = value % base  # floor modulus in [0, base)
        if d >= half:
            d -= base
        out.append(d)
        value = (value - d) >> bits
    return out


def decompose(moduli: Sequence[int], poly, levels: int, bits: int = 30) -> np.ndarray:
    poly = np.asarray(poly)
    Q = math.prod(moduli)
    n = poly.shape[1]
    out = np.zeros((levels, n), dtype=np.int64)
    for i in range(n):
        x = centred(crt(moduli, [int(poly[l, i]) for l in range(len(moduli))]), Q)
        out[:, i] = balanced_digits(x, levels, bits)
    return out


def convert_centred(src_moduli: Sequence[int], residues: Sequence[int], target: int) -> int:
    Q = math.prod(src_moduli)
    return centred(crt(src_moduli, residues), Q) % target


def mod_down(q_moduli: Sequence[int], p_moduli: Sequence[int], poly) -> np.ndarray:
    poly = np.asarray(poly)
    lq, lp = len(q_moduli), len(p_moduli)
    P = math.prod(p_moduli)
    n = poly.shape[1]
    out = np.zeros((lq, n), dtype=np.uint64)
    for i in range(n):
        xp = centred(crt(p_moduli, [int(poly[lq + k, i]) for k in range(lp)]), P)
        for j, q in enumerate(q_moduli):
            out[j, i] = ((int(poly[j, i]) - xp) * pow(P % q, -1, q)) % q
    return out


def rescale(moduli: Sequence[int], poly) -> np.ndarray:
    poly = np.asarray(poly)
    ql = moduli[-1]
    n = poly.shape[1]
    out = np.zeros((len(moduli) - 1, n), dtype=np.uint64)
    for i in range(n):
        c = centred(int(poly[-1, i]), ql)
        for j, q in enumerate(moduli[:-1]):
            out[j, i] = ((int(poly[j, i]) - c) * pow(ql % q, -1, q)) % q
    return out
