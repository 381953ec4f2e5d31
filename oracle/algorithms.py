"""CPU ORACLE (test infrastructure only): the crate's `src/algorithms` routines and the BSGS diagonal
linear transform, restated step by step over the oracle's ciphertext ops (`oracle.c` via `oracle.py`).

Each routine follows the reference's schedule literally (one `mult_plain` per BSGS term, one rotation at a
time), with its scale/level bookkeeping, so the GPU routines can be compared with it residue for residue.
Keys are coefficient-form arrays in the reference layout `[digits][2][limbs][N]`; the digit count of a key
is its first dimension.  Only tests use this module.

Reference files: `src/algorithms/halevi_shoup.rs:46-71`, `total_sum.rs:45-60`,
`src/ckks/bootstrapping/linear_transform.rs:27-272`, `src/algorithms/packed_diagonal.rs:60-77`,
`src/algorithms/paterson_stockmeyer.rs:18-349`, ops from `src/rns/context/ops.rs` and `rotation.rs`.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Dict, List, Optional, Sequence

import numpy as np

import oracle as O


@dataclass
class Ct:
    """RnsCiphertext (ciphertexts.rs:41-58): level = limbs - 1."""
    c0: np.ndarray
    c1: np.ndarray
    scale_bits: int

    @property
    def level(self) -> int:
        return self.c0.shape[0] - 1

    def truncate_levels(self, count: int) -> "Ct":
        """ciphertexts.rs:90-99."""
        assert 0 < count <= self.c0.shape[0]
        return Ct(self.c0[:count].copy(), self.c1[:count].copy(), self.scale_bits)


class Context:
    """The subset of RnsCkksContext the algorithms call, on the oracle."""

    def __init__(self, n: int, q_primes: Sequence, p_primes: Sequence):
        """q_primes / p_primes: objects with `modulus` and `primitive_root` (RnsPrime)."""
        self.n = n
        self.q = [x.modulus for x in q_primes]
        self.p = [x.modulus for x in p_primes]
        self.qpl = O.Plans(n, list(q_primes))
        self.ppl = O.Plans(n, list(p_primes)) if self.p else None
        self._enc = {}

    def num_slots(self) -> int:
        return self.n // 2

    def _plans(self, limbs: int) -> O.Plans:
        return self.qpl.prefix(limbs)

    def encode_at_level_and_scale(self, slots, level: int, scale_bits: int) -> np.ndarray:
        """context/encoding.rs -> encode_integer_coeffs + from_bigint_coeffs (memoised on the slot bytes)."""
        s = np.ascontiguousarray(np.asarray(slots, dtype=np.complex128))
        key = (s.tobytes(), level, scale_bits)
        if key not in self._enc:
            coeffs = O.encode_integer_coeffs(self.n, float(2.0 ** scale_bits), s)
            self._enc[key] = O.poly_from_bigint_coeffs(self.q[: level + 1], coeffs)
        return self._enc[key]

    def multiply_plain_rns(self, ct: Ct, plain: np.ndarray) -> Ct:
        """ops.rs:54-66 (scale unchanged)."""
        pl = self._plans(ct.level + 1)
        return Ct(O.rns_mul(pl, ct.c0, plain), O.rns_mul(pl, ct.c1, plain), ct.scale_bits)

    def mult_plain(self, ct: Ct, plain: np.ndarray) -> Ct:
        """context/ops.rs:20-30 (scale doubles)."""
        r = self.multiply_plain_rns(ct, plain)
        return Ct(r.c0, r.c1, ct.scale_bits + ct.scale_bits)

    def rescale(self, ct: Ct) -> Ct:
        """ops.rs:68-82: drop the last prime, scale_bits -= floor(log2 q_last) (saturating)."""
        pl = self._plans(ct.level + 1)
        drop = self.q[ct.level].bit_length() - 1
        return Ct(O.rescale_poly(pl, ct.c0), O.rescale_poly(pl, ct.c1), max(0, ct.scale_bits - drop))

    def mult_plain_slots_real(self, ct: Ct, slots) -> Ct:
        """context/ops.rs:39-48."""
        plain = self.encode_at_level_and_scale(np.asarray(slots, dtype=np.float64).astype(np.complex128),
                                               ct.level, ct.scale_bits)
        return self.rescale(self.mult_plain(ct, plain))

    def add(self, a: Ct, b: Ct) -> Ct:
        """ciphertexts.rs:60-69."""
        assert a.scale_bits == b.scale_bits, "ciphertexts must share the same scale to add"
        assert a.level == b.level, "ciphertexts must be at the same level to add"
        pl = self._plans(a.level + 1)
        return Ct(O.rns_add(pl, a.c0, b.c0), O.rns_add(pl, a.c1, b.c1), a.scale_bits)

    def rotate(self, ct: Ct, key) -> Ct:
        """context/rotation.rs:104-127; key = (galois_element, coefficient key)."""
        g, k = key
        r0, r1 = O.rotate(self._plans(ct.level + 1), self.ppl, ct.c0, ct.c1, g, k, k.shape[0])
        return Ct(r0, r1, ct.scale_bits)

    def mult_relinearized(self, a: Ct, b: Ct, key) -> Ct:
        """context/ops.rs:124-133."""
        assert a.level == b.level and a.scale_bits == b.scale_bits
        m0, m1 = O.mult_relinearized(self._plans(a.level + 1), self.ppl, a.c0, a.c1, b.c0, b.c1, key, key.shape[0])
        drop = self.q[a.level].bit_length() - 1
        return Ct(m0, m1, max(0, a.scale_bits + b.scale_bits - drop))


def _fold_steps(active_slots: int) -> List[int]:
    """halevi_shoup.rs:15-26 / total_sum.rs:14-25."""
    steps, step = [], 1
    width = 1
    while width < active_slots:
        width <<= 1
    while step < width:
        steps.append(step)
        step <<= 1
    return steps


def halevi_shoup_dot_product(ctx: Context, ct: Ct, plaintext_slots, rotation_keys: Dict[int, tuple]) -> Ct:
    """halevi_shoup.rs:46-71."""
    padded = np.zeros(ctx.num_slots())
    padded[: len(plaintext_slots)] = plaintext_slots
    acc = ctx.mult_plain_slots_real(ct, padded)
    for step in _fold_steps(len(plaintext_slots)):
        acc = ctx.add(acc, ctx.rotate(acc, rotation_keys[step]))
    return acc


def total_sum(ctx: Context, ct: Ct, active_slots: int, rotation_keys: Dict[int, tuple]) -> Ct:
    """total_sum.rs:45-60."""
    acc = ct
    for step in _fold_steps(active_slots):
        acc = ctx.add(acc, ctx.rotate(acc, rotation_keys[step]))
    return acc


def bsgs_baby_step(dimension: int) -> int:
    """linear_transform.rs:152-158."""
    b = 1
    while b * b < dimension:
        b += 1
    return b


def pack_bsgs_diagonals(ctx: Context, matrix, level: int, scale_bits: int,
                        baby_step: Optional[int] = None) -> List[List[Optional[np.ndarray]]]:
    """linear_transform.rs:160-211: giant_step_diagonals[g][j] = diagonal g*b+j, pre-rotated by the giant
    shift g*b and tiled with period `dimension`.  `baby_step` overrides the crate's ceil(sqrt(d)) split (a
    variant the crate does not offer; the same packing rule with another b)."""
    m = [list(map(complex, row)) for row in matrix]
    d = len(m)
    b = baby_step or bsgs_baby_step(d)
    out = []
    for g in range((d + b - 1) // b):
        shift = (g * b) % d
        row = []
        for j in range(b):
            k = g * b + j
            if k >= d:
                row.append(None)
                continue
            slots = []
            for slot in range(ctx.num_slots()):
                r = slot % d
                src = (r + d - shift) % d
                slots.append(m[src][(k + src) % d])
            row.append(ctx.encode_at_level_and_scale(np.array(slots), level, scale_bits))
        out.append(row)
    return out


def apply_diagonal_linear_transform(ctx: Context, ct: Ct, giant_step_diagonals, dimension: int,
                                    rotation_keys: Dict[int, tuple], baby_step: Optional[int] = None) -> Ct:
    """linear_transform.rs:109-150 with 213-252 (`baby_step` as in pack_bsgs_diagonals)."""
    b = baby_step or bsgs_baby_step(dimension)
    babies = [ct] + [ctx.rotate(ct, rotation_keys[s]) for s in range(1, min(b, dimension))]
    acc = None
    for g, diags in enumerate(giant_step_diagonals):
        inner = None
        for j, dg in enumerate(diags):
            if dg is None:
                continue
            term = ctx.mult_plain(babies[j], dg)
            inner = term if inner is None else ctx.add(inner, term)
        if inner is None:
            continue
        if g != 0:
            inner = ctx.rotate(inner, rotation_keys[g * b])
        acc = inner if acc is None else ctx.add(acc, inner)
    return ctx.rescale(acc)


def ps_block_size(term_count: int) -> int:
    """paterson_stockmeyer.rs:18-26."""
    b = 1
    while b * b < term_count:
        b += 1
    return b


def ps_required_levels(level: int, term_count: int) -> List[int]:
    """paterson_stockmeyer.rs:110-126."""
    if term_count == 1:
        return []
    b = ps_block_size(term_count)
    blocks = -(-term_count // b)
    final = level - (b - 1) - (blocks - 1)
    return list(range(level, final, -1))


def paterson_stockmeyer_eval(ctx: Context, ct: Ct, coefficients: Sequence[float],
                             relin_keys: Dict[int, np.ndarray]) -> Ct:
    """paterson_stockmeyer.rs:28-108 with the helpers at 146-349."""

    def constant_plain(value, level, scale_bits):
        return ctx.encode_at_level_and_scale(np.full(ctx.num_slots(), complex(value, 0.0)), level, scale_bits)

    def lift(c: Ct, target: int) -> Ct:
        assert c.scale_bits <= target, "cannot lower ciphertext scale with a plaintext-one lift"
        if c.scale_bits == target:
            return c
        r = ctx.multiply_plain_rns(c, constant_plain(1.0, c.level, target - c.scale_bits))
        return Ct(r.c0, r.c1, target)

    def add_constant(c: Ct, value: float) -> Ct:
        if value == 0.0:
            return c
        p = constant_plain(value, c.level, c.scale_bits)
        return Ct(O.rns_add(ctx._plans(c.level + 1), c.c0, p), c.c1, c.scale_bits)

    def constant_ct(level, scale_bits, value) -> Ct:
        z = np.zeros((level + 1, ctx.n), dtype=np.uint64)
        return add_constant(Ct(z, z.copy(), scale_bits), value)

    coeffs = [float(c) for c in coefficients]
    if len(coeffs) == 1:
        return constant_ct(ct.level, ct.scale_bits, coeffs[0])
    b = ps_block_size(len(coeffs))
    blocks = -(-len(coeffs) // b)
    working = min(ctx.q[lv].bit_length() - 1 for lv in ps_required_levels(ct.level, len(coeffs)))
    coeff_scale = working - ct.scale_bits
    assert coeff_scale >= 0
    # baby powers x, x^2, ..., x^b, each lifted to the input scale
    base = lift(ct, ct.scale_bits)
    powers = [base]
    for _ in range(2, b + 1):
        prev = powers[-1]
        nxt = ctx.mult_relinearized(lift(prev, ct.scale_bits), base.truncate_levels(prev.level + 1),
                                    relin_keys[prev.level])
        powers.append(lift(nxt, ct.scale_bits))
    giant = powers[-1]
    top = giant.level
    assert giant.level + 1 >= blocks
    block_cts = []
    for bi in range(blocks):
        target = top - (blocks - 1 - bi)
        acc = constant_ct(target, working, 0.0)
        for off in range(b):
            k = bi * b + off
            if k >= len(coeffs):
                break
            c = coeffs[k]
            if c == 0.0:
                continue
            if off == 0:
                acc = add_constant(acc, c)
                continue
            pw = powers[off - 1]
            aligned = lift(pw.truncate_levels(target + 1), pw.scale_bits)
            term = ctx.multiply_plain_rns(aligned, constant_plain(c, aligned.level, coeff_scale))
            acc = ctx.add(acc, Ct(term.c0, term.c1, aligned.scale_bits + coeff_scale))
        block_cts.append(acc)
    result = block_cts[-1]
    for blk in reversed(block_cts[:-1]):
        g = lift(giant.truncate_levels(result.level + 1), result.scale_bits)
        m = ctx.mult_relinearized(result, g, relin_keys[result.level])
        result = ctx.add(lift(m, result.scale_bits), blk)
    return result
