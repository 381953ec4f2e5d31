"""The crate's `src/algorithms` routines (and the BSGS diagonal linear transform they use) on the GPU ops.

Each function keeps the reference's name, argument meaning, rotation/relinearization schedule, scale and
level bookkeeping and panic messages, so its output residues equal the reference's for the same keys and
inputs.  What changes is how the work reaches the GPU:

* rotations that do not depend on one another (BSGS baby steps, BSGS giant steps, and the same step applied
  to a batch of ciphertexts) go through one batched keyswitch call, so a rotation key is read once per batch;
* a BSGS inner sum  sum_b mult_plain(rot_b(ct), diag_{g,b})  is one `rc_mult_plain_accumulate` call over
  baby-step rotations and diagonals transformed once, instead of one multiply (three transforms) per term.
  The sum of products is the same modular value however it is grouped, so the residues are unchanged.

Reference files: `src/algorithms/halevi_shoup.rs`, `total_sum.rs`, `packed_diagonal.rs`,
`paterson_stockmeyer.rs`, `src/ckks/bootstrapping/linear_transform.rs`.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence

import numpy as np
import torch

from ._lib import RcError
from .context import RnsCiphertext, RnsCkksContext, RnsKeySwitchingKey, RnsPolynomial, RnsRotationKey


def _panic(msg: str) -> None:
    raise RcError(1, msg)


def _fold_steps(active_slots: int) -> List[int]:
    if active_slots <= 0:
        _panic("active_slots must be positive")
    steps, step = [], 1
    width = 1 << (active_slots - 1).bit_length()  # next_power_of_two
    while step < width:
        steps.append(step)
        step <<= 1
    return steps


def _rotate_all(ctx: RnsCkksContext, cts: Sequence[RnsCiphertext], keys: Sequence[RnsRotationKey]):
    """Independent rotations in one batched call (jobs sharing a key are kept adjacent)."""
    if not cts:
        return []
    return ctx.rotate_batch(list(cts), list(keys))


# --------------------------------------------------------------------------------------------------------
# Halevi-Shoup dot product, src/algorithms/halevi_shoup.rs
# --------------------------------------------------------------------------------------------------------

def halevi_shoup_dot_product_rotation_steps(active_slots: int) -> List[int]:
    """halevi_shoup.rs:15-26: 1, 2, 4, ... below next_power_of_two(active_slots)."""
    return _fold_steps(active_slots)


def generate_halevi_shoup_dot_product_rotation_keys(ctx: RnsCkksContext, secret_key, public_key, level: int,
                                                    active_slots: int) -> Dict[int, RnsRotationKey]:
    """halevi_shoup.rs:28-44."""
    return {step: ctx.generate_rotation_key_at_level(secret_key, public_key, step, level)
            for step in halevi_shoup_dot_product_rotation_steps(active_slots)}


def _padded(ctx: RnsCkksContext, plaintext_slots) -> np.ndarray:
    v = np.asarray(plaintext_slots, dtype=np.float64)
    if v.size > ctx.num_slots():
        _panic("plaintext slot vector cannot exceed the CKKS slot count")
    if v.size == 0:
        _panic("plaintext slot vector cannot be empty")
    out = np.zeros(ctx.num_slots(), dtype=np.float64)
    out[: v.size] = v
    return out


def halevi_shoup_dot_product(ctx: RnsCkksContext, ciphertext: RnsCiphertext, plaintext_slots,
                             rotation_keys: Dict[int, RnsRotationKey]) -> RnsCiphertext:
    """halevi_shoup.rs:46-71: mult_plain_slots_real, then rotate-and-add over the fold steps."""
    return halevi_shoup_dot_product_batch(ctx, [ciphertext], [plaintext_slots], rotation_keys)[0]


def halevi_shoup_dot_product_batch(ctx: RnsCkksContext, ciphertexts: Sequence[RnsCiphertext],
                                   plaintext_slots: Sequence, rotation_keys: Dict[int, RnsRotationKey]
                                   ) -> List[RnsCiphertext]:
    """`halevi_shoup_dot_product` for many independent (ciphertext, plaintext) pairs: every fold step rotates
    the whole batch in one call.  Each result equals the single-pair routine's."""
    lengths = {len(np.atleast_1d(p)) for p in plaintext_slots}
    # mult_plain_slots_real (context/ops.rs:39-48) for every pair: encode at the ciphertext's level and scale,
    # mult_plain (scale doubles), rescale -- the products and rescales as batched calls
    cts = list(ciphertexts)
    plains = [ctx.encode_at_level_and_scale(_padded(ctx, p).astype(np.complex128), ct.level, ct.scale_bits)
              for ct, p in zip(cts, plaintext_slots)]
    for ct, p in zip(cts, plains):
        if p.levels() != ct.level + 1:
            _panic("plaintext levels must match the multiplication context")
    prods = [RnsCiphertext(m.data, ct.scale_bits + ct.scale_bits, m.level)
             for m, ct in zip(ctx.multiply_plain_rns_batch(cts, plains), cts)]
    accs = ctx.rescale_batch(prods)
    if len(lengths) != 1:  # different fold widths: run each pair's schedule on its own
        return [_fold(ctx, [a], len(np.atleast_1d(p)), rotation_keys, "missing rotation key for step {}")[0]
                for a, p in zip(accs, plaintext_slots)]
    return _fold(ctx, accs, lengths.pop(), rotation_keys, "missing rotation key for step {}")


def _fold(ctx, accs, active_slots, rotation_keys, missing):
    for step in _fold_steps(active_slots):
        key = rotation_keys.get(step)
        if key is None:
            _panic(missing.format(step))
        rotated = _rotate_all(ctx, accs, [key] * len(accs))
        accs = ctx.add_batch(accs, rotated)
    return accs


# --------------------------------------------------------------------------------------------------------
# Total sum, src/algorithms/total_sum.rs
# --------------------------------------------------------------------------------------------------------

def total_sum_rotation_steps(active_slots: int) -> List[int]:
    """total_sum.rs:14-25."""
    return _fold_steps(active_slots)


def generate_total_sum_rotation_keys(ctx: RnsCkksContext, secret_key, public_key, level: int,
                                     active_slots: int) -> Dict[int, RnsRotationKey]:
    """total_sum.rs:27-43."""
    return {step: ctx.generate_rotation_key_at_level(secret_key, public_key, step, level)
            for step in total_sum_rotation_steps(active_slots)}


def total_sum(ctx: RnsCkksContext, ciphertext: RnsCiphertext, active_slots: int,
              rotation_keys: Dict[int, RnsRotationKey]) -> RnsCiphertext:
    """total_sum.rs:45-60."""
    return total_sum_batch(ctx, [ciphertext], active_slots, rotation_keys)[0]


def total_sum_batch(ctx: RnsCkksContext, ciphertexts: Sequence[RnsCiphertext], active_slots: int,
                    rotation_keys: Dict[int, RnsRotationKey]) -> List[RnsCiphertext]:
    """`total_sum` over many ciphertexts, one batched rotation per fold step."""
    return _fold(ctx, list(ciphertexts), active_slots, rotation_keys,
                 "missing total-sum rotation key for step {}")


# --------------------------------------------------------------------------------------------------------
# BSGS diagonal linear transform, src/ckks/bootstrapping/linear_transform.rs
# --------------------------------------------------------------------------------------------------------

@dataclass
class DiagonalTransformRotationKeys:
    """linear_transform.rs:7-10."""
    by_step: Dict[int, RnsRotationKey] = field(default_factory=dict)


@dataclass
class DiagonalTransformPlaintexts:
    """linear_transform.rs:12-20, plus the NTT-domain copies of the BSGS diagonals the GPU path reuses."""
    diagonals: List[RnsPolynomial]
    dimension: int
    baby_step: int
    giant_step_diagonals: List[List[Optional[RnsPolynomial]]]
    level: int
    scale_bits: int
    giant_step_diagonals_ntt: List[List[Optional[torch.Tensor]]] = field(default_factory=list)


def diagonal_transform_rotation_steps(dimension: int) -> List[int]:
    """linear_transform.rs:22-25."""
    if dimension <= 0:
        _panic("transform dimension must be positive")
    return list(range(1, dimension))


def diagonal_transform_bsgs_baby_step(dimension: int) -> int:
    """linear_transform.rs:152-158: ceil(sqrt(dimension)) by the crate's loop (12 for 128)."""
    b = 1
    while b * b < dimension:
        b += 1
    return b


def _baby_step_for(dimension: int, baby_step: Optional[int]) -> int:
    """The crate's split (ceil(sqrt(dimension))) unless a baby step is given.  Another split is a variant the
    crate does not offer: the same rotations and packing rule with another b, not the crate's residues."""
    if baby_step is None:
        return diagonal_transform_bsgs_baby_step(dimension)
    if baby_step <= 0 or baby_step > dimension:
        _panic("BSGS baby step must be in 1..=dimension")
    return baby_step


def diagonal_transform_bsgs_rotation_steps(dimension: int, baby_step: Optional[int] = None) -> List[int]:
    """linear_transform.rs:27-50: baby steps 1..b-1 and giant steps g*b below dimension."""
    if dimension <= 0:
        _panic("transform dimension must be positive")
    if dimension == 1:
        return []
    b = _baby_step_for(dimension, baby_step)
    giants = (dimension + b - 1) // b
    steps = set(range(1, min(b, dimension)))
    steps.update(g * b for g in range(1, giants) if g * b < dimension)
    return sorted(steps)


def generate_diagonal_transform_rotation_keys(ctx: RnsCkksContext, secret_key, public_key, ciphertext_level: int,
                                              dimension: int,
                                              baby_step: Optional[int] = None) -> DiagonalTransformRotationKeys:
    """linear_transform.rs:52-67."""
    return DiagonalTransformRotationKeys({
        step: ctx.generate_rotation_key_at_level(secret_key, public_key, step, ciphertext_level)
        for step in diagonal_transform_bsgs_rotation_steps(dimension, baby_step)})


def repeat_block_slots(values, slot_count: int) -> np.ndarray:
    """linear_transform.rs:69-77."""
    v = np.asarray(values)
    if v.size == 0:
        _panic("input block cannot be empty")
    if v.size > slot_count:
        _panic("input block cannot exceed slot count")
    if slot_count % v.size != 0:
        _panic("slot count must be a multiple of the active block length")
    return np.array([v[i % v.size] for i in range(slot_count)])


def _validate_square_matrix(matrix, slot_count: int) -> int:
    """linear_transform.rs:254-263."""
    if len(matrix) == 0:
        _panic("matrix cannot be empty")
    d = len(matrix)
    if d & (d - 1):
        _panic("matrix dimension must be a power of two")
    if d > slot_count:
        _panic("matrix dimension cannot exceed slot count")
    for row in matrix:
        if len(row) != d:
            _panic("current diagonal transform implementation expects a square matrix")
    return d


def _packed_diagonal_slots(m: np.ndarray, diagonal: int, slot_count: int) -> np.ndarray:
    """linear_transform.rs:265-272: zero-padded generalized diagonal."""
    d = m.shape[0]
    out = np.zeros(slot_count, dtype=np.complex128)
    rows = np.arange(d)
    out[:d] = m[rows, (diagonal + rows) % d]
    return out


def _packed_bsgs_diagonal_slots(m: np.ndarray, diagonal_step: int, giant_shift: int, slot_count: int) -> np.ndarray:
    """linear_transform.rs:193-211: diagonal pre-rotated by the giant shift, tiled with period `dimension`."""
    d = m.shape[0]
    shift = giant_shift % d
    row = np.arange(slot_count) % d
    src = (row + d - shift) % d
    return m[src, (diagonal_step + src) % d]


def pack_diagonal_transform_plaintexts(ctx: RnsCkksContext, matrix, level: int, scale_bits: int,
                                       baby_step: Optional[int] = None) -> DiagonalTransformPlaintexts:
    """linear_transform.rs:79-107 (+ 160-191); `baby_step` as in diagonal_transform_bsgs_rotation_steps."""
    d = _validate_square_matrix(matrix, ctx.num_slots())
    m = np.asarray(matrix, dtype=np.complex128)
    b = _baby_step_for(d, baby_step)
    giants = (d + b - 1) // b
    # every diagonal and every pre-rotated BSGS diagonal in one batched GPU encode (each plaintext equals the
    # single host encode of its slots)
    slots = [_packed_diagonal_slots(m, k, ctx.num_slots()) for k in range(d)]
    where = []
    for g in range(giants):
        for j in range(b):
            k = g * b + j
            if k < d:
                where.append((g, j))
                slots.append(_packed_bsgs_diagonal_slots(m, k, g * b, ctx.num_slots()))
    encoded = []
    for c0 in range(0, len(slots), 256):
        encoded += ctx.encode_device_batch(slots[c0:c0 + 256], level, scale_bits)
    diagonals = encoded[:d]
    gsd: List[List[Optional[RnsPolynomial]]] = [[None] * b for _ in range(giants)]
    for (g, j), p in zip(where, encoded[d:]):
        gsd[g][j] = p
    gsd_ntt = [[None if p is None else ctx.ntt_forward_copy(p.data) for p in row] for row in gsd]
    return DiagonalTransformPlaintexts(diagonals, d, b, gsd, level, scale_bits, gsd_ntt)


def apply_diagonal_linear_transform(ctx: RnsCkksContext, ciphertext: RnsCiphertext,
                                    diagonals: DiagonalTransformPlaintexts,
                                    rotation_keys: DiagonalTransformRotationKeys) -> RnsCiphertext:
    """linear_transform.rs:109-150."""
    return apply_diagonal_linear_transform_batch(ctx, [ciphertext], diagonals, rotation_keys)[0]


def apply_diagonal_linear_transform_batch(ctx: RnsCkksContext, ciphertexts: Sequence[RnsCiphertext],
                                          diagonals: DiagonalTransformPlaintexts,
                                          rotation_keys: DiagonalTransformRotationKeys) -> List[RnsCiphertext]:
    """The BSGS transform of linear_transform.rs:109-150 applied to many ciphertexts with one set of
    diagonals: baby-step rotations of all ciphertexts in one batched call, every inner sum as one
    NTT-domain plaintext multiply-accumulate, giant-step rotations of all (ciphertext, giant) pairs in one
    batched call, then the adds and the single rescale of the reference."""
    cts = list(ciphertexts)
    for ct in cts:
        if diagonals.level != ct.level:
            _panic("packed diagonals must match the ciphertext level")
        if diagonals.scale_bits != ct.scale_bits:
            _panic("packed diagonals must match the ciphertext scale")
    b = min(diagonals.baby_step, diagonals.dimension)
    # precompute_baby_rotations (linear_transform.rs:213-232)
    jobs, keys = [], []
    for step in range(1, b):
        key = rotation_keys.by_step.get(step)
        if key is None:
            _panic(f"missing input rotation key for BSGS baby step {step}")
        jobs += cts
        keys += [key] * len(cts)
    rotated = _rotate_all(ctx, jobs, keys)
    babies = [[ct] + [rotated[(s - 1) * len(cts) + i] for s in range(1, b)] for i, ct in enumerate(cts)]
    baby_ntt = [[RnsCiphertext(ctx.ntt_forward_copy(r.data), r.scale_bits, r.level) for r in row] for row in babies]
    # apply_giant_step_terms (linear_transform.rs:234-252) for every giant index and ciphertext
    inner: List[List[Optional[RnsCiphertext]]] = []
    for i in range(len(cts)):
        row = []
        for g, gd in enumerate(diagonals.giant_step_diagonals_ntt):
            terms = [(baby_ntt[i][j], p) for j, p in enumerate(gd) if p is not None]
            row.append(ctx.mult_plain_accumulate([t[0] for t in terms], [t[1] for t in terms], True, True)
                       if terms else None)
        inner.append(row)
    # giant-step rotations of the unrescaled inner sums
    jobs, keys, where = [], [], []
    for i in range(len(cts)):
        for g, s in enumerate(inner[i]):
            if g == 0 or s is None:
                continue
            step = g * diagonals.baby_step
            key = rotation_keys.by_step.get(step)
            if key is None:
                _panic(f"missing input rotation key for BSGS giant step {step}")
            jobs.append(s)
            keys.append(key)
            where.append((i, g))
    order = sorted(range(len(jobs)), key=lambda k: (where[k][1], where[k][0]))  # same key adjacent
    rot = _rotate_all(ctx, [jobs[k] for k in order], [keys[k] for k in order])
    for k, r in zip(order, rot):
        i, g = where[k]
        inner[i][g] = r
    # the adds of the reference's giant-step order, one batched call per giant step over all ciphertexts
    terms = [[t for t in inner[i] if t is not None] for i in range(len(cts))]
    if any(not t for t in terms):
        _panic("diagonal transform must contain at least one non-empty giant-step block")
    accs = [t[0] for t in terms]
    for g in range(1, max(len(t) for t in terms)):
        idx = [i for i in range(len(cts)) if g < len(terms[i])]
        summed = ctx.add_batch([accs[i] for i in idx], [terms[i][g] for i in idx])
        for i, v in zip(idx, summed):
            accs[i] = v
    return [ctx.rescale(a) for a in accs]


# --------------------------------------------------------------------------------------------------------
# Packed-diagonal matvec, src/algorithms/packed_diagonal.rs
# --------------------------------------------------------------------------------------------------------

PackedDiagonalRotationKeys = DiagonalTransformRotationKeys
PackedDiagonalPlaintexts = DiagonalTransformPlaintexts


def packed_diagonal_rotation_steps(row_count: int) -> List[int]:
    """packed_diagonal.rs:29-31."""
    return diagonal_transform_rotation_steps(row_count)


def generate_packed_diagonal_rotation_keys(ctx, secret_key, public_key, ciphertext_level: int,
                                           row_count: int, baby_step: Optional[int] = None) -> PackedDiagonalRotationKeys:
    """packed_diagonal.rs:33-41 (BSGS steps)."""
    return generate_diagonal_transform_rotation_keys(ctx, secret_key, public_key, ciphertext_level, row_count,
                                                     baby_step)


def repeat_real_vector_blocks(values, slot_count: int) -> np.ndarray:
    """packed_diagonal.rs:43-45."""
    return repeat_block_slots(np.asarray(values, dtype=np.float64), slot_count)


def pack_diagonal_plaintexts(ctx, matrix, level: int, scale_bits: int,
                             baby_step: Optional[int] = None) -> PackedDiagonalPlaintexts:
    """packed_diagonal.rs:47-58 (real matrix)."""
    return pack_diagonal_transform_plaintexts(ctx, np.asarray(matrix, dtype=np.float64).astype(np.complex128),
                                              level, scale_bits, baby_step)


def packed_diagonal_matvec_prepacked(ctx, ciphertext, diagonals, rotation_keys) -> RnsCiphertext:
    """packed_diagonal.rs:60-67."""
    return apply_diagonal_linear_transform(ctx, ciphertext, diagonals, rotation_keys)


def packed_diagonal_matvec(ctx, ciphertext, matrix, rotation_keys) -> RnsCiphertext:
    """packed_diagonal.rs:69-77."""
    diagonals = pack_diagonal_plaintexts(ctx, matrix, ciphertext.level, ciphertext.scale_bits)
    return packed_diagonal_matvec_prepacked(ctx, ciphertext, diagonals, rotation_keys)


# --------------------------------------------------------------------------------------------------------
# Paterson-Stockmeyer, src/algorithms/paterson_stockmeyer.rs
# --------------------------------------------------------------------------------------------------------

def paterson_stockmeyer_block_size(term_count: int) -> int:
    """paterson_stockmeyer.rs:18-26."""
    if term_count <= 0:
        _panic("term_count must be positive")
    b = 1
    while b * b < term_count:
        b += 1
    return b


def paterson_stockmeyer_required_levels(ciphertext_level: int, term_count: int) -> List[int]:
    """paterson_stockmeyer.rs:110-126."""
    if term_count <= 0:
        _panic("term_count must be positive")
    if term_count == 1:
        return []
    b = paterson_stockmeyer_block_size(term_count)
    blocks = -(-term_count // b)
    top = ciphertext_level - (b - 1)
    if top < 0:
        _panic("polynomial degree is too large for the available CKKS level budget")
    final = top - (blocks - 1)
    if final < 0:
        _panic("polynomial degree is too large for the available CKKS level budget")
    return list(range(ciphertext_level, final, -1))


def generate_paterson_stockmeyer_relinearization_keys(ctx: RnsCkksContext, secret_key, public_key,
                                                      ciphertext_level: int,
                                                      term_count: int) -> Dict[int, RnsKeySwitchingKey]:
    """paterson_stockmeyer.rs:128-144."""
    return {lvl: ctx.generate_relinearization_key_at_level(secret_key, public_key, lvl)
            for lvl in paterson_stockmeyer_required_levels(ciphertext_level, term_count)}


class _Plains:
    """Encoded constant plaintexts, memoised per (value, level, scale): the host FP64 encoder is the
    expensive part of a constant and the same ones recur across blocks and across a batch."""

    def __init__(self, ctx: RnsCkksContext):
        self.ctx, self.memo = ctx, {}

    def constant(self, value: float, level: int, scale_bits: int) -> RnsPolynomial:
        key = (float(value), level, scale_bits)
        if key not in self.memo:
            slots = np.full(self.ctx.num_slots(), complex(value, 0.0))
            self.memo[key] = self.ctx.encode_at_level_and_scale(slots, level, scale_bits)
        return self.memo[key]


def _align_ciphertext_to_level(ct: RnsCiphertext, target_level: int) -> RnsCiphertext:
    """paterson_stockmeyer.rs:221-228."""
    if target_level > ct.level:
        _panic("target level cannot exceed ciphertext level")
    return ct.truncate_levels(target_level + 1)


def _constant_ciphertext(ctx, pl: _Plains, level: int, scale_bits: int, constant: float) -> RnsCiphertext:
    """paterson_stockmeyer.rs:311-323."""
    ctx.level_moduli(level)
    zero = torch.zeros((2, level + 1, ctx.params.poly_degree), dtype=torch.int64, device="cuda")
    return _add_constant_term(ctx, pl, RnsCiphertext(zero, scale_bits, level), constant)


def _add_constant_term(ctx, pl: _Plains, ct: RnsCiphertext, constant: float) -> RnsCiphertext:
    """paterson_stockmeyer.rs:325-336."""
    if constant == 0.0:
        return ct
    plain = pl.constant(constant, ct.level, ct.scale_bits)
    c0 = ctx._poly_add(ct.data[0].contiguous(), plain.data)
    return RnsCiphertext(torch.stack([c0, ct.data[1]]), ct.scale_bits, ct.level)


def _working_scale_bits(ctx: RnsCkksContext, ciphertext_level: int, term_count: int) -> int:
    """paterson_stockmeyer.rs:290-309: min floor(log2 q_level) over the multiplication levels."""
    lv = paterson_stockmeyer_required_levels(ciphertext_level, term_count)
    if not lv:
        _panic("Paterson-Stockmeyer multiplication levels must be non-empty")
    return min(ctx.q_moduli[level].bit_length() - 1 for level in lv)


def _mult_relin_all(ctx, lhs, rhs, relin_keys: Dict[int, RnsKeySwitchingKey]):
    keys = []
    for a in lhs:
        k = relin_keys.get(a.level)
        if k is None:
            _panic(f"missing Paterson-Stockmeyer relinearization key at level {a.level}")
        keys.append(k)
    if len(lhs) == 1:
        return [ctx.mult_relinearized(lhs[0], rhs[0], keys[0])]
    return ctx.mult_relinearized_batch(lhs, rhs, keys)


def paterson_stockmeyer_eval(ctx: RnsCkksContext, ciphertext: RnsCiphertext, coefficients: Sequence[float],
                             relin_keys: Dict[int, RnsKeySwitchingKey]) -> RnsCiphertext:
    """paterson_stockmeyer.rs:28-108."""
    return paterson_stockmeyer_eval_batch(ctx, [ciphertext], coefficients, relin_keys)[0]


def constant_plaintext_cache(ctx: RnsCkksContext) -> "_Plains":
    """A cache of encoded constant plaintexts that callers may keep across `paterson_stockmeyer_eval_batch`
    calls on the same context (the encodings are deterministic)."""
    return _Plains(ctx)


def paterson_stockmeyer_eval_batch(ctx: RnsCkksContext, ciphertexts: Sequence[RnsCiphertext],
                                   coefficients: Sequence[float],
                                   relin_keys: Dict[int, RnsKeySwitchingKey],
                                   plains: Optional["_Plains"] = None) -> List[RnsCiphertext]:
    """`paterson_stockmeyer_eval` of one polynomial on many ciphertexts (same level and scale): each baby
    power and each outer product runs as one batched `mult_relinearized` over the batch."""
    coeffs = [float(c) for c in coefficients]
    if not coeffs:
        _panic("polynomial must contain at least one coefficient")
    cts = list(ciphertexts)
    pl = plains if plains is not None else _Plains(ctx)
    if len(coeffs) == 1:
        return [_constant_ciphertext(ctx, pl, ct.level, ct.scale_bits, coeffs[0]) for ct in cts]
    level, in_scale = cts[0].level, cts[0].scale_bits
    for ct in cts:
        if ct.level != level or ct.scale_bits != in_scale:
            raise RcError(1, "a batch must share level and scale")
    b = paterson_stockmeyer_block_size(len(coeffs))
    blocks = -(-len(coeffs) // b)
    working = _working_scale_bits(ctx, level, len(coeffs))
    coeff_scale = working - in_scale
    if coeff_scale < 0:
        _panic("Paterson-Stockmeyer working scale must dominate the input ciphertext scale")
    def lift_all(cs: List[RnsCiphertext], target: int) -> List[RnsCiphertext]:
        """_lift_ciphertext_scale (paterson_stockmeyer.rs:230-254) over a batch that shares level and scale,
        one batched call."""
        if cs[0].scale_bits > target:
            _panic("cannot lower ciphertext scale with a plaintext-one lift")
        if cs[0].scale_bits == target:
            return cs
        one = pl.constant(1.0, cs[0].level, target - cs[0].scale_bits)
        return [RnsCiphertext(x.data, target, x.level) for x in ctx.multiply_plain_rns_batch(cs, [one] * len(cs))]

    # precompute_baby_powers (146-173): note the crate lifts to the INPUT scale here
    base = lift_all(cts, in_scale)
    powers = [base]
    for _ in range(2, b + 1):
        prev = powers[-1]
        aligned_prev = lift_all(prev, in_scale)
        aligned_base = [_align_ciphertext_to_level(x, p.level) for x, p in zip(base, prev)]
        nxt = _mult_relin_all(ctx, aligned_prev, aligned_base, relin_keys)
        powers.append(lift_all(nxt, in_scale))
    giant = powers[-1]
    if giant[0].level + 1 < blocks:
        _panic("polynomial degree is too large for the available CKKS level budget")
    top = giant[0].level

    def evaluate_block(block_index: int, target_level: int) -> List[RnsCiphertext]:
        """paterson_stockmeyer.rs:175-219, every ciphertext of the batch per step."""
        accs = [_constant_ciphertext(ctx, pl, target_level, working, 0.0) for _ in cts]
        for offset in range(b):
            k = block_index * b + offset
            if k >= len(coeffs):
                break
            c = coeffs[k]
            if c == 0.0:
                continue
            if offset == 0:
                accs = [_add_constant_term(ctx, pl, a, c) for a in accs]
                continue
            power = [p[offset - 1] for p in per_ct_powers]
            aligned = lift_all([_align_ciphertext_to_level(x, target_level) for x in power], power[0].scale_bits)
            plain = pl.constant(c, aligned[0].level, coeff_scale)
            terms = [RnsCiphertext(t.data, aligned[0].scale_bits + coeff_scale, t.level)
                     for t in ctx.multiply_plain_rns_batch(aligned, [plain] * len(aligned))]
            accs = ctx.add_batch(accs, terms)
        return accs

    per_ct_powers = [[powers[e][i] for e in range(b)] for i in range(len(cts))]
    blocks_out = [evaluate_block(bi, top - (blocks - 1 - bi)) for bi in range(blocks)]
    result = blocks_out[-1]
    for bi in range(blocks - 2, -1, -1):
        aligned_giant = lift_all([_align_ciphertext_to_level(gs, result[0].level) for gs in giant],
                                 result[0].scale_bits)
        multiplied = _mult_relin_all(ctx, result, aligned_giant, relin_keys)
        lifted = lift_all(multiplied, result[0].scale_bits)
        result = ctx.add_batch(lifted, blocks_out[bi])
    return result


# --------------------------------------------------------------------------------------------------------
# the same schedules run natively (rc_total_sum_batch, rc_halevi_shoup_batch, rc_paterson_stockmeyer_batch):
# one library call per batch, no per-step host glue; residues equal the routines above
# --------------------------------------------------------------------------------------------------------

def _raw_in(cts):
    from ._lib import RcCiphertext
    n = len(cts)
    return (RcCiphertext * n)(*[c.raw() for c in cts])


def _raw_out(ctx, levels):
    from ._lib import RcCiphertext
    outs = [torch.empty((2, lv + 1, ctx.params.poly_degree), dtype=torch.int64, device="cuda") for lv in levels]
    return outs, (RcCiphertext * len(outs))(*[RcCiphertext(o.data_ptr(), 0, 0) for o in outs])


def _step_keys(rotation_keys: Dict[int, RnsRotationKey], active_slots: int):
    import ctypes
    steps = _fold_steps(active_slots)
    return (ctypes.c_void_p * max(1, len(steps)))(
        *[(rotation_keys[s].keyswitch_key.handle if s in rotation_keys else None) for s in steps]), len(steps)


def total_sum_native(ctx: RnsCkksContext, ciphertexts: Sequence[RnsCiphertext], active_slots: int,
                     rotation_keys: Dict[int, RnsRotationKey]) -> List[RnsCiphertext]:
    """`total_sum` (total_sum.rs:45-60) of a batch in one call (rc_total_sum_batch)."""
    from ._lib import call
    from .context import _stream
    cts = list(ciphertexts)
    if not cts:
        return []
    keys, nk = _step_keys(rotation_keys, active_slots)
    outs, O = _raw_out(ctx, [c.level for c in cts])
    call("rc_total_sum_batch", ctx.handle, len(cts), _raw_in(cts), active_slots, keys, nk, O, _stream())
    return [RnsCiphertext(o, O[i].scale_bits, O[i].level) for i, o in enumerate(outs)]


def halevi_shoup_dot_product_native(ctx: RnsCkksContext, ciphertexts: Sequence[RnsCiphertext], plaintext_slots,
                                    rotation_keys: Dict[int, RnsRotationKey]) -> List[RnsCiphertext]:
    """`halevi_shoup_dot_product` (halevi_shoup.rs:46-71) of a batch sharing one plaintext length, in one call
    (rc_halevi_shoup_batch); plaintext_slots is one real vector per ciphertext."""
    from ._lib import call
    from .context import _stream
    cts = list(ciphertexts)
    if not cts:
        return []
    plain = np.ascontiguousarray(np.asarray(plaintext_slots, dtype=np.float64).reshape(len(cts), -1))
    keys, nk = _step_keys(rotation_keys, plain.shape[1])
    outs, O = _raw_out(ctx, [max(c.level - 1, 0) for c in cts])
    call("rc_halevi_shoup_batch", ctx.handle, len(cts), _raw_in(cts), plain.ctypes.data, plain.shape[1], keys, nk,
         O, _stream())
    return [RnsCiphertext(o, O[i].scale_bits, O[i].level) for i, o in enumerate(outs)]


def paterson_stockmeyer_eval_native(ctx: RnsCkksContext, ciphertexts: Sequence[RnsCiphertext],
                                    coefficients: Sequence[float],
                                    relin_keys: Dict[int, RnsKeySwitchingKey]) -> List[RnsCiphertext]:
    """`paterson_stockmeyer_eval` (paterson_stockmeyer.rs:28-108) of one polynomial on a batch sharing level
    and scale, in one call (rc_paterson_stockmeyer_batch)."""
    import ctypes
    from ._lib import call
    from .context import _stream
    cts = list(ciphertexts)
    if not cts:
        return []
    coeffs = np.ascontiguousarray(np.asarray(coefficients, dtype=np.float64))
    levels = ctx.levels()
    keys = (ctypes.c_void_p * levels)(*[(relin_keys[l].handle if l in relin_keys else None) for l in range(levels)])
    outs, O = _raw_out(ctx, [c.level for c in cts])  # results are at or below the input level
    call("rc_paterson_stockmeyer_batch", ctx.handle, len(cts), _raw_in(cts), coeffs.ctypes.data, coeffs.size, keys,
         levels, O, _stream())
    n = ctx.params.poly_degree
    # the library wrote [c0][c1] with the result's limb count at the front of each buffer
    return [RnsCiphertext(o.view(-1)[: 2 * (O[i].level + 1) * n].view(2, O[i].level + 1, n).clone(), O[i].scale_bits,
                          O[i].level) for i, o in enumerate(outs)]


def apply_diagonal_linear_transform_native(ctx: RnsCkksContext, ciphertexts: Sequence[RnsCiphertext],
                                           diagonals: DiagonalTransformPlaintexts,
                                           rotation_keys: DiagonalTransformRotationKeys) -> List[RnsCiphertext]:
    """The BSGS transform (linear_transform.rs:109-150) of a batch with one set of diagonals, as one library call
    (rc_bsgs_apply_batch); the same residues as `apply_diagonal_linear_transform_batch`."""
    import ctypes
    from ._lib import call
    from .context import _stream
    cts = list(ciphertexts)
    if not cts:
        return []
    b, g = diagonals.baby_step, len(diagonals.giant_step_diagonals_ntt)
    diag = (ctypes.c_void_p * (g * b))(*[(p.data_ptr() if p is not None else None)
                                          for row in diagonals.giant_step_diagonals_ntt for p in row])
    ks = rotation_keys.by_step
    baby = (ctypes.c_void_p * max(1, b - 1))(
        *[(ks[s].keyswitch_key.handle if s in ks else None) for s in range(1, b)])
    giant = (ctypes.c_void_p * max(1, g - 1))(
        *[(ks[k * b].keyswitch_key.handle if k * b in ks else None) for k in range(1, g)])
    outs, O = _raw_out(ctx, [max(c.level - 1, 0) for c in cts])
    call("rc_bsgs_apply_batch", ctx.handle, len(cts), _raw_in(cts), diagonals.dimension, b, diag, g,
         diagonals.level, diagonals.scale_bits, baby, giant, O, _stream())
    return [RnsCiphertext(o, O[i].scale_bits, O[i].level) for i, o in enumerate(outs)]
