"""CPU ORACLE (test infrastructure only): the crate's CKKS bootstrapping scaffold (`src/ckks/bootstrapping`),
restated over the oracle's ciphertext ops (`algorithms.py`, `oracle.py`).

ModRaise lifts a ciphertext to the eval-key basis Q u P with the exact centred basis extension; the
roundtrips project back to Q, run CoeffToSlot (a BSGS diagonal transform of the exact sparse or dense
canonical-embedding matrices), EvalMod (Paterson-Stockmeyer on odd sine Taylor coefficients) and
SlotToCoeff.  The exact transform matrices are FP64 host computations with the reference's FFT
(`canonical_embedding.rs`), operation for operation.  Only tests use this module.

Reference files: `src/ckks/bootstrapping/{mod_raise,exact_transforms,coeff_to_slot,slot_to_coeff,eval_mod,
keys,params,roundtrip}.rs`.
"""
from __future__ import annotations

import math
from typing import Dict, List, Sequence, Tuple

import numpy as np

import algorithms as OA
import oracle as O


# --------------------------------------------------------------------------------------------------------
# params.rs:14-60
# --------------------------------------------------------------------------------------------------------

def bootstrap_parameters(ctx: OA.Context, ciphertext_level: int, active_slots: int) -> dict:
    """BootstrapParameters::new (params.rs:14-60), the same checks in the same order."""
    if not ctx.p:
        raise ValueError("bootstrapping requires an auxiliary evaluation basis")
    if ciphertext_level >= len(ctx.q):
        raise ValueError(f"ciphertext level must be in 0..{len(ctx.q)}, got {ciphertext_level}")
    if active_slots == 0:
        raise ValueError("active_slots must be positive")
    if active_slots & (active_slots - 1):
        raise ValueError("active_slots must be a power of two")
    if active_slots > ctx.num_slots():
        raise ValueError(f"active_slots cannot exceed the CKKS slot count {ctx.num_slots()}; got {active_slots}")
    q_count = ciphertext_level + 1
    return {"ciphertext_level": ciphertext_level, "q_level_count": q_count,
            "eval_level_count": q_count + len(ctx.p), "aux_level_count": len(ctx.p),
            "slot_count": ctx.num_slots(), "active_slots": active_slots}


# --------------------------------------------------------------------------------------------------------
# mod_raise.rs:29-45
# --------------------------------------------------------------------------------------------------------

def mod_raise(ctx: OA.Context, ct: OA.Ct) -> Tuple[OA.Ct, int, int]:
    """lift_poly_to_context of c0 and c1 to Q_level u P; returns (raised ct, q_level, aux_level_count)."""
    q = ctx._plans(ct.level + 1)
    r0 = O.lift(q, ctx.ppl, ct.c0)
    r1 = O.lift(q, ctx.ppl, ct.c1)
    return OA.Ct(r0, r1, ct.scale_bits), ct.level, len(ctx.p)


# --------------------------------------------------------------------------------------------------------
# exact_transforms.rs
# --------------------------------------------------------------------------------------------------------

def _xi(n: int) -> complex:
    """primitive_2n_root (exact_transforms.rs:315-317): Complex64::from_polar(1, pi / N)."""
    return complex(math.cos(math.pi / n), math.sin(math.pi / n))


def _eval_index(exponent: int) -> int:
    return (exponent - 1) // 2


_TWIST: Dict[Tuple[int, int], np.ndarray] = {}


def _twist(n: int, sign: int) -> np.ndarray:
    """xi^(sign * i) for i < n by num-complex `powi`, memoised per ring degree."""
    key = (n, sign)
    if key not in _TWIST:
        xi = _xi(n)
        _TWIST[key] = np.array([O._powi(xi, sign * i) for i in range(n)], dtype=np.complex128)
    return _TWIST[key]


def _cmul_vec(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """num-complex Mul elementwise: (ar*br - ai*bi) + (ar*bi + ai*br)i, no fused multiply-add."""
    ar, ai, br, bi = a.real, a.imag, b.real, b.imag
    return (ar * br - ai * bi) + 1j * (ar * bi + ai * br)


def dense_complex_coeffs_to_slots(n: int, coeffs) -> np.ndarray:
    """exact_transforms.rs:210-229: twist by xi^i, canonical_embedding_forward, read the 5^j slots."""
    twisted = _cmul_vec(np.asarray(coeffs, dtype=np.complex128), _twist(n, 1))
    evals = O.fft_in_place(twisted, False)
    idx = [_eval_index(e) for e in O.slot_exponents(n)]
    return evals[idx]


def dense_slots_to_real_coeffs(n: int, slots) -> np.ndarray:
    """exact_transforms.rs:180-200: conjugate-symmetric evaluations, canonical_embedding_backward, untwist,
    real part."""
    evals = np.zeros(n, dtype=np.complex128)
    for value, e in zip(slots, O.slot_exponents(n)):
        value = complex(value)
        evals[_eval_index(e)] = value
        evals[_eval_index((2 * n - e) % (2 * n))] = value.conjugate()
    coeffs = O.fft_in_place(evals, True)
    return _cmul_vec(coeffs, _twist(n, -1)).real


def exact_coeff_to_slot_matrix(n: int, active_slots: int) -> np.ndarray:
    """exact_transforms.rs:21-36 with compressed_coeffs_to_slots / expand_sparse_compressed_coeffs."""
    stride = (n // 2) // active_slots
    cols = []
    for column in range(active_slots):
        coeffs = np.zeros(n, dtype=np.complex128)
        coeffs[column * stride] = 1.0  # the basis vector's real part; its imaginary part is 0
        cols.append(dense_complex_coeffs_to_slots(n, coeffs)[:active_slots])
    return np.array(cols).T


def exact_slot_to_coeff_matrix(n: int, active_slots: int) -> np.ndarray:
    """exact_transforms.rs:38-53 with slots_to_compressed_coeffs / compress_sparse_real_coeffs."""
    slots = n // 2
    stride = slots // active_slots
    cols = []
    for column in range(active_slots):
        basis = np.zeros(active_slots, dtype=np.complex128)
        basis[column] = 1.0
        full = np.array([basis[i % active_slots] for i in range(slots)])
        rc = dense_slots_to_real_coeffs(n, full)
        cols.append(np.array([complex(rc[i * stride], rc[(i + active_slots) * stride]) for i in range(active_slots)]))
    return np.array(cols).T


def exact_dense_coeff_to_slot_matrices(n: int):
    """exact_transforms.rs:55-88: (upper_from_slots, upper_from_conjugates, lower_from_slots,
    lower_from_conjugates)."""
    s = n // 2
    uf, uc, lf, lc = (np.zeros((s, s), dtype=np.complex128) for _ in range(4))
    i = complex(0.0, 1.0)
    for column in range(s):
        rb = np.zeros(s, dtype=np.complex128)
        rb[column] = 1.0
        rr = dense_slots_to_real_coeffs(n, rb)
        ib = np.zeros(s, dtype=np.complex128)
        ib[column] = i
        ir = dense_slots_to_real_coeffs(n, ib)
        for row in range(s):
            ru, rl, iu, il = complex(rr[row]), complex(rr[row + s]), complex(ir[row]), complex(ir[row + s])
            uf[row, column] = (ru - O._cmul(i, iu)) * 0.5
            uc[row, column] = (ru + O._cmul(i, iu)) * 0.5
            lf[row, column] = (rl - O._cmul(i, il)) * 0.5
            lc[row, column] = (rl + O._cmul(i, il)) * 0.5
    return uf, uc, lf, lc


def exact_dense_slot_to_coeff_matrices(n: int):
    """exact_transforms.rs:90-117: (slots_from_upper, slots_from_lower)."""
    s = n // 2
    fu = np.zeros((s, s), dtype=np.complex128)
    fl = np.zeros((s, s), dtype=np.complex128)
    for column in range(s):
        c = np.zeros(n)
        c[column] = 1.0
        fu[:, column] = dense_complex_coeffs_to_slots(n, c)
        c = np.zeros(n)
        c[column + s] = 1.0
        fl[:, column] = dense_complex_coeffs_to_slots(n, c)
    return fu, fl


# --------------------------------------------------------------------------------------------------------
# coeff_to_slot.rs / slot_to_coeff.rs / eval_mod.rs
# --------------------------------------------------------------------------------------------------------

def linear_transform(ctx: OA.Context, ct: OA.Ct, matrix, keys: Dict[int, tuple]) -> OA.Ct:
    """coeff_to_slot / slot_to_coeff (coeff_to_slot.rs:221-233, slot_to_coeff.rs:196-209): the BSGS
    diagonal transform of `matrix` packed at the ciphertext's level and scale."""
    diags = OA.pack_bsgs_diagonals(ctx, matrix, ct.level, ct.scale_bits)
    return OA.apply_diagonal_linear_transform(ctx, ct, diags, len(matrix), keys)


def coeff_to_slot_dense(ctx: OA.Ct, ct: OA.Ct, conj: OA.Ct, mats, keys) -> Tuple[OA.Ct, OA.Ct]:
    """coeff_to_slot.rs:262-307 with apply_dense_branch (332-343)."""
    uf, uc, lf, lc = mats
    upper = ctx.add(linear_transform(ctx, ct, uf, keys), linear_transform(ctx, conj, uc, keys))
    lower = ctx.add(linear_transform(ctx, ct, lf, keys), linear_transform(ctx, conj, lc, keys))
    return upper, lower


def slot_to_coeff_dense(ctx: OA.Context, upper: OA.Ct, lower: OA.Ct, mats, keys) -> OA.Ct:
    """slot_to_coeff.rs:243-280."""
    fu, fl = mats
    return ctx.add(linear_transform(ctx, upper, fu, keys), linear_transform(ctx, lower, fl, keys))


def sine_taylor_coefficients(degree: int, sine_scale: float) -> List[float]:
    """eval_mod.rs:158-173 (factorial as the f64 fold of 191-193)."""
    assert degree > 0 and degree % 2 == 1
    out = [0.0] * (degree + 1)
    for d in range(1, degree + 1, 2):
        sign = 1.0 if ((d - 1) // 2) % 2 == 0 else -1.0
        fact = 1.0
        for f in range(1, d + 1):
            fact *= float(f)
        out[d] = sign * _powi_f64(sine_scale, d) / fact
    return out


def _powi_f64(x: float, e: int) -> float:
    """f64::powi for the small positive exponents used here: repeated multiplication by squaring."""
    r, b = 1.0, x
    while e:
        if e & 1:
            r *= b
        b *= b
        e >>= 1
    return r


def eval_mod(ctx: OA.Context, ct: OA.Ct, coefficients: Sequence[float], relin_keys: Dict[int, np.ndarray]) -> OA.Ct:
    """eval_mod.rs:133-156: Paterson-Stockmeyer on the sine coefficients."""
    for lv in OA.ps_required_levels(ct.level, len(coefficients)):
        if lv not in relin_keys:
            raise ValueError(f"missing EvalMod relinearization key at level {lv}")
    return OA.paterson_stockmeyer_eval(ctx, ct, coefficients, relin_keys)


def sparse_eval_mod_roundtrip(ctx: OA.Context, ct: OA.Ct, active_slots: int, coefficients, keys) -> OA.Ct:
    """roundtrip.rs:77-99 (bootstrap_exact_sparse_eval_mod_roundtrip_from_mod_raise) after mod_raise.

    keys: {"c2s": rotation keys at ct.level, "eval_mod": relin keys by level, "s2c": rotation keys at the
    EvalMod output level}."""
    raised, q_level, _ = mod_raise(ctx, ct)
    projected = raised.truncate_levels(q_level + 1)
    slots = linear_transform(ctx, projected, exact_coeff_to_slot_matrix(ctx.n, active_slots), keys["c2s"])
    evaluated = eval_mod(ctx, slots, coefficients, keys["eval_mod"])
    return linear_transform(ctx, evaluated, exact_slot_to_coeff_matrix(ctx.n, active_slots), keys["s2c"])
