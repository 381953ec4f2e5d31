"""The crate's CKKS bootstrapping scaffold (`src/ckks/bootstrapping`) on the GPU ops.

ModRaise is the exact centred lift to the eval-key basis (`rc_mod_raise`); CoeffToSlot and SlotToCoeff are
BSGS diagonal transforms of the exact canonical-embedding matrices (the batched BSGS of `algorithms.py`);
EvalMod is Paterson-Stockmeyer on odd sine Taylor coefficients.  Names, arguments, level and scale rules
and error messages follow the reference; its `Result::Err(String)` becomes `BootstrapError`.

The exact transform matrices are FP64 host work, as in the reference, built from the library's two
slot/coefficient maps (`rc_slots_to_real_coeffs`, `rc_complex_coeffs_to_slots`) with the reference's
operation order.  What the GPU form adds is reuse: `SparseBootstrapper` packs the diagonals and generates
the key set once and runs many ciphertexts through each stage as batched calls.

Reference files: `src/ckks/bootstrapping/{params,mod_raise,exact_transforms,coeff_to_slot,slot_to_coeff,
eval_mod,keys,roundtrip}.rs`.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np
import torch

from . import algorithms as A
from ._lib import RcCiphertext, call
from .context import RnsCiphertext, RnsCkksContext, RnsKeySwitchingKey, RnsPolynomial, RnsRotationKey, _stream


class BootstrapError(ValueError):
    """The reference's `Err(String)` results."""


# --------------------------------------------------------------------------------------------------------
# params.rs
# --------------------------------------------------------------------------------------------------------

@dataclass(frozen=True)
class BootstrapParameters:
    """params.rs:4-12."""
    ciphertext_level: int
    q_level_count: int
    eval_level_count: int
    aux_level_count: int
    slot_count: int
    active_slots: int

    @staticmethod
    def new(ctx: RnsCkksContext, ciphertext_level: int, active_slots: int) -> "BootstrapParameters":
        """params.rs:14-60."""
        if not ctx.has_aux_basis():
            raise BootstrapError("bootstrapping requires an auxiliary evaluation basis")
        if ciphertext_level >= ctx.levels():
            raise BootstrapError(f"ciphertext level must be in 0..{ctx.levels()}, got {ciphertext_level}")
        if active_slots == 0:
            raise BootstrapError("active_slots must be positive")
        if active_slots & (active_slots - 1):
            raise BootstrapError("active_slots must be a power of two")
        if active_slots > ctx.num_slots():
            raise BootstrapError(
                f"active_slots cannot exceed the CKKS slot count {ctx.num_slots()}; got {active_slots}")
        q_count = ciphertext_level + 1
        eval_count = len(ctx.eval_key_level_moduli(ciphertext_level))
        return BootstrapParameters(ciphertext_level, q_count, eval_count, eval_count - q_count, ctx.num_slots(),
                                   active_slots)

    @staticmethod
    def from_ciphertext(ctx: RnsCkksContext, ciphertext: RnsCiphertext, active_slots: int) -> "BootstrapParameters":
        return BootstrapParameters.new(ctx, ciphertext.level, active_slots)


# --------------------------------------------------------------------------------------------------------
# mod_raise.rs
# --------------------------------------------------------------------------------------------------------

@dataclass
class ModRaisedCiphertext:
    """mod_raise.rs:4-28: `ciphertext` holds [2][q_level + 1 + aux][N] over Q_q_level u P; its level is the
    eval-key context's (q_level + aux)."""
    ciphertext: RnsCiphertext
    _q_level: int
    _aux_level_count: int

    def q_level(self) -> int:
        return self._q_level

    def aux_level_count(self) -> int:
        return self._aux_level_count

    def eval_level(self) -> int:
        return self.ciphertext.level

    def project_to_q_ciphertext(self) -> RnsCiphertext:
        """truncate_levels(q_level + 1): the Q limbs of c0 and c1."""
        q = self._q_level + 1
        return RnsCiphertext(self.ciphertext.data[:, :q].contiguous(), self.ciphertext.scale_bits, self._q_level)


def mod_raise(ctx: RnsCkksContext, ciphertext: RnsCiphertext) -> ModRaisedCiphertext:
    """mod_raise.rs:29-45 on the GPU (one lift launch for c0 and c1)."""
    return mod_raise_batch(ctx, [ciphertext])[0]


def mod_raise_batch(ctx: RnsCkksContext, ciphertexts: Sequence[RnsCiphertext]) -> List[ModRaisedCiphertext]:
    if not ctx.has_aux_basis():
        raise BootstrapError("ModRaise requires an auxiliary evaluation basis")
    out = []
    K = len(ctx.p_moduli)
    for ct in ciphertexts:
        limbs = ct.level + 1
        data = torch.empty((2, limbs + K, ctx.params.poly_degree), dtype=torch.int64, device="cuda")
        o = RcCiphertext(data.data_ptr(), 0, 0)
        call("rc_mod_raise", ctx.handle, ctypes.byref(ct.raw()), ctypes.byref(o), _stream())
        out.append(ModRaisedCiphertext(RnsCiphertext(data, o.scale_bits, o.level), ct.level, K))
    return out


def decrypt_mod_raised(ctx: RnsCkksContext, ciphertext: ModRaisedCiphertext, secret_key) -> RnsPolynomial:
    """mod_raise.rs:48-67 (testing): c0 + c1 * s over Q_q_level u P with the lifted secret."""
    moduli = ctx.eval_key_level_moduli(ciphertext.q_level())
    s = ctx._secret_over(secret_key, moduli)
    d = ciphertext.ciphertext.data
    c1s = ctx._poly_mul(d[1].contiguous(), s, with_aux=True)
    return RnsPolynomial(ctx._poly_add(d[0].contiguous(), c1s, with_aux=True))


# --------------------------------------------------------------------------------------------------------
# exact_transforms.rs
# --------------------------------------------------------------------------------------------------------

def _interleave(z: np.ndarray) -> np.ndarray:
    out = np.empty(2 * z.size, dtype=np.float64)
    out[0::2], out[1::2] = z.real, z.imag
    return out


def _dense_slots_to_real_coeffs(n: int, slots: np.ndarray) -> np.ndarray:
    """exact_transforms.rs:180-200 (rc_slots_to_real_coeffs)."""
    src = np.ascontiguousarray(_interleave(np.asarray(slots, dtype=np.complex128)))
    out = np.empty(n, dtype=np.float64)
    call("rc_slots_to_real_coeffs", n, src.ctypes.data, out.ctypes.data)
    return out


def _dense_complex_coeffs_to_slots(n: int, coeffs: np.ndarray) -> np.ndarray:
    """exact_transforms.rs:210-229 (rc_complex_coeffs_to_slots)."""
    src = np.ascontiguousarray(_interleave(np.asarray(coeffs, dtype=np.complex128)))
    out = np.empty(n, dtype=np.float64)
    call("rc_complex_coeffs_to_slots", n, src.ctypes.data, out.ctypes.data)
    return out[0::2] + 1j * out[1::2]


def _validate_active_slots(ctx: RnsCkksContext, active_slots: int) -> None:
    """exact_transforms.rs:119-133."""
    if active_slots == 0:
        raise BootstrapError("active_slots must be positive")
    if active_slots & (active_slots - 1):
        raise BootstrapError("active_slots must be a power of two")
    if active_slots > ctx.num_slots():
        raise BootstrapError(
            f"active_slots cannot exceed the CKKS slot count {ctx.num_slots()}; got {active_slots}")


def coeff_to_slot_matrix(n: int, active_slots: int) -> np.ndarray:
    """exact_transforms.rs:21-36 for ring degree n: column c = the first active_slots slots of the polynomial
    whose coefficient c * stride is 1 (expand_sparse_compressed_coeffs of the c-th real basis vector)."""
    stride = (n // 2) // active_slots
    cols = []
    for column in range(active_slots):
        coeffs = np.zeros(n, dtype=np.complex128)
        coeffs[column * stride] = 1.0
        cols.append(_dense_complex_coeffs_to_slots(n, coeffs)[:active_slots])
    return np.array(cols).T.copy()


def slot_to_coeff_matrix(n: int, active_slots: int) -> np.ndarray:
    """exact_transforms.rs:38-53 for ring degree n: column c = the compressed coefficients
    (c_{i*stride} + i c_{(i+a)*stride}) of the c-th slot basis vector repeated over all slots."""
    slots = n // 2
    stride = slots // active_slots
    cols = []
    for column in range(active_slots):
        full = np.zeros(slots, dtype=np.complex128)
        full[column::active_slots] = 1.0
        rc = _dense_slots_to_real_coeffs(n, full)
        idx = np.arange(active_slots) * stride
        cols.append(rc[idx] + 1j * rc[idx + active_slots * stride])
    return np.array(cols).T.copy()


@dataclass
class DenseCoeffToSlotMatrices:
    """exact_transforms.rs:7-13."""
    upper_from_slots: np.ndarray
    upper_from_conjugates: np.ndarray
    lower_from_slots: np.ndarray
    lower_from_conjugates: np.ndarray


@dataclass
class DenseSlotToCoeffMatrices:
    """exact_transforms.rs:15-19."""
    slots_from_upper: np.ndarray
    slots_from_lower: np.ndarray


def _times_i(z: np.ndarray) -> np.ndarray:
    """num-complex (0 + 1i) * z: (0*re - 1*im) + (0*im + 1*re)i."""
    return (0.0 * z.real - 1.0 * z.imag) + 1j * (0.0 * z.imag + 1.0 * z.real)


def dense_coeff_to_slot_matrices(n: int) -> DenseCoeffToSlotMatrices:
    """exact_transforms.rs:55-88 for ring degree n."""
    s = n // 2
    mats = [np.zeros((s, s), dtype=np.complex128) for _ in range(4)]
    for column in range(s):
        basis = np.zeros(s, dtype=np.complex128)
        basis[column] = 1.0
        real = _dense_slots_to_real_coeffs(n, basis).astype(np.complex128)
        basis[column] = 1j
        imag = _times_i(_dense_slots_to_real_coeffs(n, basis).astype(np.complex128))
        ru, rl, iu, il = real[:s], real[s:], imag[:s], imag[s:]
        mats[0][:, column] = (ru - iu) * 0.5
        mats[1][:, column] = (ru + iu) * 0.5
        mats[2][:, column] = (rl - il) * 0.5
        mats[3][:, column] = (rl + il) * 0.5
    return DenseCoeffToSlotMatrices(*mats)


def dense_slot_to_coeff_matrices(n: int) -> DenseSlotToCoeffMatrices:
    """exact_transforms.rs:90-117 for ring degree n."""
    s = n // 2
    fu = np.zeros((s, s), dtype=np.complex128)
    fl = np.zeros((s, s), dtype=np.complex128)
    for column in range(s):
        c = np.zeros(n, dtype=np.complex128)
        c[column] = 1.0
        fu[:, column] = _dense_complex_coeffs_to_slots(n, c)
        c = np.zeros(n, dtype=np.complex128)
        c[column + s] = 1.0
        fl[:, column] = _dense_complex_coeffs_to_slots(n, c)
    return DenseSlotToCoeffMatrices(fu, fl)


def exact_coeff_to_slot_matrix(ctx: RnsCkksContext, active_slots: int) -> np.ndarray:
    """exact_transforms.rs:21-36."""
    _validate_active_slots(ctx, active_slots)
    return coeff_to_slot_matrix(ctx.params.poly_degree, active_slots)


def exact_slot_to_coeff_matrix(ctx: RnsCkksContext, active_slots: int) -> np.ndarray:
    """exact_transforms.rs:38-53."""
    _validate_active_slots(ctx, active_slots)
    return slot_to_coeff_matrix(ctx.params.poly_degree, active_slots)


def exact_dense_coeff_to_slot_matrices(ctx: RnsCkksContext) -> DenseCoeffToSlotMatrices:
    """exact_transforms.rs:55-88."""
    return dense_coeff_to_slot_matrices(ctx.params.poly_degree)


def exact_dense_slot_to_coeff_matrices(ctx: RnsCkksContext) -> DenseSlotToCoeffMatrices:
    """exact_transforms.rs:90-117."""
    return dense_slot_to_coeff_matrices(ctx.params.poly_degree)


def _identity(d: int) -> np.ndarray:
    return np.eye(d, dtype=np.complex128)


def _validate_transform_matrix(matrix, expected: int, stage: str) -> None:
    """coeff_to_slot.rs:345-367 / slot_to_coeff.rs:298-320."""
    if len(matrix) == 0:
        raise BootstrapError(f"{stage} transform matrix cannot be empty")
    if len(matrix) != expected:
        raise BootstrapError(f"{stage} transform matrix dimension {len(matrix)} did not match plan dimension "
                             f"{expected}")
    for i, row in enumerate(matrix):
        if len(row) != expected:
            raise BootstrapError(f"{stage} transform row {i} had length {len(row)}, expected {expected}")


# --------------------------------------------------------------------------------------------------------
# coeff_to_slot.rs / slot_to_coeff.rs
# --------------------------------------------------------------------------------------------------------

@dataclass
class _TransformPlan:
    """CoeffToSlotPlan / SlotToCoeffPlan (coeff_to_slot.rs:28-59, slot_to_coeff.rs:28-59)."""
    bootstrap: BootstrapParameters
    transform_dimension: int
    rotation_steps: List[int]

    @classmethod
    def new(cls, bootstrap: BootstrapParameters):
        d = bootstrap.active_slots
        return cls(bootstrap, d, A.diagonal_transform_bsgs_rotation_steps(d))

    @classmethod
    def from_ciphertext(cls, ctx: RnsCkksContext, ciphertext: RnsCiphertext, active_slots: int):
        return cls.new(BootstrapParameters.from_ciphertext(ctx, ciphertext, active_slots))


class CoeffToSlotPlan(_TransformPlan):
    STAGE = "CoeffToSlot"


class SlotToCoeffPlan(_TransformPlan):
    STAGE = "SlotToCoeff"


@dataclass
class _Runtime:
    """CoeffToSlotRuntime / SlotToCoeffRuntime (coeff_to_slot.rs:193-219, slot_to_coeff.rs:171-194)."""
    plan: _TransformPlan
    ciphertext_level: int
    ciphertext_scale_bits: int

    @classmethod
    def new(cls, plan: _TransformPlan, ciphertext: RnsCiphertext):
        if ciphertext.level != plan.bootstrap.ciphertext_level:
            raise BootstrapError(f"ciphertext level {ciphertext.level} did not match {plan.STAGE} plan level "
                                 f"{plan.bootstrap.ciphertext_level}")
        return cls(plan, ciphertext.level, ciphertext.scale_bits)


CoeffToSlotRuntime = _Runtime
SlotToCoeffRuntime = _Runtime


@dataclass
class _TransformPrecomputed:
    """CoeffToSlotPrecomputed / SlotToCoeffPrecomputed (coeff_to_slot.rs:62-125, slot_to_coeff.rs:62-124)."""
    plan: _TransformPlan
    diagonals: A.DiagonalTransformPlaintexts

    @classmethod
    def new(cls, ctx: RnsCkksContext, plan: _TransformPlan, matrix, ciphertext_scale_bits: int):
        _validate_transform_matrix(matrix, plan.transform_dimension, plan.STAGE)
        return cls(plan, A.pack_diagonal_transform_plaintexts(ctx, matrix, plan.bootstrap.ciphertext_level,
                                                              ciphertext_scale_bits))

    @classmethod
    def identity(cls, ctx: RnsCkksContext, plan: _TransformPlan, ciphertext_scale_bits: int):
        return cls.new(ctx, plan, _identity(plan.transform_dimension), ciphertext_scale_bits)


class CoeffToSlotPrecomputed(_TransformPrecomputed):
    @classmethod
    def exact(cls, ctx: RnsCkksContext, plan: CoeffToSlotPlan, ciphertext_scale_bits: int):
        return cls.new(ctx, plan, exact_coeff_to_slot_matrix(ctx, plan.transform_dimension), ciphertext_scale_bits)


class SlotToCoeffPrecomputed(_TransformPrecomputed):
    @classmethod
    def exact(cls, ctx: RnsCkksContext, plan: SlotToCoeffPlan, ciphertext_scale_bits: int):
        return cls.new(ctx, plan, exact_slot_to_coeff_matrix(ctx, plan.transform_dimension), ciphertext_scale_bits)


@dataclass
class DenseCoeffToSlotPrecomputed:
    """coeff_to_slot.rs:68-74,127-191."""
    plan: CoeffToSlotPlan
    upper_from_slots: A.DiagonalTransformPlaintexts
    upper_from_conjugates: A.DiagonalTransformPlaintexts
    lower_from_slots: A.DiagonalTransformPlaintexts
    lower_from_conjugates: A.DiagonalTransformPlaintexts

    @classmethod
    def new(cls, ctx: RnsCkksContext, plan: CoeffToSlotPlan, upper_from_slots, upper_from_conjugates,
            lower_from_slots, lower_from_conjugates, ciphertext_scale_bits: int):
        mats = (upper_from_slots, upper_from_conjugates, lower_from_slots, lower_from_conjugates)
        for m in mats:
            _validate_transform_matrix(m, ctx.num_slots(), "CoeffToSlot")
        lvl = plan.bootstrap.ciphertext_level
        return cls(plan, *[A.pack_diagonal_transform_plaintexts(ctx, m, lvl, ciphertext_scale_bits) for m in mats])

    @classmethod
    def exact(cls, ctx: RnsCkksContext, plan: CoeffToSlotPlan, ciphertext_scale_bits: int):
        m = exact_dense_coeff_to_slot_matrices(ctx)
        return cls.new(ctx, plan, m.upper_from_slots, m.upper_from_conjugates, m.lower_from_slots,
                       m.lower_from_conjugates, ciphertext_scale_bits)


@dataclass
class DenseSlotToCoeffPrecomputed:
    """slot_to_coeff.rs:67-72,124-168."""
    plan: SlotToCoeffPlan
    slots_from_upper: A.DiagonalTransformPlaintexts
    slots_from_lower: A.DiagonalTransformPlaintexts

    @classmethod
    def new(cls, ctx: RnsCkksContext, plan: SlotToCoeffPlan, slots_from_upper, slots_from_lower,
            ciphertext_scale_bits: int):
        for m in (slots_from_upper, slots_from_lower):
            _validate_transform_matrix(m, ctx.num_slots(), "SlotToCoeff")
        lvl = plan.bootstrap.ciphertext_level
        return cls(plan, A.pack_diagonal_transform_plaintexts(ctx, slots_from_upper, lvl, ciphertext_scale_bits),
                   A.pack_diagonal_transform_plaintexts(ctx, slots_from_lower, lvl, ciphertext_scale_bits))

    @classmethod
    def exact(cls, ctx: RnsCkksContext, plan: SlotToCoeffPlan, ciphertext_scale_bits: int):
        m = exact_dense_slot_to_coeff_matrices(ctx)
        return cls.new(ctx, plan, m.slots_from_upper, m.slots_from_lower, ciphertext_scale_bits)


def _transform_batch(ctx, cts: Sequence[RnsCiphertext], pre: _TransformPrecomputed,
                     rotation_keys: A.DiagonalTransformRotationKeys) -> List[RnsCiphertext]:
    for ct in cts:
        _Runtime.new(pre.plan, ct)
    return A.apply_diagonal_linear_transform_native(ctx, list(cts), pre.diagonals, rotation_keys)


def coeff_to_slot(ctx: RnsCkksContext, ciphertext: RnsCiphertext, precomputed: CoeffToSlotPrecomputed,
                  rotation_keys: A.DiagonalTransformRotationKeys) -> RnsCiphertext:
    """coeff_to_slot.rs:221-233."""
    return _transform_batch(ctx, [ciphertext], precomputed, rotation_keys)[0]


def coeff_to_slot_batch(ctx, ciphertexts, precomputed, rotation_keys) -> List[RnsCiphertext]:
    """`coeff_to_slot` of many ciphertexts with one set of diagonals: every BSGS step is one batched call."""
    return _transform_batch(ctx, ciphertexts, precomputed, rotation_keys)


def slot_to_coeff(ctx: RnsCkksContext, ciphertext: RnsCiphertext, precomputed: SlotToCoeffPrecomputed,
                  rotation_keys: A.DiagonalTransformRotationKeys) -> RnsCiphertext:
    """slot_to_coeff.rs:196-209."""
    return _transform_batch(ctx, [ciphertext], precomputed, rotation_keys)[0]


def slot_to_coeff_batch(ctx, ciphertexts, precomputed, rotation_keys) -> List[RnsCiphertext]:
    return _transform_batch(ctx, ciphertexts, precomputed, rotation_keys)


def _check_pair(a: RnsCiphertext, b: RnsCiphertext, what_a: str, what_b: str) -> None:
    if a.level != b.level:
        raise BootstrapError(f"{what_a} level {a.level} did not match {what_b} level {b.level}")
    if a.scale_bits != b.scale_bits:
        raise BootstrapError(f"{what_a} scale {a.scale_bits} did not match {what_b} scale {b.scale_bits}")


def coeff_to_slot_dense(ctx: RnsCkksContext, ciphertext: RnsCiphertext, conjugated_ciphertext: RnsCiphertext,
                        precomputed: DenseCoeffToSlotPrecomputed,
                        rotation_keys: A.DiagonalTransformRotationKeys) -> Tuple[RnsCiphertext, RnsCiphertext]:
    """coeff_to_slot.rs:262-307 with apply_dense_branch (332-343)."""
    _Runtime.new(precomputed.plan, ciphertext)
    _check_pair(conjugated_ciphertext, ciphertext, "conjugated ciphertext", "CoeffToSlot input")
    def lt(ctx_, ct, diags, keys):
        return A.apply_diagonal_linear_transform_native(ctx_, [ct], diags, keys)[0]

    def branch(from_slots, from_conj):
        return lt(ctx, ciphertext, from_slots, rotation_keys).add(
            lt(ctx, conjugated_ciphertext, from_conj, rotation_keys))

    upper = branch(precomputed.upper_from_slots, precomputed.upper_from_conjugates)
    lower = branch(precomputed.lower_from_slots, precomputed.lower_from_conjugates)
    return upper, lower


def slot_to_coeff_dense(ctx: RnsCkksContext, upper: RnsCiphertext, lower: RnsCiphertext,
                        precomputed: DenseSlotToCoeffPrecomputed,
                        rotation_keys: A.DiagonalTransformRotationKeys) -> RnsCiphertext:
    """slot_to_coeff.rs:243-280."""
    _Runtime.new(precomputed.plan, upper)
    _check_pair(lower, upper, "lower dense SlotToCoeff ciphertext", "upper")
    def lt(ctx_, ct, diags, keys):
        return A.apply_diagonal_linear_transform_native(ctx_, [ct], diags, keys)[0]
    return lt(ctx, upper, precomputed.slots_from_upper, rotation_keys).add(
        lt(ctx, lower, precomputed.slots_from_lower, rotation_keys))


# --------------------------------------------------------------------------------------------------------
# eval_mod.rs
# --------------------------------------------------------------------------------------------------------

@dataclass
class EvalModPlan:
    """eval_mod.rs:20-80."""
    bootstrap: BootstrapParameters
    input_scale: float
    sine_scale: float
    polynomial_degree: int

    @staticmethod
    def new(bootstrap: BootstrapParameters, input_scale: float, sine_scale: float,
            polynomial_degree: int) -> "EvalModPlan":
        if input_scale <= 0.0:
            raise BootstrapError("EvalMod input_scale must be positive")
        if sine_scale == 0.0:
            raise BootstrapError("EvalMod sine_scale must be non-zero")
        if polynomial_degree == 0:
            raise BootstrapError("EvalMod polynomial_degree must be positive")
        if polynomial_degree % 2 == 0:
            raise BootstrapError("EvalMod polynomial_degree must be odd for a sine approximation")
        return EvalModPlan(bootstrap, input_scale, sine_scale, polynomial_degree)

    @staticmethod
    def from_ciphertext(ctx, ciphertext, active_slots, input_scale, sine_scale, polynomial_degree) -> "EvalModPlan":
        return EvalModPlan.new(BootstrapParameters.from_ciphertext(ctx, ciphertext, active_slots), input_scale,
                               sine_scale, polynomial_degree)

    def polynomial_term_count(self) -> int:
        return self.polynomial_degree + 1

    def required_levels(self) -> List[int]:
        return A.paterson_stockmeyer_required_levels(self.bootstrap.ciphertext_level, self.polynomial_term_count())


def _powi(x: float, e: int) -> float:
    """f64::powi for a small positive exponent (exponentiation by squaring)."""
    r, b = 1.0, x
    while e:
        if e & 1:
            r *= b
        b *= b
        e >>= 1
    return r


def sine_taylor_coefficients(polynomial_degree: int, sine_scale: float) -> List[float]:
    """eval_mod.rs:158-173: c_d = (-1)^((d-1)/2) s^d / d! for odd d."""
    if polynomial_degree <= 0:
        raise BootstrapError("polynomial_degree must be positive")
    if polynomial_degree % 2 != 1:
        raise BootstrapError("polynomial_degree must be odd")
    out = [0.0] * (polynomial_degree + 1)
    for d in range(1, polynomial_degree + 1, 2):
        sign = 1.0 if ((d - 1) // 2) % 2 == 0 else -1.0
        fact = 1.0
        for f in range(1, d + 1):
            fact *= float(f)
        out[d] = sign * _powi(sine_scale, d) / fact
    return out


def _validate_sine_coefficients(polynomial_degree: int, coefficients: Sequence[float]) -> None:
    """eval_mod.rs:175-193."""
    if len(coefficients) != polynomial_degree + 1:
        raise BootstrapError(f"EvalMod coefficient vector length {len(coefficients)} did not match polynomial "
                             f"degree {polynomial_degree}")
    for d in range(2, polynomial_degree + 1, 2):
        if coefficients[d] != 0.0:
            raise BootstrapError(f"EvalMod sine approximation requires zero coefficient for even degree {d}")


@dataclass
class EvalModPrecomputed:
    """eval_mod.rs:84-101."""
    plan: EvalModPlan
    coefficients: List[float]

    @staticmethod
    def new(plan: EvalModPlan, coefficients: Sequence[float]) -> "EvalModPrecomputed":
        _validate_sine_coefficients(plan.polynomial_degree, coefficients)
        return EvalModPrecomputed(plan, [float(c) for c in coefficients])

    @staticmethod
    def sine_taylor(plan: EvalModPlan) -> "EvalModPrecomputed":
        return EvalModPrecomputed.new(plan, sine_taylor_coefficients(plan.polynomial_degree, plan.sine_scale))


@dataclass
class EvalModRuntime:
    """eval_mod.rs:104-131."""
    ciphertext_level: int
    ciphertext_scale_bits: int
    required_relinearization_levels: List[int]

    @staticmethod
    def new(plan: EvalModPlan, ciphertext: RnsCiphertext) -> "EvalModRuntime":
        if ciphertext.level != plan.bootstrap.ciphertext_level:
            raise BootstrapError(f"ciphertext level {ciphertext.level} did not match EvalMod plan level "
                                 f"{plan.bootstrap.ciphertext_level}")
        return EvalModRuntime(ciphertext.level, ciphertext.scale_bits, plan.required_levels())


def eval_mod_batch(ctx: RnsCkksContext, ciphertexts: Sequence[RnsCiphertext], precomputed: EvalModPrecomputed,
                   relinearization_keys: Dict[int, RnsKeySwitchingKey], plains=None) -> List[RnsCiphertext]:
    """eval_mod (eval_mod.rs:133-156) of many ciphertexts: each Paterson-Stockmeyer product is one batched call."""
    if not ciphertexts:
        return []
    for ct in ciphertexts:
        runtime = EvalModRuntime.new(precomputed.plan, ct)
    for level in runtime.required_relinearization_levels:
        if level not in relinearization_keys:
            raise BootstrapError(f"missing EvalMod relinearization key at level {level}")
    return A.paterson_stockmeyer_eval_batch(ctx, list(ciphertexts), precomputed.coefficients, relinearization_keys,
                                            plains)


def eval_mod(ctx: RnsCkksContext, ciphertext: RnsCiphertext, precomputed: EvalModPrecomputed,
             relinearization_keys: Dict[int, RnsKeySwitchingKey]) -> RnsCiphertext:
    """eval_mod.rs:133-156."""
    return eval_mod_batch(ctx, [ciphertext], precomputed, relinearization_keys)[0]


# --------------------------------------------------------------------------------------------------------
# keys.rs
# --------------------------------------------------------------------------------------------------------

@dataclass
class BootstrapKeySet:
    """keys.rs:6-12; the constructors generate the keys on the GPU."""
    coeff_to_slot_rotation_keys: Dict[int, RnsRotationKey] = field(default_factory=dict)
    slot_to_coeff_rotation_keys: Dict[int, RnsRotationKey] = field(default_factory=dict)
    eval_mod_relinearization_keys: Dict[int, RnsKeySwitchingKey] = field(default_factory=dict)
    conjugation_key: Optional[RnsRotationKey] = None

    @staticmethod
    def empty() -> "BootstrapKeySet":
        return BootstrapKeySet()

    @staticmethod
    def for_eval_mod(ctx, key_pair, ciphertext_level: int, polynomial_term_count: int) -> "BootstrapKeySet":
        """keys.rs:19-36."""
        return BootstrapKeySet(eval_mod_relinearization_keys=A.generate_paterson_stockmeyer_relinearization_keys(
            ctx, key_pair.secret_key, key_pair.public_key, ciphertext_level, polynomial_term_count))

    @staticmethod
    def for_coeff_to_slot(ctx, key_pair, ciphertext_level: int, active_slots: int) -> "BootstrapKeySet":
        """keys.rs:38-55."""
        return BootstrapKeySet(coeff_to_slot_rotation_keys=A.generate_diagonal_transform_rotation_keys(
            ctx, key_pair.secret_key, key_pair.public_key, ciphertext_level, active_slots).by_step)

    @staticmethod
    def for_slot_to_coeff(ctx, key_pair, ciphertext_level: int, active_slots: int) -> "BootstrapKeySet":
        """keys.rs:57-74."""
        return BootstrapKeySet(slot_to_coeff_rotation_keys=A.generate_diagonal_transform_rotation_keys(
            ctx, key_pair.secret_key, key_pair.public_key, ciphertext_level, active_slots).by_step)

    @staticmethod
    def for_dense_coeff_to_slot(ctx, key_pair, ciphertext_level: int) -> "BootstrapKeySet":
        """keys.rs:76-97."""
        rot = A.generate_diagonal_transform_rotation_keys(ctx, key_pair.secret_key, key_pair.public_key,
                                                          ciphertext_level, ctx.num_slots())
        conj = ctx.generate_conjugation_key_at_level(key_pair.secret_key, key_pair.public_key, ciphertext_level)
        return BootstrapKeySet(coeff_to_slot_rotation_keys=rot.by_step, conjugation_key=conj)

    @staticmethod
    def for_dense_slot_to_coeff(ctx, key_pair, ciphertext_level: int) -> "BootstrapKeySet":
        """keys.rs:99-115."""
        return BootstrapKeySet(slot_to_coeff_rotation_keys=A.generate_diagonal_transform_rotation_keys(
            ctx, key_pair.secret_key, key_pair.public_key, ciphertext_level, ctx.num_slots()).by_step)


# --------------------------------------------------------------------------------------------------------
# the *_exact / *_identity entry points (keys generated per call, as in the reference)
# --------------------------------------------------------------------------------------------------------

def _rk(by_step: Dict[int, RnsRotationKey]) -> A.DiagonalTransformRotationKeys:
    return A.DiagonalTransformRotationKeys(by_step)


def coeff_to_slot_exact(ctx, ciphertext, key_pair, active_slots: int) -> RnsCiphertext:
    """coeff_to_slot.rs:235-249."""
    plan = CoeffToSlotPlan.from_ciphertext(ctx, ciphertext, active_slots)
    pre = CoeffToSlotPrecomputed.exact(ctx, plan, ciphertext.scale_bits)
    keys = BootstrapKeySet.for_coeff_to_slot(ctx, key_pair, ciphertext.level, active_slots)
    return coeff_to_slot(ctx, ciphertext, pre, _rk(keys.coeff_to_slot_rotation_keys))


def coeff_to_slot_identity(ctx, ciphertext, key_pair, active_slots: int) -> RnsCiphertext:
    """coeff_to_slot.rs:251-265."""
    plan = CoeffToSlotPlan.from_ciphertext(ctx, ciphertext, active_slots)
    pre = CoeffToSlotPrecomputed.identity(ctx, plan, ciphertext.scale_bits)
    keys = BootstrapKeySet.for_coeff_to_slot(ctx, key_pair, ciphertext.level, active_slots)
    return coeff_to_slot(ctx, ciphertext, pre, _rk(keys.coeff_to_slot_rotation_keys))


def coeff_to_slot_dense_exact(ctx, ciphertext, key_pair) -> Tuple[RnsCiphertext, RnsCiphertext]:
    """coeff_to_slot.rs:309-330."""
    keys = BootstrapKeySet.for_dense_coeff_to_slot(ctx, key_pair, ciphertext.level)
    if keys.conjugation_key is None:
        raise BootstrapError("dense CoeffToSlot key scaffold did not include a conjugation key")
    conj = ctx.conjugate(ciphertext, keys.conjugation_key)
    plan = CoeffToSlotPlan.from_ciphertext(ctx, ciphertext, ctx.num_slots())
    pre = DenseCoeffToSlotPrecomputed.exact(ctx, plan, ciphertext.scale_bits)
    return coeff_to_slot_dense(ctx, ciphertext, conj, pre, _rk(keys.coeff_to_slot_rotation_keys))


def slot_to_coeff_exact(ctx, ciphertext, key_pair, active_slots: int) -> RnsCiphertext:
    """slot_to_coeff.rs:211-225."""
    plan = SlotToCoeffPlan.from_ciphertext(ctx, ciphertext, active_slots)
    pre = SlotToCoeffPrecomputed.exact(ctx, plan, ciphertext.scale_bits)
    keys = BootstrapKeySet.for_slot_to_coeff(ctx, key_pair, ciphertext.level, active_slots)
    return slot_to_coeff(ctx, ciphertext, pre, _rk(keys.slot_to_coeff_rotation_keys))


def slot_to_coeff_identity(ctx, ciphertext, key_pair, active_slots: int) -> RnsCiphertext:
    """slot_to_coeff.rs:227-241."""
    plan = SlotToCoeffPlan.from_ciphertext(ctx, ciphertext, active_slots)
    pre = SlotToCoeffPrecomputed.identity(ctx, plan, ciphertext.scale_bits)
    keys = BootstrapKeySet.for_slot_to_coeff(ctx, key_pair, ciphertext.level, active_slots)
    return slot_to_coeff(ctx, ciphertext, pre, _rk(keys.slot_to_coeff_rotation_keys))


def slot_to_coeff_dense_exact(ctx, upper, lower, key_pair) -> RnsCiphertext:
    """slot_to_coeff.rs:282-296."""
    plan = SlotToCoeffPlan.from_ciphertext(ctx, upper, ctx.num_slots())
    pre = DenseSlotToCoeffPrecomputed.exact(ctx, plan, upper.scale_bits)
    keys = BootstrapKeySet.for_dense_slot_to_coeff(ctx, key_pair, upper.level)
    return slot_to_coeff_dense(ctx, upper, lower, pre, _rk(keys.slot_to_coeff_rotation_keys))


def _eval_mod_exact(ctx, ciphertext, key_pair, active_slots, sine_scale, polynomial_degree) -> RnsCiphertext:
    """roundtrip.rs:121-147."""
    plan = EvalModPlan.from_ciphertext(ctx, ciphertext, active_slots, 1.0, sine_scale, polynomial_degree)
    pre = EvalModPrecomputed.sine_taylor(plan)
    keys = BootstrapKeySet.for_eval_mod(ctx, key_pair, ciphertext.level, len(pre.coefficients))
    return eval_mod(ctx, ciphertext, pre, keys.eval_mod_relinearization_keys)


# --------------------------------------------------------------------------------------------------------
# roundtrip.rs
# --------------------------------------------------------------------------------------------------------

def bootstrap_identity_roundtrip_from_mod_raise(ctx, raised: ModRaisedCiphertext, key_pair,
                                                active_slots: int) -> RnsCiphertext:
    """roundtrip.rs:64-75."""
    projected = raised.project_to_q_ciphertext()
    slots = coeff_to_slot_identity(ctx, projected, key_pair, active_slots)
    return slot_to_coeff_identity(ctx, slots, key_pair, active_slots)


def bootstrap_identity_roundtrip(ctx, ciphertext, key_pair, active_slots: int) -> RnsCiphertext:
    """roundtrip.rs:16-24."""
    return bootstrap_identity_roundtrip_from_mod_raise(ctx, mod_raise(ctx, ciphertext), key_pair, active_slots)


def bootstrap_exact_sparse_eval_mod_roundtrip_from_mod_raise(ctx, raised: ModRaisedCiphertext, key_pair,
                                                             active_slots: int, sine_scale: float,
                                                             polynomial_degree: int) -> RnsCiphertext:
    """roundtrip.rs:77-99."""
    projected = raised.project_to_q_ciphertext()
    slots = coeff_to_slot_exact(ctx, projected, key_pair, active_slots)
    evaluated = _eval_mod_exact(ctx, slots, key_pair, active_slots, sine_scale, polynomial_degree)
    return slot_to_coeff_exact(ctx, evaluated, key_pair, active_slots)


def bootstrap_exact_sparse_eval_mod_roundtrip(ctx, ciphertext, key_pair, active_slots: int, sine_scale: float,
                                              polynomial_degree: int) -> RnsCiphertext:
    """roundtrip.rs:26-44."""
    return bootstrap_exact_sparse_eval_mod_roundtrip_from_mod_raise(
        ctx, mod_raise(ctx, ciphertext), key_pair, active_slots, sine_scale, polynomial_degree)


def bootstrap_exact_dense_eval_mod_roundtrip_from_mod_raise(ctx, raised: ModRaisedCiphertext, key_pair,
                                                            sine_scale: float,
                                                            polynomial_degree: int) -> RnsCiphertext:
    """roundtrip.rs:101-119 with eval_mod_exact_pair (149-175)."""
    projected = raised.project_to_q_ciphertext()
    upper, lower = coeff_to_slot_dense_exact(ctx, projected, key_pair)
    eu = _eval_mod_exact(ctx, upper, key_pair, ctx.num_slots(), sine_scale, polynomial_degree)
    el = _eval_mod_exact(ctx, lower, key_pair, ctx.num_slots(), sine_scale, polynomial_degree)
    return slot_to_coeff_dense_exact(ctx, eu, el, key_pair)


def bootstrap_exact_dense_eval_mod_roundtrip(ctx, ciphertext, key_pair, sine_scale: float,
                                             polynomial_degree: int) -> RnsCiphertext:
    """roundtrip.rs:46-62."""
    return bootstrap_exact_dense_eval_mod_roundtrip_from_mod_raise(ctx, mod_raise(ctx, ciphertext), key_pair,
                                                                   sine_scale, polynomial_degree)


# --------------------------------------------------------------------------------------------------------
# prepared form: diagonals and keys built once, many ciphertexts per call
# --------------------------------------------------------------------------------------------------------

class SparseBootstrapper:
    """`bootstrap_exact_sparse_eval_mod_roundtrip` with its precomputation hoisted: the CoeffToSlot and
    SlotToCoeff diagonals, the sine coefficients and the key set (rotation keys at the two transform levels,
    relinearization keys at the EvalMod levels) are built once for ciphertexts at `ciphertext_level` and
    `scale_bits`; `run_batch` takes each stage of many ciphertexts as batched calls.  Each result equals the
    reference routine's for the same keys."""

    def __init__(self, ctx: RnsCkksContext, key_pair, ciphertext_level: int, scale_bits: int, active_slots: int,
                 sine_scale: float, polynomial_degree: int, keys: Optional[BootstrapKeySet] = None):
        self.ctx, self.active_slots = ctx, active_slots
        self.level, self.scale_bits = ciphertext_level, scale_bits
        b = BootstrapParameters.new(ctx, ciphertext_level, active_slots)
        c2s_plan = CoeffToSlotPlan.new(b)
        self.c2s = CoeffToSlotPrecomputed.exact(ctx, c2s_plan, scale_bits)
        # CoeffToSlot ends with one rescale
        self.em_level = ciphertext_level - 1
        em_plan = EvalModPlan.new(BootstrapParameters.new(ctx, self.em_level, active_slots), 1.0, sine_scale,
                                  polynomial_degree)
        self.em = EvalModPrecomputed.sine_taylor(em_plan)
        self.s2c_level = self.em_level - (len(em_plan.required_levels()))
        self.plains = A.constant_plaintext_cache(ctx)
        if keys is None:
            keys = BootstrapKeySet(
                coeff_to_slot_rotation_keys=BootstrapKeySet.for_coeff_to_slot(
                    ctx, key_pair, ciphertext_level, active_slots).coeff_to_slot_rotation_keys,
                eval_mod_relinearization_keys=BootstrapKeySet.for_eval_mod(
                    ctx, key_pair, self.em_level, em_plan.polynomial_term_count()).eval_mod_relinearization_keys,
                slot_to_coeff_rotation_keys=BootstrapKeySet.for_slot_to_coeff(
                    ctx, key_pair, self.s2c_level, active_slots).slot_to_coeff_rotation_keys)
        self.keys = keys
        self._s2c: Dict[Tuple[int, int], SlotToCoeffPrecomputed] = {}

    def _s2c_for(self, level: int, scale_bits: int) -> SlotToCoeffPrecomputed:
        key = (level, scale_bits)
        if key not in self._s2c:
            plan = SlotToCoeffPlan.new(BootstrapParameters.new(self.ctx, level, self.active_slots))
            self._s2c[key] = SlotToCoeffPrecomputed.exact(self.ctx, plan, scale_bits)
        return self._s2c[key]

    def run_batch(self, ciphertexts: Sequence[RnsCiphertext]) -> List[RnsCiphertext]:
        ctx = self.ctx
        raised = mod_raise_batch(ctx, ciphertexts)
        projected = [r.project_to_q_ciphertext() for r in raised]
        slots = coeff_to_slot_batch(ctx, projected, self.c2s, _rk(self.keys.coeff_to_slot_rotation_keys))
        evaluated = eval_mod_batch(ctx, slots, self.em, self.keys.eval_mod_relinearization_keys, self.plains)
        s2c = self._s2c_for(evaluated[0].level, evaluated[0].scale_bits)
        return slot_to_coeff_batch(ctx, evaluated, s2c, _rk(self.keys.slot_to_coeff_rotation_keys))

    def run(self, ciphertext: RnsCiphertext) -> RnsCiphertext:
        return self.run_batch([ciphertext])[0]
