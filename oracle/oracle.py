"""CPU ORACLE (test infrastructure only) — Python side.

ctypes bindings to `oracle/_build/liboracle.so` (the C restatement in
`oracle/oracle.c`) plus the reference's scheme-level compositions that are
plain glue in the reference: encrypt/decrypt (`src/rns/ops.rs:8-52`), key
generation (`src/rns/keys.rs:153-166`, `src/rns/keyswitching.rs:44-128`),
noiseless test keys (`src/rns/tests.rs:36-114`) and the FP64 CKKS encoder and
decoder (`src/rns/encoding.rs:9-88`, `src/math/canonical_embedding.rs:21-79`).

Only tests, the smoke check and the CPU-baseline leg of the benchmark use this
module.  All polynomials are numpy uint64 arrays shaped (limbs, N).
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess
from pathlib import Path
from typing import List, Optional, Sequence

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "liboracle.so"
DECOMP_BITS = 30  # RNS_DECOMP_BITS, src/rns/mod.rs:1


class OrcPlan(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in
                ("modulus", "size", "root", "root_inv", "negacyclic_twiddle", "negacyclic_twiddle_inv", "size_inv")]


_PLAN_ERRORS = {
    1: "NTT size must be a non-zero power of two",
    2: "modulus must be an odd prime larger than 2",
    3: "size must divide modulus - 1",
    4: "2 * size must divide modulus - 1 for negacyclic NTTs",
    5: "primitive_root does not generate a size-th root of unity",
    6: "root is not primitive for the requested size",
    7: "root is not invertible",
    8: "size is not invertible modulo modulus",
    9: "primitive_root does not generate a valid negacyclic twiddle",
    10: "negacyclic twiddle is not invertible",
}


def build() -> Path:
    """Compile the oracle with its Makefile (gcc, no external libraries)."""
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            build()
        L = ctypes.CDLL(str(LIB_PATH))
        P = ctypes.POINTER(OrcPlan)
        u64p = ctypes.POINTER(ctypes.c_uint64)
        i64p = ctypes.POINTER(ctypes.c_int64)
        sz, u64 = ctypes.c_size_t, ctypes.c_uint64
        sig = {
            "orc_set_threads": (None, [ctypes.c_int]),
            "orc_get_threads": (ctypes.c_int, []),
            "orc_ntt_plan_new": (ctypes.c_int, [u64, u64, u64, P]),
            "orc_ntt_forward": (None, [P, u64p]),
            "orc_ntt_inverse": (None, [P, u64p]),
            "orc_poly_add": (None, [u64p, u64p, u64p, sz, u64]),
            "orc_poly_sub": (None, [u64p, u64p, u64p, sz, u64]),
            "orc_poly_mul_naive": (None, [u64p, u64p, u64p, sz, u64]),
            "orc_poly_automorphism": (None, [u64p, u64p, sz, u64, u64]),
            "orc_poly_mul_ntt": (None, [P, u64p, u64p, u64p]),
            "orc_rns_mul_ntt": (None, [P, sz, u64p, u64p, u64p]),
            "orc_rns_add": (None, [P, sz, u64p, u64p, u64p]),
            "orc_rns_sub": (None, [P, sz, u64p, u64p, u64p]),
            "orc_rns_automorphism": (None, [P, sz, u64p, u64p, u64]),
            "orc_tensor": (None, [P, sz, u64p, u64p, u64p, u64p, u64p, u64p, u64p]),
            "orc_rescale_poly": (None, [P, sz, u64p, u64p]),
            "orc_decompose": (None, [P, sz, u64p, sz, sz, i64p, u64p]),
            "orc_lift": (None, [P, sz, P, sz, u64p, u64p]),
            "orc_mod_down": (None, [P, sz, P, sz, u64p, u64p]),
            "orc_num_decomp_digits": (sz, [sz, sz]),
            "orc_modulus_bits": (sz, [u64p, sz]),
            "orc_keyswitch": (None, [P, sz, P, sz, u64p, u64p, sz, u64p, u64p]),
            "orc_relinearize": (None, [P, sz, P, sz, u64p, u64p, u64p, u64p, sz, u64p, u64p]),
            "orc_mult_relinearized": (None, [P, sz, P, sz, u64p, u64p, u64p, u64p, u64p, sz, u64p, u64p]),
            "orc_rotate": (None, [P, sz, P, sz, u64p, u64p, u64, u64p, sz, u64p, u64p]),
            "orc_mul_scalar": (None, [u64p, u64p, sz, u64, u64]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def set_threads(n: int) -> None:
    lib().orc_set_threads(int(n))


def _p(a: np.ndarray):
    assert a.dtype in (np.uint64, np.int64) and a.flags["C_CONTIGUOUS"], (a.dtype, a.flags)
    t = ctypes.c_uint64 if a.dtype == np.uint64 else ctypes.c_int64
    return a.ctypes.data_as(ctypes.POINTER(t))


def _u(x) -> np.ndarray:
    return np.ascontiguousarray(x, dtype=np.uint64)


class Plans:
    """An ordered RNS basis: one NttPlan per prime (`RnsContext`, src/rns/basis.rs:25-112)."""

    def __init__(self, n: int, primes: Sequence, roots: Optional[Sequence[int]] = None):
        if roots is None:  # accept RnsPrime-like objects
            roots = [p.primitive_root for p in primes]
            primes = [p.modulus for p in primes]
        self.n = int(n)
        self.moduli = [int(q) for q in primes]
        self.roots = [int(g) for g in roots]
        self.arr = (OrcPlan * max(1, len(self.moduli)))()
        for i, (q, g) in enumerate(zip(self.moduli, self.roots)):
            err = lib().orc_ntt_plan_new(self.n, q, g, ctypes.byref(self.arr[i]))
            if err:
                raise ValueError(f"invalid RNS prime {q}: {_PLAN_ERRORS[err]}")

    def __len__(self):
        return len(self.moduli)

    def prefix(self, count: int) -> "Plans":
        """`RnsContext::at_level` (basis.rs:87-95)."""
        if count == 0 or count > len(self):
            raise ValueError(f"level_count must be in 1..={len(self)}, got {count}")
        return Plans(self.n, self.moduli[:count], self.roots[:count])

    def concat(self, other: "Plans") -> "Plans":
        return Plans(self.n, self.moduli + other.moduli, self.roots + other.roots)

    @property
    def ptr(self):
        return ctypes.cast(self.arr, ctypes.POINTER(OrcPlan))

    def plan(self, i: int) -> OrcPlan:
        return self.arr[i]

    def total_modulus(self) -> int:
        return math.prod(self.moduli)

    def total_modulus_bits(self) -> int:
        return self.total_modulus().bit_length()


# ----------------------------------------------------------------------------------
# single-limb primitives
# ----------------------------------------------------------------------------------

def ntt_forward(plans: Plans, i: int, values) -> np.ndarray:
    v = _u(values).copy()
    lib().orc_ntt_forward(ctypes.byref(plans.arr[i]), _p(v))
    return v


def ntt_inverse(plans: Plans, i: int, values) -> np.ndarray:
    v = _u(values).copy()
    lib().orc_ntt_inverse(ctypes.byref(plans.arr[i]), _p(v))
    return v


def poly_mul_naive(a, b, q: int) -> np.ndarray:
    a, b = _u(a), _u(b)
    out = np.zeros_like(a)
    lib().orc_poly_mul_naive(_p(a), _p(b), _p(out), a.size, q)
    return out


def poly_mul_ntt(plans: Plans, i: int, a, b) -> np.ndarray:
    a, b = _u(a), _u(b)
    out = np.zeros_like(a)
    lib().orc_poly_mul_ntt(ctypes.byref(plans.arr[i]), _p(a), _p(b), _p(out))
    return out


def poly_automorphism(a, q: int, g: int) -> np.ndarray:
    a = _u(a)
    out = np.zeros_like(a)
    lib().orc_poly_automorphism(_p(a), _p(out), a.size, q, g)
    return out


# ----------------------------------------------------------------------------------
# RNS polynomials (limbs, N)
# ----------------------------------------------------------------------------------

def rns_mul(plans: Plans, a, b) -> np.ndarray:
    a, b = _u(a), _u(b)
    out = np.zeros_like(a)
    lib().orc_rns_mul_ntt(plans.ptr, a.shape[0], _p(a), _p(b), _p(out))
    return out


def rns_add(plans: Plans, a, b) -> np.ndarray:
    a, b = _u(a), _u(b)
    out = np.zeros_like(a)
    lib().orc_rns_add(plans.ptr, a.shape[0], _p(a), _p(b), _p(out))
    return out


def rns_sub(plans: Plans, a, b) -> np.ndarray:
    a, b = _u(a), _u(b)
    out = np.zeros_like(a)
    lib().orc_rns_sub(plans.ptr, a.shape[0], _p(a), _p(b), _p(out))
    return out


def rns_automorphism(plans: Plans, a, g: int) -> np.ndarray:
    a = _u(a)
    out = np.zeros_like(a)
    lib().orc_rns_automorphism(plans.ptr, a.shape[0], _p(a), _p(out), g)
    return out


def tensor(plans: Plans, a0, a1, b0, b1):
    a0, a1, b0, b1 = map(_u, (a0, a1, b0, b1))
    c0, c1, c2 = (np.zeros_like(a0) for _ in range(3))
    lib().orc_tensor(plans.ptr, a0.shape[0], _p(a0), _p(a1), _p(b0), _p(b1), _p(c0), _p(c1), _p(c2))
    return c0, c1, c2


def rescale_poly(plans: Plans, a) -> np.ndarray:
    a = _u(a)
    out = np.zeros((a.shape[0] - 1, a.shape[1]), dtype=np.uint64)
    lib().orc_rescale_poly(plans.ptr, a.shape[0], _p(a), _p(out))
    return out


def decompose(plans: Plans, poly, levels: int, decomp_bits: int = DECOMP_BITS):
    """Returns (signed digits int64[levels][N], digit residues uint64[levels][limbs][N])."""
    poly = _u(poly)
    L, n = poly.shape
    digits = np.zeros((levels, n), dtype=np.int64)
    res = np.zeros((levels, L, n), dtype=np.uint64)
    lib().orc_decompose(plans.ptr, L, _p(poly), decomp_bits, levels, _p(digits), _p(res))
    return digits, res


def lift(q: Plans, p: Plans, poly) -> np.ndarray:
    poly = _u(poly)
    out = np.zeros((len(q) + len(p), poly.shape[1]), dtype=np.uint64)
    lib().orc_lift(q.ptr, len(q), p.ptr, len(p), _p(poly), _p(out))
    return out


def mod_down(q: Plans, p: Plans, poly) -> np.ndarray:
    poly = _u(poly)
    out = np.zeros((len(q), poly.shape[1]), dtype=np.uint64)
    lib().orc_mod_down(q.ptr, len(q), p.ptr, len(p), _p(poly), _p(out))
    return out


def num_decomp_digits(total_bits: int, decomp_bits: int = DECOMP_BITS) -> int:
    return (total_bits + decomp_bits - 1) // decomp_bits


def _no_plans() -> Plans:
    empty = Plans.__new__(Plans)
    empty.n, empty.moduli, empty.roots = 0, [], []
    empty.arr = (OrcPlan * 1)()
    return empty


def keyswitch(q: Plans, p: Optional[Plans], poly, ksk, decomp_levels: int):
    """keyswitch_rns (Q-only, p None/empty) or keyswitch_rns_hybrid; ksk shaped
    (digits, 2, limbs_q + limbs_p, N)."""
    p = p if p is not None and len(p) else _no_plans()
    poly, ksk = _u(poly), _u(ksk)
    c0 = np.zeros_like(poly)
    c1 = np.zeros_like(poly)
    lib().orc_keyswitch(q.ptr, len(q), p.ptr, len(p), _p(poly), _p(ksk), decomp_levels, _p(c0), _p(c1))
    return c0, c1


def relinearize(q: Plans, p: Optional[Plans], c0, c1, c2, ksk, decomp_levels: int):
    p = p if p is not None and len(p) else _no_plans()
    c0, c1, c2, ksk = map(_u, (c0, c1, c2, ksk))
    o0, o1 = np.zeros_like(c0), np.zeros_like(c0)
    lib().orc_relinearize(q.ptr, len(q), p.ptr, len(p), _p(c0), _p(c1), _p(c2), _p(ksk), decomp_levels, _p(o0), _p(o1))
    return o0, o1


def mult_relinearized(q: Plans, p: Optional[Plans], a0, a1, b0, b1, ksk, decomp_levels: int):
    p = p if p is not None and len(p) else _no_plans()
    a0, a1, b0, b1, ksk = map(_u, (a0, a1, b0, b1, ksk))
    L, n = a0.shape
    o0 = np.zeros((L - 1, n), dtype=np.uint64)
    o1 = np.zeros((L - 1, n), dtype=np.uint64)
    lib().orc_mult_relinearized(q.ptr, L, p.ptr, len(p), _p(a0), _p(a1), _p(b0), _p(b1), _p(ksk), decomp_levels,
                                _p(o0), _p(o1))
    return o0, o1


def rotate(q: Plans, p: Optional[Plans], c0, c1, galois_element: int, ksk, decomp_levels: int):
    p = p if p is not None and len(p) else _no_plans()
    c0, c1, ksk = map(_u, (c0, c1, ksk))
    o0, o1 = np.zeros_like(c0), np.zeros_like(c0)
    lib().orc_rotate(q.ptr, len(q), p.ptr, len(p), _p(c0), _p(c1), galois_element, _p(ksk), decomp_levels,
                     _p(o0), _p(o1))
    return o0, o1


# ----------------------------------------------------------------------------------
# scheme glue (reference compositions) with caller-supplied samples
# ----------------------------------------------------------------------------------

def from_signed(coeffs, moduli: Sequence[int]) -> np.ndarray:
    """Signed small integers -> canonical residues per limb (the lifts in keys.rs:102-151)."""
    c = np.asarray(coeffs, dtype=np.int64)
    return np.stack([(c % np.int64(q)).astype(np.uint64) for q in moduli])


def keygen(plans: Plans, s_coeffs, p1, error_coeffs):
    """`rns_keygen` (keys.rs:153-166): p0 = e - p1*s.  Returns (sk, p0, p1, e)."""
    s = from_signed(s_coeffs, plans.moduli)
    e = from_signed(error_coeffs, plans.moduli)
    p1 = _u(p1)
    p0 = rns_sub(plans, e, rns_mul(plans, p1, s))
    return s, p0, p1, e


def encrypt_with_samples(plans: Plans, pt, p0, p1, u, e0, e1):
    """`encrypt_rns_with_samples` (ops.rs:25-42)."""
    c0 = rns_add(plans, rns_add(plans, rns_mul(plans, p0, u), e0), pt)
    c1 = rns_add(plans, rns_mul(plans, p1, u), e1)
    return c0, c1


def decrypt(plans: Plans, c0, c1, s):
    """`decrypt_rns` (ops.rs:44-52)."""
    return rns_add(plans, c0, rns_mul(plans, c1, s))


def decrypt_quadratic(plans: Plans, c0, c1, c2, s):
    """`decrypt_quadratic_rns` (ops.rs:102-113)."""
    s2 = rns_mul(plans, s, s)
    return rns_add(plans, rns_add(plans, c0, rns_mul(plans, c1, s)), rns_mul(plans, c2, s2))


def _pow_mod_b(i: int, q: int, bits: int = DECOMP_BITS) -> int:
    return pow(2, bits * i, q)


def keyswitch_key_q(plans: Plans, src, p0, p1, samples: List[tuple], digits: Optional[int] = None,
                    decomp_bits: int = DECOMP_BITS):
    """`generate_keyswitch_key_rns` (keyswitching.rs:44-79): digit i encrypts
    (src * B^i mod Q) under the public key with scale 0; samples[i] = (u, e0, e1).
    Returns the key shaped (digits, 2, limbs, N)."""
    src = _u(src)
    D = digits if digits is not None else num_decomp_digits(plans.total_modulus_bits(), decomp_bits)
    out = np.zeros((D, 2) + src.shape, dtype=np.uint64)
    for i in range(D):
        pt = _scale_rows(src, [_pow_mod_b(i, q, decomp_bits) for q in plans.moduli], plans.moduli)
        u, e0, e1 = samples[i]
        out[i, 0], out[i, 1] = encrypt_with_samples(plans, pt, p0, p1, u, e0, e1)
    return out


def keyswitch_key_hybrid(q: Plans, p: Plans, src, s_q, samples: List[tuple], decomp_bits: int = DECOMP_BITS):
    """`generate_keyswitch_key_rns_hybrid` (keyswitching.rs:81-128): digit i is
    (P*B^i*centred(src) + e - a1*s', a1) over Q u P, s' the centred lift of the
    secret; samples[i] = (a1, e).  Returns (digits, 2, lq+lp, N)."""
    src, s_q = _u(src), _u(s_q)
    qp = q.concat(p)
    D = num_decomp_digits(q.total_modulus_bits(), decomp_bits)
    P = p.total_modulus()
    target = lift(q, p, s_q)
    out = np.zeros((D, 2, len(qp), src.shape[1]), dtype=np.uint64)
    for i in range(D):
        pt = np.zeros((len(qp), src.shape[1]), dtype=np.uint64)
        pt[: len(q)] = _scale_rows(src, [(pow(2, decomp_bits * i, m) * (P % m)) % m for m in q.moduli], q.moduli)
        a1, e = samples[i]
        a1 = _u(a1)
        out[i, 0] = rns_sub(qp, rns_add(qp, pt, e), rns_mul(qp, a1, target))
        out[i, 1] = a1
    return out


def noiseless_key_q(plans: Plans, src, decomp_bits: int = DECOMP_BITS):
    """`noiseless_rotation_key` (tests.rs:36-67): ksk_i = (src*B^i mod Q, 0)."""
    src = _u(src)
    D = num_decomp_digits(plans.total_modulus_bits(), decomp_bits)
    out = np.zeros((D, 2) + src.shape, dtype=np.uint64)
    for i in range(D):
        out[i, 0] = _scale_rows(src, [_pow_mod_b(i, q, decomp_bits) for q in plans.moduli], plans.moduli)
    return out


def noiseless_key_hybrid(q: Plans, p: Plans, src, decomp_bits: int = DECOMP_BITS):
    """`noiseless_hybrid_rotation_key_at_level` (tests.rs:69-114): (P*B^i*centred(src), 0) over Q u P."""
    src = _u(src)
    D = num_decomp_digits(q.total_modulus_bits(), decomp_bits)
    P = p.total_modulus()
    out = np.zeros((D, 2, len(q) + len(p), src.shape[1]), dtype=np.uint64)
    for i in range(D):
        out[i, 0, : len(q)] = _scale_rows(src, [(pow(2, decomp_bits * i, m) * (P % m)) % m for m in q.moduli], q.moduli)
    return out


def _scale_rows(a: np.ndarray, factors: Sequence[int], moduli: Sequence[int]) -> np.ndarray:
    """out[i] = a[i] * factors[i] mod moduli[i] (u128 arithmetic in the C oracle)."""
    a = _u(a)
    out = np.empty_like(a)
    for i, (f, m) in enumerate(zip(factors, moduli)):
        row_in = np.ascontiguousarray(a[i])
        row_out = np.empty_like(row_in)
        lib().orc_mul_scalar(_p(row_in), _p(row_out), row_in.size, int(f) % int(m), int(m))
        out[i] = row_out
    return out


# ----------------------------------------------------------------------------------
# FP64 encode / decode (src/rns/encoding.rs, src/math/canonical_embedding.rs)
# ----------------------------------------------------------------------------------

def _bit_reverse_permute(v: np.ndarray) -> np.ndarray:
    n = v.size
    idx = np.arange(n)
    bits = n.bit_length() - 1
    rev = np.zeros(n, dtype=np.int64)
    for b in range(bits):
        rev |= ((idx >> b) & 1) << (bits - 1 - b)
    return v[rev]


def _cmul(a: complex, b: complex) -> complex:
    """num-complex Mul: (ar*br - ai*bi) + (ar*bi + ai*br)i."""
    return complex(a.real * b.real - a.imag * b.imag, a.real * b.imag + a.imag * b.real)


def fft_in_place(values: np.ndarray, inverse: bool) -> np.ndarray:
    """`fft_in_place` (canonical_embedding.rs:44-79): bit reversal, radix-2 DIT with
    the twiddle advanced by recurrence w *= w_len, then 1/n for the inverse."""
    v = _bit_reverse_permute(np.asarray(values, dtype=np.complex128).copy())
    n = v.size
    length = 2
    while length <= n:
        angle = (-2.0 if inverse else 2.0) * math.pi / length
        w_len = complex(math.cos(angle), math.sin(angle))  # Complex64::from_polar(1, angle)
        half = length // 2
        ws = np.empty(half, dtype=np.complex128)
        w = complex(1.0, 0.0)
        for i in range(half):
            ws[i] = w
            w = _cmul(w, w_len)
        blocks = v.reshape(-1, length)
        u = blocks[:, :half].copy()
        x = blocks[:, half:]
        xr, xi = x.real, x.imag
        t = (xr * ws.real - xi * ws.imag) + 1j * (xr * ws.imag + xi * ws.real)
        blocks[:, :half] = u + t
        blocks[:, half:] = u - t
        v = blocks.reshape(-1)
        length *= 2
    if inverse:
        v = v * (1.0 / n)
    return v


def _powi(z: complex, e: int) -> complex:
    """num-complex `powi` (i32): inverse for negative exponents, then num-traits'
    exponentiation by squaring with its multiplication order."""
    if e < 0:
        zr, zi = z.real, z.imag
        d = zr * zr + zi * zi
        z = complex(zr / d, 0.0 - zi / d)
        e = -e
    if e == 0:
        return complex(1.0, 0.0)
    base = z
    while e & 1 == 0:
        base = _cmul(base, base)
        e >>= 1
    if e == 1:
        return base
    acc = base
    while e > 1:
        e >>= 1
        base = _cmul(base, base)
        if e & 1:
            acc = _cmul(acc, base)
    return acc


def slot_exponents(n: int) -> List[int]:
    """encoding.rs:68-79: 5^j mod 2N."""
    out, cur = [], 1
    for _ in range(n // 2):
        out.append(cur)
        cur = cur * 5 % (2 * n)
    return out


def encode_integer_coeffs(n: int, scale: float, slots) -> List[int]:
    """`encode_integer_coeffs` (encoding.rs:9-31)."""
    slots = np.asarray(slots, dtype=np.complex128)
    assert slots.size == n // 2, "slot count must be N/2"
    evals = np.zeros(n, dtype=np.complex128)
    for value, e in zip(slots, slot_exponents(n)):
        evals[(e - 1) // 2] = value
        evals[((2 * n - e) % (2 * n) - 1) // 2] = np.conj(value)
    xi = complex(math.cos(math.pi / n), math.sin(math.pi / n))
    coeffs = fft_in_place(evals, True)
    out = []
    for i, c in enumerate(coeffs):
        tw = _cmul(complex(c), _powi(xi, -i))
        out.append(int(round_half_away(tw.real * scale)))
    return out


def round_half_away(x: float) -> float:
    """f64::round: half-way cases away from zero."""
    return math.floor(x + 0.5) if x >= 0 else -math.floor(-x + 0.5)


def poly_from_bigint_coeffs(moduli: Sequence[int], coeffs: Sequence[int]) -> np.ndarray:
    """`from_bigint_coeffs` (polynomial.rs:78-85): centred big ints -> residues."""
    Q = math.prod(moduli)
    red = [c % Q for c in coeffs]
    return np.array([[x % q for x in red] for q in moduli], dtype=np.uint64)


def reconstruct(moduli: Sequence[int], poly) -> List[int]:
    """`reconstruct_coefficients` (polynomial.rs:162-201), exact CRT."""
    Q = math.prod(moduli)
    terms = []
    for q in moduli:
        part = Q // q
        terms.append((part, pow(part % q, -1, q)))
    poly = np.asarray(poly)
    out = []
    for i in range(poly.shape[1]):
        acc = 0
        for l, (part, inv) in enumerate(terms):
            acc += int(poly[l, i]) * part * inv
        out.append(acc % Q)
    return out


def decode_integer_coeffs(n: int, scale: float, moduli: Sequence[int], poly) -> np.ndarray:
    """`decode_integer_coeffs` (encoding.rs:33-66)."""
    Q = math.prod(moduli)
    half = Q >> 1
    vals = reconstruct(moduli, poly)
    inv_delta = 1.0 / scale
    xi = complex(math.cos(math.pi / n), math.sin(math.pi / n))
    b = np.empty(n, dtype=np.complex128)
    for i, v in enumerate(vals):
        c = v if v <= half else v - Q
        b[i] = _cmul(complex(float(c) * inv_delta, 0.0), _powi(xi, i))
    evals = fft_in_place(b, False)
    return np.array([evals[(e - 1) // 2] for e in slot_exponents(n)], dtype=np.complex128)


def galois_element_for_rotation(n: int, steps: int) -> int:
    """`galois_element_for_rotation` (rotation.rs:14-26)."""
    m = 2 * n
    g = 5 % m
    if steps >= 0:
        return pow(g, steps, m)
    return pow(pow(g, -1, m), -steps, m)
