"""Host-side mirror of the reference's public API (`RnsCkksContext` and friends,
src/rns/context/*.rs, src/rns/{ciphertexts,keys,keyswitching,rotation}.rs) over
the C ABI of librnsckks_gpu.so.

Names, argument meaning and level/scale bookkeeping follow the reference.
Ciphertexts and keys live in GPU memory; only encode/decode (FP64 canonical
embedding) and sampling run on the host, as in the reference.  Precondition
failures raise `RcError` (code RC_ERR_INVALID_ARGUMENT) with the reference's
panic message.

Device memory is held in torch int64 tensors (residues are < 2^61, so the bit
patterns equal the reference's u64 values); torch is only the allocator and
stream provider here, every computation is a library call.
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np
import torch

from . import _lib
from ._lib import RcCiphertext, RcError, RcParams, RcPrime, call, lib
from .params import RnsCkksParams, RnsPrime, num_decomp_digits

DECOMP_BITS = 30  # RNS_DECOMP_BITS, src/rns/mod.rs:1
GALOIS_GENERATOR = 5  # src/rns/rotation.rs:6
GAUSSIAN_SIGMA = 3.19  # sample_gaussian_i64, src/rns/keys.rs:83-86


def _stream() -> ctypes.c_void_p:
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _ptr(t: torch.Tensor) -> ctypes.c_void_p:
    assert t.is_cuda and t.is_contiguous() and t.dtype == torch.int64
    return ctypes.c_void_p(t.data_ptr())


def to_device(a: np.ndarray) -> torch.Tensor:
    a = np.ascontiguousarray(a, dtype=np.uint64)
    return torch.from_numpy(a.view(np.int64)).to("cuda")


def to_host(t: torch.Tensor) -> np.ndarray:
    return t.detach().cpu().numpy().view(np.uint64)


def galois_element_for_rotation(poly_degree: int, steps: int) -> int:
    """src/rns/rotation.rs:14-26: 5^steps mod 2N (5^-1 for negative steps)."""
    m = 2 * poly_degree
    g = GALOIS_GENERATOR % m
    if steps >= 0:
        return pow(g, steps, m)
    return pow(pow(g, -1, m), -steps, m)


# --------------------------------------------------------------------------------------
# data types
# --------------------------------------------------------------------------------------

class RnsPolynomial:
    """`RnsPolynomial` (src/rns/polynomial.rs:9-11): device tensor (limbs, N)."""

    def __init__(self, data: torch.Tensor):
        self.data = data.contiguous()

    def levels(self) -> int:
        return self.data.shape[0]

    def degree(self) -> int:
        return self.data.shape[1]

    def truncate_levels(self, level_count: int) -> "RnsPolynomial":
        """polynomial.rs:154-160."""
        if level_count <= 0:
            raise RcError(1, "level_count must be positive")
        if level_count > self.levels():
            raise RcError(1, "level_count cannot exceed polynomial levels")
        return RnsPolynomial(self.data[:level_count].clone())

    def drop_last_level(self) -> "RnsPolynomial":
        if self.levels() <= 1:
            raise RcError(1, "cannot drop the last RNS level")
        return self.truncate_levels(self.levels() - 1)

    def numpy(self) -> np.ndarray:
        return to_host(self.data)

    def __eq__(self, other) -> bool:
        return isinstance(other, RnsPolynomial) and torch.equal(self.data, other.data)


class RnsCiphertext:
    """`RnsCiphertext{c0, c1, scale_bits, level}` (src/rns/ciphertexts.rs:4-9):
    data is a device tensor (2, level+1, N)."""

    def __init__(self, data: torch.Tensor, scale_bits: int, level: Optional[int] = None):
        self.data = data.contiguous()
        self.scale_bits = int(scale_bits)
        self.level = self.data.shape[1] - 1 if level is None else int(level)

    @staticmethod
    def new(c0: RnsPolynomial, c1: RnsPolynomial, scale_bits: int) -> "RnsCiphertext":
        """ciphertexts.rs:48-58."""
        if c0.levels() != c1.levels():
            raise RcError(1, "ciphertext components must have the same number of RNS levels")
        return RnsCiphertext(torch.stack([c0.data, c1.data]), scale_bits)

    @property
    def c0(self) -> RnsPolynomial:
        return RnsPolynomial(self.data[0])

    @property
    def c1(self) -> RnsPolynomial:
        return RnsPolynomial(self.data[1])

    def raw(self) -> RcCiphertext:
        return RcCiphertext(self.data.data_ptr(), self.level, self.scale_bits)

    def add(self, other: "RnsCiphertext") -> "RnsCiphertext":
        """ciphertexts.rs:60-69 (on the GPU, through the most recent context)."""
        if not _LAST_CTX:
            raise RcError(1, "no RnsCkksContext is alive")
        return _LAST_CTX[-1].add(self, other)

    def truncate_levels(self, level_count: int) -> "RnsCiphertext":
        """ciphertexts.rs:90-98."""
        if level_count <= 0:
            raise RcError(1, "level_count must be positive")
        if level_count > self.level + 1:
            raise RcError(1, "level_count cannot exceed ciphertext levels")
        return RnsCiphertext(self.data[:, :level_count].clone(), self.scale_bits)

    def drop_last_level(self) -> "RnsCiphertext":
        """ciphertexts.rs:80-88."""
        if self.level == 0:
            raise RcError(1, "cannot drop the last ciphertext level")
        return self.truncate_levels(self.level)

    def numpy(self) -> np.ndarray:
        return to_host(self.data)


class RnsQuadraticCiphertext(RnsCiphertext):
    """`RnsQuadraticCiphertext{c0, c1, c2, scale_bits, level}`: device tensor (3, level+1, N)."""

    @property
    def c2(self) -> RnsPolynomial:
        return RnsPolynomial(self.data[2])


_LAST_CTX: List["RnsCkksContext"] = []


@dataclass
class RnsSecretKey:
    """`RnsSecretKey` (src/rns/keys.rs:8-52); `coeffs` keeps the ternary integers."""
    coeffs: np.ndarray  # int64 in {-1, 0, 1}
    poly: RnsPolynomial  # residues over the full Q chain


@dataclass
class RnsPublicKey:
    """`RnsPublicKey{p0, p1}` (keys.rs:54-72)."""
    p0: RnsPolynomial
    p1: RnsPolynomial

    def truncate_levels(self, level_count: int) -> "RnsPublicKey":
        return RnsPublicKey(self.p0.truncate_levels(level_count), self.p1.truncate_levels(level_count))


@dataclass
class RnsKeyPair:
    """`RnsKeyPair{secret_key, public_key, error}` (keys.rs:74-79)."""
    secret_key: RnsSecretKey
    public_key: RnsPublicKey
    error: RnsPolynomial


class RnsKeySwitchingKey:
    """`RnsKeySwitchingKey{ksk, decomp_bits, level, aux_level_count}`
    (src/rns/keyswitching.rs:13-18), device-resident behind an rc_ksk handle."""

    def __init__(self, ctx: "RnsCkksContext", handle: ctypes.c_void_p, galois_element: int = 0,
                 owner: Optional["RnsKeySwitchingKey"] = None):
        self.ctx = ctx
        self.handle = handle
        d, lv, aux, g = ctypes.c_uint32(), ctypes.c_int32(), ctypes.c_uint32(), ctypes.c_uint64()
        call("rc_ksk_info", handle, ctypes.byref(d), ctypes.byref(lv), ctypes.byref(aux), ctypes.byref(g))
        self.digits = d.value  # ksk.len()
        self.level = lv.value
        self.aux_level_count = aux.value
        self.decomp_bits = DECOMP_BITS
        self.galois_element = g.value
        self._owner = owner

    def __del__(self):
        try:
            if self.handle:
                lib().rc_ksk_destroy(self.handle)
                self.handle = None
        except Exception:
            pass

    def drop_last_level(self) -> "RnsKeySwitchingKey":
        """keyswitching.rs:21-30."""
        if self.level == 0:
            raise RcError(1, "cannot drop the last keyswitch level")
        return self.truncate_levels(self.level)

    def truncate_levels(self, level_count: int) -> "RnsKeySwitchingKey":
        """keyswitching.rs:32-41."""
        out = ctypes.c_void_p()
        call("rc_ksk_truncate", self.ctx.handle, self.handle, level_count - 1, ctypes.byref(out))
        return RnsKeySwitchingKey(self.ctx, out, owner=self)

    def to_bytes(self) -> bytes:
        """The resident key as a serialised record (rc_ksk_serialize)."""
        size = ctypes.c_uint64()
        call("rc_ksk_serialized_size", self.handle, ctypes.byref(size))
        buf = torch.empty(size.value, dtype=torch.uint8, pin_memory=torch.cuda.is_available())
        call("rc_ksk_serialize", self.ctx.handle, self.handle, buf.data_ptr(), size.value, _stream())
        return buf.numpy().tobytes()

    def save(self, path) -> None:
        with open(path, "wb") as f:
            f.write(self.to_bytes())


@dataclass
class RnsRotationKey:
    """`RnsRotationKey{galois_element, keyswitch_key}` (src/rns/rotation.rs:9-12)."""
    galois_element: int
    keyswitch_key: RnsKeySwitchingKey


# --------------------------------------------------------------------------------------
# samplers (src/rns/keys.rs) over a seeded generator
# --------------------------------------------------------------------------------------

class Sampler:
    """The reference's distributions with a seeded generator (the reference uses
    an unseeded thread_rng, keys.rs:23,154)."""

    def __init__(self, seed: int = 0):
        self.rng = np.random.default_rng(seed)

    def sparse_ternary(self, n: int, hamming_weight: int) -> np.ndarray:
        """`sample_sparse_ternary` (keys.rs:18-52)."""
        if hamming_weight > n:
            raise RcError(1, "hamming_weight must be <= poly_degree")
        c = np.zeros(n, dtype=np.int64)
        idx = self.rng.choice(n, hamming_weight, replace=False)
        c[idx] = np.where(self.rng.random(hamming_weight) < 0.5, 1, -1)
        return c

    def gaussian(self, n: int) -> np.ndarray:
        """`sample_gaussian_i64` (keys.rs:83-86): N(0, 3.19) rounded half away from zero."""
        x = self.rng.normal(0.0, GAUSSIAN_SIGMA, n)
        return (np.sign(x) * np.floor(np.abs(x) + 0.5)).astype(np.int64)

    def ternary(self, n: int) -> np.ndarray:
        """`sample_ternary_poly` (keys.rs:126-151): uniform over {0, 1, -1}."""
        v = self.rng.integers(0, 3, n)
        return np.where(v == 0, 0, np.where(v == 1, 1, -1)).astype(np.int64)

    def uniform(self, moduli: Sequence[int], n: int) -> np.ndarray:
        """`sample_uniform_poly` (keys.rs:88-100): per limb, u64 % q."""
        out = np.empty((len(moduli), n), dtype=np.uint64)
        for i, q in enumerate(moduli):
            out[i] = self.rng.integers(0, 2 ** 64, n, dtype=np.uint64, endpoint=False) % np.uint64(q)
        return out


class DeviceSampler:
    """The same distributions drawn on the GPU (`rc_sample_uniform/error/ternary`, Philox4x32-10): each draw
    takes the next stream id, so the seed fixes the whole sequence and a polynomial is one launch with no
    host-to-device copy.  Draws are residue tensors [limbs][N] over the first `limbs` chain primes, or over
    Q_(limbs-aux) u P with `with_aux`.  The secret key's fixed-weight ternary draw (a choice of positions)
    stays on the host generator."""

    def __init__(self, ctx: "RnsCkksContext", seed: int = 0):
        self.ctx, self.seed, self.next_id = ctx, int(seed) & (2 ** 64 - 1), 0
        self.host = Sampler(seed)

    def _draw(self, fn: str, limbs: int, with_aux: bool) -> torch.Tensor:
        out = torch.empty((limbs, self.ctx.params.poly_degree), dtype=torch.int64, device="cuda")
        call(fn, self.ctx.handle, self.seed, self.next_id, _ptr(out), limbs, int(with_aux), _stream())
        self.next_id += 1
        return out

    def uniform_residues(self, limbs: int, with_aux: bool = False) -> torch.Tensor:
        return self._draw("rc_sample_uniform", limbs, with_aux)

    def error_residues(self, limbs: int, with_aux: bool = False) -> torch.Tensor:
        return self._draw("rc_sample_error", limbs, with_aux)

    def ternary_residues(self, limbs: int, with_aux: bool = False) -> torch.Tensor:
        return self._draw("rc_sample_ternary", limbs, with_aux)

    def sparse_ternary(self, n: int, hamming_weight: int) -> np.ndarray:
        return self.host.sparse_ternary(n, hamming_weight)


def signed_to_residues(coeffs: np.ndarray, moduli: Sequence[int]) -> np.ndarray:
    c = np.asarray(coeffs, dtype=np.int64)
    return np.stack([(c % np.int64(q)).astype(np.uint64) for q in moduli])


# --------------------------------------------------------------------------------------
# the context
# --------------------------------------------------------------------------------------

class RnsCkksContext:
    """`RnsCkksContext` (src/rns/context.rs:23-28 and context/*.rs) on the GPU."""

    def __init__(self, params: RnsCkksParams):
        self.params = params
        q = (RcPrime * max(1, len(params.primes)))(*[RcPrime(p.modulus, p.primitive_root) for p in params.primes])
        p = (RcPrime * max(1, len(params.aux_primes)))(
            *[RcPrime(x.modulus, x.primitive_root) for x in params.aux_primes])
        raw = RcParams(params.poly_degree, q, len(params.primes), p, len(params.aux_primes), params.scale_bits)
        self.handle = ctypes.c_void_p()
        call("rc_context_create", ctypes.byref(raw), ctypes.byref(self.handle))
        self.q_moduli = [x.modulus for x in params.primes]
        self.p_moduli = [x.modulus for x in params.aux_primes]
        _LAST_CTX.append(self)

    def __del__(self):
        try:
            if self.handle:
                torch.cuda.synchronize()
                lib().rc_context_destroy(self.handle)
                self.handle = None
        except Exception:
            pass

    # ---- context.rs:57-118 ----
    def num_slots(self) -> int:
        return self.params.poly_degree // 2

    def levels(self) -> int:
        return len(self.params.primes)

    def has_aux_basis(self) -> bool:
        return bool(self.params.aux_primes)

    def total_modulus_bits(self) -> int:
        return math.prod(self.q_moduli).bit_length()

    def level_moduli(self, level: int) -> List[int]:
        """Primes of `level_context(level)` (context.rs:100-102)."""
        if level + 1 <= 0 or level + 1 > self.levels():
            raise RcError(1, f"level_count must be in 1..={self.levels()}, got {level + 1}")
        return self.q_moduli[: level + 1]

    def eval_key_level_moduli(self, level: int) -> List[int]:
        """context.rs:104-118."""
        if not self.p_moduli:
            raise RcError(1, "eval-key level context requires an auxiliary basis")
        if level >= self.levels():
            raise RcError(1, f"level must be in 0..{self.levels()}, got {level}")
        return self.q_moduli[: level + 1] + self.p_moduli

    def decomp_digits(self, level: int) -> int:
        d = ctypes.c_uint32()
        call("rc_decomp_digits", self.handle, level, ctypes.byref(d))
        return d.value

    def reserve(self, max_level: int, max_batch: int = 1) -> None:
        call("rc_reserve", self.handle, max_level, max_batch, _stream())

    # ---- encoding, context/encoding.rs ----
    def encode(self, slots) -> RnsPolynomial:
        return self.encode_at_level_and_scale(slots, self.levels() - 1, self.params.scale_bits)

    def encode_real(self, slots) -> RnsPolynomial:
        return self.encode(np.asarray(slots, dtype=np.float64).astype(np.complex128))

    def encode_host(self, slots, level: int, scale_bits: int) -> np.ndarray:
        s = np.asarray(slots, dtype=np.complex128)
        if s.size != self.num_slots():
            raise RcError(1, "slot count must be N/2")
        inter = np.ascontiguousarray(np.stack([s.real, s.imag], axis=1).reshape(-1))
        out = np.empty((level + 1, self.params.poly_degree), dtype=np.uint64)
        call("rc_encode", self.handle, inter.ctypes.data, level, scale_bits, out.ctypes.data)
        return out

    def encode_at_level_and_scale(self, slots, level: int, scale_bits: int) -> RnsPolynomial:
        """context/encoding.rs: encoded on the GPU (the same residues as the host encoder, `encode_host`)."""
        return self.encode_device_batch([slots], level, scale_bits)[0]

    def encode_device_batch(self, slots_list: Sequence, level: int, scale_bits: int) -> List[RnsPolynomial]:
        """Encode many slot vectors on the GPU (rc_encode_device): the same residues as `encode_host`."""
        if not len(slots_list):
            return []
        s = np.asarray(slots_list, dtype=np.complex128).reshape(len(slots_list), -1)
        if s.shape[1] != self.num_slots():
            raise RcError(1, "slot count must be N/2")
        src = torch.from_numpy(np.ascontiguousarray(np.stack([s.real, s.imag], axis=2))).to("cuda")
        out = torch.empty((len(slots_list), level + 1, self.params.poly_degree), dtype=torch.int64, device="cuda")
        call("rc_encode_device", self.handle, ctypes.c_void_p(src.data_ptr()), len(slots_list), level, scale_bits,
             _ptr(out), _stream())
        return [RnsPolynomial(out[i]) for i in range(out.shape[0])]

    def decode_device_batch(self, polys: Sequence[RnsPolynomial], scale_bits: int) -> np.ndarray:
        """Decode many polynomials of one level on the GPU (rc_decode_device): the same values as
        `decode_host`; returns [count][N/2] complex."""
        data = torch.stack([p.data for p in polys]).contiguous()
        out = torch.empty((data.shape[0], self.num_slots(), 2), dtype=torch.float64, device="cuda")
        call("rc_decode_device", self.handle, _ptr(data), data.shape[0], data.shape[1] - 1, scale_bits,
             ctypes.c_void_p(out.data_ptr()), _stream())
        h = out.cpu().numpy()
        return h[..., 0] + 1j * h[..., 1]

    def decode_host(self, poly: np.ndarray, scale_bits: int) -> np.ndarray:
        poly = np.ascontiguousarray(poly, dtype=np.uint64)
        out = np.empty(self.params.poly_degree, dtype=np.float64)
        call("rc_decode", self.handle, poly.ctypes.data, poly.shape[0] - 1, scale_bits, out.ctypes.data)
        return out[0::2] + 1j * out[1::2]

    def decode(self, poly: RnsPolynomial) -> np.ndarray:
        return self.decode_at_scale(poly, self.params.scale_bits)

    def decode_real(self, poly: RnsPolynomial) -> np.ndarray:
        return self.decode(poly).real

    def decode_at_scale(self, poly: RnsPolynomial, scale_bits: int) -> np.ndarray:
        """context/encoding.rs: decoded on the GPU (the same doubles as the host decoder, `decode_host`)."""
        return self.decode_device_batch([poly], scale_bits)[0]

    def decode_real_at_scale(self, poly: RnsPolynomial, scale_bits: int) -> np.ndarray:
        return self.decode_at_scale(poly, scale_bits).real

    # ---- polynomial helpers on the GPU ----
    def _poly_mul(self, a: torch.Tensor, b: torch.Tensor, with_aux: bool = False) -> torch.Tensor:
        out = torch.empty_like(a)
        call("rc_poly_multiply", self.handle, _ptr(a), _ptr(b), _ptr(out), a.shape[0], int(with_aux), _stream())
        return out

    def _poly_add(self, a: torch.Tensor, b: torch.Tensor, with_aux: bool = False) -> torch.Tensor:
        out = torch.empty_like(a)
        call("rc_poly_add", self.handle, _ptr(a), _ptr(b), _ptr(out), a.shape[0], int(with_aux), _stream())
        return out

    def _poly_sub(self, a: torch.Tensor, b: torch.Tensor, with_aux: bool = False) -> torch.Tensor:
        out = torch.empty_like(a)
        call("rc_poly_sub", self.handle, _ptr(a), _ptr(b), _ptr(out), a.shape[0], int(with_aux), _stream())
        return out

    def _poly_scalar(self, a: torch.Tensor, scalars: Sequence[int], with_aux: bool = False) -> torch.Tensor:
        out = torch.empty_like(a)
        arr = np.ascontiguousarray(np.array([int(x) for x in scalars], dtype=np.uint64))
        call("rc_poly_mul_scalar", self.handle, _ptr(a), arr.ctypes.data, _ptr(out), a.shape[0], int(with_aux),
             _stream())
        return out

    def _poly_aut(self, a: torch.Tensor, g: int) -> torch.Tensor:
        out = torch.empty_like(a)
        call("rc_poly_automorphism", self.handle, _ptr(a), _ptr(out), a.shape[0], g, _stream())
        return out

    # ---- keys, src/rns/keys.rs + context/keys.rs ----
    def keygen(self, hamming_weight: int, sampler: Optional[Sampler] = None,
               samples: Optional[Tuple[np.ndarray, np.ndarray, np.ndarray]] = None) -> RnsKeyPair:
        """`rns_keygen` (keys.rs:153-166): p0 = e - p1*s.  `samples` = (s, p1, e)."""
        n = self.params.poly_degree
        if isinstance(sampler, DeviceSampler) and samples is None:
            s = sampler.sparse_ternary(n, hamming_weight)
            p1d = sampler.uniform_residues(len(self.q_moduli))
            ed = sampler.error_residues(len(self.q_moduli))
        else:
            if samples is None:
                sampler = sampler or Sampler()
                s = sampler.sparse_ternary(n, hamming_weight)
                p1 = sampler.uniform(self.q_moduli, n)
                e = sampler.gaussian(n)
            else:
                s, p1, e = samples
            ed = to_device(signed_to_residues(e, self.q_moduli))
            p1d = to_device(p1)
        sd = to_device(signed_to_residues(s, self.q_moduli))
        p0 = self._poly_sub(ed, self._poly_mul(p1d, sd))
        return RnsKeyPair(RnsSecretKey(np.asarray(s, dtype=np.int64), RnsPolynomial(sd)),
                          RnsPublicKey(RnsPolynomial(p0), RnsPolynomial(p1d)), RnsPolynomial(ed))

    def _secret_over(self, sk: RnsSecretKey, moduli: Sequence[int], galois_element: int = 0) -> torch.Tensor:
        coeffs = sk.coeffs
        if galois_element:
            coeffs = _automorphism_signed(coeffs, galois_element)
        return to_device(signed_to_residues(coeffs, moduli))

    def _keyswitch_key_hybrid(self, source: torch.Tensor, sk: RnsSecretKey, level: int, galois_element: int,
                              sampler: Sampler, samples=None, return_coeff: bool = False):
        """`generate_keyswitch_key_rns_hybrid` (keyswitching.rs:81-128) on the GPU:
        digit i = (P*B^i*centred(src) + e - a1*s', a1) over Q_level u P."""
        qm = self.level_moduli(level)
        allm = qm + self.p_moduli
        n = self.params.poly_degree
        D = num_decomp_digits(math.prod(qm).bit_length())
        P = math.prod(self.p_moduli)
        target = self._secret_over(sk, allm)
        key = torch.empty((D, 2, len(allm), n), dtype=torch.int64, device="cuda")
        ext = torch.zeros((len(allm), n), dtype=torch.int64, device="cuda")
        for i in range(D):
            scal = [(pow(2, DECOMP_BITS * i, m) * (P % m)) % m for m in qm] + [0] * len(self.p_moduli)
            ext[: len(qm)] = source[: len(qm)]
            pt = self._poly_scalar(ext, scal, with_aux=True)
            if samples is not None:
                a1, e = samples[i]
                a1d = to_device(a1)
                ed = to_device(signed_to_residues(e, allm) if np.asarray(e).ndim == 1 else e)
            elif isinstance(sampler, DeviceSampler):
                a1d = sampler.uniform_residues(len(allm), True)
                ed = sampler.error_residues(len(allm), True)
            else:
                a1d = to_device(sampler.uniform(allm, n))
                ed = to_device(signed_to_residues(sampler.gaussian(n), allm))
            a1s = self._poly_mul(a1d, target, with_aux=True)
            key[i, 0] = self._poly_sub(self._poly_add(pt, ed, True), a1s, True)
            key[i, 1] = a1d
        return self._upload_key(key, D, level, len(self.p_moduli), galois_element, return_coeff)

    def _keyswitch_key_q(self, source: torch.Tensor, pk: RnsPublicKey, level: int, galois_element: int,
                         sampler: Sampler, samples=None, return_coeff: bool = False):
        """`generate_keyswitch_key_rns` (keyswitching.rs:44-79): digit i encrypts
        src*B^i (mod Q) under the public key with scale 0."""
        qm = self.level_moduli(level)
        n = self.params.poly_degree
        D = num_decomp_digits(math.prod(qm).bit_length())
        key = torch.empty((D, 2, len(qm), n), dtype=torch.int64, device="cuda")
        p0 = pk.p0.data[: len(qm)].contiguous()
        p1 = pk.p1.data[: len(qm)].contiguous()
        src = source[: len(qm)].contiguous()
        for i in range(D):
            pt = self._poly_scalar(src, [pow(2, DECOMP_BITS * i, m) for m in qm])
            if samples is not None:
                u, e0, e1 = samples[i]
            elif isinstance(sampler, DeviceSampler):
                lq = len(qm)
                u, e0, e1 = sampler.ternary_residues(lq), sampler.error_residues(lq), sampler.error_residues(lq)
            else:
                u, e0, e1 = sampler.ternary(n), sampler.gaussian(n), sampler.gaussian(n)
            c0, c1 = self._encrypt_raw(pt, p0, p1, u, e0, e1, qm)
            key[i, 0] = c0
            key[i, 1] = c1
        return self._upload_key(key, D, level, 0, galois_element, return_coeff)

    def _upload_key(self, key: torch.Tensor, digits: int, level: int, aux: int, galois_element: int,
                    return_coeff: bool):
        handle = ctypes.c_void_p()
        torch.cuda.synchronize()
        call("rc_ksk_upload_device", self.handle, _ptr(key), digits, level, aux, galois_element,
             ctypes.byref(handle))
        k = RnsKeySwitchingKey(self, handle)
        return (k, key) if return_coeff else k

    def upload_keyswitch_key(self, host_key: np.ndarray, level: int, aux_level_count: int,
                             galois_element: int = 0) -> RnsKeySwitchingKey:
        """Upload a coefficient-form key [digits][2][limbs][N] (reference layout)."""
        host_key = np.ascontiguousarray(host_key, dtype=np.uint64)
        handle = ctypes.c_void_p()
        call("rc_ksk_upload", self.handle, host_key.ctypes.data, host_key.shape[0], level, aux_level_count,
             galois_element, ctypes.byref(handle))
        return RnsKeySwitchingKey(self, handle)

    # ---- serialised keys and ciphertexts (csrc/serialize.cu) ----
    def keyswitch_key_from_bytes(self, data) -> RnsKeySwitchingKey:
        """A key saved by `RnsKeySwitchingKey.to_bytes`/`save` on a context with the same modulus chain."""
        buf = np.frombuffer(data, dtype=np.uint8)
        out = ctypes.c_void_p()
        call("rc_ksk_deserialize", self.handle, buf.ctypes.data, buf.size, ctypes.byref(out))
        return RnsKeySwitchingKey(self, out)

    def load_keyswitch_key(self, path) -> RnsKeySwitchingKey:
        with open(path, "rb") as f:
            return self.keyswitch_key_from_bytes(f.read())

    def load_rotation_key(self, path) -> "RnsRotationKey":
        k = self.load_keyswitch_key(path)
        return RnsRotationKey(k.galois_element, k)

    def ciphertext_to_bytes(self, ct: "RnsCiphertext") -> bytes:
        comps = ct.data.shape[0]
        size = ctypes.c_uint64()
        call("rc_ct_serialized_size", self.handle, ct.level, comps, ctypes.byref(size))
        buf = np.empty(size.value, dtype=np.uint8)
        call("rc_ct_serialize", self.handle, ctypes.byref(ct.raw()), comps, buf.ctypes.data, size.value, _stream())
        return buf.tobytes()

    def ciphertext_from_bytes(self, data) -> "RnsCiphertext":
        buf = np.frombuffer(data, dtype=np.uint8)
        n, lv, sb, comps = ctypes.c_uint64(), ctypes.c_int32(), ctypes.c_int32(), ctypes.c_uint32()
        call("rc_ct_header", buf.ctypes.data, buf.size, ctypes.byref(n), ctypes.byref(lv), ctypes.byref(sb),
             ctypes.byref(comps))
        if n.value != self.params.poly_degree or not (0 <= lv.value < self.levels()) or comps.value not in (2, 3):
            raise RcError(1, "serialized ciphertext was made for another modulus chain")
        data_t = torch.empty((comps.value, lv.value + 1, n.value), dtype=torch.int64, device="cuda")
        o = RcCiphertext(data_t.data_ptr(), 0, 0)
        call("rc_ct_deserialize", self.handle, buf.ctypes.data, buf.size, ctypes.byref(o),
             data_t.numel() * 8, _stream())
        cls = RnsQuadraticCiphertext if comps.value == 3 else RnsCiphertext
        return cls(data_t, o.scale_bits, o.level)

    def _source_square(self, sk: RnsSecretKey, level: int) -> torch.Tensor:
        s = sk.poly.data[: level + 1].contiguous()
        return self._poly_mul(s, s)

    def generate_relinearization_key(self, sk: RnsSecretKey, pk: RnsPublicKey,
                                     sampler: Optional[Sampler] = None, samples=None, return_coeff=False):
        """context/keys.rs:33-44."""
        return self.generate_relinearization_key_at_level(sk, pk, self.levels() - 1, sampler, samples,
                                                          return_coeff)

    def generate_relinearization_key_at_level(self, sk: RnsSecretKey, pk: RnsPublicKey, level: int,
                                              sampler: Optional[Sampler] = None, samples=None, return_coeff=False):
        """context/keys.rs:46-63."""
        sampler = sampler or Sampler(level + 1000)
        src = self._source_square(sk, level)
        if self.has_aux_basis():
            return self._keyswitch_key_hybrid(src, sk, level, 0, sampler, samples, return_coeff)
        return self._keyswitch_key_q(src, pk, level, 0, sampler, samples, return_coeff)

    def generate_relinearization_key_dnum(self, sk: RnsSecretKey, alpha: int, level: Optional[int] = None,
                                          sampler: Optional[Sampler] = None, return_coeff: bool = False):
        """An RNS-hybrid ("dnum") relinearization key (no counterpart in the reference, whose gadget is balanced
        base-2^30 digits): the level's chain cut into groups of `alpha` limbs (alpha <= the aux prime count),
        group b's pair (e_b - a_b s + g_b s^2, a_b) over Q_level u P with g_b = P mod q_i on the group's limbs
        and 0 elsewhere.  Relinearizing with it decrypts to the same values as with the reference's gadget,
        not to the same residues."""
        if not self.has_aux_basis():
            raise RcError(1, "RNS-hybrid keys need an auxiliary basis")
        level = self.levels() - 1 if level is None else level
        qm = self.level_moduli(level)
        allm = qm + self.p_moduli
        n = self.params.poly_degree
        dnum = -(-len(qm) // alpha)
        P = math.prod(self.p_moduli)
        sampler = sampler or Sampler(level + 4000)
        s_all = self._secret_over(sk, allm)
        s2 = self._poly_mul(s_all, s_all, with_aux=True)
        key = torch.empty((dnum, 2, len(allm), n), dtype=torch.int64, device="cuda")
        for b in range(dnum):
            lo, hi = b * alpha, min((b + 1) * alpha, len(qm))
            gs2 = self._poly_scalar(s2, [P % m if lo <= i < hi else 0 for i, m in enumerate(qm)]
                                    + [0] * len(self.p_moduli), with_aux=True)
            if isinstance(sampler, DeviceSampler):
                a = sampler.uniform_residues(len(allm), True)
                e = sampler.error_residues(len(allm), True)
            else:
                a = to_device(sampler.uniform(allm, n))
                e = to_device(signed_to_residues(sampler.gaussian(n), allm))
            key[b, 0] = self._poly_add(self._poly_sub(e, self._poly_mul(a, s_all, True), True), gs2, True)
            key[b, 1] = a
        torch.cuda.synchronize()
        handle = ctypes.c_void_p()
        call("rc_ksk_upload_dnum", self.handle, _ptr(key), 1, alpha, level, ctypes.byref(handle))
        k = RnsKeySwitchingKey(self, handle)
        return (k, key) if return_coeff else k

    def galois_element_for_rotation(self, steps: int) -> int:
        return galois_element_for_rotation(self.params.poly_degree, steps)

    def conjugation_galois_element(self) -> int:
        """context/rotation.rs:63-65."""
        return 2 * self.params.poly_degree - 1

    def _rotation_key(self, sk, pk, g, level, sampler, samples, return_coeff):
        src = self._secret_over(sk, self.level_moduli(level), g)
        sampler = sampler or Sampler(g * 7919 + level)
        if self.has_aux_basis():
            r = self._keyswitch_key_hybrid(src, sk, level, g, sampler, samples, return_coeff)
        else:
            r = self._keyswitch_key_q(src, pk, level, g, sampler, samples, return_coeff)
        if return_coeff:
            return RnsRotationKey(g, r[0]), r[1]
        return RnsRotationKey(g, r)

    def generate_rotation_key(self, sk, pk, steps: int, sampler=None, samples=None, return_coeff=False):
        """context/rotation.rs:24-41."""
        return self._rotation_key(sk, pk, self.galois_element_for_rotation(steps), self.levels() - 1, sampler,
                                  samples, return_coeff)

    def generate_rotation_key_at_level(self, sk, pk, steps: int, level: int, sampler=None, samples=None,
                                       return_coeff=False):
        """context/rotation.rs:43-61."""
        return self._rotation_key(sk, pk, self.galois_element_for_rotation(steps), level, sampler, samples,
                                  return_coeff)

    def generate_conjugation_key(self, sk, pk, sampler=None, return_coeff=False):
        return self._rotation_key(sk, pk, self.conjugation_galois_element(), self.levels() - 1, sampler, None,
                                  return_coeff)

    def generate_conjugation_key_at_level(self, sk, pk, level: int, sampler=None, return_coeff=False):
        return self._rotation_key(sk, pk, self.conjugation_galois_element(), level, sampler, None, return_coeff)

    # ---- encryption, src/rns/ops.rs:8-52 ----
    def _encrypt_raw(self, pt, p0, p1, u, e0, e1, moduli):
        def residues(x):
            if isinstance(x, torch.Tensor):  # already device residues (DeviceSampler)
                return x
            return to_device(signed_to_residues(x, moduli)) if np.asarray(x).ndim == 1 else to_device(x)
        ud, e0d, e1d = residues(u), residues(e0), residues(e1)
        c0 = self._poly_add(self._poly_add(self._poly_mul(p0, ud), e0d), pt)
        c1 = self._poly_add(self._poly_mul(p1, ud), e1d)
        return c0, c1

    def encrypt(self, plaintext: RnsPolynomial, public_key: RnsPublicKey, sampler: Optional[Sampler] = None,
                samples=None) -> RnsCiphertext:
        """context/ops.rs:8-10 -> encrypt_rns (ops.rs:8-23).  samples = (u, e0, e1)."""
        if plaintext.levels() != self.levels():
            raise RcError(1, "plaintext levels must match the active RNS context")
        n = self.params.poly_degree
        if samples is None and isinstance(sampler, DeviceSampler):
            lq = len(self.q_moduli)
            samples = (sampler.ternary_residues(lq), sampler.error_residues(lq), sampler.error_residues(lq))
        elif samples is None:
            sampler = sampler or Sampler()
            samples = (sampler.ternary(n), sampler.gaussian(n), sampler.gaussian(n))
        c0, c1 = self._encrypt_raw(plaintext.data, public_key.p0.data, public_key.p1.data, *samples, self.q_moduli)
        return RnsCiphertext(torch.stack([c0, c1]), self.params.scale_bits)

    def decrypt(self, ct: RnsCiphertext, sk: RnsSecretKey) -> RnsPolynomial:
        """context/ops.rs:12-18 -> decrypt_rns (ops.rs:44-52)."""
        self.level_moduli(ct.level)
        s = sk.poly.data[: ct.level + 1].contiguous()
        c0 = ct.data[0].contiguous()
        c1 = ct.data[1].contiguous()
        return RnsPolynomial(self._poly_add(c0, self._poly_mul(c1, s)))

    def decrypt_quadratic(self, ct: RnsQuadraticCiphertext, sk: RnsSecretKey) -> RnsPolynomial:
        """context/ops.rs:72-83 -> decrypt_quadratic_rns (ops.rs:102-113)."""
        s = sk.poly.data[: ct.level + 1].contiguous()
        s2 = self._poly_mul(s, s)
        d = self._poly_add(ct.data[0].contiguous(), self._poly_mul(ct.data[1].contiguous(), s))
        return RnsPolynomial(self._poly_add(d, self._poly_mul(ct.data[2].contiguous(), s2)))

    # ---- ciphertext ops, context/ops.rs ----
    def _ct_out(self, comps: int, limbs: int) -> torch.Tensor:
        return torch.empty((comps, limbs, self.params.poly_degree), dtype=torch.int64, device="cuda")

    def add(self, lhs: RnsCiphertext, rhs: RnsCiphertext) -> RnsCiphertext:
        out = self._ct_out(2, lhs.level + 1)
        r = RcCiphertext(out.data_ptr(), 0, 0)
        call("rc_add", self.handle, ctypes.byref(lhs.raw()), ctypes.byref(rhs.raw()), ctypes.byref(r), _stream())
        return RnsCiphertext(out, r.scale_bits, r.level)

    def mult_plain(self, ct: RnsCiphertext, plain: RnsPolynomial) -> RnsCiphertext:
        """context/ops.rs:20-30."""
        if plain.levels() != ct.level + 1:
            raise RcError(1, "plaintext levels must match the multiplication context")
        out = self._ct_out(2, ct.level + 1)
        r = RcCiphertext(out.data_ptr(), 0, 0)
        call("rc_mult_plain", self.handle, ctypes.byref(ct.raw()), _ptr(plain.data), ctypes.byref(r), _stream())
        return RnsCiphertext(out, r.scale_bits, r.level)

    def add_batch(self, lhs: Sequence[RnsCiphertext], rhs: Sequence[RnsCiphertext]) -> List[RnsCiphertext]:
        """`add` of many independent pairs in one call (rc_add_batch)."""
        n = len(lhs)
        if n == 0:
            return []
        outs = [self._ct_out(2, a.level + 1) for a in lhs]
        A = (RcCiphertext * n)(*[a.raw() for a in lhs])
        B = (RcCiphertext * n)(*[b.raw() for b in rhs])
        O = (RcCiphertext * n)(*[RcCiphertext(o.data_ptr(), 0, 0) for o in outs])
        call("rc_add_batch", self.handle, n, A, B, O, _stream())
        return [RnsCiphertext(o, O[i].scale_bits, O[i].level) for i, o in enumerate(outs)]

    def multiply_plain_rns_batch(self, cts: Sequence[RnsCiphertext], plains: Sequence) -> List[RnsCiphertext]:
        """`multiply_plain_rns` of many independent pairs in one call (rc_multiply_plain_rns_batch)."""
        n = len(cts)
        if n == 0:
            return []
        outs = [self._ct_out(2, c.level + 1) for c in cts]
        C = (RcCiphertext * n)(*[c.raw() for c in cts])
        P = (ctypes.c_void_p * n)(*[(p.data if isinstance(p, RnsPolynomial) else p).data_ptr() for p in plains])
        O = (RcCiphertext * n)(*[RcCiphertext(o.data_ptr(), 0, 0) for o in outs])
        call("rc_multiply_plain_rns_batch", self.handle, n, C, P, O, _stream())
        return [RnsCiphertext(o, O[i].scale_bits, O[i].level) for i, o in enumerate(outs)]

    def rescale_batch(self, cts: Sequence[RnsCiphertext]) -> List[RnsCiphertext]:
        """`rescale` of many ciphertexts in one call (rc_rescale_batch)."""
        n = len(cts)
        if n == 0:
            return []
        outs = [self._ct_out(2, max(c.level, 1)) for c in cts]
        C = (RcCiphertext * n)(*[c.raw() for c in cts])
        O = (RcCiphertext * n)(*[RcCiphertext(o.data_ptr(), 0, 0) for o in outs])
        call("rc_rescale_batch", self.handle, n, C, O, _stream())
        return [RnsCiphertext(o, O[i].scale_bits, O[i].level) for i, o in enumerate(outs)]

    def multiply_plain_rns(self, ct: RnsCiphertext, plain: RnsPolynomial) -> RnsCiphertext:
        """src/rns/ops.rs:54-66 (scale unchanged)."""
        if plain.levels() != ct.level + 1:
            raise RcError(1, "plaintext levels must match the multiplication context")
        out = self._ct_out(2, ct.level + 1)
        r = RcCiphertext(out.data_ptr(), 0, 0)
        call("rc_multiply_plain_rns", self.handle, ctypes.byref(ct.raw()), _ptr(plain.data), ctypes.byref(r),
             _stream())
        return RnsCiphertext(out, r.scale_bits, r.level)

    def ntt_forward_copy(self, data: torch.Tensor) -> torch.Tensor:
        """NTT-domain copy of a stack of Q-basis polynomials shaped (..., limbs, N) (rc_ntt_forward)."""
        out = data.contiguous().clone()
        limbs = out.shape[-2]
        call("rc_ntt_forward", self.handle, _ptr(out), out.numel() // (limbs * self.params.poly_degree), limbs, 0,
             _stream())
        return out

    def mult_plain_accumulate(self, cts: Sequence[RnsCiphertext], plains: Sequence, cts_ntt: bool = False,
                              plains_ntt: bool = False) -> RnsCiphertext:
        """Sum of mult_plain(cts[k], plains[k]) (linear_transform.rs:234-252), one inverse transform.
        With cts_ntt / plains_ntt the inputs are NTT-domain tensors from `ntt_forward_copy`."""
        n = len(cts)
        out = self._ct_out(2, cts[0].level + 1)
        C = (RcCiphertext * n)(*[c.raw() for c in cts])
        P = (ctypes.c_void_p * n)(*[(p.data if isinstance(p, RnsPolynomial) else p).data_ptr() for p in plains])
        r = RcCiphertext(out.data_ptr(), 0, 0)
        call("rc_mult_plain_accumulate", self.handle, n, C, int(cts_ntt), P, int(plains_ntt), ctypes.byref(r),
             _stream())
        return RnsCiphertext(out, r.scale_bits, r.level)

    def rescale(self, ct: RnsCiphertext) -> RnsCiphertext:
        """context/ops.rs:32-37."""
        out = self._ct_out(2, max(ct.level, 1))
        r = RcCiphertext(out.data_ptr(), 0, 0)
        call("rc_rescale", self.handle, ctypes.byref(ct.raw()), ctypes.byref(r), _stream())
        return RnsCiphertext(out, r.scale_bits, r.level)

    def mult_plain_slots(self, ct: RnsCiphertext, plain_slots) -> RnsCiphertext:
        """context/ops.rs:39-43."""
        plain = self.encode_at_level_and_scale(plain_slots, ct.level, ct.scale_bits)
        return self.rescale(self.mult_plain(ct, plain))

    def mult_plain_slots_real(self, ct: RnsCiphertext, plain_slots) -> RnsCiphertext:
        return self.mult_plain_slots(ct, np.asarray(plain_slots, dtype=np.float64).astype(np.complex128))

    def mult_plain_slots_preserve_scale(self, ct: RnsCiphertext, plain_slots) -> RnsCiphertext:
        """context/ops.rs:50-56."""
        plain = self.encode_at_level_and_scale(plain_slots, ct.level, 0)
        return self.multiply_plain_rns(ct, plain)

    def mult(self, lhs: RnsCiphertext, rhs: RnsCiphertext) -> RnsQuadraticCiphertext:
        """context/ops.rs:63-70."""
        out = self._ct_out(3, lhs.level + 1)
        r = RcCiphertext(out.data_ptr(), 0, 0)
        call("rc_mult", self.handle, ctypes.byref(lhs.raw()), ctypes.byref(rhs.raw()), ctypes.byref(r), _stream())
        return RnsQuadraticCiphertext(out, r.scale_bits, r.level)

    def rescale_quadratic(self, ct: RnsQuadraticCiphertext) -> RnsQuadraticCiphertext:
        """context/ops.rs:85-90."""
        out = self._ct_out(3, max(ct.level, 1))
        r = RcCiphertext(out.data_ptr(), 0, 0)
        call("rc_rescale_quadratic", self.handle, ctypes.byref(ct.raw()), ctypes.byref(r), _stream())
        return RnsQuadraticCiphertext(out, r.scale_bits, r.level)

    def mult_slots(self, lhs: RnsCiphertext, rhs: RnsCiphertext) -> RnsQuadraticCiphertext:
        """context/ops.rs:92-95."""
        return self.rescale_quadratic(self.mult(lhs, rhs))

    def keyswitch(self, poly: RnsPolynomial, ksk: RnsKeySwitchingKey) -> RnsCiphertext:
        """context/ops.rs:97-109."""
        out = self._ct_out(2, poly.levels())
        r = RcCiphertext(out.data_ptr(), 0, 0)
        call("rc_keyswitch", self.handle, _ptr(poly.data), poly.levels() - 1, ksk.handle, ctypes.byref(r), _stream())
        return RnsCiphertext(out, r.scale_bits, r.level)

    def relinearize(self, ct: RnsQuadraticCiphertext, relin_key: RnsKeySwitchingKey) -> RnsCiphertext:
        """context/ops.rs:111-122."""
        out = self._ct_out(2, ct.level + 1)
        r = RcCiphertext(out.data_ptr(), 0, 0)
        call("rc_relinearize", self.handle, ctypes.byref(ct.raw()), relin_key.handle, ctypes.byref(r), _stream())
        return RnsCiphertext(out, r.scale_bits, r.level)

    def mult_relinearized(self, lhs: RnsCiphertext, rhs: RnsCiphertext,
                          relin_key: RnsKeySwitchingKey) -> RnsCiphertext:
        """context/ops.rs:124-133."""
        out = self._ct_out(2, max(lhs.level, 1))
        r = RcCiphertext(out.data_ptr(), 0, 0)
        call("rc_mult_relinearized", self.handle, ctypes.byref(lhs.raw()), ctypes.byref(rhs.raw()),
             relin_key.handle, ctypes.byref(r), _stream())
        return RnsCiphertext(out, r.scale_bits, r.level)

    def mult_relinearized_batch(self, lhs: Sequence[RnsCiphertext], rhs: Sequence[RnsCiphertext],
                                keys: Sequence[RnsKeySwitchingKey]) -> List[RnsCiphertext]:
        n = len(lhs)
        outs = [self._ct_out(2, max(a.level, 1)) for a in lhs]
        L = (RcCiphertext * n)(*[a.raw() for a in lhs])
        R = (RcCiphertext * n)(*[b.raw() for b in rhs])
        O = (RcCiphertext * n)(*[RcCiphertext(o.data_ptr(), 0, 0) for o in outs])
        K = (ctypes.c_void_p * n)(*[k.handle for k in keys])
        call("rc_mult_relinearized_batch", self.handle, n, L, R, K, O, _stream())
        return [RnsCiphertext(o, O[i].scale_bits, O[i].level) for i, o in enumerate(outs)]

    def relinearize_batch(self, cts: Sequence[RnsQuadraticCiphertext],
                          keys: Sequence[RnsKeySwitchingKey]) -> List[RnsCiphertext]:
        """relinearize (context/ops.rs:111-122) of many quadratic ciphertexts (mixed levels) in one call."""
        n = len(cts)
        outs = [self._ct_out(2, c.level + 1) for c in cts]
        Q = (RcCiphertext * n)(*[c.raw() for c in cts])
        O = (RcCiphertext * n)(*[RcCiphertext(o.data_ptr(), 0, 0) for o in outs])
        K = (ctypes.c_void_p * n)(*[k.handle for k in keys])
        call("rc_relinearize_batch", self.handle, n, Q, K, O, _stream())
        return [RnsCiphertext(o, O[i].scale_bits, O[i].level) for i, o in enumerate(outs)]

    def relinearize_rescale_batch(self, cts: Sequence[RnsQuadraticCiphertext],
                                  keys: Sequence[RnsKeySwitchingKey], outs: Optional[Sequence[torch.Tensor]] = None
                                  ) -> List[RnsCiphertext]:
        """relinearize + rescale of many quadratic ciphertexts (mixed levels) in one call."""
        n = len(cts)
        outs = list(outs) if outs is not None else [self._ct_out(2, c.level) for c in cts]
        Q = (RcCiphertext * n)(*[c.raw() for c in cts])
        O = (RcCiphertext * n)(*[RcCiphertext(o.data_ptr(), 0, 0) for o in outs])
        K = (ctypes.c_void_p * n)(*[k.handle for k in keys])
        call("rc_relinearize_rescale_batch", self.handle, n, Q, K, O, _stream())
        return [RnsCiphertext(o, O[i].scale_bits, O[i].level) for i, o in enumerate(outs)]

    def capture_graph(self, fn) -> "CudaGraph":
        """Record every library call `fn` makes on the current (non-default) stream into a CUDA graph."""
        s = _stream()
        call("rc_graph_begin", self.handle, s)
        h = ctypes.c_void_p()
        try:
            fn()
        except BaseException:
            if lib().rc_graph_end(self.handle, s, ctypes.byref(h)) == 0:
                lib().rc_graph_destroy(h)
            raise
        call("rc_graph_end", self.handle, s, ctypes.byref(h))
        return CudaGraph(h)

    # ---- rotation, context/rotation.rs ----
    def apply_galois_automorphism(self, poly: RnsPolynomial, galois_element: int) -> RnsPolynomial:
        """context/rotation.rs:6-10."""
        if galois_element >= 2 * self.params.poly_degree:
            raise RcError(1, "galois element must be reduced modulo 2N")
        return RnsPolynomial(self._poly_aut(poly.data, galois_element))

    def rotate_plain_raw(self, poly: RnsPolynomial, steps: int) -> RnsPolynomial:
        return RnsPolynomial(self._poly_aut(poly.data, self.galois_element_for_rotation(steps)))

    def rotate_raw(self, ct: RnsCiphertext, steps: int) -> RnsCiphertext:
        return self.automorphism(ct, self.galois_element_for_rotation(steps))

    def conjugate_raw(self, ct: RnsCiphertext) -> RnsCiphertext:
        return self.automorphism(ct, self.conjugation_galois_element())

    def automorphism(self, ct: RnsCiphertext, galois_element: int) -> RnsCiphertext:
        """RnsCiphertext::apply_galois_automorphism (ciphertexts.rs:71-78)."""
        out = self._ct_out(2, ct.level + 1)
        r = RcCiphertext(out.data_ptr(), 0, 0)
        call("rc_automorphism", self.handle, ctypes.byref(ct.raw()), galois_element, ctypes.byref(r), _stream())
        return RnsCiphertext(out, r.scale_bits, r.level)

    def rotate(self, ct: RnsCiphertext, rotation_key: RnsRotationKey) -> RnsCiphertext:
        """context/rotation.rs:104-127."""
        out = self._ct_out(2, ct.level + 1)
        r = RcCiphertext(out.data_ptr(), 0, 0)
        call("rc_rotate", self.handle, ctypes.byref(ct.raw()), rotation_key.keyswitch_key.handle, ctypes.byref(r),
             _stream())
        return RnsCiphertext(out, r.scale_bits, r.level)

    def conjugate(self, ct: RnsCiphertext, conjugation_key: RnsRotationKey) -> RnsCiphertext:
        """context/rotation.rs:133-135."""
        return self.rotate(ct, conjugation_key)

    def rotate_batch(self, cts: Sequence[RnsCiphertext], keys: Sequence[RnsRotationKey]) -> List[RnsCiphertext]:
        n = len(cts)
        outs = [self._ct_out(2, c.level + 1) for c in cts]
        C = (RcCiphertext * n)(*[c.raw() for c in cts])
        O = (RcCiphertext * n)(*[RcCiphertext(o.data_ptr(), 0, 0) for o in outs])
        K = (ctypes.c_void_p * n)(*[k.keyswitch_key.handle for k in keys])
        call("rc_rotate_batch", self.handle, n, C, K, O, _stream())
        return [RnsCiphertext(o, O[i].scale_bits, O[i].level) for i, o in enumerate(outs)]

    def rotate_hoisted(self, cts: Sequence[RnsCiphertext], keys: Sequence[RnsRotationKey]) -> List[List[RnsCiphertext]]:
        """out[i][r] = rotate(cts[i], keys[r]) with one decomposition of each ciphertext shared by its rotations
        (rc_rotate_hoisted); the same residues as `rotate`."""
        n, m = len(cts), len(keys)
        if n == 0 or m == 0:
            return [[] for _ in range(n)]
        outs = [self._ct_out(2, c.level + 1) for c in cts for _ in range(m)]
        C = (RcCiphertext * n)(*[c.raw() for c in cts])
        O = (RcCiphertext * (n * m))(*[RcCiphertext(o.data_ptr(), 0, 0) for o in outs])
        K = (ctypes.c_void_p * m)(*[k.keyswitch_key.handle for k in keys])
        call("rc_rotate_hoisted", self.handle, n, C, m, K, O, _stream())
        return [[RnsCiphertext(outs[i * m + r], O[i * m + r].scale_bits, O[i * m + r].level) for r in range(m)]
                for i in range(n)]


class CudaGraph:
    """An executable CUDA graph of library calls (rc_graph_*): replays on the captured buffers."""

    def __init__(self, handle: ctypes.c_void_p):
        self.handle = handle

    def launch(self) -> None:
        call("rc_graph_launch", self.handle, _stream())

    def __del__(self):
        try:
            if self.handle:
                lib().rc_graph_destroy(self.handle)
                self.handle = None
        except Exception:
            pass


def _automorphism_signed(coeffs: np.ndarray, g: int) -> np.ndarray:
    """X -> X^g on signed integer coefficients (poly/mod.rs:110-131 without the modulus)."""
    n = coeffs.size
    out = np.zeros(n, dtype=np.int64)
    idx = (np.arange(n, dtype=np.int64) * g) % (2 * n)
    pos = idx < n
    out[idx[pos]] += coeffs[pos]
    out[idx[~pos] - n] -= coeffs[~pos]
    return out
