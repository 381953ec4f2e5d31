"""RNS-CKKS parameter sets and the NTT-friendly prime search.

The prime search follows the reference's `find_primes.py:1-79`: candidates are
`q = k * 2N + 1` scanned upward from a start value, kept when prime, paired with
the smallest primitive root modulo q (found by factoring q - 1,
`find_primes.py:12-32`), and accepted only when `verify_ntt`
(`find_primes.py:34-55`) holds: 2N | q - 1, w = g^((q-1)/N) has order exactly N,
and psi = g^((q-1)/2N) satisfies psi^N = -1.  Primality is decided with a
deterministic Miller-Rabin test instead of trial division; both decide the
same mathematical fact, the Miller-Rabin bases below being exact for every
integer below 3.3e24.

Parameter presets mirror `RnsCkksParams` (`src/rns/context/params.rs:9-46`):
`toy`, `small` and `realistic_8_level` are restated with the reference's own
primes, and the build adds the workloads it is measured on (ring degrees
2^13..2^16), each generated by the search above.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from functools import lru_cache
from typing import List, Sequence, Tuple

_MR_BASES = (2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37, 41)


def is_prime(n: int) -> bool:
    if n < 2:
        return False
    for p in _MR_BASES:
        if n % p == 0:
            return n == p
    d, s = n - 1, 0
    while d % 2 == 0:
        d //= 2
        s += 1
    for a in _MR_BASES:
        x = pow(a, d, n)
        if x in (1, n - 1):
            continue
        for _ in range(s - 1):
            x = x * x % n
            if x == n - 1:
                break
        else:
            return False
    return True


def _prime_factors(n: int) -> List[int]:
    factors = []
    d = 2
    while d * d <= n:
        if n % d == 0:
            factors.append(d)
            while n % d == 0:
                n //= d
        d += 1 if d == 2 else 2
    if n > 1:
        factors.append(n)
    return factors


def primitive_root(p: int) -> int:
    """Smallest generator of (Z/pZ)^*, as `get_primitive_root` in find_primes.py:12-32."""
    phi = p - 1
    factors = _prime_factors(phi)
    for g in range(2, p):
        if all(pow(g, phi // f, p) != 1 for f in factors):
            return g
    raise ValueError(f"no primitive root for {p}")


def verify_ntt(n: int, q: int, root: int) -> bool:
    """The NttPlan acceptance test (`src/math/ntt.rs:17-60`, find_primes.py:34-55)."""
    if (q - 1) % (2 * n) != 0:
        return False
    w = pow(root, (q - 1) // n, q)
    if pow(w, n, q) != 1 or (n > 1 and pow(w, n // 2, q) == 1):
        return False
    psi = pow(root, (q - 1) // (2 * n), q)
    return pow(psi, 2 * n, q) == 1 and pow(psi, n, q) == q - 1


def find_ntt_primes(n: int, bits: int, count: int, exclude: Sequence[int] = (),
                    start: int | None = None) -> List[Tuple[int, int]]:
    """Return `count` primes q = k*2n+1 >= start (default 2^(bits-1)+1) with q < 2^bits.

    Scans k upward exactly as find_primes.py:59-79 does.
    """
    step = 2 * n
    lo = (1 << (bits - 1)) + 1 if start is None else start
    k = max(1, (lo - 1 + step - 1) // step)
    found: List[Tuple[int, int]] = []
    excluded = set(exclude)
    while len(found) < count:
        q = k * step + 1
        if q >= (1 << bits):
            raise ValueError(f"ran out of {bits}-bit primes for N={n}")
        if q not in excluded and is_prime(q):
            g = primitive_root(q)
            if verify_ntt(n, q, g):
                found.append((q, g))
        k += 1
    return found


@dataclass(frozen=True)
class RnsPrime:
    """`RnsPrime{modulus, primitive_root}` (`src/rns/basis.rs:8-22`)."""
    modulus: int
    primitive_root: int


@dataclass
class RnsCkksParams:
    """`RnsCkksParams{poly_degree, primes, aux_primes, scale_bits}` (`src/rns/context.rs:16-21`)."""
    poly_degree: int
    primes: List[RnsPrime]
    aux_primes: List[RnsPrime] = field(default_factory=list)
    scale_bits: int = 40

    # ---- presets restated from src/rns/context/params.rs:9-46 -------------------------
    @staticmethod
    def toy() -> "RnsCkksParams":
        return RnsCkksParams(8, default_rns_primes(), [], 30)

    @staticmethod
    def small() -> "RnsCkksParams":
        return RnsCkksParams(1024, default_rns_primes(), [], 40)

    @staticmethod
    def realistic_8_level() -> "RnsCkksParams":
        q = [(1_125_899_908_022_273, 3), (1_125_899_908_612_097, 3), (1_125_899_909_398_529, 3),
             (1_125_899_910_316_033, 5), (1_125_899_911_168_001, 3), (1_125_899_911_364_609, 3),
             (1_125_899_913_527_297, 3), (1_125_899_914_510_337, 3)]
        p = [(562_949_954_142_209, 3), (562_949_955_125_249, 3)]
        return RnsCkksParams(1 << 15, [RnsPrime(*x) for x in q], [RnsPrime(*x) for x in p], 45)

    def validate(self) -> None:
        """`RnsCkksParams::validate` (`src/rns/context/params.rs:48-73`); raises ValueError."""
        if self.scale_bits == 0:
            raise ValueError("scale_bits must be greater than zero")
        if self.scale_bits >= 60:
            raise ValueError("scale_bits must stay below 60 bits per rescale step in this RNS scaffold")
        qs = [p.modulus for p in self.primes]
        for a in self.aux_primes:
            if a.modulus in qs:
                raise ValueError(f"auxiliary eval-key modulus {a.modulus} must be distinct from the ciphertext modulus chain")
        for chain in (self.primes, self.aux_primes, self.primes + self.aux_primes):
            if chain is self.aux_primes and not chain:
                continue
            validate_chain(self.poly_degree, chain)

    def q_moduli(self) -> List[int]:
        return [p.modulus for p in self.primes]

    def p_moduli(self) -> List[int]:
        return [p.modulus for p in self.aux_primes]


def validate_chain(n: int, primes: Sequence[RnsPrime]) -> None:
    """`RnsContext::new` checks (`src/rns/basis.rs:32-59`) and `NttPlan::new` (`ntt.rs:17-60`)."""
    if n == 0 or n & (n - 1):
        raise ValueError("poly_degree must be a non-zero power of two")
    if not primes:
        raise ValueError("RNS basis must contain at least one prime")
    seen = set()
    for p in primes:
        if p.modulus in seen:
            raise ValueError(f"duplicate RNS modulus {p.modulus}")
        seen.add(p.modulus)
        q, g = p.modulus, p.primitive_root
        err = ntt_plan_error(n, q, g)
        if err:
            raise ValueError(f"invalid RNS prime {q}: {err}")


def ntt_plan_error(size: int, modulus: int, root: int) -> str:
    """Error string of `NttPlan::new` (`src/math/ntt.rs:17-60`), '' when the plan is valid."""
    if size == 0 or size & (size - 1):
        return "NTT size must be a non-zero power of two"
    if modulus < 3:
        return "modulus must be an odd prime larger than 2"
    if (modulus - 1) % size:
        return "size must divide modulus - 1"
    if (modulus - 1) % (2 * size):
        return "2 * size must divide modulus - 1 for negacyclic NTTs"
    w = pow(root % modulus, (modulus - 1) // size, modulus)
    if pow(w, size, modulus) != 1:
        return "primitive_root does not generate a size-th root of unity"
    if size > 1 and pow(w, size // 2, modulus) == 1:
        return "root is not primitive for the requested size"
    psi = pow(root % modulus, (modulus - 1) // (2 * size), modulus)
    if pow(psi, 2 * size, modulus) != 1 or pow(psi, size, modulus) != modulus - 1:
        return "primitive_root does not generate a valid negacyclic twiddle"
    return ""


def default_rns_primes() -> List[RnsPrime]:
    """`default_rns_primes` (`src/rns/basis.rs:139-147`)."""
    return [RnsPrime(998_244_353, 3), RnsPrime(1_004_535_809, 3), RnsPrime(469_762_049, 3),
            RnsPrime(754_974_721, 11), RnsPrime(167_772_161, 3), RnsPrime(1_224_736_769, 3)]


# ---------------------------------------------------------------------------------------
# Workload parameter sets (generated by the search above; cached per process).
# ---------------------------------------------------------------------------------------

@lru_cache(maxsize=None)
def _chain(n: int, bits: int, count: int, exclude: Tuple[int, ...] = ()) -> Tuple[Tuple[int, int], ...]:
    return tuple(find_ntt_primes(n, bits, count, exclude))


def plain_small_params() -> RnsCkksParams:
    """N=2^13, one 60-bit base prime plus two scaling primes just above 2^40, scale 2^40, no aux basis.

    The scaling primes have floor(log2 q) = 40, so the reference's integer rescale rule
    (`scale_bits -= floor(log2 q)`, `src/rns/ops.rs:74-79`) returns the scale to 2^40 exactly.
    """
    n = 1 << 13
    base = _chain(n, 60, 1)
    scaling = tuple(find_ntt_primes(n, 41, 2, start=(1 << 40) + 1))
    primes = [RnsPrime(*x) for x in base + scaling]
    return RnsCkksParams(n, primes, [], 40)


def hybrid_params(log_n: int, limbs: int, aux: int = 2, bits: int = 50, scale_bits: int | None = None) -> RnsCkksParams:
    """`limbs` Q primes and `aux` P primes, all `bits`-bit NTT-friendly for N=2^log_n.

    Primes are the first ones found scanning up from 2^(bits-1) (find_primes.py:59-79):
    the first `limbs` form Q, the next `aux` form P, as `realistic_8_level` pairs a Q
    chain with a disjoint two-prime auxiliary basis (`src/rns/context/params.rs:24-46`).
    """
    n = 1 << log_n
    chain = _chain(n, bits, limbs + aux)
    q = [RnsPrime(*x) for x in chain[:limbs]]
    p = [RnsPrime(*x) for x in chain[limbs:]]
    sb = scale_bits if scale_bits is not None else (bits - 1)
    return RnsCkksParams(n, q, p, sb)


def scheme_params(log_n: int, limbs: int, aux: int = 2, scale_bits: int = 40) -> RnsCkksParams:
    """A precision-friendly chain: one 60-bit base prime, `limbs-1` primes just above 2^scale_bits
    (so each rescale removes exactly scale_bits bits), and `aux` 60-bit aux primes.
    Used by the algorithm workloads that decode their results."""
    n = 1 << log_n
    base = _chain(n, 60, 1 + aux)
    scaling = tuple(find_ntt_primes(n, scale_bits + 1, limbs - 1, start=(1 << scale_bits) + 1))
    q = [RnsPrime(*base[0])] + [RnsPrime(*x) for x in scaling]
    p = [RnsPrime(*x) for x in base[1:1 + aux]]
    return RnsCkksParams(n, q, p, scale_bits)


def bench_params() -> RnsCkksParams:
    """HMult+relin workload: N=2^16, 24 Q limbs and 2 P limbs of 50-bit primes."""
    return hybrid_params(16, 24, 2, 50)


def num_decomp_digits(total_modulus_bits: int, decomp_bits: int = 30) -> int:
    """`num_decomp_digits` (`src/rns/keyswitching.rs:238-240`)."""
    return (total_modulus_bits + decomp_bits - 1) // decomp_bits


def modulus_bits(moduli: Sequence[int]) -> int:
    return math.prod(moduli).bit_length()
