"""Python models of integer tricks the CUDA kernels rely on, checked exhaustively or on random inputs against
exact arithmetic (CPU only).

* the centred CRT's quotient estimate: each term y/q in 32-bit fixed point, truncated, at most 3 units of
  2^-31 below its value, so floor(sum) is exact or one low (the kernel's correction handles one);
* the BSGS inner sums' split products: x = x1 2^26 + x0, three 32x32->64 products per term summed in 64-bit
  columns, recombined and reduced once, equal sum(x y) mod q for primes below 2^52 and up to 16 terms;
* the lazy finalize's negated-constant Shoup companions: floor((q - w) 2^64 / q) = 2^64 - 1 - floor(w 2^64 / q);
* the transforms' approximate Shoup product (mul_shoup_apx): the quotient from three of the four 32-bit partial
  products, remainder in [0, 4q); the unreduced forward pass it feeds stays below (4 log N + 1) q < 2^64 for
  primes below 2^57, and the unreduced inverse column pass keeps its 2^(c+1) q bounds;
* the tensor pass's middle term by Karatsuba: (a0 + a1)(b0 + b1) - a0 b0 - a1 b1 in two 64-bit words with
  borrows equals the 128-bit a0 b1 + a1 b0 for inputs below 4q, q < 2^61, and for the forward row pass's
  unreduced outputs (below (4 log N + 1) q) wherever the host allows them (2 B^2 q < 2^64): every Montgomery
  input then stays below q 2^64;
* the inverse transforms' scale folded into their last stage: (x + y) n and (x - y + off)(w1 n) equal the
  unfolded stage followed by the product by n;
* the key product's Montgomery 64 -> 32-bit reduction (mont64_32) over the four internal primes: x 2^-32 mod q
  in [0, q) for every 64-bit x, with no 64-bit overflow on the way.
"""
import random

import pytest

M64 = (1 << 64) - 1


def _primes(bits, count, n=1 << 16):
    import importlib.util
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parent.parent
    if "rnsckks_gb300" not in sys.modules:
        spec = importlib.util.spec_from_file_location("rnsckks_gb300", root / "rns-ckks-rust_gb300" / "__init__.py",
                                                      submodule_search_locations=[str(root / "rns-ckks-rust_gb300")])
        mod = importlib.util.module_from_spec(spec)
        sys.modules["rnsckks_gb300"] = mod
        spec.loader.exec_module(mod)
    from rnsckks_gb300 import params
    return [q for q, _ in params.find_ntt_primes(n, bits, count)]


def _fx(q):
    """(n << 32) | floor(2^95 / (q << n)), n = 64 - bits(q): the table entry the library stores per prime."""
    n = 64 - q.bit_length()
    return n, (1 << 95) // (q << n)


def _term(y, n, r):
    """umulhi32((y << n) >> 32, r): the kernel's fixed-point y / q * 2^31."""
    yh = ((y << n) & M64) >> 32
    return (yh * r) >> 32


@pytest.mark.parametrize("bits", [30, 41, 50, 60, 61])
def test_fixed_point_quotient_terms_are_at_most_three_units_low(bits):
    rng = random.Random(bits)
    for q in _primes(bits, 3):
        n, r = _fx(q)
        assert r < 1 << 32
        for y in [0, 1, q - 1, q // 2, q // 2 + 1] + [rng.randrange(q) for _ in range(2000)]:
            exact_units = (y << 31) / q  # the value in units of 2^-31
            f = _term(y, n, r)
            assert f <= exact_units and exact_units - f < 3, (q, y)


def test_fixed_point_quotient_floor_is_exact_or_one_low():
    rng = random.Random(7)
    qs = _primes(50, 24)
    for _ in range(3000):
        ys = [rng.randrange(q) for q in qs]
        fsum = sum(_term(y, *_fx(q)) for y, q in zip(ys, qs))
        k = fsum >> 31
        exact = sum(__import__("fractions").Fraction(y, q) for y, q in zip(ys, qs))
        assert k in (int(exact), int(exact) - 1)


def _split_sum(xs, ys, q):
    """The k_bsgs_inner split-26 path: three 32x32 products per term in 64-bit columns, then one reduction."""
    mask = (1 << 26) - 1
    p00 = p11 = pk = 0
    for x, y in zip(xs, ys):
        x0, x1, y0, y1 = x & mask, x >> 26, y & mask, y >> 26
        p00 = (p00 + x0 * y0) & M64
        p11 = (p11 + x1 * y1) & M64
        pk = (pk + (x0 + x1) * (y0 + y1)) & M64
    cross = (pk - p00 - p11) & M64
    t = p00 + (cross << 26) + (p11 << 52)  # the 128-bit value the kernel assembles
    assert t < q << 64  # Barrett's precondition
    return t % q


@pytest.mark.parametrize("bits", [30, 41, 50, 52])
def test_bsgs_split_products_equal_the_modular_sum(bits):
    rng = random.Random(bits + 100)
    for q in _primes(bits, 2):
        assert q < 1 << 52
        for terms in (1, 2, 12, 16):
            for _ in range(200):
                xs = [rng.randrange(q) for _ in range(terms)]
                ys = [rng.randrange(q) for _ in range(terms)]
                assert _split_sum(xs, ys, q) == sum(x * y for x, y in zip(xs, ys)) % q
            worst = [q - 1] * terms
            assert _split_sum(worst, worst, q) == (terms * (q - 1) ** 2) % q


def test_negated_shoup_companion():
    rng = random.Random(3)
    for q in _primes(50, 2) + _primes(60, 2):
        for w in [1, 2, q - 1, q // 2] + [rng.randrange(1, q) for _ in range(500)]:
            ws = (w << 64) // q
            assert ((q - w) << 64) // q == M64 - ws


def _shoup_lazy(x, w, q):
    """The kernels' mul_shoup_lazy: x w - floor(x floor(w 2^64 / q) / 2^64) q, mod 2^64."""
    ws = (w << 64) // q
    return (x * w - ((x * ws) >> 64) * q) & M64


def _shoup_apx(x, w, q):
    """The kernels' mul_shoup_apx: x w - qh q mod 2^64 with qh = a1 s1 + hi32(a1 s0) + hi32(a0 s1), where
    (a1, a0) and (s1, s0) are the 32-bit halves of x and floor(w 2^64 / q)."""
    ws = (w << 64) // q
    a0, a1, s0, s1 = x & 0xFFFFFFFF, x >> 32, ws & 0xFFFFFFFF, ws >> 32
    qh = (a1 * s1 + ((a1 * s0) >> 32) + ((a0 * s1) >> 32)) & M64
    return (x * w - qh * q) & M64


@pytest.mark.parametrize("bits", [30, 41, 50, 56, 61])
def test_approximate_shoup_product_is_below_4q_and_congruent(bits):
    rng = random.Random(bits * 3)
    for q in _primes(bits, 2):
        for _ in range(3000):
            w = rng.randrange(q)
            for x in (rng.randrange(1 << 64), M64, rng.randrange(q), (1 << 64) - rng.randrange(1, 1 << 32)):
                r = _shoup_apx(x, w, q)
                assert r < 4 * q and r % q == x * w % q, (q, w, x)


@pytest.mark.parametrize("bits", [50, 56])
def test_lazy_forward_transform_with_approximate_products_stays_below_2_64(bits):
    """The unreduced Cooley-Tukey forward transform (both four-step passes of N = 2^16, 16 stages) with
    approximate Shoup products: x' = x + t, y' = x - t + 4q, t < 4q, so values grow by < 4q per stage from
    inputs below q; modelled on one butterfly chain per stage with adversarial x and t, and on a 2^8-point
    sub-transform for the congruence."""
    q = _primes(bits, 1)[0]
    assert q < 1 << 57
    bound = q  # worst case per stage: x at its bound, t = 4q - 1
    for _ in range(16):
        bound = bound + 4 * q
        assert bound < 1 << 64
    assert bound == 65 * q
    rng = random.Random(bits)
    M = 8
    tw = {(s, j): rng.randrange(1, q) for s in range(M) for j in range(1 << s)}
    vals = [q - 1 if i % 3 else rng.randrange(q) for i in range(1 << M)]
    ref = list(vals)
    for s in range(M):
        t = (1 << M) >> (s + 1)
        for blk in range(0, 1 << M, 2 * t):
            for i in range(blk, blk + t):
                w = tw[(s, i >> (M - s))]
                x, y = vals[i], vals[i + t]
                p = _shoup_apx(y, w, q)
                assert p < 4 * q
                vals[i], vals[i + t] = x + p, x - p + 4 * q
                assert vals[i] < (1 + 4 * (s + 1)) * q and vals[i + t] < (1 + 4 * (s + 1)) * q
                rx, ry = ref[i], ref[i + t]
                ref[i], ref[i + t] = (rx + ry * w) % q, (rx - ry * w) % q
    assert [v % q for v in vals] == ref


@pytest.mark.parametrize("bits", [50, 54])
def test_lazy_inverse_pass_stays_below_2_64_and_matches_the_reduced_pass(bits):
    """The unreduced Gentleman-Sande pass of the inverse column phase (primes below 2^55, M = 8 stages,
    inputs below 2q): the sum path's bound doubles per stage, the difference path adds 2^(c+1) q before its
    approximate Shoup product (below 4q, within the 2^(c+1) q bound from the second stage on); every
    intermediate stays below 2^64 and every output is congruent to the reduced pass's, here on a 256-point
    sub-transform with random twiddles and adversarial (all 2q - 1) inputs."""
    rng = random.Random(bits)
    q = _primes(bits, 1)[0]
    assert q < 1 << 55
    M = 8
    tw = {(s, j): rng.randrange(1, q) for s in range(M) for j in range(1 << s)}
    for inputs in ([2 * q - 1] * (1 << M), [rng.randrange(2 * q) for _ in range(1 << M)]):
        lazy, ref = list(inputs), [x % q for x in inputs]
        for c, s in enumerate(reversed(range(M))):  # stage s = M-1 .. 0; c stages done before it
            t = 1 << (M - 1 - s)
            for blk in range(0, 1 << M, 2 * t):
                for i in range(blk, blk + t):
                    w = tw[(s, i >> (M - s))] if (i >> (M - s)) < (1 << s) else tw[(s, 0)]
                    x, y = lazy[i], lazy[i + t]
                    assert x < (2 << c) * q and y < (2 << c) * q
                    d = x - y + (q << (c + 1))
                    assert 0 <= d < 1 << 64 and x + y < 1 << 64
                    lazy[i], lazy[i + t] = x + y, _shoup_apx(d, w, q)
                    assert lazy[i + t] < 4 * q
                    rx, ry = ref[i], ref[i + t]
                    ref[i], ref[i + t] = (rx + ry) % q, (rx - ry) * w % q
        assert all(v < (2 << M) * q for v in lazy)
        assert [v % q for v in lazy] == ref


def _u128_sub(hi, lo, x):
    """The kernel's sub_from on (hi, lo) words: borrow from the low word into the high one."""
    borrow = 1 if lo < (x & M64) else 0
    return (hi - (x >> 64) - borrow) & M64, (lo - (x & M64)) & M64


@pytest.mark.parametrize("bits", [36, 50, 60])
def test_karatsuba_middle_term_equals_the_two_products(bits):
    rng = random.Random(bits)
    for q in _primes(bits, 2):
        for _ in range(3000):
            a0, a1, b0, b1 = (rng.randrange(4 * q) for _ in range(4))
            if rng.random() < 0.05:
                a0 = a1 = b0 = b1 = 4 * q - 1
            s_a, s_b = a0 + a1, b0 + b1
            assert s_a <= M64 and s_b <= M64
            m = s_a * s_b
            assert m < 1 << 128
            hi, lo = m >> 64, m & M64
            hi, lo = _u128_sub(hi, lo, a0 * b0)
            hi, lo = _u128_sub(hi, lo, a1 * b1)
            assert (hi << 64) | lo == a0 * b1 + a1 * b0


@pytest.mark.parametrize("bits", [30, 50, 55])
def test_inverse_scale_folded_into_the_last_stage(bits):
    rng = random.Random(bits + 1)
    for q in _primes(bits, 2):
        n = pow(1 << 16, -1, q)
        for _ in range(3000):
            w1 = rng.randrange(1, q)
            x, y = rng.randrange(2 * q), rng.randrange(2 * q)
            # unfolded: Gentleman-Sande stage, then every output times n
            u, v = (x + y) % q * n % q, (x - y) * w1 % q * n % q
            # folded: two products by the precomputed n and w1 n (offset 2q keeps x - y non-negative)
            assert (x + y) * n % q == u
            assert (x - y + 2 * q) * (w1 * n % q) % q == v


def _internal_primes():
    """The four largest primes k 2^17 + 1 below 2^29 (the wide key product's internal primes)."""
    out = []
    k = ((1 << 29) - 2) >> 17
    while len(out) < 4 and k > 0:
        q = (k << 17) + 1
        if all(q % d for d in range(3, int(q ** 0.5) + 1, 2)):
            out.append(q)
        k -= 1
    return out


def _mont64_32(x, q, qn, kq):
    """The kernel's steps, with every intermediate checked against its machine width."""
    if x >> 63:
        x -= kq << 32
        assert x >= 0
    m = ((x & 0xFFFFFFFF) * qn) & 0xFFFFFFFF
    s = x + m * q
    assert s < 1 << 64 and s & 0xFFFFFFFF == 0
    t = s >> 32
    assert t < 8 * q and t < 1 << 32
    for c in (4, 2, 1):
        if t >= c * q:
            t -= c * q
    return t


def test_montgomery_64_to_32_reduction_over_the_internal_primes():
    rng = random.Random(64)
    primes = _internal_primes()
    assert len(primes) == 4 and all(q < 1 << 29 for q in primes)
    for q in primes:
        qn = (-pow(q, -1, 1 << 32)) % (1 << 32)
        kq = ((1 << 31) // q) * q
        rinv = pow(1 << 32, -1, q)
        xs = [rng.randrange(1 << 64) for _ in range(20000)]
        xs += [0, 1, q, (1 << 63) - 1, 1 << 63, (1 << 64) - 1, 40 * (q - 1) ** 2, 64 * (q - 1) ** 2 + q - 1]
        for x in xs:
            assert _mont64_32(x, q, qn, kq) == x * rinv % q


def _raw_out_allowed(q, log_n, lazy):
    """The host's condition for unreduced forward outputs into the tensor (B = 4 log N + 1 lazy, else 4)."""
    b = 4 * log_n + 1 if lazy else 4
    return 2 * b * b * q < 1 << 64, b


@pytest.mark.parametrize("bits", [40, 50, 51])
def test_unreduced_forward_outputs_keep_the_tensor_exact(bits):
    rng = random.Random(bits + 7)
    for q in _primes(bits, 2):
        for log_n, lazy in ((16, True), (12, True), (16, False)):
            ok, b = _raw_out_allowed(q, log_n, lazy)
            if not ok:
                assert bits == 51 and lazy  # 51-bit primes exceed the lazy bound: canonical outputs instead
                continue
            for _ in range(2000):
                a0, a1, b0, b1 = (rng.randrange(b * q) for _ in range(4))
                if rng.random() < 0.05:
                    a0 = a1 = b0 = b1 = b * q - 1
                assert a0 + a1 <= M64 and b0 + b1 <= M64
                m = (a0 + a1) * (b0 + b1)
                hi, lo = m >> 64, m & M64
                hi, lo = _u128_sub(hi, lo, a0 * b0)
                hi, lo = _u128_sub(hi, lo, a1 * b1)
                mid = (hi << 64) | lo
                assert mid == a0 * b1 + a1 * b0
                for t in (a0 * b0, mid, a1 * b1):  # the Montgomery reduction's input bound
                    assert t < q << 64
