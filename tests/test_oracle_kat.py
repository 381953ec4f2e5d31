"""The CPU oracle pinned against the reference's own known-answer tests and
exact identities (values restated from the reference test files named in
each test), plus cross-checks against the independent big-integer restatement."""
import math

import numpy as np
import pytest

import bigint_ref as B


def test_ntt_round_trip_kats(oracle):
    # src/math/ntt.rs:194-204 and tests/math/ntt_tests.rs:3-15
    p8 = oracle.Plans(8, [998_244_353], [3])
    v = [1, 2, 3, 4, 5, 6, 7, 8]
    assert list(oracle.ntt_inverse(p8, 0, oracle.ntt_forward(p8, 0, v))) == v
    p16 = oracle.Plans(16, [998_244_353], [3])
    fib = [0, 1, 2, 3, 5, 8, 13, 21, 34, 55, 89, 144, 233, 377, 610, 987]
    assert list(oracle.ntt_inverse(p16, 0, oracle.ntt_forward(p16, 0, fib))) == fib


def test_ntt_plan_rejections(oracle):
    # ntt.rs:206-211, tests/math/ntt_tests.rs:17-29
    with pytest.raises(ValueError, match="2 \\* size must divide modulus - 1"):
        oracle.Plans(8, [41], [6])
    with pytest.raises(ValueError):
        oracle.Plans(12, [998_244_353], [3])
    with pytest.raises(ValueError):
        oracle.Plans(7, [998_244_353], [3])


def test_poly_add_sub_kat(oracle):
    # src/poly/mod.rs:204-211 (mod 17)
    L = oracle.lib()
    a = np.array([14, 1, 9, 0], dtype=np.uint64)
    b = np.array([5, 16, 12, 3], dtype=np.uint64)
    s, d = np.zeros_like(a), np.zeros_like(a)
    L.orc_poly_add(oracle._p(a), oracle._p(b), oracle._p(s), 4, 17)
    L.orc_poly_sub(oracle._p(a), oracle._p(b), oracle._p(d), 4, 17)
    assert list(s) == [2, 0, 4, 3]
    assert list(d) == [9, 2, 14, 14]


def test_negacyclic_product_kat(oracle):
    # src/poly/mod.rs:214-224
    p = oracle.Plans(8, [998_244_353], [3])
    got = oracle.poly_mul_ntt(p, 0, [1, 2, 3, 4, 5, 6, 7, 8], [8, 7, 6, 5, 4, 3, 2, 1])
    assert list(got) == [998_244_193, 998_244_243, 998_244_297, 0, 56, 110, 160, 204]
    assert list(oracle.poly_mul_naive([1, 2, 3, 4, 5, 6, 7, 8], [8, 7, 6, 5, 4, 3, 2, 1], 998_244_353)) == list(got)


def test_ntt_product_matches_naive(oracle):
    # tests/math/poly_tests.rs:22-32 and rns/tests.rs:139-154
    p = oracle.Plans(8, [998_244_353], [3])
    a, b = [11, 22, 33, 44, 55, 66, 77, 88], [3, 1, 4, 1, 5, 9, 2, 6]
    assert list(oracle.poly_mul_ntt(p, 0, a, b)) == list(oracle.poly_mul_naive(a, b, 998_244_353))
    ctx = oracle.Plans(8, [998_244_353, 1_004_535_809, 469_762_049], [3, 3, 3])
    lhs = oracle.from_signed([1, 2, 3, 4, 0, 0, 0, 0], ctx.moduli)
    rhs = oracle.from_signed([4, 3, 2, 1, 0, 0, 0, 0], ctx.moduli)
    prod = oracle.rns_mul(ctx, lhs, rhs)
    for l, q in enumerate(ctx.moduli):
        assert list(prod[l]) == list(oracle.poly_mul_naive(lhs[l], rhs[l], q))


def test_automorphism_kat(oracle):
    # src/poly/mod.rs:227-233
    assert list(oracle.poly_automorphism([1, 2, 3, 4], 17, 3)) == [1, 4, 14, 2]


def test_galois_elements_kat(oracle):
    # src/rns/tests.rs:313-321
    assert oracle.galois_element_for_rotation(8, 0) == 1
    assert oracle.galois_element_for_rotation(8, 1) == 5
    assert oracle.galois_element_for_rotation(8, 2) == 9
    assert oracle.galois_element_for_rotation(8, -1) == 13


def test_rns_add_reconstructs(oracle):
    # src/rns/tests.rs:124-136
    ctx = oracle.Plans(8, [998_244_353, 1_004_535_809, 469_762_049], [3, 3, 3])
    a = oracle.from_signed([10, 20, 30, 40, 0, 0, 0, 0], ctx.moduli)
    b = oracle.from_signed([3, 4, 5, 6, 0, 0, 0, 0], ctx.moduli)
    rec = oracle.reconstruct(ctx.moduli, oracle.rns_add(ctx, a, b))
    assert rec[:4] == [13, 24, 35, 46]


def _rand_poly(rng, moduli, n):
    return np.stack([rng.integers(0, q, n, dtype=np.uint64) for q in moduli])


@pytest.mark.parametrize("limbs,levels_extra", [(1, 0), (3, 0), (3, 2), (5, 0)])
def test_decompose_matches_bigint(oracle, limbs, levels_extra):
    rng = np.random.default_rng(7 + limbs)
    q = [998_244_353, 1_004_535_809, 469_762_049, 754_974_721, 167_772_161][:limbs]
    plans = oracle.Plans(16, q, [3, 3, 3, 11, 3][:limbs])
    poly = _rand_poly(rng, q, 16)
    # the centring boundary and its neighbours
    Q = math.prod(q)
    for k, x in enumerate([Q // 2, Q // 2 + 1, 0, Q - 1, (1 << 29), Q // 2 - 1]):
        poly[:, k] = [x % m for m in q]
    levels = oracle.num_decomp_digits(Q.bit_length()) + levels_extra
    digits, res = oracle.decompose(plans, poly, levels)
    assert np.array_equal(digits, B.decompose(q, poly, levels))
    assert digits.min() >= -(1 << 29) and digits.max() < (1 << 29)
    for d in range(levels):
        for l, m in enumerate(q):
            assert np.array_equal(res[d, l], (digits[d] % m).astype(np.uint64))


def test_mod_down_and_lift_match_bigint(oracle):
    rng = np.random.default_rng(11)
    q = [998_244_353, 1_004_535_809, 469_762_049]
    p = [754_974_721, 167_772_161]
    qp, pp = oracle.Plans(16, q, [3, 3, 3]), oracle.Plans(16, p, [11, 3])
    poly = _rand_poly(rng, q + p, 16)
    P = math.prod(p)
    poly[3:, 0] = [(P // 2) % m for m in p]       # tie: counts as positive
    poly[3:, 1] = [(P // 2 + 1) % m for m in p]
    assert np.array_equal(oracle.mod_down(qp, pp, poly), B.mod_down(q, p, poly))
    src = _rand_poly(rng, q, 16)
    lifted = oracle.lift(qp, pp, src)
    for i in range(16):
        for k, m in enumerate(p):
            assert int(lifted[3 + k, i]) == B.convert_centred(q, [int(src[l, i]) for l in range(3)], m)


def test_rescale_matches_bigint(oracle):
    rng = np.random.default_rng(3)
    q = [998_244_353, 1_004_535_809, 469_762_049]
    plans = oracle.Plans(16, q, [3, 3, 3])
    poly = _rand_poly(rng, q, 16)
    poly[2, 0] = q[2] // 2
    poly[2, 1] = q[2] // 2 + 1
    assert np.array_equal(oracle.rescale_poly(plans, poly), B.rescale(q, poly))


def test_encode_decode_round_trip(oracle):
    # src/rns/tests.rs:585-600 (tolerance 1e-3), toy-sized context with 3 primes and scale 2^40
    q = [998_244_353, 1_004_535_809, 469_762_049]
    slots = [0.125 - 0.25j, -0.75 + 0.5j, 0.3125j, 0.625 - 0.4375j]
    coeffs = oracle.encode_integer_coeffs(8, 2.0 ** 40, slots)
    poly = oracle.poly_from_bigint_coeffs(q, coeffs)
    back = oracle.decode_integer_coeffs(8, 2.0 ** 40, q, poly)
    assert np.max(np.abs(back - np.array(slots))) <= 1e-3


def test_noiseless_encrypt_identity(oracle):
    # src/rns/tests.rs:651-677: decrypt(enc(pt; u=1+X^2, e=0)) == pt + e_pk * u exactly
    rng = np.random.default_rng(5)
    q = [998_244_353, 1_004_535_809, 469_762_049]
    plans = oracle.Plans(8, q, [3, 3, 3])
    s = np.zeros(8, dtype=np.int64)
    s[[1, 4, 6]] = [1, -1, 1]
    e = rng.integers(-6, 7, 8)
    s_rns, p0, p1, e_rns = oracle.keygen(plans, s, _rand_poly(rng, q, 8), e)
    pt = oracle.poly_from_bigint_coeffs(q, oracle.encode_integer_coeffs(8, 2.0 ** 40, [0.125 - 0.25j, -0.0625 + 0.1875j, 0.03125 + 0.09375j, -0.125 - 0.0625j]))
    mask = oracle.from_signed([1, 0, 1, 0, 0, 0, 0, 0], q)
    zero = np.zeros_like(pt)
    c0, c1 = oracle.encrypt_with_samples(plans, pt, p0, p1, mask, zero, zero)
    dec = oracle.decrypt(plans, c0, c1, s_rns)
    assert np.array_equal(dec, oracle.rns_add(plans, pt, oracle.rns_mul(plans, e_rns, mask)))


@pytest.mark.slow
def test_noiseless_hybrid_keyswitch_identity_realistic(oracle, pkg):
    # src/rns/tests.rs:437-456: realistic_8_level, noiseless hybrid key for rotation 1
    # at level 7; decrypt(keyswitch([1,2,3,4])) == input * sigma_5(s) exactly.
    params = pkg.RnsCkksParams.realistic_8_level()
    n = params.poly_degree
    qpl = oracle.Plans(n, params.primes)
    ppl = oracle.Plans(n, params.aux_primes)
    rng = np.random.default_rng(64)
    s = np.zeros(n, dtype=np.int64)
    idx = rng.choice(n, 64, replace=False)
    s[idx] = rng.choice([-1, 1], 64)
    s_rns = oracle.from_signed(s, qpl.moduli)
    g = oracle.galois_element_for_rotation(n, 1)
    src = oracle.rns_automorphism(qpl, s_rns, g)
    key = oracle.noiseless_key_hybrid(qpl, ppl, src)
    x = oracle.from_signed(np.r_[[1, 2, 3, 4], np.zeros(n - 4, dtype=np.int64)], qpl.moduli)
    D = oracle.num_decomp_digits(qpl.total_modulus_bits())
    c0, c1 = oracle.keyswitch(qpl, ppl, x, key, D)
    assert np.array_equal(oracle.decrypt(qpl, c0, c1, s_rns), oracle.rns_mul(qpl, x, src))
