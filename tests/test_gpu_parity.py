"""GPU path (C ABI) vs the CPU oracle, bit-exact on residues."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # collected on CPU-only machines, never run there
    pytest.skip("needs a CUDA GPU", allow_module_level=True)


@pytest.fixture(scope="module")
def C(pkg):
    pkg.lib()
    from rnsckks_gb300 import context as C
    return C


def rand_poly(rng, moduli, n):
    return np.stack([rng.integers(0, q, n, dtype=np.uint64) for q in moduli])


def rand_ct(rng, moduli, n, comps=2):
    return np.stack([rand_poly(rng, moduli, n) for _ in range(comps)])


def bitrev(x, bits):
    return int(format(x, f"0{bits}b")[::-1], 2) if bits else 0


PARAM_CASES = {
    "toy_q3": lambda P: P.RnsCkksParams(8, P.default_rns_primes()[:3], [], 40),
    "small_q6": lambda P: P.RnsCkksParams.small(),
    "plain_n13": lambda P: P.plain_small_params(),
    "hybrid_n12": lambda P: P.hybrid_params(12, 6, 2, 50),
    "hybrid_n11_k3": lambda P: P.hybrid_params(11, 5, 3, 45),
}


@pytest.fixture(scope="module", params=list(PARAM_CASES))
def setup(request, pkg, C, oracle):
    params = PARAM_CASES[request.param](pkg.params)
    ctx = C.RnsCkksContext(params)
    n = params.poly_degree
    qpl = oracle.Plans(n, params.primes)
    ppl = oracle.Plans(n, params.aux_primes) if params.aux_primes else None
    return ctx, params, qpl, ppl


@pytest.mark.parametrize("log_n", [3, 4, 5, 10, 13, 16])
def test_ntt_forward_matches_reference_ordering(C, pkg, oracle, log_n):
    n = 1 << log_n
    params = pkg.params.hybrid_params(log_n, 3, 1, 50) if log_n >= 10 else pkg.params.RnsCkksParams(
        n, pkg.params.default_rns_primes()[:3], [], 40)
    ctx = C.RnsCkksContext(params)
    rng = np.random.default_rng(log_n)
    q = params.q_moduli()
    a = rand_poly(rng, q, n)
    d = C.to_device(a)
    C.call("rc_ntt_forward", ctx.handle, C._ptr(d), 1, len(q), 0, C._stream())
    got = C.to_host(d)
    pl = oracle.Plans(n, params.primes)
    for l, m in enumerate(q):
        psi = pl.plan(l).negacyclic_twiddle
        tw = np.array([(int(a[l, i]) * pow(psi, i, m)) % m for i in range(n)], dtype=np.uint64)
        ref = oracle.ntt_forward(pl, l, tw)
        perm = np.array([bitrev(k, log_n) for k in range(n)])
        assert np.array_equal(got[l, perm], ref)
    C.call("rc_ntt_inverse", ctx.handle, C._ptr(d), 1, len(q), 0, C._stream())
    assert np.array_equal(C.to_host(d), a)


def test_ntt_round_trip_many_polys_with_aux(C, pkg):
    params = pkg.params.hybrid_params(13, 4, 2, 50)
    ctx = C.RnsCkksContext(params)
    rng = np.random.default_rng(3)
    allm = params.q_moduli() + params.p_moduli()
    a = np.stack([rand_poly(rng, allm, params.poly_degree) for _ in range(70)])
    d = C.to_device(a)
    C.call("rc_ntt_forward", ctx.handle, C._ptr(d), 70, len(allm), 1, C._stream())
    assert not np.array_equal(C.to_host(d), a)
    C.call("rc_ntt_inverse", ctx.handle, C._ptr(d), 70, len(allm), 1, C._stream())
    assert np.array_equal(C.to_host(d), a)


def test_poly_ops_match_oracle(setup, C, oracle):
    ctx, params, qpl, _ = setup
    n, q = params.poly_degree, params.q_moduli()
    rng = np.random.default_rng(11)
    a, b = rand_poly(rng, q, n), rand_poly(rng, q, n)
    da, db = C.to_device(a), C.to_device(b)
    assert np.array_equal(C.to_host(ctx._poly_mul(da, db)), oracle.rns_mul(qpl, a, b))
    assert np.array_equal(C.to_host(ctx._poly_add(da, db)), oracle.rns_add(qpl, a, b))
    assert np.array_equal(C.to_host(ctx._poly_sub(da, db)), oracle.rns_sub(qpl, a, b))
    for g in (5, 2 * n - 1, 3 if n > 4 else 1):
        assert np.array_equal(C.to_host(ctx._poly_aut(da, g)), oracle.rns_automorphism(qpl, a, g))


def test_tensor_and_rescale_match_oracle(setup, C, oracle):
    ctx, params, qpl, _ = setup
    n, q = params.poly_degree, params.q_moduli()
    rng = np.random.default_rng(12)
    a, b = rand_ct(rng, q, n), rand_ct(rng, q, n)
    lhs = C.RnsCiphertext(C.to_device(a), 40)
    rhs = C.RnsCiphertext(C.to_device(b), 40)
    quad = ctx.mult(lhs, rhs)
    ref = oracle.tensor(qpl, a[0], a[1], b[0], b[1])
    got = quad.numpy()
    for k in range(3):
        assert np.array_equal(got[k], ref[k])
    assert quad.scale_bits == 80 and quad.level == len(q) - 1
    r = ctx.rescale(lhs)
    assert np.array_equal(r.numpy()[0], oracle.rescale_poly(qpl, a[0]))
    assert np.array_equal(r.numpy()[1], oracle.rescale_poly(qpl, a[1]))
    assert r.level == len(q) - 2
    assert r.scale_bits == max(0, 40 - (q[-1].bit_length() - 1))
    rq = ctx.rescale_quadratic(quad)
    for k in range(3):
        assert np.array_equal(rq.numpy()[k], oracle.rescale_poly(qpl, ref[k]))


def test_mult_plain_matches_oracle(setup, C, oracle):
    ctx, params, qpl, _ = setup
    n, q = params.poly_degree, params.q_moduli()
    rng = np.random.default_rng(13)
    a, p = rand_ct(rng, q, n), rand_poly(rng, q, n)
    ct = C.RnsCiphertext(C.to_device(a), 30)
    out = ctx.mult_plain(ct, C.RnsPolynomial(C.to_device(p)))
    assert out.scale_bits == 60
    assert np.array_equal(out.numpy()[0], oracle.rns_mul(qpl, a[0], p))
    assert np.array_equal(out.numpy()[1], oracle.rns_mul(qpl, a[1], p))
    keep = ctx.multiply_plain_rns(ct, C.RnsPolynomial(C.to_device(p)))
    assert keep.scale_bits == 30 and np.array_equal(keep.numpy(), out.numpy())


def _random_key(rng, params, limbs_q, hybrid):
    n = params.poly_degree
    qm = params.q_moduli()[:limbs_q]
    allm = qm + (params.p_moduli() if hybrid else [])
    D = math.ceil(math.prod(qm).bit_length() / 30)
    return np.stack([rand_ct(rng, allm, n) for _ in range(D)]), D


@pytest.mark.parametrize("level_drop", [0, 1])
def test_keyswitch_relin_mult_relin_match_oracle(setup, C, oracle, level_drop):
    ctx, params, qpl_full, ppl = setup
    n, qall = params.poly_degree, params.q_moduli()
    limbs = len(qall) - level_drop
    if limbs < 2:
        pytest.skip("needs two limbs")
    qpl = qpl_full.prefix(limbs)
    q = qall[:limbs]
    hybrid = bool(params.aux_primes)
    rng = np.random.default_rng(100 + limbs)
    key, D = _random_key(rng, params, limbs, hybrid)
    ksk = ctx.upload_keyswitch_key(key, limbs - 1, len(params.aux_primes) if hybrid else 0)
    # keyswitch of a single polynomial
    x = rand_poly(rng, q, n)
    ks = ctx.keyswitch(C.RnsPolynomial(C.to_device(x)), ksk)
    r0, r1 = oracle.keyswitch(qpl, ppl, x, key, D)
    assert np.array_equal(ks.numpy()[0], r0) and np.array_equal(ks.numpy()[1], r1)
    assert ks.scale_bits == limbs  # RnsCiphertext::new(c0, c1, poly.levels())
    # relinearize
    quad = rand_ct(rng, q, n, 3)
    qct = C.RnsQuadraticCiphertext(C.to_device(quad), 70)
    rl = ctx.relinearize(qct, ksk)
    o0, o1 = oracle.relinearize(qpl, ppl, quad[0], quad[1], quad[2], key, D)
    assert np.array_equal(rl.numpy()[0], o0) and np.array_equal(rl.numpy()[1], o1)
    assert rl.scale_bits == 70
    # mult_relinearized = tensor + relinearize + rescale
    a, b = rand_ct(rng, q, n), rand_ct(rng, q, n)
    out = ctx.mult_relinearized(C.RnsCiphertext(C.to_device(a), 35), C.RnsCiphertext(C.to_device(b), 35), ksk)
    m0, m1 = oracle.mult_relinearized(qpl, ppl, a[0], a[1], b[0], b[1], key, D)
    assert np.array_equal(out.numpy()[0], m0) and np.array_equal(out.numpy()[1], m1)
    assert out.level == limbs - 2
    assert out.scale_bits == max(0, 70 - (q[-1].bit_length() - 1))


def test_rotate_matches_oracle(setup, C, oracle):
    ctx, params, qpl, ppl = setup
    n, q = params.poly_degree, params.q_moduli()
    hybrid = bool(params.aux_primes)
    rng = np.random.default_rng(21)
    key, D = _random_key(rng, params, len(q), hybrid)
    for steps in (1, -1, 3):
        g = ctx.galois_element_for_rotation(steps)
        ksk = ctx.upload_keyswitch_key(key, len(q) - 1, len(params.aux_primes) if hybrid else 0, g)
        rk = C.RnsRotationKey(g, ksk)
        a = rand_ct(rng, q, n)
        out = ctx.rotate(C.RnsCiphertext(C.to_device(a), 40), rk)
        r0, r1 = oracle.rotate(qpl, ppl, a[0], a[1], g, key, D)
        assert np.array_equal(out.numpy()[0], r0) and np.array_equal(out.numpy()[1], r1)
    g = ctx.conjugation_galois_element()
    ksk = ctx.upload_keyswitch_key(key, len(q) - 1, len(params.aux_primes) if hybrid else 0, g)
    a = rand_ct(rng, q, n)
    out = ctx.conjugate(C.RnsCiphertext(C.to_device(a), 40), C.RnsRotationKey(g, ksk))
    r0, r1 = oracle.rotate(qpl, ppl, a[0], a[1], g, key, D)
    assert np.array_equal(out.numpy()[0], r0) and np.array_equal(out.numpy()[1], r1)


def test_q_only_truncated_key_uses_all_key_digits(C, pkg, oracle):
    # keyswitch_rns decomposes into ksk.ksk.len() digits even after
    # truncate_levels (keyswitching.rs:21-41, 138): the extra digits carry the
    # sign extension.
    params = pkg.params.RnsCkksParams.small()
    ctx = C.RnsCkksContext(params)
    n, q = params.poly_degree, params.q_moduli()
    qpl = oracle.Plans(n, params.primes)
    rng = np.random.default_rng(5)
    key, D = _random_key(rng, params, len(q), False)
    ksk = ctx.upload_keyswitch_key(key, len(q) - 1, 0)
    for lv in (3, 1, 0):
        tk = ksk.truncate_levels(lv + 1)
        assert tk.digits == D and tk.level == lv
        x = rand_poly(rng, q[: lv + 1], n)
        ks = ctx.keyswitch(C.RnsPolynomial(C.to_device(x)), tk)
        tkey = np.ascontiguousarray(key[:, :, : lv + 1])
        r0, r1 = oracle.keyswitch(qpl.prefix(lv + 1), None, x, tkey, D)
        assert np.array_equal(ks.numpy()[0], r0) and np.array_equal(ks.numpy()[1], r1)


def test_centring_boundaries(C, pkg, oracle):
    # coefficients at floor(Q/2), floor(Q/2)+1, 0, Q-1 and at the P/2 tie for ModDown
    params = pkg.params.hybrid_params(11, 3, 2, 50)
    ctx = C.RnsCkksContext(params)
    n, q, p = params.poly_degree, params.q_moduli(), params.p_moduli()
    qpl, ppl = oracle.Plans(n, params.primes), oracle.Plans(n, params.aux_primes)
    rng = np.random.default_rng(9)
    Q = math.prod(q)
    x = rand_poly(rng, q, n)
    for k, v in enumerate([Q // 2, Q // 2 + 1, 0, Q - 1, 1 << 29, (1 << 29) - 1, Q - (1 << 29)]):
        x[:, k] = [v % m for m in q]
    key, D = _random_key(rng, params, len(q), True)
    ksk = ctx.upload_keyswitch_key(key, len(q) - 1, len(p))
    ks = ctx.keyswitch(C.RnsPolynomial(C.to_device(x)), ksk)
    r0, r1 = oracle.keyswitch(qpl, ppl, x, key, D)
    assert np.array_equal(ks.numpy()[0], r0) and np.array_equal(ks.numpy()[1], r1)


def test_batch_mixed_levels_equals_per_op(C, pkg, oracle):
    params = pkg.params.hybrid_params(12, 6, 2, 50)
    ctx = C.RnsCkksContext(params)
    n, q = params.poly_degree, params.q_moduli()
    rng = np.random.default_rng(33)
    keys, lhs, rhs = [], [], []
    key_np = {}
    for lv in (5, 3, 5, 2, 4, 3, 5):
        if lv not in key_np:
            key_np[lv] = ctx.upload_keyswitch_key(_random_key(rng, params, lv + 1, True)[0], lv, 2)
        keys.append(key_np[lv])
        lhs.append(C.RnsCiphertext(C.to_device(rand_ct(rng, q[: lv + 1], n)), 40))
        rhs.append(C.RnsCiphertext(C.to_device(rand_ct(rng, q[: lv + 1], n)), 40))
    batch = ctx.mult_relinearized_batch(lhs, rhs, keys)
    for a, b, k, out in zip(lhs, rhs, keys, batch):
        single = ctx.mult_relinearized(a, b, k)
        assert single.level == out.level and single.scale_bits == out.scale_bits
        assert np.array_equal(single.numpy(), out.numpy())


def test_host_entry_point_equals_device_path(C, pkg):
    import ctypes
    params = pkg.params.hybrid_params(11, 4, 2, 50)
    ctx = C.RnsCkksContext(params)
    n, q = params.poly_degree, params.q_moduli()
    rng = np.random.default_rng(44)
    key = ctx.upload_keyswitch_key(_random_key(rng, params, len(q), True)[0], len(q) - 1, 2)
    a, b = rand_ct(rng, q, n), rand_ct(rng, q, n)
    dev = ctx.mult_relinearized(C.RnsCiphertext(C.to_device(a), 40), C.RnsCiphertext(C.to_device(b), 40), key)
    out = np.zeros((2, len(q) - 1, n), dtype=np.uint64)
    sb = ctypes.c_int32()
    C.call("rc_mult_relinearized_host", ctx.handle, a.ctypes.data, b.ctypes.data, len(q) - 1, 40, key.handle,
           out.ctypes.data, ctypes.byref(sb), C._stream())
    assert np.array_equal(out, dev.numpy()) and sb.value == dev.scale_bits


def test_pipelined_host_batch_equals_device_path(C, pkg):
    # more jobs than one pipeline chunk, mixed levels, repeated calls reusing the staging slots; N=2^12 so the
    # wide key product (and with it the phased form for one-level batches) is in use
    import ctypes
    params = pkg.params.hybrid_params(12, 5, 2, 50)
    ctx = C.RnsCkksContext(params)
    n, q = params.poly_degree, params.q_moduli()
    rng = np.random.default_rng(45)
    keys = {lv: ctx.upload_keyswitch_key(_random_key(rng, params, lv + 1, True)[0], lv, 2) for lv in (2, 3, 4)}
    cases = [(21, None), (3, None), (11, 4), (11, 4)]  # mixed levels (chunked pipeline); one level (phased)
    for case, (count, fixed) in enumerate(cases):
        if case == 3:  # the same batch with the phased form switched off
            C.call("rc_tune_set", ctx.handle, b"host_phased", 0)
        levels = [int(x) for x in rng.integers(2, 5, count)] if fixed is None else [fixed] * count
        A = [np.ascontiguousarray(rand_ct(rng, q[: lv + 1], n)) for lv in levels]
        B = [np.ascontiguousarray(rand_ct(rng, q[: lv + 1], n)) for lv in levels]
        outs = [np.zeros((2, lv, n), dtype=np.uint64) for lv in levels]
        P = lambda arrs: (ctypes.c_void_p * count)(*[x.ctypes.data for x in arrs])
        LV = (ctypes.c_int32 * count)(*levels)
        SB = (ctypes.c_int32 * count)(*([40] * count))
        K = (ctypes.c_void_p * count)(*[keys[lv].handle for lv in levels])
        OSB = (ctypes.c_int32 * count)()
        C.call("rc_mult_relinearized_batch_host", ctx.handle, count, P(A), P(B), LV, SB, K, P(outs), OSB,
               C._stream())
        for i, lv in enumerate(levels):
            dev = ctx.mult_relinearized(C.RnsCiphertext(C.to_device(A[i]), 40), C.RnsCiphertext(C.to_device(B[i]), 40),
                                        keys[lv])
            assert np.array_equal(outs[i], dev.numpy()) and OSB[i] == dev.scale_bits


@pytest.mark.parametrize("phased", [2, 1, 0])
def test_async_host_batches_back_to_back_equal_device_path(C, pkg, phased):
    # several asynchronous batches in a row (their copies and kernels overlap; the staging slots alternate),
    # then one join and a synchronisation: every batch's results equal the device path's; the last batch
    # reuses the first batch's output buffers after the join.  phased 0 (the staged form) runs synchronously.
    import ctypes
    params = pkg.params.hybrid_params(12, 5, 2, 50)
    ctx = C.RnsCkksContext(params)
    C.call("rc_tune_set", ctx.handle, b"host_phased", phased)
    C.call("rc_tune_set", ctx.handle, b"host_chunk", 2)
    n, q = params.poly_degree, params.q_moduli()
    rng = np.random.default_rng(46 + phased)
    lv, count = 4, 7
    key = ctx.upload_keyswitch_key(_random_key(rng, params, lv + 1, True)[0], lv, 2)
    P = lambda arrs: (ctypes.c_void_p * count)(*[x.ctypes.data for x in arrs])
    LV = (ctypes.c_int32 * count)(*([lv] * count))
    SB = (ctypes.c_int32 * count)(*([40] * count))
    K = (ctypes.c_void_p * count)(*([key.handle] * count))
    def pinned(a):  # page-locked host memory, as the entry point expects (numpy view of a pinned tensor)
        return torch.from_numpy(np.ascontiguousarray(a).view(np.int64)).pin_memory().numpy().view(np.uint64)

    batches = []
    for _ in range(4):
        A = [pinned(rand_ct(rng, q, n)) for _ in range(count)]
        B = [pinned(rand_ct(rng, q, n)) for _ in range(count)]
        outs = [pinned(np.zeros((2, lv, n), dtype=np.uint64)) for _ in range(count)]
        batches.append((A, B, outs, (ctypes.c_int32 * count)()))
    s = C._stream()
    for A, B, outs, OSB in batches[:3]:
        C.call("rc_mult_relinearized_batch_host_async", ctx.handle, count, P(A), P(B), LV, SB, K, P(outs), OSB, s)
    C.call("rc_host_join", ctx.handle, s)
    torch.cuda.synchronize()
    A3, B3, _, OSB3 = batches[3]
    first = [o.copy() for o in batches[0][2]]
    C.call("rc_mult_relinearized_batch_host_async", ctx.handle, count, P(A3), P(B3), LV, SB, K, P(batches[0][2]),
           OSB3, s)
    C.call("rc_host_join", ctx.handle, s)
    torch.cuda.synchronize()
    results = [(batches[0][0], batches[0][1], first, batches[0][3])] + batches[1:3] + [(A3, B3, batches[0][2], OSB3)]
    for A, B, outs, OSB in results:
        for i in range(count):
            dev = ctx.mult_relinearized(C.RnsCiphertext(C.to_device(A[i]), 40), C.RnsCiphertext(C.to_device(B[i]), 40),
                                        key)
            assert np.array_equal(outs[i], dev.numpy()) and OSB[i] == dev.scale_bits


def test_precondition_errors_carry_reference_messages(C, pkg):
    params = pkg.params.hybrid_params(11, 4, 2, 50)
    ctx = C.RnsCkksContext(params)
    n, q = params.poly_degree, params.q_moduli()
    rng = np.random.default_rng(45)
    a = C.RnsCiphertext(C.to_device(rand_ct(rng, q, n)), 40)
    b = C.RnsCiphertext(C.to_device(rand_ct(rng, q[:3], n)), 40)
    with pytest.raises(C.RcError, match="same level to multiply"):
        ctx.mult(a, b)
    c = C.RnsCiphertext(C.to_device(rand_ct(rng, q, n)), 41)
    with pytest.raises(C.RcError, match="same scale to add"):
        ctx.add(a, c)
    key = ctx.upload_keyswitch_key(_random_key(rng, params, 3, True)[0], 2, 2)
    with pytest.raises(C.RcError, match="keyswitch key level must match the active Q chain"):
        ctx.relinearize(C.RnsQuadraticCiphertext(C.to_device(rand_ct(rng, q, n, 3)), 80), key)
    with pytest.raises(C.RcError, match="rescale requires at least two levels"):
        ctx.rescale(C.RnsCiphertext(C.to_device(rand_ct(rng, q[:1], n)), 40))
    with pytest.raises(C.RcError, match="distinct from the ciphertext modulus chain"):
        P = pkg.params
        C.RnsCkksContext(P.RnsCkksParams(8, [P.RnsPrime(998_244_353, 3)], [P.RnsPrime(998_244_353, 3)], 30))


def test_encode_decode_matches_oracle(C, pkg, oracle):
    params = pkg.params.plain_small_params()
    ctx = C.RnsCkksContext(params)
    n = params.poly_degree
    rng = np.random.default_rng(7)
    slots = rng.uniform(-1, 1, n // 2) + 1j * rng.uniform(-1, 1, n // 2)
    got = ctx.encode_host(slots, len(params.primes) - 1, 40)
    ref = oracle.poly_from_bigint_coeffs(params.q_moduli(), oracle.encode_integer_coeffs(n, 2.0 ** 40, slots))
    assert np.array_equal(got, ref)
    back = ctx.decode_host(got, 40)
    ref_back = oracle.decode_integer_coeffs(n, 2.0 ** 40, params.q_moduli(), ref)
    assert np.max(np.abs(back - ref_back)) <= 1e-12
    assert np.max(np.abs(back - slots)) <= 1e-6


@pytest.mark.parametrize("log_n,limbs,aux", [(12, 5, 2), (13, 4, 0), (14, 6, 2), (12, 4, 1), (12, 4, 3)])
def test_wide_and_standard_key_products_agree(C, pkg, oracle, monkeypatch, log_n, limbs, aux):
    """The exact integer key product (two internal primes) and the per-limb
    product give the same residues, equal to the oracle's."""
    params = pkg.params.hybrid_params(log_n, limbs, aux, 50) if aux else pkg.params.RnsCkksParams(
        1 << log_n, [pkg.params.RnsPrime(*x) for x in pkg.params.find_ntt_primes(1 << log_n, 50, limbs)], [], 40)
    n, q = params.poly_degree, params.q_moduli()
    rng = np.random.default_rng(log_n * 7 + limbs)
    key, D = _random_key(rng, params, len(q), aux > 0)
    a, b = rand_ct(rng, q, n), rand_ct(rng, q, n)
    outs = []
    for wide in ("1", "0"):
        monkeypatch.setenv("RNSCKKS_WIDE", wide)
        ctx = C.RnsCkksContext(params)
        ksk = ctx.upload_keyswitch_key(key, len(q) - 1, aux)
        out = ctx.mult_relinearized(C.RnsCiphertext(C.to_device(a), 40), C.RnsCiphertext(C.to_device(b), 40), ksk)
        outs.append(out.numpy())
    qpl = oracle.Plans(n, params.primes)
    ppl = oracle.Plans(n, params.aux_primes) if aux else None
    m0, m1 = oracle.mult_relinearized(qpl, ppl, a[0], a[1], b[0], b[1], key, D)
    for o in outs:
        assert np.array_equal(o[0], m0) and np.array_equal(o[1], m1)
