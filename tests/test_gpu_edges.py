"""Edge cases of the batch entry points: empty batches, batches larger than one launch, the lowest level,
and plaintext sums past one pass of the multiply-accumulate."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # collected on CPU-only machines, never run there
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

from test_gpu_parity import _random_key, rand_ct  # noqa: E402


@pytest.fixture(scope="module")
def C(pkg):
    pkg.lib()
    from rnsckks_gb300 import context as C
    return C


@pytest.fixture(scope="module")
def small(pkg, C):
    params = pkg.params.hybrid_params(12, 4, 2, 50)
    return params, C.RnsCkksContext(params)


def test_empty_batches_are_no_ops(C, small):
    params, ctx = small
    one = (C.RcCiphertext * 1)()
    ptrs = (ctypes.c_void_p * 1)()
    i32 = (ctypes.c_int32 * 1)()
    s = C._stream()
    h = ctx.handle
    C.call("rc_mult_relinearized_batch", h, 0, one, one, ptrs, one, s)
    C.call("rc_relinearize_batch", h, 0, one, ptrs, one, s)
    C.call("rc_rotate_batch", h, 0, one, ptrs, one, s)
    C.call("rc_relinearize_rescale_batch", h, 0, one, ptrs, one, s)
    C.call("rc_add_batch", h, 0, one, one, one, s)
    C.call("rc_rescale_batch", h, 0, one, one, s)
    C.call("rc_multiply_plain_rns_batch", h, 0, one, ptrs, one, s)
    C.call("rc_mult_relinearized_batch_host", h, 0, ptrs, ptrs, i32, i32, ptrs, ptrs, i32, s)
    coeffs = np.zeros(4)
    C.call("rc_total_sum_batch", h, 0, one, 4, ptrs, 1, one, s)
    C.call("rc_halevi_shoup_batch", h, 0, one, coeffs.ctypes.data, 4, ptrs, 1, one, s)
    C.call("rc_paterson_stockmeyer_batch", h, 0, one, coeffs.ctypes.data, 4, ptrs, 1, one, s)
    C.call("rc_bsgs_apply_batch", h, 0, one, 4, 2, ptrs, 2, 3, 40, ptrs, ptrs, one, s)
    torch.cuda.synchronize()
    assert ctx.mult_relinearized_batch([], [], []) == []
    from rnsckks_gb300 import algorithms as A
    assert A.total_sum_native(ctx, [], 4, {}) == []
    assert A.apply_diagonal_linear_transform_native(ctx, [], None, None) == []


def test_batch_beyond_one_launch_equals_per_op(C, small):
    """70 jobs: more than one key-product launch (32 jobs) and more than one tensor chunk (16 jobs)."""
    params, ctx = small
    n, q = params.poly_degree, params.q_moduli()
    rng = np.random.default_rng(70)
    key = ctx.upload_keyswitch_key(_random_key(rng, params, len(q), True)[0], len(q) - 1, 2)
    lhs = [C.RnsCiphertext(C.to_device(rand_ct(rng, q, n)), 40) for _ in range(70)]
    rhs = [C.RnsCiphertext(C.to_device(rand_ct(rng, q, n)), 40) for _ in range(70)]
    batch = ctx.mult_relinearized_batch(lhs, rhs, [key] * 70)
    for i in (0, 31, 32, 47, 63, 64, 69):
        single = ctx.mult_relinearized(lhs[i], rhs[i], key)
        assert np.array_equal(single.numpy(), batch[i].numpy())


def test_lowest_level_matches_oracle(C, small, oracle):
    """mult_relinearized from two limbs down to one, and a keyswitch at one limb, against the oracle."""
    params, ctx = small
    n = params.poly_degree
    rng = np.random.default_rng(2)
    qpl = oracle.Plans(n, params.primes).prefix(2)
    ppl = oracle.Plans(n, params.aux_primes)
    q = params.q_moduli()[:2]
    key, D = _random_key(rng, params, 2, True)
    ksk = ctx.upload_keyswitch_key(key, 1, 2)
    a, b = rand_ct(rng, q, n), rand_ct(rng, q, n)
    out = ctx.mult_relinearized(C.RnsCiphertext(C.to_device(a), 35), C.RnsCiphertext(C.to_device(b), 35), ksk)
    m0, m1 = oracle.mult_relinearized(qpl, ppl, a[0], a[1], b[0], b[1], key, D)
    assert out.level == 0
    assert np.array_equal(out.numpy()[0], m0) and np.array_equal(out.numpy()[1], m1)
    qpl1 = oracle.Plans(n, params.primes).prefix(1)
    key1, D1 = _random_key(rng, params, 1, True)
    ksk1 = ctx.upload_keyswitch_key(key1, 0, 2)
    x = rand_ct(rng, params.q_moduli()[:1], n, 1)[0]
    ks = ctx.keyswitch(C.RnsPolynomial(C.to_device(x)), ksk1)
    r0, r1 = oracle.keyswitch(qpl1, ppl, x, key1, D1)
    assert np.array_equal(ks.numpy()[0], r0) and np.array_equal(ks.numpy()[1], r1)


def test_plain_accumulate_past_one_pass_equals_sum_of_products(C, small):
    """40 terms: three passes of the 16-term multiply-accumulate, against mult_plain + add term by term."""
    params, ctx = small
    n, q = params.poly_degree, params.q_moduli()
    rng = np.random.default_rng(40)
    cts = [C.RnsCiphertext(C.to_device(rand_ct(rng, q, n)), 40) for _ in range(40)]
    plains = [C.to_device(np.stack([rng.integers(0, m, n, dtype=np.uint64) for m in q])) for _ in range(40)]
    out = torch.zeros((2, len(q), n), dtype=torch.int64, device="cuda")
    CT = (C.RcCiphertext * 40)(*[c.raw() for c in cts])
    PT = (ctypes.c_void_p * 40)(*[p.data_ptr() for p in plains])
    O = C.RcCiphertext(out.data_ptr(), 0, 0)
    C.call("rc_mult_plain_accumulate", ctx.handle, 40, CT, 0, PT, 0, ctypes.byref(O), C._stream())
    want = None
    for c, p in zip(cts, plains):
        term = ctx.multiply_plain_rns(c, C.RnsPolynomial(p))
        want = term if want is None else want.add(term)
    assert np.array_equal(C.to_host(out), want.numpy())


def _rot_keys(C, ctx, params, rng, gals):
    q = params.q_moduli()
    key = _random_key(rng, params, len(q), True)[0]
    return [C.RnsRotationKey(g, ctx.upload_keyswitch_key(key, len(q) - 1, 2, g)) for g in gals]


def test_hoisted_rotations_equal_ordinary_rotations(C, small):
    """rc_rotate_hoisted (one decomposition per ciphertext, the automorphism applied to its digit transforms)
    against rc_rotate for steps 1, 2, 5, -1, -7 and the conjugation, three ciphertexts."""
    params, ctx = small
    n, q = params.poly_degree, params.q_moduli()
    rng = np.random.default_rng(5)
    gals = [ctx.galois_element_for_rotation(st) for st in (1, 2, 5, -1, -7)] + [ctx.conjugation_galois_element()]
    keys = _rot_keys(C, ctx, params, rng, gals)
    cts = [C.RnsCiphertext(C.to_device(rand_ct(rng, q, n)), 40) for _ in range(3)]
    got = ctx.rotate_hoisted(cts, keys)
    for i, ct in enumerate(cts):
        for r, k in enumerate(keys):
            want = ctx.rotate(ct, k)
            assert (got[i][r].level, got[i][r].scale_bits) == (want.level, want.scale_bits)
            assert np.array_equal(got[i][r].numpy(), want.numpy()), (i, r)


def test_hoisted_rotation_of_a_balanced_digit_tie(C, small):
    """Coefficients whose centred value has a base-2^30 digit at exactly 2^29 (the balanced rule's tie, where
    the digits of -X are not the negated digits of X) moved with a sign flip by the conjugation: the hoisted
    call must still equal the ordinary rotation."""
    params, ctx = small
    n, q = params.poly_degree, params.q_moduli()
    rng = np.random.default_rng(6)
    keys = _rot_keys(C, ctx, params, rng, [ctx.conjugation_galois_element(), ctx.galois_element_for_rotation(3)])
    a = rand_ct(rng, q, n)
    for j, X in ((1, 1 << 29), (2, (1 << 29) + (5 << 30)), (3, -(1 << 29)), (7, 3 << 59)):
        for limb, m in enumerate(q):
            a[1][limb][j] = X % m
    cts = [C.RnsCiphertext(C.to_device(a), 40), C.RnsCiphertext(C.to_device(rand_ct(rng, q, n)), 40)]
    got = ctx.rotate_hoisted(cts, keys)
    for i, ct in enumerate(cts):
        for r, k in enumerate(keys):
            assert np.array_equal(got[i][r].numpy(), ctx.rotate(ct, k).numpy()), (i, r)


def test_hoisted_rotations_fall_back_where_they_cannot_hoist(C, pkg):
    """A ring below the wide key product's sizes (N=2^11) and a batch of mixed levels run as ordinary
    rotations with the same results."""
    params = pkg.params.hybrid_params(11, 3, 2, 50)
    ctx = C.RnsCkksContext(params)
    n, q = params.poly_degree, params.q_moduli()
    rng = np.random.default_rng(11)
    keys = _rot_keys(C, ctx, params, rng, [ctx.galois_element_for_rotation(1), ctx.conjugation_galois_element()])
    cts = [C.RnsCiphertext(C.to_device(rand_ct(rng, q, n)), 40) for _ in range(2)]
    got = ctx.rotate_hoisted(cts, keys)
    for i, ct in enumerate(cts):
        for r, k in enumerate(keys):
            assert np.array_equal(got[i][r].numpy(), ctx.rotate(ct, k).numpy())
    params2 = pkg.params.hybrid_params(12, 4, 2, 50)
    ctx2 = C.RnsCkksContext(params2)
    q2 = params2.q_moduli()
    low = C.RnsCiphertext(C.to_device(rand_ct(rng, q2[:3], params2.poly_degree)), 40)
    top = C.RnsCiphertext(C.to_device(rand_ct(rng, q2, params2.poly_degree)), 40)
    with pytest.raises(Exception, match="rotation key level must match the ciphertext level"):
        ctx2.rotate_hoisted([top, low], _rot_keys(C, ctx2, params2, rng, [ctx2.galois_element_for_rotation(1)]))


def test_key_products_report_no_copy_timeouts(C, small):
    """The key product's bulk copies complete within the kernel's bounded wait (the device flag stays 0)."""
    params, ctx = small
    n, q = params.poly_degree, params.q_moduli()
    rng = np.random.default_rng(9)
    key = ctx.upload_keyswitch_key(_random_key(rng, params, len(q), True)[0], len(q) - 1, 2)
    cts = [C.RnsCiphertext(C.to_device(rand_ct(rng, q, n)), 40) for _ in range(9)]
    ctx.mult_relinearized_batch(cts, cts[::-1], [key] * 9)
    flags = ctypes.c_int32(-1)
    C.call("rc_kernel_errors", ctypes.byref(flags), 1)
    assert flags.value == 0


def test_key_product_wait_that_runs_out_raises_the_flag_and_recovers(C, small):
    """The key product's first wait for its staged digit transforms is bounded.  A poll limit of 0 makes every
    CTA give up at once: the CTA drains its copies (the second wait keeps its full bound, so nothing is left in
    flight), raises the device flag and writes nothing.  rc_kernel_errors reports the flag, clearing it works,
    and with the limit restored the same batch is bit-exact again."""
    params, ctx = small
    n, q = params.poly_degree, params.q_moduli()
    rng = np.random.default_rng(77)
    key = ctx.upload_keyswitch_key(_random_key(rng, params, len(q), True)[0], len(q) - 1, 2)
    cts = [C.RnsCiphertext(C.to_device(rand_ct(rng, q, n)), 40) for _ in range(3)]
    flags = ctypes.c_int32(-1)
    C.call("rc_kernel_errors", ctypes.byref(flags), 1)
    assert flags.value == 0
    ref = [o.numpy() for o in ctx.mult_relinearized_batch(cts, cts[::-1], [key] * 3)]
    default = ctypes.c_int32(0)
    C.call("rc_tune_get", ctx.handle, b"mac_wait_polls", ctypes.byref(default))
    assert default.value == 1 << 22
    C.call("rc_tune_set", ctx.handle, b"mac_wait_polls", 0)
    try:
        ctx.mult_relinearized_batch(cts, cts[::-1], [key] * 3)
        torch.cuda.synchronize()
    finally:
        C.call("rc_tune_set", ctx.handle, b"mac_wait_polls", default.value)
    C.call("rc_kernel_errors", ctypes.byref(flags), 0)
    assert flags.value == 1
    C.call("rc_kernel_errors", ctypes.byref(flags), 1)  # read and clear
    assert flags.value == 1
    C.call("rc_kernel_errors", ctypes.byref(flags), 0)
    assert flags.value == 0
    got = [o.numpy() for o in ctx.mult_relinearized_batch(cts, cts[::-1], [key] * 3)]
    C.call("rc_kernel_errors", ctypes.byref(flags), 1)
    assert flags.value == 0
    for g, r in zip(got, ref):
        assert np.array_equal(g, r)
    with pytest.raises(C.RcError, match="mac_wait_polls must be in"):
        C.call("rc_tune_set", ctx.handle, b"mac_wait_polls", -1)


def test_nvtx_ranges_leave_results_unchanged(C, small):
    """With NVTX ranges on (per entry point and per kernel launch), also inside a captured graph, the residues
    are the same as with instrumentation off."""
    params, ctx = small
    n, q = params.poly_degree, params.q_moduli()
    rng = np.random.default_rng(78)
    key = ctx.upload_keyswitch_key(_random_key(rng, params, len(q), True)[0], len(q) - 1, 2)
    cts = [C.RnsCiphertext(C.to_device(rand_ct(rng, q, n)), 40) for _ in range(2)]
    lib = C.lib()
    ref = [o.numpy() for o in ctx.mult_relinearized_batch(cts, cts[::-1], [key] * 2)]
    try:
        assert lib.rc_profile_enable(2) == 0
        got = [o.numpy() for o in ctx.mult_relinearized_batch(cts, cts[::-1], [key] * 2)]
        side = torch.cuda.Stream()
        with torch.cuda.stream(side):
            ctx.reserve(len(q) - 1, 2)
            outs = [torch.zeros((2, len(q) - 1, n), dtype=torch.int64, device="cuda") for _ in range(2)]
            quads = [ctx.mult(a, b) for a, b in zip(cts, cts[::-1])]
            graph = ctx.capture_graph(lambda: ctx.relinearize_rescale_batch(quads, [key] * 2, outs))
            graph.launch()
            side.synchronize()
            direct = ctx.relinearize_rescale_batch(quads, [key] * 2)
            side.synchronize()
    finally:
        lib.rc_profile_enable(0)
    torch.cuda.synchronize()
    for g, r in zip(got, ref):
        assert np.array_equal(g, r)
    for o, d in zip(outs, direct):
        assert torch.equal(o, d.data)


def test_hoisted_rotations_past_one_launch(C, small):
    """34 ciphertexts: two chunks of the hoisted path (32 jobs per key-product launch)."""
    params, ctx = small
    n, q = params.poly_degree, params.q_moduli()
    rng = np.random.default_rng(34)
    keys = _rot_keys(C, ctx, params, rng, [ctx.galois_element_for_rotation(s) for s in (1, -3)])
    cts = [C.RnsCiphertext(C.to_device(rand_ct(rng, q, n)), 40) for _ in range(34)]
    got = ctx.rotate_hoisted(cts, keys)
    for i in (0, 31, 32, 33):
        for r, k in enumerate(keys):
            assert np.array_equal(got[i][r].numpy(), ctx.rotate(cts[i], k).numpy()), (i, r)
