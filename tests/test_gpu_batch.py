"""Mixed-level batched relinearize+rescale and CUDA-graph capture of library calls, bit-exact against the
per-op path and the oracle (relinearize: context/ops.rs:111-122, rescale: context/ops.rs:32-37)."""
import ctypes
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # collected on CPU-only machines, never run there
    pytest.skip("needs a CUDA GPU", allow_module_level=True)


@pytest.fixture(scope="module")
def env(pkg, oracle):
    pkg.lib()
    from rnsckks_gb300 import context as C
    params = pkg.params.hybrid_params(12, 8, 2, 50)
    ctx = C.RnsCkksContext(params)
    q, p = params.q_moduli(), params.p_moduli()
    rng = np.random.default_rng(77)
    keys, host_keys = {}, {}
    for lv in range(1, len(q)):
        qm = q[: lv + 1]
        D = math.ceil(math.prod(qm).bit_length() / 30)
        k = np.stack([np.stack([np.stack([rng.integers(0, m, params.poly_degree, dtype=np.uint64)
                                          for m in qm + p]) for _ in range(2)]) for _ in range(D)])
        host_keys[lv] = k
        keys[lv] = ctx.upload_keyswitch_key(k, lv, len(p))
    return C, ctx, params, keys, host_keys, oracle


def _quad(C, rng, params, level, scale_bits=80):
    q = params.q_moduli()[: level + 1]
    d = np.stack([np.stack([rng.integers(0, m, params.poly_degree, dtype=np.uint64) for m in q]) for _ in range(3)])
    return C.RnsQuadraticCiphertext(C.to_device(d), scale_bits), d


def test_relinearize_rescale_batch_mixed_levels(env):
    C, ctx, params, keys, host_keys, O = env
    rng = np.random.default_rng(5)
    levels = [int(x) for x in rng.integers(1, 8, 21)]
    cts, raw = zip(*[_quad(C, rng, params, lv, 60 + lv) for lv in levels])
    outs = ctx.relinearize_rescale_batch(list(cts), [keys[lv] for lv in levels])
    for ct, out, lv in zip(cts, outs, levels):
        ref = ctx.rescale(ctx.relinearize(ct, keys[lv]))
        assert out.level == lv - 1 == ref.level and out.scale_bits == ref.scale_bits
        assert np.array_equal(out.numpy(), ref.numpy())
    # one job against the oracle: relinearize then rescale of both components
    i = int(np.argmax(levels))
    lv = levels[i]
    qpl = O.Plans(params.poly_degree, params.primes[: lv + 1])
    ppl = O.Plans(params.poly_degree, params.aux_primes)
    d = raw[i]
    r0, r1 = O.relinearize(qpl, ppl, d[0], d[1], d[2], host_keys[lv], host_keys[lv].shape[0])
    h = outs[i].numpy()
    assert np.array_equal(h[0], O.rescale_poly(qpl, r0)) and np.array_equal(h[1], O.rescale_poly(qpl, r1))
    assert outs[i].scale_bits == max(0, 60 + lv - (params.q_moduli()[lv].bit_length() - 1))


def test_graph_capture_replays_the_batch(env):
    C, ctx, params, keys, host_keys, O = env
    rng = np.random.default_rng(6)
    levels = [7, 3, 5, 7, 2, 6, 4, 7, 1]
    cts = [_quad(C, rng, params, lv)[0] for lv in levels]
    ks = [keys[lv] for lv in levels]
    side = torch.cuda.Stream()
    with torch.cuda.stream(side):
        ctx.reserve(7, 16)
        outs = [torch.zeros((2, lv, params.poly_degree), dtype=torch.int64, device="cuda") for lv in levels]
        direct = [r.data.clone() for r in ctx.relinearize_rescale_batch(cts, ks, [o.clone() for o in outs])]
        graph = ctx.capture_graph(lambda: ctx.relinearize_rescale_batch(cts, ks, outs))
        for o in outs:
            o.zero_()
        graph.launch()
        side.synchronize()
        for o, d in zip(outs, direct):
            assert torch.equal(o, d)
        # the graph reads the captured buffers: new contents give the new result
        fresh = _quad(C, rng, params, levels[0])[0]
        cts[0].data.copy_(fresh.data)
        graph.launch()
        side.synchronize()
        expect = ctx.rescale(ctx.relinearize(cts[0], ks[0]))
        assert np.array_equal(C.to_host(outs[0]), expect.numpy())
    torch.cuda.synchronize()


def test_graph_capture_refuses_to_grow_scratch(env):
    C, ctx, params, keys, host_keys, O = env
    rng = np.random.default_rng(7)
    ct = _quad(C, rng, params, 7)[0]
    side = torch.cuda.Stream()  # a stream with no reserved scratch
    with torch.cuda.stream(side):
        with pytest.raises(C.RcError, match="reserved"):
            ctx.capture_graph(lambda: ctx.relinearize_rescale_batch([ct], [keys[7]]))
    torch.cuda.synchronize()
    with pytest.raises(C.RcError, match="non-default stream"):
        ctx.capture_graph(lambda: None)


def test_fused_and_unfused_tensor_agree(env):
    C, ctx, params, keys, host_keys, O = env
    rng = np.random.default_rng(9)
    q, n = params.q_moduli(), params.poly_degree
    mk = lambda: C.RnsCiphertext(C.to_device(np.stack([np.stack([rng.integers(0, m, n, dtype=np.uint64) for m in q])
                                                       for _ in range(2)])), 40)
    a, b = [mk() for _ in range(5)], [mk() for _ in range(5)]
    import ctypes
    got = {}
    for fuse in (0, 1):
        C.call("rc_tune_set", ctx.handle, b"fuse_tensor", fuse)
        got[fuse] = ([x.numpy() for x in ctx.mult_relinearized_batch(a, b, [keys[len(q) - 1]] * 5)],
                     ctx.mult(a[0], b[0]).numpy())
    C.call("rc_tune_set", ctx.handle, b"fuse_tensor", 1)
    for u, v in zip(got[0][0], got[1][0]):
        assert np.array_equal(u, v)
    assert np.array_equal(got[0][1], got[1][1])


def test_add_and_multiply_plain_batches_equal_single_calls(env):
    C, ctx, params, keys, host_keys, O = env
    rng = np.random.default_rng(10)
    q, n = params.q_moduli(), params.poly_degree
    levels = [3, 6, 3, 7, 1]
    mk = lambda lv: C.RnsCiphertext(C.to_device(np.stack([np.stack([rng.integers(0, m, n, dtype=np.uint64)
                                                                      for m in q[: lv + 1]]) for _ in range(2)])), 33)
    a, b = [mk(lv) for lv in levels], [mk(lv) for lv in levels]
    pts = [C.RnsPolynomial(C.to_device(np.stack([rng.integers(0, m, n, dtype=np.uint64) for m in q[: lv + 1]])))
           for lv in levels]
    for got, x, y in zip(ctx.add_batch(a, b), a, b):
        ref = ctx.add(x, y)
        assert np.array_equal(got.numpy(), ref.numpy()) and got.scale_bits == ref.scale_bits
    for got, x, p in zip(ctx.multiply_plain_rns_batch(a, pts), a, pts):
        ref = ctx.multiply_plain_rns(x, p)
        assert np.array_equal(got.numpy(), ref.numpy()) and got.scale_bits == 33
    with pytest.raises(C.RcError, match="same scale to add"):
        ctx.add_batch([a[0]], [C.RnsCiphertext(b[0].data, 34)])


def test_one_graph_spans_ring_degrees(env, pkg):
    """Jobs of uneven ring degree and level in one replayable launch: the batched calls of two contexts
    (N = 2^12 and N = 2^13) captured into one CUDA graph on one stream; the replay equals the direct calls."""
    C, ctx, params, keys, host_keys, O = env
    params2 = pkg.params.hybrid_params(13, 6, 2, 50)
    ctx2 = C.RnsCkksContext(params2)
    q2, p2 = params2.q_moduli(), params2.p_moduli()
    rng = np.random.default_rng(8)
    keys2 = {}
    for lv in (3, 5):
        D = math.ceil(math.prod(q2[: lv + 1]).bit_length() / 30)
        k = np.stack([np.stack([np.stack([rng.integers(0, m, params2.poly_degree, dtype=np.uint64)
                                          for m in q2[: lv + 1] + p2]) for _ in range(2)]) for _ in range(D)])
        keys2[lv] = ctx2.upload_keyswitch_key(k, lv, len(p2))
    lv1, lv2 = [7, 2, 5], [5, 3, 5]
    cts1 = [_quad(C, rng, params, lv)[0] for lv in lv1]
    cts2 = [_quad(C, rng, params2, lv)[0] for lv in lv2]
    side = torch.cuda.Stream()
    with torch.cuda.stream(side):
        ctx.reserve(7, 8)
        ctx2.reserve(5, 8)
        o1 = [torch.zeros((2, lv, params.poly_degree), dtype=torch.int64, device="cuda") for lv in lv1]
        o2 = [torch.zeros((2, lv, params2.poly_degree), dtype=torch.int64, device="cuda") for lv in lv2]
        d1 = [r.data.clone() for r in ctx.relinearize_rescale_batch(cts1, [keys[lv] for lv in lv1])]
        d2 = [r.data.clone() for r in ctx2.relinearize_rescale_batch(cts2, [keys2[lv] for lv in lv2])]

        def both():
            ctx.relinearize_rescale_batch(cts1, [keys[lv] for lv in lv1], o1)
            ctx2.relinearize_rescale_batch(cts2, [keys2[lv] for lv in lv2], o2)
        graph = ctx.capture_graph(both)
        graph.launch()
        side.synchronize()
        for o, d in zip(o1 + o2, d1 + d2):
            assert torch.equal(o, d)
    torch.cuda.synchronize()


def test_mixed_levels_run_one_launch_per_pass(env):
    """A batch of seven levels runs each pass of the key switch (decompose, digit transforms, key product,
    inverse transforms, finalize) as one launch over all levels; its residues equal the level-by-level path
    (mixed_levels off) and the per-op path, also when the batch is cut into chunks of 5 jobs."""
    import ctypes
    import json
    C, ctx, params, keys, host_keys, O = env
    rng = np.random.default_rng(55)
    levels = [int(x) for x in rng.integers(1, 8, 23)]
    assert len(set(levels)) >= 5
    cts = [_quad(C, rng, params, lv)[0] for lv in levels]
    ks = [keys[lv] for lv in levels]
    lib = C.lib()
    buf = ctypes.create_string_buffer(1 << 16)
    torch.cuda.synchronize()
    lib.rc_profile_enable(1)
    lib.rc_profile_report(buf, len(buf))  # reset
    mixed = [o.numpy() for o in ctx.relinearize_rescale_batch(cts, ks)]
    lib.rc_profile_report(buf, len(buf))
    lib.rc_profile_enable(0)
    prof = json.loads(buf.value.decode())
    for name in ("decompose", "wide_digit_ntt", "wide_mac", "wide_inv_rows", "wide_inv_cols", "finalize"):
        assert prof[name]["launches"] == 1, (name, prof)
    plain = [o.numpy() for o in ctx.relinearize_batch(cts, ks)]
    try:
        C.call("rc_tune_set", ctx.handle, b"mixed_levels", 0)
        by_level = [o.numpy() for o in ctx.relinearize_rescale_batch(cts, ks)]
        plain_by_level = [o.numpy() for o in ctx.relinearize_batch(cts, ks)]
        C.call("rc_tune_set", ctx.handle, b"mixed_levels", 1)
        C.call("rc_tune_set", ctx.handle, b"ml_jobs", 5)
        chunked = [o.numpy() for o in ctx.relinearize_rescale_batch(cts, ks)]
    finally:
        C.call("rc_tune_set", ctx.handle, b"mixed_levels", 1)
        C.call("rc_tune_set", ctx.handle, b"ml_jobs", 128)
    for i, lv in enumerate(levels):
        assert np.array_equal(mixed[i], by_level[i]), i
        assert np.array_equal(mixed[i], chunked[i]), i
        assert np.array_equal(plain[i], plain_by_level[i]), i
    for i in (0, int(np.argmin(levels))):
        assert np.array_equal(mixed[i], ctx.rescale(ctx.relinearize(cts[i], ks[i])).numpy())


def test_mixed_levels_with_q_only_keys(pkg, oracle):
    """The one-launch-per-pass form with Q-only keys (no aux basis; the digit count is the key's) on the plain
    small chain (N=2^13, 60 + 41 + 41 bits): equal to the level-by-level form, to the per-op path and, for one
    job, to the oracle's relinearize then rescale."""
    import ctypes
    import json
    from rnsckks_gb300 import context as C
    params = pkg.params.plain_small_params()
    ctx = C.RnsCkksContext(params)
    n, q = params.poly_degree, params.q_moduli()
    rng = np.random.default_rng(91)
    keys, host = {}, {}
    for lv in (1, 2):
        qm = q[: lv + 1]
        D = math.ceil(math.prod(qm).bit_length() / 30)
        k = np.stack([np.stack([np.stack([rng.integers(0, m, n, dtype=np.uint64) for m in qm])
                                for _ in range(2)]) for _ in range(D)])
        host[lv] = k
        keys[lv] = ctx.upload_keyswitch_key(k, lv, 0)
    levels = [2, 1, 2, 1, 1, 2]
    raw = [np.stack([np.stack([rng.integers(0, m, n, dtype=np.uint64) for m in q[: lv + 1]]) for _ in range(3)])
           for lv in levels]
    cts = [C.RnsQuadraticCiphertext(C.to_device(r), 80) for r in raw]
    ks = [keys[lv] for lv in levels]
    lib = C.lib()
    buf = ctypes.create_string_buffer(1 << 16)
    torch.cuda.synchronize()
    lib.rc_profile_enable(1)
    lib.rc_profile_report(buf, len(buf))
    mixed = [o.numpy() for o in ctx.relinearize_rescale_batch(cts, ks)]
    lib.rc_profile_report(buf, len(buf))
    lib.rc_profile_enable(0)
    assert json.loads(buf.value.decode())["wide_mac"]["launches"] == 1
    try:
        C.call("rc_tune_set", ctx.handle, b"mixed_levels", 0)
        by_level = [o.numpy() for o in ctx.relinearize_rescale_batch(cts, ks)]
    finally:
        C.call("rc_tune_set", ctx.handle, b"mixed_levels", 1)
    for i in range(len(levels)):
        assert np.array_equal(mixed[i], by_level[i]), i
        assert np.array_equal(mixed[i], ctx.rescale(ctx.relinearize(cts[i], ks[i])).numpy()), i
    lv = levels[0]
    qpl = oracle.Plans(n, params.primes[: lv + 1])
    d = raw[0]
    r0, r1 = oracle.relinearize(qpl, None, d[0], d[1], d[2], host[lv], host[lv].shape[0])
    assert np.array_equal(mixed[0][0], oracle.rescale_poly(qpl, r0))
    assert np.array_equal(mixed[0][1], oracle.rescale_poly(qpl, r1))


def test_persistent_key_product_matches_the_per_tile_form(env):
    """The persistent key product (one CTA per SM taking (tile, limb) units, the next tile's digit transforms
    copied while the current one is used) gives the residues of the one-CTA-per-tile form: ragged job groups
    (11 jobs in groups of 8 and of 4), fewer limbs than the CTA has warps (6 limbs at level 3), and the hoisted
    rotation's permuted digit tiles; the batch also equals the per-op calls."""
    C, ctx, params, keys, host_keys, O = env
    n, q, p = params.poly_degree, params.q_moduli(), params.p_moduli()
    rng = np.random.default_rng(91)

    def lin(lv):
        return C.RnsCiphertext(C.to_device(np.stack([np.stack([rng.integers(0, m, n, dtype=np.uint64)
                                                               for m in q[: lv + 1]]) for _ in range(2)])), 40)

    g = 5  # rotation by one slot
    rk = {}
    for lv in (7, 3):
        k = np.stack([np.stack([np.stack([rng.integers(0, m, n, dtype=np.uint64) for m in q[: lv + 1] + p])
                                for _ in range(2)]) for _ in range(host_keys[lv].shape[0])])
        rk[lv] = C.RnsRotationKey(g, ctx.upload_keyswitch_key(k, lv, len(p), g))
    cases = {lv: ([lin(lv) for _ in range(11)], [lin(lv) for _ in range(11)]) for lv in (7, 3)}

    def run():
        out = {}
        for lv, (a, b) in cases.items():
            out[("mult", lv)] = [o.numpy() for o in ctx.mult_relinearized_batch(a, b, [keys[lv]] * len(a))]
            out[("rot", lv)] = [o.numpy() for row in ctx.rotate_hoisted(a, [rk[lv]]) for o in row]
        return out

    old = {}
    for name in ("mac_persistent", "mac_bc"):
        v = ctypes.c_int32()
        C.call("rc_tune_get", ctx.handle, name.encode(), ctypes.byref(v))
        old[name] = v.value
    try:
        results = {}
        for bc in (8, 4):
            for pers in (1, 0):
                C.call("rc_tune_set", ctx.handle, b"mac_bc", bc)
                C.call("rc_tune_set", ctx.handle, b"mac_persistent", pers)
                results[(bc, pers)] = run()
    finally:
        for name, v in old.items():
            C.call("rc_tune_set", ctx.handle, name.encode(), v)
    flags = ctypes.c_int32(-1)
    C.call("rc_kernel_errors", ctypes.byref(flags), 1)
    assert flags.value == 0
    ref = results[(8, 0)]
    for cfg, res in results.items():
        for k in ref:
            for x, y in zip(res[k], ref[k]):
                assert np.array_equal(x, y), (cfg, k)
    for lv, (a, b) in cases.items():
        for i in (0, 10):
            assert np.array_equal(ctx.mult_relinearized(a[i], b[i], keys[lv]).numpy(), ref[("mult", lv)][i])
            assert np.array_equal(ctx.rotate(a[i], rk[lv]).numpy(), ref[("rot", lv)][i])
