"""Autotuner: candidate enumeration, choice and the per-shape cache (CPU); tuning on the GPU leaves results
bit-identical and applies the chosen launch shapes."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def T(pkg):
    from rnsckks_gb300 import autotune
    return autotune


def test_candidates_cover_the_space(T):
    c = T.candidates({"a": (1, 2), "b": (3, 4, 5)})
    assert len(c) == 6 and {"a": 2, "b": 5} in c and all(set(x) == {"a", "b"} for x in c)


def test_choose_fastest_and_skip_failed(T):
    trials = [{"config": {"x": 1}, "ms": 3.0}, {"config": {"x": 2}, "ms": None}, {"config": {"x": 3}, "ms": 1.5},
              {"config": {"x": 4}, "ms": 1.5}]
    assert T.choose(trials)["config"] == {"x": 3}
    with pytest.raises(RuntimeError):
        T.choose([{"config": {}, "ms": None}])


def test_cache_round_trip(T, tmp_path):
    p = tmp_path / "sub" / "tune.json"
    k = T.shape_key("GB300", 65536, 24, 2, 23, 32, "mult_relinearized_batch")
    assert T.load_cache(p) == {}
    T.store_cache(p, k, {"choice": {"ks_jobs": 32}, "ms": 1.0})
    T.store_cache(p, "other", {"choice": {}, "ms": 2.0})
    data = T.load_cache(p)
    assert data[k]["choice"] == {"ks_jobs": 32} and "other" in data


@pytest.mark.gpu
def test_tuning_keeps_results_and_applies_choice(pkg, T, tmp_path):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    from rnsckks_gb300 import context as C
    params = pkg.params.hybrid_params(12, 6, 2, 50)
    ctx = C.RnsCkksContext(params)
    n, q, p = params.poly_degree, params.q_moduli(), params.p_moduli()
    rng = np.random.default_rng(3)
    D = ctx.decomp_digits(len(q) - 1)
    key = ctx.upload_keyswitch_key(np.stack([np.stack([np.stack([rng.integers(0, m, n, dtype=np.uint64)
                                                                 for m in q + p]) for _ in range(2)])
                                             for _ in range(D)]), len(q) - 1, len(p))
    mk = lambda: C.RnsCiphertext(C.to_device(np.stack([np.stack([rng.integers(0, m, n, dtype=np.uint64)
                                                                 for m in q]) for _ in range(2)])), 40)
    lhs, rhs = [mk() for _ in range(12)], [mk() for _ in range(12)]
    ref = [r.numpy() for r in ctx.mult_relinearized_batch(lhs, rhs, [key] * 12)]
    outs = [torch.empty((2, len(q) - 1, n), dtype=torch.int64, device="cuda") for _ in range(12)]
    rep = T.tune_mult_relinearized(ctx, lhs, rhs, [key] * 12, outs, reps=1, cache=tmp_path / "t.json")
    assert not rep["cached"] and T.current(ctx, rep["choice"]) == rep["choice"]
    assert len(rep["trials"]) == 32  # 4 x 2 x 2 x 2 candidates, all primes below 2^58
    # kernel shapes after that: 2 x 2 x 2 (column CTAs, row polynomials, persistent key product), times the
    # splits 6x6 only at N = 2^12
    assert len(rep["shape_trials"]) == 8 and set(rep["choice"]) >= {"col_ctas", "row_polys", "mac_persistent"}
    for o, r in zip(ctx.mult_relinearized_batch(lhs, rhs, [key] * 12), ref):
        assert np.array_equal(o.numpy(), r)
    again = T.tune_mult_relinearized(ctx, lhs, rhs, [key] * 12, outs, reps=1, cache=tmp_path / "t.json")
    assert again["cached"] and again["choice"] == rep["choice"]
    with pytest.raises(C.RcError, match="unknown tunable"):
        T.apply(ctx, {"nope": 1})
    with pytest.raises(C.RcError, match="ks_jobs must be"):
        T.apply(ctx, {"ks_jobs": 65})
    with pytest.raises(C.RcError, match="ntt_split must leave"):
        T.apply(ctx, {"ntt_split": 7})  # 2^12 = 2^7 x 2^5: the row phase would be below 2^6


def test_split_candidates(T):
    assert T.split_candidates(16) == [8]
    assert T.split_candidates(15) == [7, 8]
    assert T.split_candidates(14) == [6, 7, 8]
    assert T.split_candidates(13) == [6, 7]
    assert T.split_candidates(12) == [6]


@pytest.mark.gpu
def test_every_kernel_shape_gives_the_same_residues(pkg, T):
    """Each four-step split at N = 2^14 and 2^15, each column-pass CTA count and row-block size: the NTT round
    trip, its forward output and a relinearized product are identical to the default shape's."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    from rnsckks_gb300 import context as C
    for log_n in (14, 15):
        params = pkg.params.hybrid_params(log_n, 4, 2, 50)
        ctx = C.RnsCkksContext(params)
        n, q, p = params.poly_degree, params.q_moduli(), params.p_moduli()
        rng = np.random.default_rng(log_n)
        D = ctx.decomp_digits(len(q) - 1)
        key = ctx.upload_keyswitch_key(np.stack([np.stack([np.stack([rng.integers(0, m, n, dtype=np.uint64)
                                                                     for m in q + p]) for _ in range(2)])
                                                 for _ in range(D)]), len(q) - 1, len(p))
        mk = lambda: C.RnsCiphertext(C.to_device(np.stack([np.stack([rng.integers(0, m, n, dtype=np.uint64)
                                                                     for m in q]) for _ in range(2)])), 40)
        lhs, rhs = [mk() for _ in range(3)], [mk() for _ in range(3)]
        polys = np.stack([np.stack([rng.integers(0, m, n, dtype=np.uint64) for m in q]) for _ in range(20)])

        def run():
            d = C.to_device(polys)
            C.call("rc_ntt_forward", ctx.handle, C._ptr(d), 20, len(q), 0, C._stream())
            fwd = C.to_host(d)
            C.call("rc_ntt_inverse", ctx.handle, C._ptr(d), 20, len(q), 0, C._stream())
            assert np.array_equal(C.to_host(d), polys)
            return fwd, [o.numpy() for o in ctx.mult_relinearized_batch(lhs, rhs, [key] * 3)]

        ref_fwd, ref_prod = run()
        for split in T.split_candidates(log_n):
            for cc in (2, 3):
                for rp in (8, 16):
                    for fuse in (0, 1):
                        T.apply(ctx, {"ntt_split": split, "col_ctas": cc, "row_polys": rp, "fuse_tensor": fuse})
                        fwd, prod = run()
                        assert np.array_equal(fwd, ref_fwd), (log_n, split, cc, rp, fuse)
                        for a, b in zip(prod, ref_prod):
                            assert np.array_equal(a, b), (log_n, split, cc, rp, fuse)
