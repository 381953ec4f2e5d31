"""The continuous-batching server on the GPU: a mixed stream of Hadamard, Halevi-Shoup and Paterson-Stockmeyer
jobs on three contexts, submitted in a burst and then with gaps; every job's result is bit-identical to the
same job run alone, and the mix was actually batched and overlapped."""
import random
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # collected on CPU-only machines, never run there
    pytest.skip("needs a CUDA GPU", allow_module_level=True)


@pytest.fixture(scope="module")
def env(pkg):
    pkg.lib()
    from rnsckks_gb300 import algorithms as A
    from rnsckks_gb300 import context as C
    from rnsckks_gb300 import server as S
    P = pkg.params
    out = {}
    # Hadamard: relinearized product at the top level
    ctx = C.RnsCkksContext(P.scheme_params(12, 6, 2, 40))
    kp = ctx.keygen(64, C.Sampler(1))
    out["hadamard"] = (ctx, kp, ctx.generate_relinearization_key(kp.secret_key, kp.public_key))
    # Halevi-Shoup dot product of length 64
    ctx = C.RnsCkksContext(P.scheme_params(12, 4, 2, 40))
    kp = ctx.keygen(64, C.Sampler(2))
    keys = A.generate_halevi_shoup_dot_product_rotation_keys(ctx, kp.secret_key, kp.public_key, ctx.levels() - 2, 64)
    out["halevi_shoup"] = (ctx, kp, keys)
    # Paterson-Stockmeyer, 8 coefficients
    ctx = C.RnsCkksContext(P.scheme_params(12, 7, 2, 40))
    kp = ctx.keygen(64, C.Sampler(3))
    keys = A.generate_paterson_stockmeyer_relinearization_keys(ctx, kp.secret_key, kp.public_key, ctx.levels() - 1, 8)
    out["paterson_stockmeyer"] = (ctx, kp, keys, A.constant_plaintext_cache(ctx))
    return A, C, S, out


def _encrypt(C, ctx, kp, rng, seed):
    slots = rng.uniform(-0.5, 0.5, ctx.num_slots())
    return ctx.encrypt(ctx.encode_real(slots), kp.public_key, C.Sampler(seed))


def test_mixed_stream_results_equal_jobs_alone(env):
    A, C, S, E = env
    rng = np.random.default_rng(7)
    coeffs = [0.5, -0.25, 0.125, 0.3, -0.2, 0.1, 0.05, -0.03]
    jobs = []
    for i in range(10):
        ctx, kp, key = E["hadamard"]
        jobs.append(S.hadamard_job(ctx, _encrypt(C, ctx, kp, rng, 100 + i), _encrypt(C, ctx, kp, rng, 200 + i), key))
        ctx, kp, keys = E["halevi_shoup"]
        jobs.append(S.halevi_shoup_job(ctx, _encrypt(C, ctx, kp, rng, 300 + i), list(rng.uniform(-1, 1, 64)), keys))
        ctx, kp, keys, plains = E["paterson_stockmeyer"]
        jobs.append(S.paterson_stockmeyer_job(ctx, _encrypt(C, ctx, kp, rng, 400 + i), coeffs, keys, plains))
    random.Random(5).shuffle(jobs)
    torch.cuda.synchronize()
    budget = sum(j.footprint for j in jobs) // 3
    sch = S.Scheduler(S.GpuExecutor(3), slots=3, memory_budget=budget, max_batch=8).start()
    try:
        for j in jobs[:15]:  # a burst: later jobs queue behind busy slots and get batched
            sch.submit(j)
        for j in jobs[15:]:
            time.sleep(0.002)
            sch.submit(j)
        sch.drain(300)
    finally:
        sch.stop()
    torch.cuda.synchronize()
    assert max(b[2] for b in sch.batches) > 1
    assert sch.peak_in_use <= budget
    st = sch.stats()
    assert st["jobs"] == len(jobs) and set(st["by_kind"]) == {"hadamard", "halevi_shoup", "paterson_stockmeyer"}
    for j in jobs:
        got = j.wait(1)
        p = j.payload
        if j.kind == "hadamard":
            alone = p["ctx"].mult_relinearized(p["lhs"], p["rhs"], p["key"])
        elif j.kind == "halevi_shoup":
            alone = A.halevi_shoup_dot_product(p["ctx"], p["ct"], p["plain"], p["keys"])
        else:
            alone = A.paterson_stockmeyer_eval(p["ctx"], p["ct"], p["coeffs"], p["keys"])
        assert got.level == alone.level and got.scale_bits == alone.scale_bits
        assert np.array_equal(got.numpy(), alone.numpy()), j.kind
