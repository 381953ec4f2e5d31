"""The optional RNS-hybrid ("dnum") key switch (rc_ksk_upload_dnum; no counterpart in the reference, whose
gadget is balanced base-2^30 digits).  Its results are not the reference's residues, so it is checked:
  * bit for bit against a CPU restatement of the same algorithm built from the oracle's primitives (ModUp by
    fast basis conversion in exact integers, NTT products and sums over Q u P, the reference's exact centred
    ModDown), for relinearize and mult_relinearized;
  * by decryption: products of real encryptions with real keys decode to the FP64 product;
  * for batching (batch = per op, RNS-hybrid and gadget keys mixed in one call) and its refusals.
"""
import ctypes
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # collected on CPU-only machines, never run there
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

from test_gpu_parity import rand_ct  # noqa: E402


@pytest.fixture(scope="module")
def C(pkg):
    pkg.lib()
    from rnsckks_gb300 import context as C
    return C


def _upload(C, ctx, key, alpha, level):
    h = ctypes.c_void_p()
    k = np.ascontiguousarray(key, dtype=np.uint64)
    C.call("rc_ksk_upload_dnum", ctx.handle, k.ctypes.data, 0, alpha, level, ctypes.byref(h))
    return C.RnsKeySwitchingKey(ctx, h)


def _modup(c2, qm, allm, alpha):
    """D_b over Q u P for each group b of alpha limbs: the group's residues on its own limbs, elsewhere
    sum_i [c_i (Q_b/q_i)^-1]_{q_i} (Q_b/q_i) mod t in exact integers."""
    groups = []
    for b in range(-(-len(qm) // alpha)):
        lo, hi = b * alpha, min((b + 1) * alpha, len(qm))
        Qb = math.prod(qm[lo:hi])
        ys = [(c2[i].astype(object) * pow(Qb // qm[i] % qm[i], -1, qm[i])) % qm[i] for i in range(lo, hi)]
        D = np.zeros((len(allm), c2.shape[1]), dtype=np.uint64)
        for t, m in enumerate(allm):
            if lo <= t < hi:
                D[t] = c2[t]
            else:
                s = sum(y * ((Qb // qm[lo + k]) % m) for k, y in enumerate(ys))
                D[t] = np.array([int(v) % m for v in s], dtype=np.uint64)
        groups.append(D)
    return groups


def _relin_restated(oracle, params, limbs, quad, key, alpha):
    n = params.poly_degree
    qpl = oracle.Plans(n, params.primes[:limbs])
    ppl = oracle.Plans(n, params.aux_primes)
    qp = qpl.concat(ppl)
    qm, pm = params.q_moduli()[:limbs], params.p_moduli()
    acc = [None, None]
    for b, D in enumerate(_modup(quad[2], qm, qm + pm, alpha)):
        for c in range(2):
            t = oracle.rns_mul(qp, D, key[b, c])
            acc[c] = t if acc[c] is None else oracle.rns_add(qp, acc[c], t)
    return [oracle.rns_add(qpl, quad[c], oracle.mod_down(qpl, ppl, acc[c])) for c in range(2)]


@pytest.mark.parametrize("alpha", [3, 2, 1])
def test_dnum_relinearize_matches_its_restatement(C, pkg, oracle, alpha):
    params = pkg.params.hybrid_params(12, 6, 3, 50)
    ctx = C.RnsCkksContext(params)
    n, q, p = params.poly_degree, params.q_moduli(), params.p_moduli()
    rng = np.random.default_rng(100 + alpha)
    for limbs in (6, 4):
        dnum = -(-limbs // alpha)
        key = np.stack([np.stack([np.stack([rng.integers(0, m, n, dtype=np.uint64) for m in q[:limbs] + p])
                                  for _ in range(2)]) for _ in range(dnum)])
        ksk = _upload(C, ctx, key, alpha, limbs - 1)
        assert ksk.digits == dnum and ksk.aux_level_count == 3
        quad = rand_ct(rng, q[:limbs], n, 3)
        got = ctx.relinearize(C.RnsQuadraticCiphertext(C.to_device(quad), 80), ksk).numpy()
        want = _relin_restated(oracle, params, limbs, quad, key, alpha)
        assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1]), (alpha, limbs)
        # mult_relinearized = tensor + this relinearization + rescale
        a, b = rand_ct(rng, q[:limbs], n), rand_ct(rng, q[:limbs], n)
        out = ctx.mult_relinearized(C.RnsCiphertext(C.to_device(a), 40), C.RnsCiphertext(C.to_device(b), 40), ksk)
        qpl = oracle.Plans(n, params.primes[:limbs])
        t = oracle.tensor(qpl, a[0], a[1], b[0], b[1])
        r = _relin_restated(oracle, params, limbs, np.stack(t), key, alpha)
        got = out.numpy()
        assert np.array_equal(got[0], oracle.rescale_poly(qpl, r[0]))
        assert np.array_equal(got[1], oracle.rescale_poly(qpl, r[1]))


def test_dnum_products_decrypt_and_batch(C, pkg):
    """Real keys: the RNS-hybrid relinearization key at alpha = 3 (2 groups) and 2 (3 groups) relinearizes
    products of encryptions that decode to the FP64 product like the gadget key's; a batch equals the per-op
    calls, also with gadget and RNS-hybrid keys mixed in one call."""
    params = pkg.params.hybrid_params(13, 6, 3, 50, 40)
    ctx = C.RnsCkksContext(params)
    ds = C.DeviceSampler(ctx, 21)
    kp = ctx.keygen(64, ds)
    gadget = ctx.generate_relinearization_key(kp.secret_key, kp.public_key, ds)
    rng = np.random.default_rng(8)
    xs = [rng.uniform(-1, 1, ctx.num_slots()) for _ in range(4)]
    cts = [ctx.encrypt(ctx.encode_real(x), kp.public_key, ds) for x in xs]
    for alpha in (3, 2):
        key = ctx.generate_relinearization_key_dnum(kp.secret_key, alpha, sampler=ds)
        for i in range(2):
            prod = ctx.mult_relinearized(cts[i], cts[i + 2], key)
            dec = ctx.decode_real_at_scale(ctx.decrypt(prod, kp.secret_key), prod.scale_bits)
            assert np.max(np.abs(dec - xs[i] * xs[i + 2])) < 1e-3
        single = [ctx.mult_relinearized(cts[i], cts[3 - i], key).numpy() for i in range(4)]
        batch = ctx.mult_relinearized_batch(cts, cts[::-1], [key] * 4)
        for s, b in zip(single, batch):
            assert np.array_equal(s, b.numpy())
        mixed = ctx.mult_relinearized_batch(cts, cts[::-1], [key, gadget, key, gadget])
        assert np.array_equal(mixed[0].numpy(), single[0]) and np.array_equal(mixed[2].numpy(), single[2])
        assert np.array_equal(mixed[1].numpy(), ctx.mult_relinearized(cts[1], cts[2], gadget).numpy())


def test_dnum_refusals(C, pkg):
    params = pkg.params.hybrid_params(12, 4, 2, 50)
    ctx = C.RnsCkksContext(params)
    n, q, p = params.poly_degree, params.q_moduli(), params.p_moduli()
    key = np.zeros((2, 2, len(q) + len(p), n), dtype=np.uint64)
    with pytest.raises(C.RcError, match="alpha must be between 1 and the number of aux primes"):
        _upload(C, ctx, key, 3, len(q) - 1)
    with pytest.raises(C.RcError, match="alpha must be between 1"):
        _upload(C, ctx, key, 0, len(q) - 1)
    ksk = _upload(C, ctx, key, 2, len(q) - 1)
    with pytest.raises(C.RcError, match="not serialisable"):
        ksk.to_bytes()
    qonly = C.RnsCkksContext(pkg.params.RnsCkksParams.small())
    with pytest.raises(C.RcError, match="need an auxiliary basis"):
        _upload(C, qonly, key, 1, 0)
    low = C.RnsQuadraticCiphertext(C.to_device(rand_ct(np.random.default_rng(1), q[:3], n, 3)), 80)
    with pytest.raises(C.RcError, match="keyswitch key level must match"):
        ctx.relinearize(low, ksk)
