"""The 16-residues-per-lane transform passes (N = 2^16 split 2^8 x 2^8, tunable `ntt_r16`: a set of pass bits,
63 = every pass, 0 = none) against the eight-residue passes and the oracle, bit-exact: the forward and inverse
NTT over RNS limbs (lazy and Harvey forward butterflies, 16-byte aligned and unaligned polynomials), the tensor
with its inverse rows, and the wide key product's transforms (key build, digit transforms of uniform and mixed-level batches, product
transforms).  The reference's transform is src/math/ntt.rs:92-130 with the twist of src/poly/mod.rs:134-175;
mult_relinearized is src/rns/context/ops.rs:124-133.
"""
import math
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # collected on CPU-only machines, never run there
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

from test_gpu_parity import rand_ct, rand_poly  # noqa: E402


@pytest.fixture(scope="module")
def C(pkg):
    pkg.lib()
    from rnsckks_gb300 import context as C
    return C


def _tune(C, ctx, name, value):
    C.call("rc_tune_set", ctx.handle, name.encode(), int(value))


def _ntt(C, ctx, t, polys, limbs, aux, forward):
    fn = "rc_ntt_forward" if forward else "rc_ntt_inverse"
    C.call(fn, ctx.handle, C._ptr(t), polys, limbs, aux, C._stream())
    torch.cuda.synchronize()


@pytest.mark.parametrize("lazy", [1, 0])
def test_r16_ntt_equals_eight_residue_passes(C, pkg, lazy):
    params = pkg.params.hybrid_params(16, 4, 2, 50)
    ctx = C.RnsCkksContext(params)
    _tune(C, ctx, "lazy_ntt", lazy)
    n = params.poly_degree
    allm = params.q_moduli() + params.p_moduli()
    rng = np.random.default_rng(16 + lazy)
    polys = 19  # more than one row block of 16 polynomials
    a = np.stack([rand_poly(rng, allm, n) for _ in range(polys)])
    fwd, back = {}, {}
    for r16 in (63, 1, 0):
        _tune(C, ctx, "ntt_r16", r16)
        d = C.to_device(a)
        _ntt(C, ctx, d, polys, len(allm), 1, True)
        fwd[r16] = C.to_host(d)
        _ntt(C, ctx, d, polys, len(allm), 1, False)
        back[r16] = C.to_host(d)
    assert np.array_equal(fwd[63], fwd[0]) and np.array_equal(fwd[1], fwd[0])
    assert all(np.array_equal(back[r], a) for r in back)
    assert int(fwd[63].max()) < max(allm)  # canonical residues
    # a polynomial array that starts 8 bytes past a 16-byte boundary takes the eight-residue passes
    _tune(C, ctx, "ntt_r16", 63)
    flat = torch.zeros(a.size + 1, dtype=torch.int64, device="cuda")
    view = flat[1:].view(a.shape)
    view.copy_(torch.from_numpy(a.view(np.int64)).cuda())
    assert view.data_ptr() % 16 == 8
    _ntt(C, ctx, view, polys, len(allm), 1, True)
    assert np.array_equal(C.to_host(view), fwd[0])
    _ntt(C, ctx, view, polys, len(allm), 1, False)
    assert np.array_equal(C.to_host(view), a)


def _key(rng, params, limbs):
    qm = params.q_moduli()[:limbs]
    allm = qm + params.p_moduli()
    D = math.ceil(math.prod(qm).bit_length() / 30)
    return np.stack([rand_ct(rng, allm, params.poly_degree) for _ in range(D)]), D


@pytest.mark.parametrize("fuse_tensor", [0, 1])
def test_r16_mult_relinearized_matches_oracle_and_eight_residue_passes(C, pkg, oracle, fuse_tensor):
    oracle.set_threads(os.cpu_count() or 1)
    params = pkg.params.hybrid_params(16, 6, 2, 50)
    n, q = params.poly_degree, params.q_moduli()
    rng = np.random.default_rng(0x16 + fuse_tensor)
    key, D = _key(rng, params, len(q))
    pairs = [(rand_ct(rng, q, n), rand_ct(rng, q, n)) for _ in range(5)]
    results = {}
    # (ntt_r16, lazy_ntt): the forward row passes leave their outputs to the tensor unreduced, below 65q (lazy)
    # or 4q, in both row forms; the results stay the same
    for r16, lazy in ((63, 1), (9, 1), (0, 1), (9, 0)):
        ctx = C.RnsCkksContext(params)
        _tune(C, ctx, "ntt_r16", r16)
        _tune(C, ctx, "fuse_tensor", fuse_tensor)
        _tune(C, ctx, "lazy_ntt", lazy)
        ksk = ctx.upload_keyswitch_key(key, len(q) - 1, 2)  # the key's wide form is built by these passes too
        lhs = [C.RnsCiphertext(C.to_device(a), 40) for a, _ in pairs]
        rhs = [C.RnsCiphertext(C.to_device(b), 40) for _, b in pairs]
        batched = [o.numpy() for o in ctx.mult_relinearized_batch(lhs, rhs, [ksk] * len(pairs))]
        single = ctx.mult_relinearized(lhs[1], rhs[1], ksk).numpy()
        assert np.array_equal(single, batched[1])
        results[r16, lazy] = batched
    for cfg in ((63, 1), (9, 1), (9, 0)):
        for x, y in zip(results[cfg], results[0, 1]):
            assert np.array_equal(x, y)
    qpl, ppl = oracle.Plans(n, params.primes), oracle.Plans(n, params.aux_primes)
    a, b = pairs[0]
    m0, m1 = oracle.mult_relinearized(qpl, ppl, a[0], a[1], b[0], b[1], key, D)
    assert np.array_equal(results[63, 1][0][0], m0) and np.array_equal(results[63, 1][0][1], m1)


def test_r16_mixed_level_relinearize_rescale_equals_eight_residue_passes(C, pkg):
    params = pkg.params.hybrid_params(16, 6, 2, 50)
    n, q = params.poly_degree, params.q_moduli()
    rng = np.random.default_rng(0x61)
    limbs_list = [6, 3, 5, 6, 2]
    host_keys = {limbs: _key(rng, params, limbs)[0] for limbs in set(limbs_list)}
    quads = [rand_ct(rng, q[:limbs], n, 3) for limbs in limbs_list]
    outs = {}
    for r16 in (63, 0):
        ctx = C.RnsCkksContext(params)
        _tune(C, ctx, "ntt_r16", r16)
        keys = {limbs: ctx.upload_keyswitch_key(k, limbs - 1, 2) for limbs, k in host_keys.items()}
        cts = [C.RnsQuadraticCiphertext(C.to_device(x), 80) for x in quads]
        res = ctx.relinearize_rescale_batch(cts, [keys[limbs] for limbs in limbs_list])
        outs[r16] = [r.numpy() for r in res]
    for x, y in zip(outs[63], outs[0]):
        assert np.array_equal(x, y)
