"""The allocation-free polynomial product (rc_poly_multiply_noalloc).

It exists for callers that may not allocate device memory through the library (a host that owns the whole
GPU pool, or a loop that cannot afford cudaMalloc's device-wide synchronisation); its scratch is a fixed
array inside the library.  These checks call it through the C ABI, first, on a fresh context and a fresh
stream (so no earlier call has grown a workspace it could silently reuse), and check:
  * its residues equal the oracle's RNS product and the allocating rc_poly_multiply's, on two calls in a row
    (the array keeps the first call's contents, which must not leak into the second result);
  * the device's free memory is the same before and after calls that follow a first (warm) call;
  * the exact fit, limbs * N = 2^20 words per operand (16 limbs at N = 2^16), is accepted and correct, and
    one limb more is refused.
This file is collected last on purpose.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)


def _rand_poly(rng, moduli, n):
    return np.stack([rng.integers(0, q, n, dtype=np.uint64) for q in moduli])


def _noalloc(C, ctx, da, db, out, limbs, with_aux, stream):
    C.call("rc_poly_multiply_noalloc", ctx.handle, C._ptr(da), C._ptr(db), C._ptr(out), limbs, with_aux,
           stream.cuda_stream)


def test_noalloc_product_allocates_nothing_and_matches_oracle(pkg, oracle):
    pkg.lib()
    from rnsckks_gb300 import context as C
    params = pkg.params.hybrid_params(13, 6, 2, 50)
    ctx = C.RnsCkksContext(params)  # fresh: no call has grown a workspace on it yet
    stream = torch.cuda.Stream()
    n = params.poly_degree
    rng = np.random.default_rng(2024)
    cases = []
    for with_aux, primes in ((0, params.primes), (1, params.primes + params.aux_primes)):
        moduli = [p.modulus for p in primes]
        for _ in range(2):  # two calls in a row on the shared scratch
            a, b = _rand_poly(rng, moduli, n), _rand_poly(rng, moduli, n)
            cases.append((with_aux, primes, a, b, C.to_device(a), C.to_device(b)))
    outs = [torch.full((len(c[1]), n), -1, dtype=torch.int64, device="cuda") for c in cases]
    torch.cuda.synchronize()
    # warm call: the first call looks up the array's device address and loads the kernels it launches
    with torch.cuda.stream(stream):
        _noalloc(C, ctx, cases[0][4], cases[0][5], outs[0], len(cases[0][1]), cases[0][0], stream)
    stream.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    with torch.cuda.stream(stream):
        for (with_aux, primes, a, b, da, db), out in zip(cases, outs):
            _noalloc(C, ctx, da, db, out, len(primes), with_aux, stream)
    stream.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, f"device free memory changed by {free0 - free1} bytes across no-alloc calls"
    for (with_aux, primes, a, b, da, db), out in zip(cases, outs):
        ref = oracle.rns_mul(oracle.Plans(n, primes), a, b)
        assert np.array_equal(C.to_host(out), ref)
        # and the allocating entry point gives the same residues
        alloc = torch.empty_like(out)
        C.call("rc_poly_multiply", ctx.handle, C._ptr(da), C._ptr(db), C._ptr(alloc), len(primes), with_aux,
               C._stream())
        torch.cuda.synchronize()
        assert torch.equal(alloc, out)


def test_noalloc_product_exact_fit_and_refusal(pkg, oracle):
    """16 limbs at N = 2^16 fill both halves of the 2^21-word array exactly; 17 limbs do not fit."""
    pkg.lib()
    from rnsckks_gb300 import context as C
    params = pkg.params.hybrid_params(16, 17, 2, 50)
    ctx = C.RnsCkksContext(params)
    n = params.poly_degree
    stream = torch.cuda.Stream()
    rng = np.random.default_rng(16)
    primes = params.primes[:16]
    moduli = [p.modulus for p in primes]
    # two calls in a row; the oracle checks the first limbs only (the full 16-limb product takes it minutes)
    for _ in range(2):
        a, b = _rand_poly(rng, moduli, n), _rand_poly(rng, moduli, n)
        da, db = C.to_device(a), C.to_device(b)
        out = torch.full((16, n), -1, dtype=torch.int64, device="cuda")
        with torch.cuda.stream(stream):
            _noalloc(C, ctx, da, db, out, 16, 0, stream)
        stream.synchronize()
        got = C.to_host(out)
        alloc = torch.empty_like(out)
        C.call("rc_poly_multiply", ctx.handle, C._ptr(da), C._ptr(db), C._ptr(alloc), 16, 0, C._stream())
        torch.cuda.synchronize()
        assert np.array_equal(got, C.to_host(alloc))
        for i in (0, 15):
            assert np.array_equal(got[i], oracle.poly_mul_ntt(oracle.Plans(n, [primes[i]]), 0, a[i], b[i]))
    x = torch.zeros((17, n), dtype=torch.int64, device="cuda")
    with pytest.raises(C.RcError, match="exceeds the static scratch limit"):
        C.call("rc_poly_multiply_noalloc", ctx.handle, C._ptr(x), C._ptr(x), C._ptr(x), 17, 0, C._stream())
