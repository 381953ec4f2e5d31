"""The allocation-free polynomial product (rc_poly_multiply_noalloc).

It exists for callers that may not allocate device memory through the library
(a host that owns the whole GPU pool, or a loop that cannot afford cudaMalloc's
device-wide synchronisation); its scratch is a fixed array inside the library.
These checks call it through the C ABI and compare it bit for bit with the
allocating rc_poly_multiply, on two calls in a row (the array keeps the first
call's contents, which must not leak into the second result), and check that
an oversized request is refused.  This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)


def _rand_poly(rng, moduli, n):
    return np.stack([rng.integers(0, q, n, dtype=np.uint64) for q in moduli])


def test_noalloc_product_matches_allocating_product_twice(pkg):
    pkg.lib()
    from rnsckks_gb300 import context as C
    params = pkg.params.hybrid_params(13, 6, 2, 50)
    ctx = C.RnsCkksContext(params)
    n = params.poly_degree
    rng = np.random.default_rng(2024)
    for with_aux, moduli in ((0, params.q_moduli()), (1, params.q_moduli() + params.p_moduli())):
        for _ in range(2):  # two calls in a row on the shared scratch
            a, b = _rand_poly(rng, moduli, n), _rand_poly(rng, moduli, n)
            da, db = C.to_device(a), C.to_device(b)
            ref = torch.empty_like(da)
            got = torch.full_like(da, -1)
            C.call("rc_poly_multiply", ctx.handle, C._ptr(da), C._ptr(db), C._ptr(ref), len(moduli), with_aux,
                   C._stream())
            C.call("rc_poly_multiply_noalloc", ctx.handle, C._ptr(da), C._ptr(db), C._ptr(got), len(moduli),
                   with_aux, C._stream())
            torch.cuda.synchronize()
            assert torch.equal(got, ref)


def test_noalloc_product_rejects_oversized_requests(pkg):
    pkg.lib()
    from rnsckks_gb300 import context as C
    params = pkg.params.hybrid_params(16, 20, 2, 50)  # 20 limbs * 2^16 > 2^20 words per operand
    ctx = C.RnsCkksContext(params)
    x = torch.zeros((20, params.poly_degree), dtype=torch.int64, device="cuda")
    with pytest.raises(C.RcError, match="exceeds the static scratch limit"):
        C.call("rc_poly_multiply_noalloc", ctx.handle, C._ptr(x), C._ptr(x), C._ptr(x), 20, 0, C._stream())
