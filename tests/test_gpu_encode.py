"""FP64 encode/decode on the GPU (csrc/encode_gpu.cu) against the host encoder (csrc/encode.cpp), which follows
src/rns/encoding.rs:9-66 and src/math/canonical_embedding.rs:44-79 operation for operation and equals the
oracle's restatement (tests/test_oracle_kat.py).  The bar is bit-exact: the same residues from encode and the
same doubles from decode, over ring degrees, levels, scales, magnitudes that take the 128-bit and saturating
paths, and many plaintexts per call.
"""
import numpy as np
import pytest


def _gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")


def _ctx(pkg, log_n, limbs, scale):
    from rnsckks_gb300 import context as C
    return C, C.RnsCkksContext(pkg.params.hybrid_params(log_n, limbs, 2, 50, scale))


@pytest.mark.gpu
@pytest.mark.parametrize("log_n,limbs,scale", [(4, 3, 30), (10, 4, 40), (12, 6, 45), (15, 8, 45), (16, 24, 50)])
def test_device_encode_decode_equal_host(pkg, log_n, limbs, scale):
    _gpu()
    C, ctx = _ctx(pkg, log_n, limbs, scale)
    rng = np.random.default_rng(log_n)
    h = ctx.num_slots()
    batch = [rng.uniform(-1, 1, h) + 1j * rng.uniform(-1, 1, h) for _ in range(3)]
    batch.append(np.full(h, 0.5 + 0.5j))  # exact halves: round-half-away cases in the rounding step
    for level in (limbs - 1, 0):
        dev = ctx.encode_device_batch(batch, level, scale)
        for s, p in zip(batch, dev):
            assert np.array_equal(p.numpy(), ctx.encode_host(s, level, scale))
        got = ctx.decode_device_batch(dev, scale)
        for i, p in enumerate(dev):
            want = ctx.decode_host(p.numpy(), scale)
            assert np.array_equal(got[i].view(np.uint64), want.view(np.uint64))


@pytest.mark.gpu
def test_device_encode_large_and_saturating_values(pkg):
    _gpu()
    C, ctx = _ctx(pkg, 12, 4, 40)
    h = ctx.num_slots()
    rng = np.random.default_rng(3)
    cases = [rng.uniform(-1, 1, h) * 2.0 ** 30,          # |x| 2^40 up to 2^70: the two-word path
             rng.uniform(-1, 1, h) * 2.0 ** 95,          # up to 2^135: saturates at +-2^127
             np.where(np.arange(h) % 2 == 0, 2.0 ** 23, -(2.0 ** 23)) + 0j,  # exactly 2^63 in magnitude
             np.zeros(h)]
    for s in cases:
        dev = ctx.encode_device_batch([s], 3, 40)[0]
        assert np.array_equal(dev.numpy(), ctx.encode_host(s, 3, 40))
    # decode of arbitrary residues (centred values up to Q/2 in magnitude)
    polys = [C.RnsPolynomial(C.to_device(C.Sampler(9 + i).uniform(ctx.q_moduli[:4], ctx.params.poly_degree)))
             for i in range(2)]
    got = ctx.decode_device_batch(polys, 40)
    for i, p in enumerate(polys):
        assert np.array_equal(got[i].view(np.uint64), ctx.decode_host(p.numpy(), 40).view(np.uint64))
