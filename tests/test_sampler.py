"""Seeded samplers on the device (csrc/sample.cu).

The reference draws from an unseeded OS generator, so its samples cannot be compared value for value; the
contract is its distributions (keys.rs: u64 % q uniform residues, round(N(0, 3.19)) errors, uniform ternary)
and, for the device samplers, reproducibility per (seed, stream id).
CPU: the oracle's Philox4x32-10 against the published known-answer vectors.  GPU: device draws equal the
oracle's restatement value for value, have the reference's distributions (moments, ranges, frequencies), and
keys and ciphertexts made from them decrypt and decode correctly.
"""
import numpy as np
import pytest

import sampler as OS


def test_philox_known_answers():
    # the generator's published known-answer vectors (counter, key) -> output
    M = 0xFFFFFFFF
    assert OS.philox4x32_10([0, 0, 0, 0], [0, 0]) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert OS.philox4x32_10([M] * 4, [M, M]) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert OS.philox4x32_10([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0]) == \
        [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def _gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")


@pytest.fixture(scope="module")
def setup(pkg):
    _gpu()
    from rnsckks_gb300 import context as C
    params = pkg.params.hybrid_params(14, 6, 2, 50, 40)
    return C, C.RnsCkksContext(params), params


def _signed(v, q):
    v = v.astype(object)
    return np.array([int(x) if int(x) <= q // 2 else int(x) - q for x in v], dtype=np.int64)


@pytest.mark.gpu
def test_device_draws_match_oracle_and_repeat(setup):
    C, ctx, params = setup
    seed = 0x0123456789ABCDEF
    s = C.DeviceSampler(ctx, seed)
    u = s.uniform_residues(6).cpu().numpy().view(np.uint64)
    t = s.ternary_residues(3).cpu().numpy().view(np.uint64)
    n = params.poly_degree
    q = ctx.q_moduli
    for j, x in [(0, 0), (0, 1), (2, 777), (5, n - 1)]:
        assert int(u[j, x]) == OS.uniform_residue(seed, 0, j * n + x, q[j])
    for x in (0, 5, 4095, n - 1):
        want = OS.ternary_value(seed, 1, x)
        assert all(int(t[j, x]) == (want % q[j]) for j in range(3))
    again = C.DeviceSampler(ctx, seed).uniform_residues(6).cpu().numpy().view(np.uint64)
    assert np.array_equal(u, again)
    other = C.DeviceSampler(ctx, seed + 1).uniform_residues(6).cpu().numpy().view(np.uint64)
    assert np.mean(u == other) < 1e-3
    # aux basis: Q_(limbs-aux) then P
    ua = s.uniform_residues(4, True).cpu().numpy().view(np.uint64)
    assert int(ua[3].max()) < ctx.p_moduli[1] and int(ua[2].max()) < ctx.p_moduli[0]


@pytest.mark.gpu
def test_device_distributions(setup):
    C, ctx, params = setup
    s = C.DeviceSampler(ctx, 99)
    n, q = params.poly_degree, ctx.q_moduli
    u = s.uniform_residues(6).cpu().numpy().view(np.uint64)
    for j in range(6):
        row = u[j].astype(np.float64) / q[j]
        assert row.max() < 1.0 and abs(row.mean() - 0.5) < 0.01
        hist = np.bincount(np.minimum((row * 16).astype(int), 15), minlength=16)
        chi2 = float(np.sum((hist - n / 16) ** 2 / (n / 16)))
        assert chi2 < 60  # 15 degrees of freedom
    e = s.error_residues(3).cpu().numpy().view(np.uint64)
    es = _signed(e[0], q[0])
    assert all(np.array_equal(_signed(e[j], q[j]), es) for j in range(3))
    assert abs(es.mean()) < 0.1 and abs(es.std() - 3.19) < 0.1 and np.abs(es).max() < 3.19 * 7
    t = s.ternary_residues(2).cpu().numpy().view(np.uint64)
    ts = _signed(t[0], q[0])
    assert set(np.unique(ts)) <= {-1, 0, 1}
    for v in (-1, 0, 1):
        assert abs(np.mean(ts == v) - 1 / 3) < 0.02
    assert np.array_equal(_signed(t[1], q[1]), ts)


@pytest.mark.gpu
def test_device_sampled_keys_and_encryption(pkg):
    _gpu()
    from rnsckks_gb300 import context as C
    params = pkg.params.hybrid_params(13, 6, 2, 50, 40)
    ctx = C.RnsCkksContext(params)
    ds = C.DeviceSampler(ctx, 7)
    kp = ctx.keygen(64, ds)
    relin = ctx.generate_relinearization_key(kp.secret_key, kp.public_key, ds)
    rot = ctx.generate_rotation_key(kp.secret_key, kp.public_key, 1, ds)
    rng = np.random.default_rng(8)
    a = rng.uniform(-1, 1, ctx.num_slots())
    b = rng.uniform(-1, 1, ctx.num_slots())
    ca = ctx.encrypt(ctx.encode_real(a), kp.public_key, ds)
    cb = ctx.encrypt(ctx.encode_real(b), kp.public_key, ds)
    prod = ctx.mult_relinearized(ca, cb, relin)
    dec = ctx.decode_real_at_scale(ctx.decrypt(prod, kp.secret_key), prod.scale_bits)
    assert np.max(np.abs(dec - a * b)) < 1e-3
    r = ctx.rotate(ca, rot)
    dr = ctx.decode_real_at_scale(ctx.decrypt(r, kp.secret_key), r.scale_bits)
    assert np.max(np.abs(dr - np.roll(a, -1))) < 1e-3
    # a Q-only context: the public-key-encrypted keys (keyswitching.rs:44-79) from device samples
    qctx = C.RnsCkksContext(pkg.params.RnsCkksParams.small())
    qs = C.DeviceSampler(qctx, 9)
    qkp = qctx.keygen(64, qs)
    qrel = qctx.generate_relinearization_key(qkp.secret_key, qkp.public_key, qs)
    x = np.linspace(-1, 1, qctx.num_slots())
    cx = qctx.encrypt(qctx.encode_real(x), qkp.public_key, qs)
    sq = qctx.mult_relinearized(cx, cx, qrel)
    dq = qctx.decode_real_at_scale(qctx.decrypt(sq, qkp.secret_key), sq.scale_bits)
    # the reference's integer scale rule (scale_bits -= floor(log2 q_last)) against the exact division by this
    # chain's last prime leaves the factor 2^floor(log2 q)/q on the decoded value
    q_last = qctx.q_moduli[-1]
    factor = 2.0 ** (q_last.bit_length() - 1) / q_last
    assert np.max(np.abs(dq - x * x * factor)) < 1e-2
