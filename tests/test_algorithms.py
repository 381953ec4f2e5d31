"""src/algorithms routines (Halevi-Shoup, total sum, BSGS packed-diagonal matvec, Paterson-Stockmeyer).

CPU: the schedule known-answer tests of the reference (halevi_shoup.rs:82-87, total_sum.rs:71-76,
linear_transform.rs:281-292, packed_diagonal.rs:92-96, paterson_stockmeyer.rs:366-380) on both the GPU
package's routines and the oracle's, and the oracle's routines end to end against the FP64 results with the
reference tests' inputs and tolerances (smaller ring so the CPU suite stays fast).
GPU: the package's routines at `realistic_8_level` (the reference tests' parameters) bit-exact against the
oracle's restatement with the same keys and inputs, decoded within the reference's tolerances, and the
batched forms equal to the single-ciphertext forms.
"""
import math

import numpy as np
import pytest

import algorithms as OA


@pytest.fixture(scope="module")
def A(pkg):
    from rnsckks_gb300 import algorithms
    return algorithms


# ---------------------------------------------------------------------------------------------------------
# schedules (CPU)
# ---------------------------------------------------------------------------------------------------------

def test_fold_steps_follow_powers_of_two(A):
    for f in (A.halevi_shoup_dot_product_rotation_steps, A.total_sum_rotation_steps, OA._fold_steps):
        assert f(1) == [] and f(4) == [1, 2] and f(5) == [1, 2, 4]
    assert A.total_sum_rotation_steps(1024) == [1 << i for i in range(10)]


def test_diagonal_and_bsgs_steps(A):
    assert A.diagonal_transform_rotation_steps(1) == [] and A.diagonal_transform_rotation_steps(4) == [1, 2, 3]
    assert A.packed_diagonal_rotation_steps(4) == [1, 2, 3]
    assert A.diagonal_transform_bsgs_rotation_steps(1) == []
    assert A.diagonal_transform_bsgs_rotation_steps(4) == [1, 2]
    assert A.diagonal_transform_bsgs_rotation_steps(8) == [1, 2, 3, 6]
    # dimension 128: ceil(sqrt) = 12 baby steps, 11 giant steps (not 16/8)
    assert A.diagonal_transform_bsgs_baby_step(128) == 12 == OA.bsgs_baby_step(128)
    steps = A.diagonal_transform_bsgs_rotation_steps(128)
    assert steps == list(range(1, 12)) + [12 * g for g in range(1, 11)]


def test_paterson_stockmeyer_schedule(A):
    for t, b in ((1, 1), (2, 2), (4, 2), (5, 3), (9, 3), (16, 4)):
        assert A.paterson_stockmeyer_block_size(t) == b == OA.ps_block_size(t)
    assert A.paterson_stockmeyer_required_levels(7, 1) == [] == OA.ps_required_levels(7, 1)
    assert A.paterson_stockmeyer_required_levels(7, 5) == [7, 6, 5] == OA.ps_required_levels(7, 5)
    with pytest.raises(Exception, match="level budget"):
        A.paterson_stockmeyer_required_levels(2, 16)


def test_repeat_block_slots(A):
    assert list(A.repeat_block_slots([1.0, 2.0], 6)) == [1.0, 2.0, 1.0, 2.0, 1.0, 2.0]
    with pytest.raises(Exception, match="multiple of the active block length"):
        A.repeat_block_slots([1.0, 2.0, 3.0], 8)


# ---------------------------------------------------------------------------------------------------------
# oracle end to end (CPU)
# ---------------------------------------------------------------------------------------------------------

class OracleKeys:
    """Seeded key material for the oracle (the reference's distributions; keys.rs, keyswitching.rs:81-128)."""

    def __init__(self, oracle, params, ctx, seed=5):
        self.O, self.ctx = oracle, ctx
        self.n = params.poly_degree
        self.q = [p.modulus for p in params.primes]
        self.p = [p.modulus for p in params.aux_primes]
        self.rng = np.random.default_rng(seed)
        s = np.zeros(self.n, dtype=np.int64)
        idx = self.rng.choice(self.n, 64, replace=False)
        s[idx] = np.where(self.rng.random(64) < 0.5, 1, -1)
        self.s = s
        qpl = ctx.qpl
        p1 = np.stack([self.rng.integers(0, q, self.n, dtype=np.uint64) for q in self.q])
        e = np.rint(self.rng.normal(0, 3.19, self.n)).astype(np.int64)
        self.s_q, self.p0, self.p1, _ = oracle.keygen(qpl, s, p1, e)

    def _ks_key(self, src_signed_or_res, level, signed=True):
        O, n = self.O, self.n
        q = self.q[: level + 1]
        qpl, ppl = self.ctx._plans(level + 1), self.ctx.ppl
        src = O.from_signed(src_signed_or_res, q) if signed else src_signed_or_res
        D = O.num_decomp_digits(math.prod(q).bit_length())
        allm = q + self.p
        samples = []
        for _ in range(D):
            a1 = np.stack([self.rng.integers(0, m, n, dtype=np.uint64) for m in allm])
            e = O.from_signed(np.rint(self.rng.normal(0, 3.19, n)).astype(np.int64), allm)
            samples.append((a1, e))
        return O.keyswitch_key_hybrid(qpl, ppl, src, O.from_signed(self.s, q), samples)

    def rotation(self, steps, level):
        g = self.O.galois_element_for_rotation(self.n, steps)
        src = np.zeros(self.n, dtype=np.int64)
        idx = (np.arange(self.n) * g) % (2 * self.n)
        pos = idx < self.n
        src[idx[pos]] += self.s[pos]
        src[idx[~pos] - self.n] -= self.s[~pos]
        return g, self._ks_key(src, level)

    def relin(self, level):
        q = self.q[: level + 1]
        s = self.O.from_signed(self.s, q)
        return self._ks_key(self.O.rns_mul(self.ctx._plans(level + 1), s, s), level, signed=False)

    def encrypt(self, ctx, slots, scale_bits):
        O, n = self.O, self.n
        pt = ctx.encode_at_level_and_scale(np.asarray(slots, dtype=np.complex128), len(self.q) - 1, scale_bits)
        u = O.from_signed(self.rng.integers(-1, 2, n), self.q)
        e0 = O.from_signed(np.rint(self.rng.normal(0, 3.19, n)).astype(np.int64), self.q)
        e1 = O.from_signed(np.rint(self.rng.normal(0, 3.19, n)).astype(np.int64), self.q)
        c0, c1 = O.encrypt_with_samples(ctx.qpl, pt, self.p0, self.p1, u, e0, e1)
        return OA.Ct(c0, c1, scale_bits)

    def decode(self, ctx, ct):
        q = self.q[: ct.level + 1]
        m = self.O.decrypt(self.ctx._plans(ct.level + 1), ct.c0, ct.c1, self.O.from_signed(self.s, q))
        return self.O.decode_integer_coeffs(self.n, float(2.0 ** ct.scale_bits), q, m).real


@pytest.fixture(scope="module")
def small_oracle(pkg, oracle):
    params = pkg.params.hybrid_params(12, 8, 2, 50, 45)
    ctx = OA.Context(params.poly_degree, params.primes, params.aux_primes)
    return ctx, OracleKeys(oracle, params, ctx), params


def test_oracle_halevi_shoup_and_total_sum_decode(small_oracle):
    ctx, K, params = small_oracle
    enc = [0.125, -0.4, 0.03125, -0.125]
    plain = [2.0, -1.0, 0.5, 4.0]
    slots = np.zeros(ctx.num_slots())
    slots[:4] = enc
    ct = K.encrypt(ctx, slots, params.scale_bits)
    keys = {s: K.rotation(s, ct.level - 1) for s in OA._fold_steps(4)}
    out = OA.halevi_shoup_dot_product(ctx, ct, plain, keys)
    assert abs(K.decode(ctx, out)[0] - float(np.dot(enc, plain))) <= 1.5e-2
    vals = [0.125, -0.4, 0.03125, -0.125, 0.375, -0.25, 0.5, 0.0625]
    slots = np.zeros(ctx.num_slots())
    slots[:8] = vals
    ct = K.encrypt(ctx, slots, params.scale_bits)
    keys = {s: K.rotation(s, ct.level) for s in OA._fold_steps(8)}
    out = OA.total_sum(ctx, ct, 8, keys)
    assert abs(K.decode(ctx, out)[0] - sum(vals)) <= 1.5e-2


MATRIX4 = [[1.0, 0.5, -0.25, 0.0], [0.0, -1.0, 0.75, 0.25], [0.5, 0.0, 1.25, -0.5], [-0.25, 0.125, 0.0, 0.75]]
VECTOR4 = [0.5, -0.25, 0.125, 0.75]
PS_COEFFS = [0.75, -0.5, 1.25, -0.25, 0.125]
PS_INPUT = [0.125, -0.2, 0.05, 0.3]


def test_oracle_bsgs_matvec_decode(small_oracle):
    ctx, K, params = small_oracle
    packed = np.array([VECTOR4[i % 4] for i in range(ctx.num_slots())])
    ct = K.encrypt(ctx, packed, params.scale_bits)
    keys = {s: K.rotation(s, ct.level) for s in [1, 2]}
    diags = OA.pack_bsgs_diagonals(ctx, MATRIX4, ct.level, ct.scale_bits)
    out = OA.apply_diagonal_linear_transform(ctx, ct, diags, 4, keys)
    dec = K.decode(ctx, out)
    expect = np.array(MATRIX4) @ np.array(VECTOR4)
    assert np.max(np.abs(dec[:4] - expect)) <= 2e-2
    assert np.max(np.abs(dec[4:8] - expect)) <= 2e-2  # periodic tail


def test_oracle_paterson_stockmeyer_decode(small_oracle):
    ctx, K, params = small_oracle
    slots = np.zeros(ctx.num_slots())
    slots[:4] = PS_INPUT
    ct = K.encrypt(ctx, slots, params.scale_bits)
    keys = {lv: K.relin(lv) for lv in OA.ps_required_levels(ct.level, len(PS_COEFFS))}
    out = OA.paterson_stockmeyer_eval(ctx, ct, PS_COEFFS, keys)
    dec = K.decode(ctx, out)
    expect = [sum(c * x ** i for i, c in enumerate(PS_COEFFS)) for x in PS_INPUT]
    assert np.max(np.abs(dec[:4] - expect)) <= 2e-2


# ---------------------------------------------------------------------------------------------------------
# GPU routines vs the oracle's (bit-exact) at the reference tests' parameters
# ---------------------------------------------------------------------------------------------------------

def _gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")


@pytest.fixture(scope="module")
def realistic(pkg, oracle):
    _gpu()
    from rnsckks_gb300 import context as C
    params = pkg.params.RnsCkksParams.realistic_8_level()
    ctx = C.RnsCkksContext(params)
    kp = ctx.keygen(64, C.Sampler(11))
    octx = OA.Context(params.poly_degree, params.primes, params.aux_primes)
    return C, ctx, kp, octx, params


def _rot_keys(ctx, kp, steps, level):
    gpu, orc = {}, {}
    for s in steps:
        rk, coeff = ctx.generate_rotation_key_at_level(kp.secret_key, kp.public_key, s, level, return_coeff=True)
        gpu[s] = rk
        orc[s] = (rk.galois_element, np.ascontiguousarray(coeff.cpu().numpy().view(np.uint64)))
    return gpu, orc


def _oct(C, ct):
    h = ct.numpy()
    return OA.Ct(h[0].copy(), h[1].copy(), ct.scale_bits)


def _same(C, gpu_ct, o):
    h = gpu_ct.numpy()
    return (gpu_ct.scale_bits == o.scale_bits and gpu_ct.level == o.level
            and np.array_equal(h[0], o.c0) and np.array_equal(h[1], o.c1))


def _encrypt(C, ctx, kp, slots, seed):
    return ctx.encrypt(ctx.encode_real(slots), kp.public_key, C.Sampler(seed))


@pytest.mark.gpu
def test_gpu_halevi_shoup_matches_oracle(A, realistic):
    C, ctx, kp, octx, params = realistic
    enc, plain = [0.125, -0.4, 0.03125, -0.125], [2.0, -1.0, 0.5, 4.0]
    slots = np.zeros(ctx.num_slots())
    slots[:4] = enc
    ct = _encrypt(C, ctx, kp, slots, 1)
    gk, ok = _rot_keys(ctx, kp, A.halevi_shoup_dot_product_rotation_steps(4), ct.level - 1)
    out = A.halevi_shoup_dot_product(ctx, ct, plain, gk)
    ref = OA.halevi_shoup_dot_product(octx, _oct(C, ct), plain, ok)
    assert _same(C, out, ref)
    dec = ctx.decode_real_at_scale(ctx.decrypt(out, kp.secret_key), out.scale_bits)
    assert abs(dec[0] - float(np.dot(enc, plain))) <= 1.5e-2
    # batch of pairs == one pair at a time
    ct2 = _encrypt(C, ctx, kp, slots[::-1].copy(), 2)
    outs = A.halevi_shoup_dot_product_batch(ctx, [ct, ct2], [plain, plain], gk)
    assert np.array_equal(outs[0].numpy(), out.numpy())
    assert np.array_equal(outs[1].numpy(), A.halevi_shoup_dot_product(ctx, ct2, plain, gk).numpy())


@pytest.mark.gpu
def test_gpu_total_sum_matches_oracle(A, realistic):
    C, ctx, kp, octx, params = realistic
    vals = [0.125, -0.4, 0.03125, -0.125, 0.375, -0.25, 0.5, 0.0625]
    slots = np.zeros(ctx.num_slots())
    slots[:8] = vals
    ct = _encrypt(C, ctx, kp, slots, 3)
    gk, ok = _rot_keys(ctx, kp, A.total_sum_rotation_steps(8), ct.level)
    out = A.total_sum(ctx, ct, 8, gk)
    assert _same(C, out, OA.total_sum(octx, _oct(C, ct), 8, ok))
    dec = ctx.decode_real_at_scale(ctx.decrypt(out, kp.secret_key), out.scale_bits)
    assert abs(dec[0] - sum(vals)) <= 1.5e-2
    with pytest.raises(Exception, match="missing total-sum rotation key for step 4"):
        A.total_sum(ctx, ct, 8, {1: gk[1], 2: gk[2]})


@pytest.mark.gpu
@pytest.mark.parametrize("dim", [4, 8])
def test_gpu_bsgs_matvec_matches_oracle(A, realistic, dim):
    C, ctx, kp, octx, params = realistic
    rng = np.random.default_rng(dim)
    matrix = MATRIX4 if dim == 4 else rng.uniform(-1, 1, (dim, dim)).tolist()
    vector = VECTOR4 if dim == 4 else rng.uniform(-1, 1, dim).tolist()
    packed = A.repeat_real_vector_blocks(vector, ctx.num_slots())
    ct = _encrypt(C, ctx, kp, packed, 4 + dim)
    gk, ok = _rot_keys(ctx, kp, A.diagonal_transform_bsgs_rotation_steps(dim), ct.level)
    keys = A.DiagonalTransformRotationKeys(gk)
    diags = A.pack_diagonal_plaintexts(ctx, matrix, ct.level, ct.scale_bits)
    out = A.packed_diagonal_matvec_prepacked(ctx, ct, diags, keys)
    odiags = OA.pack_bsgs_diagonals(octx, matrix, ct.level, ct.scale_bits)
    for g, row in enumerate(odiags):  # the plaintexts themselves agree
        for j, p in enumerate(row):
            if p is not None:
                assert np.array_equal(diags.giant_step_diagonals[g][j].numpy(), p)
    ref = OA.apply_diagonal_linear_transform(octx, _oct(C, ct), odiags, dim, ok)
    assert _same(C, out, ref)
    dec = ctx.decode_real_at_scale(ctx.decrypt(out, kp.secret_key), out.scale_bits)
    expect = np.array(matrix) @ np.array(vector)
    assert np.max(np.abs(dec[:dim] - expect)) <= 2e-2
    assert np.max(np.abs(dec[dim:2 * dim] - expect)) <= 2e-2
    # matrix entry point and batch entry point give the same residues
    assert np.array_equal(A.packed_diagonal_matvec(ctx, ct, matrix, keys).numpy(), out.numpy())
    ct2 = _encrypt(C, ctx, kp, packed[::-1].copy(), 40 + dim)
    outs = A.apply_diagonal_linear_transform_batch(ctx, [ct, ct2], diags, keys)
    assert np.array_equal(outs[0].numpy(), out.numpy())
    assert np.array_equal(outs[1].numpy(), A.apply_diagonal_linear_transform(ctx, ct2, diags, keys).numpy())


@pytest.mark.gpu
def test_gpu_paterson_stockmeyer_matches_oracle(A, realistic):
    C, ctx, kp, octx, params = realistic
    slots = np.zeros(ctx.num_slots())
    slots[:4] = PS_INPUT
    ct = _encrypt(C, ctx, kp, slots, 5)
    gk, ok = {}, {}
    for lv in A.paterson_stockmeyer_required_levels(ct.level, len(PS_COEFFS)):
        k, coeff = ctx.generate_relinearization_key_at_level(kp.secret_key, kp.public_key, lv, return_coeff=True)
        gk[lv] = k
        ok[lv] = np.ascontiguousarray(coeff.cpu().numpy().view(np.uint64))
    out = A.paterson_stockmeyer_eval(ctx, ct, PS_COEFFS, gk)
    ref = OA.paterson_stockmeyer_eval(octx, _oct(C, ct), PS_COEFFS, ok)
    assert _same(C, out, ref)
    dec = ctx.decode_real_at_scale(ctx.decrypt(out, kp.secret_key), out.scale_bits)
    expect = [sum(c * x ** i for i, c in enumerate(PS_COEFFS)) for x in PS_INPUT]
    assert np.max(np.abs(dec[:4] - expect)) <= 2e-2
    ct2 = _encrypt(C, ctx, kp, slots[::-1].copy(), 6)
    outs = A.paterson_stockmeyer_eval_batch(ctx, [ct, ct2], PS_COEFFS, gk)
    assert np.array_equal(outs[0].numpy(), out.numpy())
    assert np.array_equal(outs[1].numpy(), A.paterson_stockmeyer_eval(ctx, ct2, PS_COEFFS, gk).numpy())


@pytest.mark.gpu
def test_gpu_mult_plain_accumulate_equals_sum_of_mult_plain(realistic):
    C, ctx, kp, octx, params = realistic
    rng = np.random.default_rng(9)
    q = ctx.q_moduli[:5]
    cts = [C.RnsCiphertext(C.to_device(np.stack([np.stack([rng.integers(0, m, ctx.params.poly_degree,
                                                                         dtype=np.uint64) for m in q])
                                                 for _ in range(2)])), 30) for _ in range(19)]
    pts = [C.RnsPolynomial(C.to_device(np.stack([rng.integers(0, m, ctx.params.poly_degree, dtype=np.uint64)
                                                 for m in q]))) for _ in range(19)]
    acc = ctx.mult_plain(cts[0], pts[0])
    for c, p in zip(cts[1:], pts[1:]):
        acc = ctx.add(acc, ctx.mult_plain(c, p))
    out = ctx.mult_plain_accumulate(cts, pts)
    assert out.scale_bits == 60 and out.level == 4
    assert np.array_equal(out.numpy(), acc.numpy())
    ntt_c = [C.RnsCiphertext(ctx.ntt_forward_copy(c.data), 30, 4) for c in cts]
    ntt_p = [ctx.ntt_forward_copy(p.data) for p in pts]
    assert np.array_equal(ctx.mult_plain_accumulate(ntt_c, ntt_p, True, True).numpy(), acc.numpy())
    with pytest.raises(Exception, match="same scale to add"):
        ctx.mult_plain_accumulate([cts[0], C.RnsCiphertext(cts[1].data, 31)], pts[:2])


# ---------------------------------------------------------------------------------------------------------
# the native schedules (one library call per batch) equal the routines above, residue for residue
# ---------------------------------------------------------------------------------------------------------

@pytest.mark.gpu
def test_gpu_native_total_sum_and_halevi_shoup(A, realistic):
    C, ctx, kp, octx, params = realistic
    rng = np.random.default_rng(31)
    cts = [_encrypt(C, ctx, kp, rng.uniform(-0.5, 0.5, ctx.num_slots()), 60 + i) for i in range(3)]
    gk, _ = _rot_keys(ctx, kp, A.total_sum_rotation_steps(8), cts[0].level)
    got = A.total_sum_native(ctx, cts, 8, gk)
    want = A.total_sum_batch(ctx, cts, 8, gk)
    for g, w in zip(got, want):
        assert (g.level, g.scale_bits) == (w.level, w.scale_bits) and np.array_equal(g.numpy(), w.numpy())
    with pytest.raises(Exception, match="missing total-sum rotation key for step 4"):
        A.total_sum_native(ctx, cts, 8, {1: gk[1], 2: gk[2]})
    # Halevi-Shoup: one plaintext per ciphertext, same length
    plains = [rng.uniform(-2, 2, 4) for _ in cts]
    hk, _ = _rot_keys(ctx, kp, A.halevi_shoup_dot_product_rotation_steps(4), cts[0].level - 1)
    got = A.halevi_shoup_dot_product_native(ctx, cts, plains, hk)
    want = A.halevi_shoup_dot_product_batch(ctx, cts, plains, hk)
    for g, w in zip(got, want):
        assert (g.level, g.scale_bits) == (w.level, w.scale_bits) and np.array_equal(g.numpy(), w.numpy())
    with pytest.raises(Exception, match="plaintext slot vector cannot exceed the CKKS slot count"):
        A.halevi_shoup_dot_product_native(ctx, cts[:1], [np.zeros(ctx.num_slots() + 1)], hk)


@pytest.mark.gpu
def test_gpu_native_paterson_stockmeyer(A, realistic):
    C, ctx, kp, octx, params = realistic
    slots = np.zeros(ctx.num_slots())
    slots[:4] = PS_INPUT
    cts = [_encrypt(C, ctx, kp, slots, 71), _encrypt(C, ctx, kp, slots[::-1].copy(), 72)]
    gk = {lv: ctx.generate_relinearization_key_at_level(kp.secret_key, kp.public_key, lv)
          for lv in A.paterson_stockmeyer_required_levels(cts[0].level, len(PS_COEFFS))}
    got = A.paterson_stockmeyer_eval_native(ctx, cts, PS_COEFFS, gk)
    want = A.paterson_stockmeyer_eval_batch(ctx, cts, PS_COEFFS, gk)
    for g, w in zip(got, want):
        assert (g.level, g.scale_bits) == (w.level, w.scale_bits) and np.array_equal(g.numpy(), w.numpy())
    dec = ctx.decode_real_at_scale(ctx.decrypt(got[0], kp.secret_key), got[0].scale_bits)
    expect = [sum(c * x ** i for i, c in enumerate(PS_COEFFS)) for x in PS_INPUT]
    assert np.max(np.abs(dec[:4] - expect)) <= 2e-2
    # a constant polynomial, a polynomial with zero terms, and a missing key
    one = A.paterson_stockmeyer_eval_native(ctx, cts[:1], [0.25], gk)[0]
    assert np.array_equal(one.numpy(), A.paterson_stockmeyer_eval(ctx, cts[0], [0.25], gk).numpy())
    sparse = [0.0, 0.5, 0.0, -0.25, 0.0]
    assert np.array_equal(A.paterson_stockmeyer_eval_native(ctx, cts[:1], sparse, gk)[0].numpy(),
                          A.paterson_stockmeyer_eval(ctx, cts[0], sparse, gk).numpy())
    with pytest.raises(Exception, match="missing Paterson-Stockmeyer relinearization key at level"):
        A.paterson_stockmeyer_eval_native(ctx, cts[:1], PS_COEFFS, {})


@pytest.mark.gpu
@pytest.mark.parametrize("dim", [4, 8, 16, 128])
def test_gpu_native_bsgs_equals_routine(A, realistic, dim):
    C, ctx, kp, octx, params = realistic
    rng = np.random.default_rng(100 + dim)
    matrix = rng.uniform(-1, 1, (dim, dim))
    cts = [_encrypt(C, ctx, kp, A.repeat_real_vector_blocks(rng.uniform(-1, 1, dim), ctx.num_slots()), 110 + i)
           for i in range(3)]
    gk, _ = _rot_keys(ctx, kp, A.diagonal_transform_bsgs_rotation_steps(dim), cts[0].level)
    keys = A.DiagonalTransformRotationKeys(gk)
    diags = A.pack_diagonal_plaintexts(ctx, matrix, cts[0].level, cts[0].scale_bits)
    got = A.apply_diagonal_linear_transform_native(ctx, cts, diags, keys)
    want = A.apply_diagonal_linear_transform_batch(ctx, cts, diags, keys)
    for g, w in zip(got, want):
        assert (g.level, g.scale_bits) == (w.level, w.scale_bits) and np.array_equal(g.numpy(), w.numpy())
    missing = dict(gk)
    missing.pop(1)
    with pytest.raises(Exception, match="missing input rotation key for BSGS baby step 1"):
        A.apply_diagonal_linear_transform_native(ctx, cts[:1], diags, A.DiagonalTransformRotationKeys(missing))
    with pytest.raises(Exception, match="packed diagonals must match the ciphertext level"):
        A.apply_diagonal_linear_transform_native(ctx, [cts[0].drop_last_level()], diags, keys)


@pytest.mark.gpu
def test_gpu_bsgs_other_baby_step_matches_oracle(A, realistic):
    """A baby step other than the crate's ceil(sqrt(d)) (the 16/8 split of a 128-wide transform, here 8/2 at
    d = 16): the same packing rule and schedule with another b, against the oracle run with that b."""
    C, ctx, kp, octx, params = realistic
    dim, baby = 16, 8
    rng = np.random.default_rng(77)
    matrix = rng.uniform(-1, 1, (dim, dim))
    vector = rng.uniform(-1, 1, dim)
    ct = _encrypt(C, ctx, kp, A.repeat_real_vector_blocks(vector, ctx.num_slots()), 78)
    steps = A.diagonal_transform_bsgs_rotation_steps(dim, baby)
    assert steps == [1, 2, 3, 4, 5, 6, 7, 8]
    gk, ok = _rot_keys(ctx, kp, steps, ct.level)
    keys = A.DiagonalTransformRotationKeys(gk)
    diags = A.pack_diagonal_plaintexts(ctx, matrix, ct.level, ct.scale_bits, baby)
    assert (diags.baby_step, len(diags.giant_step_diagonals)) == (8, 2)
    odiags = OA.pack_bsgs_diagonals(octx, matrix, ct.level, ct.scale_bits, baby)
    ref = OA.apply_diagonal_linear_transform(octx, _oct(C, ct), odiags, dim, ok, baby)
    native = A.apply_diagonal_linear_transform_native(ctx, [ct], diags, keys)[0]
    assert _same(C, native, ref)
    assert np.array_equal(A.apply_diagonal_linear_transform(ctx, ct, diags, keys).numpy(), native.numpy())
    dec = ctx.decode_real_at_scale(ctx.decrypt(native, kp.secret_key), native.scale_bits)
    assert np.max(np.abs(dec[:dim] - matrix @ vector)) <= 2e-2


def test_bsgs_baby_step_override_validation(A):
    assert A.diagonal_transform_bsgs_rotation_steps(128) == list(range(1, 12)) + [12 * g for g in range(1, 11)]
    assert A.diagonal_transform_bsgs_rotation_steps(128, 16) == list(range(1, 16)) + [16 * g for g in range(1, 8)]
    for bad in (0, 129):
        with pytest.raises(Exception, match="BSGS baby step must be in"):
            A.diagonal_transform_bsgs_rotation_steps(128, bad)


@pytest.mark.gpu
def test_gpu_native_bsgs_16_8_split_equals_routine(A, realistic):
    """The 16/8 split of a 128-wide transform: the fused inner-sum kernel at its largest register tile against
    the routine's per-giant multiply-accumulate (an independent code path)."""
    C, ctx, kp, octx, params = realistic
    rng = np.random.default_rng(128)
    matrix = rng.standard_normal((128, 128))
    cts = [_encrypt(C, ctx, kp, A.repeat_real_vector_blocks(rng.uniform(-1, 1, 128), ctx.num_slots()), 130 + i)
           for i in range(2)]
    gk, _ = _rot_keys(ctx, kp, A.diagonal_transform_bsgs_rotation_steps(128, 16), cts[0].level)
    keys = A.DiagonalTransformRotationKeys(gk)
    diags = A.pack_diagonal_plaintexts(ctx, matrix, cts[0].level, cts[0].scale_bits, 16)
    got = A.apply_diagonal_linear_transform_native(ctx, cts, diags, keys)
    want = A.apply_diagonal_linear_transform_batch(ctx, cts, diags, keys)
    for g, w in zip(got, want):
        assert np.array_equal(g.numpy(), w.numpy())


@pytest.mark.gpu
def test_gpu_native_bsgs_with_60_bit_base_prime_matches_oracle(pkg, oracle, A):
    """A chain with a 60-bit base prime (the inner sums' per-term Barrett branch on that limb, the split
    branch on the 41-bit scaling limbs) against the oracle."""
    _gpu()
    from rnsckks_gb300 import context as C
    params = pkg.params.scheme_params(13, 4, 2, 40)
    ctx = C.RnsCkksContext(params)
    kp = ctx.keygen(64, C.Sampler(21))
    octx = OA.Context(params.poly_degree, params.primes, params.aux_primes)
    dim = 16
    rng = np.random.default_rng(16)
    matrix = rng.uniform(-1, 1, (dim, dim))
    vector = rng.uniform(-1, 1, dim)
    ct = _encrypt(C, ctx, kp, A.repeat_real_vector_blocks(vector, ctx.num_slots()), 22)
    gk, ok = _rot_keys(ctx, kp, A.diagonal_transform_bsgs_rotation_steps(dim), ct.level)
    diags = A.pack_diagonal_plaintexts(ctx, matrix, ct.level, ct.scale_bits)
    out = A.apply_diagonal_linear_transform_native(ctx, [ct], diags, A.DiagonalTransformRotationKeys(gk))[0]
    ref = OA.apply_diagonal_linear_transform(octx, _oct(C, ct), OA.pack_bsgs_diagonals(octx, matrix, ct.level,
                                                                                      ct.scale_bits), dim, ok)
    assert _same(C, out, ref)
    dec = ctx.decode_real_at_scale(ctx.decrypt(out, kp.secret_key), out.scale_bits)
    assert np.max(np.abs(dec[:dim] - matrix @ vector)) <= 1e-3


@pytest.mark.gpu
def test_gpu_native_bsgs_with_61_bit_primes_equals_routine(pkg, A):
    """Primes in [2^60, 2^61): the inner sums' per-term reduction branch, against the routine's multiply-
    accumulate."""
    _gpu()
    from rnsckks_gb300 import context as C
    params = pkg.params.hybrid_params(13, 3, 2, 61, 40)
    assert all(p.modulus >> 60 == 1 for p in params.primes)
    ctx = C.RnsCkksContext(params)
    kp = ctx.keygen(64, C.Sampler(31))
    dim = 8
    rng = np.random.default_rng(8)
    matrix = rng.uniform(-1, 1, (dim, dim))
    ct = _encrypt(C, ctx, kp, A.repeat_real_vector_blocks(rng.uniform(-1, 1, dim), ctx.num_slots()), 32)
    gk, _ = _rot_keys(ctx, kp, A.diagonal_transform_bsgs_rotation_steps(dim), ct.level)
    keys = A.DiagonalTransformRotationKeys(gk)
    diags = A.pack_diagonal_plaintexts(ctx, matrix, ct.level, ct.scale_bits)
    got = A.apply_diagonal_linear_transform_native(ctx, [ct], diags, keys)[0]
    want = A.apply_diagonal_linear_transform(ctx, ct, diags, keys)
    assert np.array_equal(got.numpy(), want.numpy())
