"""CKKS bootstrapping scaffold (src/ckks/bootstrapping).

CPU: the exact transform matrices of the package (built from the library's host FP64 slot/coefficient maps)
equal the oracle's restatement bit for bit and are mutual inverses (exact_transforms.rs:309-343); the
schedule and validation known answers of params.rs, coeff_to_slot.rs, eval_mod.rs; the oracle's sparse
EvalMod roundtrip end to end against the FP64 plaintext pipeline (roundtrip.rs:247-303) at N=2^12.
GPU: ModRaise, CoeffToSlot, EvalMod, SlotToCoeff and the roundtrips bit-exact against the oracle with the
same keys at `realistic_8_level` (the reference tests' parameters) and at the reference's 16-coefficient
dense context, decoded within the reference tests' tolerances; the prepared batched form equal to the
reference routine per ciphertext.
"""
import math

import numpy as np
import pytest

import algorithms as OA
import bootstrapping as OB

BASIS8 = [complex(0.5, -0.125), complex(-0.25, 0.75), complex(0.125, 0.5), complex(0.875, -0.25),
          complex(-0.5, 0.125), complex(0.375, -0.5), complex(-0.125, 0.25), complex(0.625, 0.375)]
SMALL8 = [complex(0.03125, -0.015625), complex(-0.05, 0.0125), complex(0.08, -0.02), complex(-0.02, 0.01),
          complex(0.0125, -0.03125), complex(-0.04, 0.02), complex(0.025, -0.0125), complex(-0.01, 0.04)]


@pytest.fixture(scope="module")
def B(pkg):
    from rnsckks_gb300 import bootstrapping
    return bootstrapping


def _poly(coeffs, z):
    acc = complex(0.0)
    for c in reversed(coeffs):
        acc = acc * z + c
    return acc


def _repeat(v, slots):
    return np.array([v[i % len(v)] for i in range(slots)], dtype=np.complex128)


# ---------------------------------------------------------------------------------------------------------
# exact transform matrices (CPU)
# ---------------------------------------------------------------------------------------------------------

@pytest.mark.parametrize("n,active", [(1 << 15, 8), (1 << 12, 16), (16, 8), (16, 2)])
def test_sparse_matrices_match_oracle_and_invert(B, n, active):
    c2s, s2c = B.coeff_to_slot_matrix(n, active), B.slot_to_coeff_matrix(n, active)
    assert np.array_equal(c2s, OB.exact_coeff_to_slot_matrix(n, active))
    assert np.array_equal(s2c, OB.exact_slot_to_coeff_matrix(n, active))
    v = np.array((BASIS8 * 2)[:active])
    # exact_sparse_transform_matrices_are_mutual_inverses (exact_transforms.rs:309-343)
    assert np.max(np.abs(s2c @ (c2s @ v) - v)) <= 1e-8


@pytest.mark.parametrize("n", [16, 64])
def test_dense_matrices_match_oracle(B, n):
    pm = B.dense_coeff_to_slot_matrices(n)
    om = OB.exact_dense_coeff_to_slot_matrices(n)
    for got, want in zip((pm.upper_from_slots, pm.upper_from_conjugates, pm.lower_from_slots,
                          pm.lower_from_conjugates), om):
        assert np.array_equal(got, want)
    ps = B.dense_slot_to_coeff_matrices(n)
    os_ = OB.exact_dense_slot_to_coeff_matrices(n)
    assert np.array_equal(ps.slots_from_upper, os_[0]) and np.array_equal(ps.slots_from_lower, os_[1])
    # the dense pair inverts: slots -> (upper, lower) coefficient halves -> slots
    z = np.array(SMALL8 * (n // 16), dtype=np.complex128)[: n // 2]
    upper = pm.upper_from_slots @ z + pm.upper_from_conjugates @ np.conj(z)
    lower = pm.lower_from_slots @ z + pm.lower_from_conjugates @ np.conj(z)
    assert np.max(np.abs(ps.slots_from_upper @ upper + ps.slots_from_lower @ lower - z)) <= 1e-9


# ---------------------------------------------------------------------------------------------------------
# schedules and validation (CPU)
# ---------------------------------------------------------------------------------------------------------

def _params(B, level=7, active=8):
    return B.BootstrapParameters(level, level + 1, level + 3, 2, 1 << 14, active)


def test_sine_taylor_coefficients(B):
    c = B.sine_taylor_coefficients(5, 1.0)
    assert c == [0.0, 1.0, 0.0, -1.0 / 6.0, 0.0, 1.0 / 120.0]
    assert c == OB.sine_taylor_coefficients(5, 1.0)
    assert B.sine_taylor_coefficients(7, 0.5) == OB.sine_taylor_coefficients(7, 0.5)
    with pytest.raises(B.BootstrapError, match="polynomial_degree must be odd"):
        B.sine_taylor_coefficients(4, 1.0)


def test_eval_mod_plan_validation(B):
    p = _params(B)
    with pytest.raises(B.BootstrapError, match="input_scale must be positive"):
        B.EvalModPlan.new(p, 0.0, 1.0, 5)
    with pytest.raises(B.BootstrapError, match="sine_scale must be non-zero"):
        B.EvalModPlan.new(p, 1.0, 0.0, 5)
    with pytest.raises(B.BootstrapError, match="polynomial_degree must be positive"):
        B.EvalModPlan.new(p, 1.0, 1.0, 0)
    with pytest.raises(B.BootstrapError, match="must be odd for a sine approximation"):
        B.EvalModPlan.new(p, 1.0, 1.0, 4)
    plan = B.EvalModPlan.new(p, 1.0, 1.0, 5)
    assert plan.polynomial_term_count() == 6
    assert plan.required_levels() == [7, 6, 5] == OA.ps_required_levels(7, 6)
    with pytest.raises(B.BootstrapError, match="requires zero coefficient for even degree 2"):
        B.EvalModPrecomputed.new(plan, [0.0, 1.0, 0.5, 0.0, 0.0, 0.0])
    with pytest.raises(B.BootstrapError, match="did not match polynomial degree 5"):
        B.EvalModPrecomputed.new(plan, [0.0, 1.0])


def test_transform_plans(B):
    plan = B.CoeffToSlotPlan.new(_params(B))
    assert plan.transform_dimension == 8 and plan.rotation_steps == [1, 2, 3, 6]
    assert B.SlotToCoeffPlan.new(_params(B, active=128)).rotation_steps == \
        sorted(set(range(1, 12)) | {12 * g for g in range(1, 11)})
    with pytest.raises(B.BootstrapError, match="did not match plan dimension 8"):
        B._validate_transform_matrix(np.ones((4, 4)), 8, "CoeffToSlot")
    with pytest.raises(B.BootstrapError, match="SlotToCoeff transform row 1 had length 3, expected 2"):
        B._validate_transform_matrix([[1, 0], [0, 1, 2]], 2, "SlotToCoeff")


def test_oracle_bootstrap_parameters(pkg):
    params = pkg.params.RnsCkksParams.realistic_8_level()
    ctx = OA.Context(params.poly_degree, params.primes, params.aux_primes)
    p = OB.bootstrap_parameters(ctx, 7, 8)
    assert (p["q_level_count"], p["eval_level_count"], p["aux_level_count"]) == (8, 10, 2)
    with pytest.raises(ValueError, match="active_slots must be a power of two"):
        OB.bootstrap_parameters(ctx, 7, 6)
    with pytest.raises(ValueError, match="ciphertext level must be in 0..8, got 8"):
        OB.bootstrap_parameters(ctx, 8, 8)


# ---------------------------------------------------------------------------------------------------------
# the oracle's sparse EvalMod roundtrip end to end (CPU, N = 2^12)
# ---------------------------------------------------------------------------------------------------------

def _expected_sparse(n, active, inp, coeffs):
    c2s = OB.exact_coeff_to_slot_matrix(n, active)
    s2c = OB.exact_slot_to_coeff_matrix(n, active)
    ev = np.array([_poly(coeffs, z) for z in c2s @ np.array(inp)])
    return s2c @ ev


def test_oracle_sparse_eval_mod_roundtrip_decodes(pkg, oracle):
    from test_algorithms import OracleKeys
    params = pkg.params.hybrid_params(12, 8, 2, 50, 45)
    ctx = OA.Context(params.poly_degree, params.primes, params.aux_primes)
    K = OracleKeys(oracle, params, ctx, seed=9)
    n = params.poly_degree
    ct = K.encrypt(ctx, _repeat(SMALL8, n // 2), 45)
    coeffs = OB.sine_taylor_coefficients(5, 1.0)
    steps = OA.bsgs_baby_step(8)
    rot = sorted(set(range(1, steps)) | {g * steps for g in range(1, -(-8 // steps)) if g * steps < 8})
    em_level = ct.level - 1
    s2c_level = em_level - len(OA.ps_required_levels(em_level, 6))
    keys = {"c2s": {s: K.rotation(s, ct.level) for s in rot},
            "eval_mod": {lv: K.relin(lv) for lv in OA.ps_required_levels(em_level, 6)},
            "s2c": {s: K.rotation(s, s2c_level) for s in rot}}
    out = OB.sparse_eval_mod_roundtrip(ctx, ct, 8, coeffs, keys)
    assert out.level == s2c_level - 1
    q = K.q[: out.level + 1]
    m = oracle.decrypt(ctx._plans(out.level + 1), out.c0, out.c1, oracle.from_signed(K.s, q))
    dec = oracle.decode_integer_coeffs(n, float(2.0 ** out.scale_bits), q, m)
    expect = _expected_sparse(n, 8, SMALL8, coeffs)
    assert np.max(np.abs(dec[:8] - expect)) <= 5e-2


# ---------------------------------------------------------------------------------------------------------
# GPU vs oracle
# ---------------------------------------------------------------------------------------------------------

def _gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")


def _oct(ct):
    h = ct.numpy()
    return OA.Ct(h[0].copy(), h[1].copy(), ct.scale_bits)


def _same(gpu_ct, o):
    h = gpu_ct.numpy()
    return (gpu_ct.scale_bits == o.scale_bits and gpu_ct.level == o.level
            and np.array_equal(h[0], o.c0) and np.array_equal(h[1], o.c1))


def _coeff_u64(t):
    return np.ascontiguousarray(t.cpu().numpy().view(np.uint64))


def _oracle_rot_keys(ctx, kp, steps, level):
    """The keys BootstrapKeySet generates (deterministic default samplers), in oracle form."""
    out = {}
    for s in steps:
        rk, coeff = ctx.generate_rotation_key_at_level(kp.secret_key, kp.public_key, s, level, return_coeff=True)
        out[s] = (rk.galois_element, _coeff_u64(coeff))
    return out


def _oracle_relin_keys(ctx, kp, levels):
    out = {}
    for lv in levels:
        _, coeff = ctx.generate_relinearization_key_at_level(kp.secret_key, kp.public_key, lv, return_coeff=True)
        out[lv] = _coeff_u64(coeff)
    return out


@pytest.fixture(scope="module")
def realistic(pkg, oracle):
    _gpu()
    from rnsckks_gb300 import context as C
    params = pkg.params.RnsCkksParams.realistic_8_level()
    ctx = C.RnsCkksContext(params)
    kp = ctx.keygen(64, C.Sampler(21))
    octx = OA.Context(params.poly_degree, params.primes, params.aux_primes)
    return C, ctx, kp, octx


@pytest.mark.gpu
def test_gpu_bootstrap_parameters(B, realistic):
    C, ctx, kp, octx = realistic
    p = B.BootstrapParameters.new(ctx, 7, 8)
    assert (p.ciphertext_level, p.q_level_count, p.eval_level_count, p.aux_level_count, p.active_slots) == \
        (7, 8, 10, 2, 8)
    for level, active, msg in [(8, 8, "ciphertext level must be in 0..8, got 8"),
                               (7, 0, "active_slots must be positive"),
                               (7, 6, "active_slots must be a power of two"),
                               (7, 1 << 15, "cannot exceed the CKKS slot count 16384")]:
        with pytest.raises(B.BootstrapError, match=msg):
            B.BootstrapParameters.new(ctx, level, active)


@pytest.mark.gpu
def test_gpu_mod_raise_matches_oracle(B, realistic):
    C, ctx, kp, octx = realistic
    inp = [0.125, -0.4, 0.03125, -0.125]
    slots = np.zeros(ctx.num_slots())
    slots[:4] = inp
    ct = ctx.encrypt(ctx.encode_real(slots), kp.public_key, C.Sampler(3))
    raised = B.mod_raise(ctx, ct)
    ref, q_level, aux = OB.mod_raise(octx, _oct(ct))
    assert (raised.q_level(), raised.aux_level_count(), raised.eval_level()) == (7, 2, 9)
    h = raised.ciphertext.numpy()
    assert np.array_equal(h[0], ref.c0) and np.array_equal(h[1], ref.c1)
    assert _same(raised.project_to_q_ciphertext(), _oct(ct))
    # mod_raise_preserves_round_trip_on_realistic_params (mod_raise.rs:74-101)
    dec = B.decrypt_mod_raised(ctx, raised, kp.secret_key)
    got = ctx.decode_real_at_scale(dec.truncate_levels(raised.q_level() + 1), raised.ciphertext.scale_bits)
    assert np.max(np.abs(got[:4] - inp)) <= 2e-2
    # a batch of one level and another
    ct2 = ct.drop_last_level()
    both = B.mod_raise_batch(ctx, [ct, ct2])
    assert np.array_equal(both[0].ciphertext.numpy(), h)
    r2, _, _ = OB.mod_raise(octx, _oct(ct2))
    assert np.array_equal(both[1].ciphertext.numpy()[0], r2.c0)


@pytest.mark.gpu
def test_gpu_coeff_to_slot_exact_matches_oracle(B, realistic):
    """exact_coeff_to_slot_executes_as_expected (exact_transforms.rs:345-400) plus residues."""
    C, ctx, kp, octx = realistic
    ct = ctx.encrypt(ctx.encode(_repeat(BASIS8, ctx.num_slots())), kp.public_key, C.Sampler(4))
    out = B.coeff_to_slot_exact(ctx, ct, kp, 8)
    keys = _oracle_rot_keys(ctx, kp, [1, 2, 3, 6], ct.level)
    ref = OB.linear_transform(octx, _oct(ct), OB.exact_coeff_to_slot_matrix(ctx.params.poly_degree, 8), keys)
    assert _same(out, ref)
    dec = ctx.decode_at_scale(ctx.decrypt(out, kp.secret_key), out.scale_bits)
    expect = B.exact_coeff_to_slot_matrix(ctx, 8) @ np.array(BASIS8)
    assert np.max(np.abs(dec[:8] - expect)) <= 4e-2
    with pytest.raises(B.BootstrapError, match="did not match CoeffToSlot plan level 7"):
        plan = B.CoeffToSlotPlan.from_ciphertext(ctx, ct, 8)
        B.CoeffToSlotRuntime.new(plan, ct.drop_last_level())


@pytest.mark.gpu
def test_gpu_identity_roundtrip(B, realistic):
    """bootstrap_identity_roundtrip_preserves_q_chain_message (roundtrip.rs:220-244)."""
    C, ctx, kp, octx = realistic
    inp = [0.5, -0.25, 0.125, 0.75, -0.5, 0.25, -0.125, 0.375]
    ct = ctx.encrypt(ctx.encode_real(np.tile(inp, ctx.num_slots() // 8)), kp.public_key, C.Sampler(5))
    out = B.bootstrap_identity_roundtrip(ctx, ct, kp, 8)
    dec = ctx.decode_real_at_scale(ctx.decrypt(out, kp.secret_key), out.scale_bits)
    assert np.max(np.abs(dec[:8] - inp)) <= 2e-2
    eye = np.eye(8, dtype=np.complex128)
    o1 = OB.linear_transform(octx, _oct(ct), eye, _oracle_rot_keys(ctx, kp, [1, 2, 3, 6], ct.level))
    o2 = OB.linear_transform(octx, o1, eye, _oracle_rot_keys(ctx, kp, [1, 2, 3, 6], o1.level))
    assert _same(out, o2)


@pytest.mark.gpu
def test_gpu_sparse_eval_mod_roundtrip_matches_oracle(B, realistic):
    """bootstrap_exact_sparse_eval_mod_matches_plaintext_pipeline (roundtrip.rs:246-303), residue for
    residue against the oracle with the same keys, and the prepared batched form."""
    C, ctx, kp, octx = realistic
    ct = ctx.encrypt(ctx.encode(_repeat(SMALL8, ctx.num_slots())), kp.public_key, C.Sampler(6))
    out = B.bootstrap_exact_sparse_eval_mod_roundtrip(ctx, ct, kp, 8, 1.0, 5)
    coeffs = B.sine_taylor_coefficients(5, 1.0)
    em_level = ct.level - 1
    ps_levels = OA.ps_required_levels(em_level, 6)
    s2c_level = em_level - len(ps_levels)
    keys = {"c2s": _oracle_rot_keys(ctx, kp, [1, 2, 3, 6], ct.level),
            "eval_mod": _oracle_relin_keys(ctx, kp, ps_levels),
            "s2c": _oracle_rot_keys(ctx, kp, [1, 2, 3, 6], s2c_level)}
    ref = OB.sparse_eval_mod_roundtrip(octx, _oct(ct), 8, coeffs, keys)
    assert _same(out, ref)
    dec = ctx.decode_at_scale(ctx.decrypt(out, kp.secret_key), out.scale_bits)
    expect = _expected_sparse(ctx.params.poly_degree, 8, SMALL8, coeffs)
    assert np.max(np.abs(dec[:8] - expect)) <= 5e-2
    # prepared form: same keys, same residues, many ciphertexts at once
    boot = B.SparseBootstrapper(ctx, kp, ct.level, ct.scale_bits, 8, 1.0, 5)
    assert boot.s2c_level == s2c_level
    ct2 = ctx.encrypt(ctx.encode(_repeat(SMALL8[::-1], ctx.num_slots())), kp.public_key, C.Sampler(7))
    outs = boot.run_batch([ct, ct2])
    assert np.array_equal(outs[0].numpy(), out.numpy())
    single = B.bootstrap_exact_sparse_eval_mod_roundtrip(ctx, ct2, kp, 8, 1.0, 5)
    assert np.array_equal(outs[1].numpy(), single.numpy())


@pytest.fixture(scope="module")
def dense(pkg, oracle):
    """sample_dense_bootstrap_context (roundtrip.rs:203-218)."""
    _gpu()
    from rnsckks_gb300 import context as C
    P = pkg.params
    primes = [P.RnsPrime(998_244_353, 3), P.RnsPrime(1_004_535_809, 3), P.RnsPrime(469_762_049, 3),
              P.RnsPrime(754_974_721, 11), P.RnsPrime(1_224_736_769, 3), P.RnsPrime(2_013_265_921, 31)]
    params = P.RnsCkksParams(16, primes, [P.RnsPrime(167_772_161, 3)], 28)
    ctx = C.RnsCkksContext(params)
    kp = ctx.keygen(16, C.Sampler(31))
    octx = OA.Context(params.poly_degree, params.primes, params.aux_primes)
    return C, ctx, kp, octx


@pytest.mark.gpu
def test_gpu_dense_coeff_to_slot_matches_oracle(B, dense):
    """dense_coeff_to_slot_exact_matches_plaintext_pipeline (roundtrip.rs:305-357)."""
    C, ctx, kp, octx = dense
    ct = ctx.encrypt(ctx.encode(np.array(SMALL8)), kp.public_key, C.Sampler(8))
    projected = B.mod_raise(ctx, ct).project_to_q_ciphertext()
    upper, lower = B.coeff_to_slot_dense_exact(ctx, projected, kp)
    n, s = ctx.params.poly_degree, ctx.num_slots()
    steps = B.A.diagonal_transform_bsgs_rotation_steps(s)
    keys = _oracle_rot_keys(ctx, kp, steps, ct.level)
    conj_key, conj_coeff = ctx.generate_conjugation_key_at_level(kp.secret_key, kp.public_key, ct.level,
                                                                 return_coeff=True)
    oct_ = _oct(projected)
    oconj = octx.rotate(oct_, (conj_key.galois_element, _coeff_u64(conj_coeff)))
    ou, ol = OB.coeff_to_slot_dense(octx, oct_, oconj, OB.exact_dense_coeff_to_slot_matrices(n), keys)
    assert _same(upper, ou) and _same(lower, ol)
    m = B.exact_dense_coeff_to_slot_matrices(ctx)
    z = np.array(SMALL8)
    eu = m.upper_from_slots @ z + m.upper_from_conjugates @ np.conj(z)
    el = m.lower_from_slots @ z + m.lower_from_conjugates @ np.conj(z)
    du = ctx.decode_at_scale(ctx.decrypt(upper, kp.secret_key), upper.scale_bits)
    dl = ctx.decode_at_scale(ctx.decrypt(lower, kp.secret_key), lower.scale_bits)
    assert np.max(np.abs(du - eu)) <= 7e-2 and np.max(np.abs(dl - el)) <= 7e-2
    # dense SlotToCoeff back: dense_coeff_to_slot_then_slot_to_coeff_exact_recovers_input
    back = B.slot_to_coeff_dense_exact(ctx, upper, lower, kp)
    okeys = _oracle_rot_keys(ctx, kp, steps, upper.level)
    oback = OB.slot_to_coeff_dense(octx, ou, ol, OB.exact_dense_slot_to_coeff_matrices(n), okeys)
    assert _same(back, oback)
    dec = ctx.decode_at_scale(ctx.decrypt(back, kp.secret_key), back.scale_bits)
    assert np.max(np.abs(dec - z)) <= 7e-2
