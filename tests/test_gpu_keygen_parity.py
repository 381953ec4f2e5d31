"""Residue parity of GPU key generation and encryption with the oracle on identical samples.

The device sampler's draws are reproducible per (seed, stream id) and equal the oracle's Philox
restatement (tests/test_sampler.py), so a second sampler with the same seed replays exactly the samples the
context consumed.  Those samples go into the oracle's restatements of
  * rns_keygen (src/rns/keys.rs:153-166): p0 = e - p1 s;
  * encrypt_rns_with_samples (src/rns/ops.rs:25-42);
  * generate_keyswitch_key_rns_hybrid (src/rns/keyswitching.rs:81-128) for the relinearization key (source
    s^2) and a rotation key (source sigma_g(s)), at realistic_8_level;
  * generate_keyswitch_key_rns (src/rns/keyswitching.rs:44-79), the public-key-encrypted Q-only key, at the
    small preset;
and every residue of the GPU's keys and ciphertexts must equal the oracle's bit for bit.
"""
import numpy as np
import pytest

import sampler as OS

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # collected on CPU-only machines, never run there
    pytest.skip("needs a CUDA GPU", allow_module_level=True)


def _signed(row, q):
    r = row.astype(object)
    return np.array([int(x) if int(x) <= q // 2 else int(x) - q for x in r], dtype=np.int64)


def _host(t):
    return t.cpu().numpy().view(np.uint64)


def test_hybrid_keygen_encrypt_and_keys_equal_oracle(pkg, oracle):
    pkg.lib()
    from rnsckks_gb300 import context as C
    params = pkg.params.RnsCkksParams.realistic_8_level()
    ctx = C.RnsCkksContext(params)
    n, qm, pm = params.poly_degree, ctx.q_moduli, ctx.p_moduli
    lq, la = len(qm), len(qm) + len(pm)
    seed = 0x5EED_0008
    ds = C.DeviceSampler(ctx, seed)
    kp = ctx.keygen(64, ds)
    relin, relin_coeff = ctx.generate_relinearization_key(kp.secret_key, kp.public_key, ds, return_coeff=True)
    rot, rot_coeff = ctx.generate_rotation_key(kp.secret_key, kp.public_key, 3, ds, return_coeff=True)
    rng = np.random.default_rng(5)
    pt = ctx.encode(rng.uniform(-1, 1, n // 2) + 1j * rng.uniform(-1, 1, n // 2))
    ct = ctx.encrypt(pt, kp.public_key, ds)
    torch.cuda.synchronize()

    # replay the same draws
    rep = C.DeviceSampler(ctx, seed)
    s = rep.sparse_ternary(n, 64)
    assert np.array_equal(s, kp.secret_key.coeffs)
    p1 = _host(rep.uniform_residues(lq))
    e = _host(rep.error_residues(lq))
    for j, x in [(0, 0), (lq - 1, n - 1)]:  # the replay is the oracle's Philox stream 0
        assert int(p1[j, x]) == OS.uniform_residue(seed, 0, j * n + x, qm[j])
    D = relin_coeff.shape[0]
    relin_samples = [(_host(rep.uniform_residues(la, True)), _host(rep.error_residues(la, True))) for _ in range(D)]
    rot_samples = [(_host(rep.uniform_residues(la, True)), _host(rep.error_residues(la, True))) for _ in range(D)]
    u, e0, e1 = (_host(rep.ternary_residues(lq)), _host(rep.error_residues(lq)), _host(rep.error_residues(lq)))

    qpl, ppl = oracle.Plans(n, params.primes), oracle.Plans(n, params.aux_primes)
    s_res, p0_ref, p1_ref, _ = oracle.keygen(qpl, s, p1, _signed(e[0], qm[0]))
    assert np.array_equal(kp.secret_key.poly.numpy(), s_res)
    assert np.array_equal(kp.public_key.p0.numpy(), p0_ref)
    assert np.array_equal(kp.public_key.p1.numpy(), p1_ref)

    c0, c1 = oracle.encrypt_with_samples(qpl, pt.numpy(), p0_ref, p1_ref, u, e0, e1)
    got = ct.numpy()
    assert np.array_equal(got[0], c0) and np.array_equal(got[1], c1)

    relin_ref = oracle.keyswitch_key_hybrid(qpl, ppl, oracle.rns_mul(qpl, s_res, s_res), s_res, relin_samples)
    assert relin_ref.shape == tuple(relin_coeff.shape)
    assert np.array_equal(_host(relin_coeff), relin_ref)

    g = ctx.galois_element_for_rotation(3)
    assert rot.galois_element == g
    rot_ref = oracle.keyswitch_key_hybrid(qpl, ppl, oracle.rns_automorphism(qpl, s_res, g), s_res, rot_samples)
    assert np.array_equal(_host(rot_coeff), rot_ref)


def test_q_only_keygen_and_key_equal_oracle(pkg, oracle):
    pkg.lib()
    from rnsckks_gb300 import context as C
    params = pkg.params.RnsCkksParams.small()
    ctx = C.RnsCkksContext(params)
    n, qm = params.poly_degree, ctx.q_moduli
    lq = len(qm)
    seed = 0x5EED_0006
    ds = C.DeviceSampler(ctx, seed)
    kp = ctx.keygen(64, ds)
    relin, relin_coeff = ctx.generate_relinearization_key(kp.secret_key, kp.public_key, ds, return_coeff=True)
    pt = ctx.encode_real(np.linspace(-1, 1, ctx.num_slots()))
    ct = ctx.encrypt(pt, kp.public_key, ds)
    torch.cuda.synchronize()

    rep = C.DeviceSampler(ctx, seed)
    s = rep.sparse_ternary(n, 64)
    p1 = _host(rep.uniform_residues(lq))
    e = _host(rep.error_residues(lq))
    D = relin_coeff.shape[0]
    samples = [(_host(rep.ternary_residues(lq)), _host(rep.error_residues(lq)), _host(rep.error_residues(lq)))
               for _ in range(D)]
    u, e0, e1 = (_host(rep.ternary_residues(lq)), _host(rep.error_residues(lq)), _host(rep.error_residues(lq)))

    qpl = oracle.Plans(n, params.primes)
    s_res, p0_ref, p1_ref, _ = oracle.keygen(qpl, s, p1, _signed(e[0], qm[0]))
    assert np.array_equal(kp.public_key.p0.numpy(), p0_ref)
    key_ref = oracle.keyswitch_key_q(qpl, oracle.rns_mul(qpl, s_res, s_res), p0_ref, p1_ref, samples, digits=D)
    assert np.array_equal(_host(relin_coeff), key_ref)
    c0, c1 = oracle.encrypt_with_samples(qpl, pt.numpy(), p0_ref, p1_ref, u, e0, e1)
    got = ct.numpy()
    assert np.array_equal(got[0], c0) and np.array_equal(got[1], c1)
