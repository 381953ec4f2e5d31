"""Serialised keys and ciphertexts (csrc/serialize.cu) and the server's key store.

The reference has no serialisation; the contract tested here is the library's own: a record reloads into a
context with the same modulus chain and gives the same residues as the original object, and a record that is
damaged, truncated or made for another chain is refused with a message, never loaded.
CPU: header parsing of ciphertext records (no context needed).  GPU: round trips of relinearization,
rotation and truncated Q-only keys and of 2- and 3-component ciphertexts, refusals, and a server key store
reopened on a fresh context.
"""
import ctypes
import struct

import numpy as np
import pytest


def _ct_header(magic=b"RCCTXT01", version=1, comps=2, n=4096, level=3, scale=40, payload=0):
    return magic + struct.pack("<IIQiiQQQQ", version, comps, n, level, scale, payload, 0, 0, 0)


def test_ct_header_parsing(pkg):
    from rnsckks_gb300._lib import call, RcError
    buf = np.frombuffer(_ct_header(), dtype=np.uint8).copy()
    assert buf.size == 64
    n, lv, sb, comps = ctypes.c_uint64(), ctypes.c_int32(), ctypes.c_int32(), ctypes.c_uint32()
    call("rc_ct_header", buf.ctypes.data, buf.size, ctypes.byref(n), ctypes.byref(lv), ctypes.byref(sb),
         ctypes.byref(comps))
    assert (n.value, lv.value, sb.value, comps.value) == (4096, 3, 40, 2)
    for bad, msg in [(_ct_header(magic=b"RCKSKEY1"), "not a serialized ciphertext"),
                     (_ct_header(version=2), "unsupported serialized ciphertext version"),
                     (_ct_header()[:40], "truncated")]:
        b = np.frombuffer(bad, dtype=np.uint8).copy()
        with pytest.raises(RcError, match=msg):
            call("rc_ct_header", b.ctypes.data, b.size, None, None, None, None)


def _gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")


@pytest.fixture(scope="module")
def setup(pkg):
    _gpu()
    from rnsckks_gb300 import context as C
    params = pkg.params.hybrid_params(12, 6, 2, 50, 40)
    ctx = C.RnsCkksContext(params)
    kp = ctx.keygen(64, C.Sampler(3))
    rng = np.random.default_rng(4)
    n = params.poly_degree
    cts = [ctx.encrypt(ctx.encode(rng.uniform(-1, 1, n // 2) + 1j * rng.uniform(-1, 1, n // 2)), kp.public_key,
                       C.Sampler(10 + i)) for i in range(2)]
    return C, ctx, kp, cts, params


@pytest.mark.gpu
def test_keyswitch_key_round_trip(setup, tmp_path):
    C, ctx, kp, cts, params = setup
    relin = ctx.generate_relinearization_key(kp.secret_key, kp.public_key)
    ref = ctx.mult_relinearized(cts[0], cts[1], relin)
    path = tmp_path / "relin.rcksk"
    relin.save(path)
    back = ctx.load_keyswitch_key(path)
    assert (back.digits, back.level, back.aux_level_count, back.galois_element) == \
        (relin.digits, relin.level, relin.aux_level_count, 0)
    assert np.array_equal(ctx.mult_relinearized(cts[0], cts[1], back).numpy(), ref.numpy())
    # rotation key (galois element travels in the record)
    rk = ctx.generate_rotation_key(kp.secret_key, kp.public_key, 3)
    rpath = tmp_path / "rot3.rcksk"
    rk.keyswitch_key.save(rpath)
    rback = ctx.load_rotation_key(rpath)
    assert rback.galois_element == rk.galois_element
    assert np.array_equal(ctx.rotate(cts[0], rback).numpy(), ctx.rotate(cts[0], rk).numpy())


@pytest.mark.gpu
def test_truncated_q_only_key_round_trip(pkg):
    _gpu()
    from rnsckks_gb300 import context as C
    params = pkg.params.RnsCkksParams.small()
    ctx = C.RnsCkksContext(params)
    kp = ctx.keygen(64, C.Sampler(5))
    key = ctx.generate_relinearization_key(kp.secret_key, kp.public_key)
    short = key.drop_last_level()
    back = ctx.keyswitch_key_from_bytes(short.to_bytes())
    assert back.level == short.level and back.digits == short.digits
    ct = ctx.encrypt(ctx.encode_real(np.linspace(-1, 1, ctx.num_slots())), kp.public_key, C.Sampler(6))
    ct = ct.drop_last_level()
    assert np.array_equal(ctx.mult_relinearized(ct, ct, back).numpy(), ctx.mult_relinearized(ct, ct, short).numpy())
    assert len(short.to_bytes()) < len(key.to_bytes())  # the prefix of limbs only


@pytest.mark.gpu
def test_ciphertext_round_trip(setup):
    C, ctx, kp, cts, params = setup
    ct = cts[0]
    back = ctx.ciphertext_from_bytes(ctx.ciphertext_to_bytes(ct))
    assert (back.level, back.scale_bits) == (ct.level, ct.scale_bits)
    assert np.array_equal(back.numpy(), ct.numpy())
    quad = ctx.mult(cts[0], cts[1])
    qb = ctx.ciphertext_from_bytes(ctx.ciphertext_to_bytes(quad))
    assert isinstance(qb, C.RnsQuadraticCiphertext)
    assert np.array_equal(qb.numpy(), quad.numpy()) and qb.scale_bits == quad.scale_bits
    low = ct.drop_last_level()
    assert np.array_equal(ctx.ciphertext_from_bytes(ctx.ciphertext_to_bytes(low)).numpy(), low.numpy())


@pytest.mark.gpu
def test_damaged_records_are_refused(setup, pkg):
    C, ctx, kp, cts, params = setup
    from rnsckks_gb300._lib import RcError
    relin = ctx.generate_relinearization_key(kp.secret_key, kp.public_key)
    rec = bytearray(relin.to_bytes())
    flipped = bytearray(rec)
    flipped[200] ^= 1
    with pytest.raises(RcError, match="checksum mismatch"):
        ctx.keyswitch_key_from_bytes(bytes(flipped))
    with pytest.raises(RcError, match="truncated"):
        ctx.keyswitch_key_from_bytes(bytes(rec[:-8]))
    with pytest.raises(RcError, match="not a serialized keyswitch key"):
        ctx.keyswitch_key_from_bytes(b"X" + bytes(rec[1:]))
    other = C.RnsCkksContext(pkg.params.hybrid_params(12, 6, 2, 49, 40))
    with pytest.raises(RcError, match="another modulus chain"):
        other.keyswitch_key_from_bytes(bytes(rec))
    crec = bytearray(ctx.ciphertext_to_bytes(cts[0]))
    crec[100] ^= 4
    with pytest.raises(RcError, match="checksum mismatch"):
        ctx.ciphertext_from_bytes(bytes(crec))
    with pytest.raises(RcError, match="another modulus chain"):
        other.ciphertext_from_bytes(ctx.ciphertext_to_bytes(cts[0]))
    # a destination sized for a lower level than the record's is refused and left untouched
    import torch
    rec = np.frombuffer(ctx.ciphertext_to_bytes(cts[0]), dtype=np.uint8)
    small = torch.full((2, cts[0].level, params.poly_degree), 7, dtype=torch.int64, device="cuda")
    o = C.RcCiphertext(small.data_ptr(), 0, 0)
    with pytest.raises(RcError, match="does not fit the destination buffer"):
        C.call("rc_ct_deserialize", ctx.handle, rec.ctypes.data, rec.size, ctypes.byref(o), small.numel() * 8,
               C._stream())
    torch.cuda.synchronize()
    assert bool((small == 7).all())


@pytest.mark.gpu
def test_key_store_survives_restart(setup, pkg, tmp_path):
    """A server's keys saved, the context dropped, a fresh context on the same chain reopens the store and
    serves the same jobs with the same residues."""
    C, ctx, kp, cts, params = setup
    from rnsckks_gb300 import algorithms as A
    from rnsckks_gb300.server import KeyStore
    relin = ctx.generate_relinearization_key(kp.secret_key, kp.public_key)
    rots = A.generate_total_sum_rotation_keys(ctx, kp.secret_key, kp.public_key, cts[0].level, 8)
    store = KeyStore(ctx, tmp_path / "keys")
    store.put("relin", relin)
    store.put_group("total_sum", rots)
    want_mul = ctx.mult_relinearized(cts[0], cts[1], relin).numpy()
    want_sum = A.total_sum(ctx, cts[0], 8, rots).numpy()
    blobs = [ctx.ciphertext_to_bytes(c) for c in cts]

    fresh = C.RnsCkksContext(params)
    reopened = KeyStore.open(fresh, tmp_path / "keys")
    a, b = (fresh.ciphertext_from_bytes(x) for x in blobs)
    assert np.array_equal(fresh.mult_relinearized(a, b, reopened.get("relin")).numpy(), want_mul)
    got_rots = reopened.get("total_sum")
    assert sorted(got_rots) == sorted(rots)
    assert np.array_equal(A.total_sum(fresh, a, 8, got_rots).numpy(), want_sum)
