"""CPU-side checks of the C ABI: the shared library loads and exports every
symbol include/rnsckks_gpu.h declares (no compute calls without a GPU), and
the Python binding table matches the header."""
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "rnsckks_gpu.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(rc_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_hot_path():
    names = declared_functions()
    for must in ("rc_context_create", "rc_mult_relinearized", "rc_mult_relinearized_batch", "rc_rotate",
                 "rc_relinearize", "rc_keyswitch", "rc_rescale", "rc_ntt_forward", "rc_ksk_upload",
                 "rc_mult_relinearized_host"):
        assert must in names


def test_library_exports_every_declared_symbol(pkg):
    pkg.build()
    lib = pkg.lib()
    for name in declared_functions():
        assert hasattr(lib, name), name


def test_profile_flags_switch_without_a_device(pkg):
    """rc_profile_enable takes RC_PROFILE_EVENTS (1) and RC_PROFILE_NVTX (2); switching is host-only."""
    text = HEADER.read_text()
    assert "#define RC_PROFILE_EVENTS 1" in text and "#define RC_PROFILE_NVTX 2" in text
    lib = pkg.lib()
    for flags in (2, 3, 1, 0):
        assert lib.rc_profile_enable(flags) == 0


def test_binding_table_covers_header(pkg):
    from rnsckks_gb300 import _lib
    bound = {s[0] for s in _lib.SIGNATURES}
    assert set(declared_functions()) == bound


def test_params_presets_validate(pkg):
    P = pkg.params
    P.RnsCkksParams.toy().validate()
    P.RnsCkksParams.small().validate()
    P.RnsCkksParams.realistic_8_level().validate()
    with pytest.raises(ValueError, match="distinct from the ciphertext modulus chain"):
        P.RnsCkksParams(8, [P.RnsPrime(998_244_353, 3)], [P.RnsPrime(998_244_353, 3)], 30).validate()
    b = P.bench_params()
    b.validate()
    assert b.poly_degree == 1 << 16 and len(b.primes) == 24 and len(b.aux_primes) == 2
    assert all(p.modulus.bit_length() == 50 for p in b.primes + b.aux_primes)
    assert P.num_decomp_digits(P.modulus_bits(b.q_moduli())) == 40
    a = P.plain_small_params()
    a.validate()
    assert [p.modulus.bit_length() for p in a.primes] == [60, 41, 41]
    assert all((p.modulus - 1) % (2 << 13) == 0 for p in a.primes)


def test_prime_search_follows_find_primes(pkg):
    P = pkg.params
    # find_primes.py scans q = k*2N + 1 upward from 2^(bits-1); every accepted prime
    # passes verify_ntt and uses its smallest primitive root
    found = P.find_ntt_primes(1 << 15, 50, 3)
    for q, g in found:
        assert (q - 1) % (1 << 16) == 0 and q.bit_length() == 50
        assert P.verify_ntt(1 << 15, q, g)
        assert g == P.primitive_root(q)
    assert [q for q, _ in found] == sorted(q for q, _ in found)
