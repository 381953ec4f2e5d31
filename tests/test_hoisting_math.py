"""The index map behind hoisted rotations, on the CPU.

The key product reads the digit transforms of sigma_g(d) as those of d permuted: in the NTT domain sigma_g is
k -> k' with 2k'+1 = g (2k+1) mod 2N, and in the library's bit-reversed storage order position x reads
src(x) = bitrev(k'(bitrev(x))).  The kernel relies on two facts checked here: (1) the 32 positions of a tile
all read one source tile, through a permutation of its lanes; (2) the map is the automorphism's, shown on the
oracle's negacyclic evaluations (twist by psi^i, then the reference's cyclic NTT) against its coefficient-
domain automorphism.
"""
import numpy as np
import pytest


def bitrev(x: int, bits: int) -> int:
    return int(format(x, f"0{bits}b")[::-1], 2) if bits else 0


def galois_source(x: int, g: int, log_n: int) -> int:
    """The same arithmetic as the kernel's galois_source (32-bit wrap included)."""
    k = bitrev(x, log_n)
    kk = ((((g * (2 * k + 1)) & 0xFFFFFFFF) & ((2 << log_n) - 1)) - 1) >> 1
    return bitrev(kk, log_n)


def _galois_elements(log_n: int):
    two_n = 2 << log_n
    out = [pow(5, e, two_n) for e in (1, 2, 3, 7, (1 << (log_n - 1)) - 1)]
    out.append(two_n - 1)  # conjugation
    return out


@pytest.mark.parametrize("log_n", [5, 6, 8, 12, 15, 16])
def test_tiles_read_one_source_tile_through_a_lane_permutation(log_n):
    n = 1 << log_n
    for g in _galois_elements(log_n):
        seen = np.zeros(n, dtype=bool)
        for tile in range(n // 32):
            src = [galois_source(tile * 32 + lane, g, log_n) for lane in range(32)]
            assert len({s >> 5 for s in src}) == 1, (log_n, g, tile)
            assert sorted(s & 31 for s in src) == list(range(32)), (log_n, g, tile)
            seen[src] = True
        assert seen.all()  # a permutation of all positions


def test_map_is_the_automorphism_in_the_ntt_domain(pkg, oracle):
    log_n = 6
    n = 1 << log_n
    q, root = pkg.params.find_ntt_primes(n, 50, 1)[0]
    plans = oracle.Plans(n, [pkg.params.RnsPrime(q, root)])
    psi = pow(root, (q - 1) // (2 * n), q)
    twist = np.array([pow(psi, i, q) for i in range(n)], dtype=object)

    def evaluations(d):  # d(psi^(2k+1)) for k = 0..n-1: twist, then the reference's cyclic NTT
        t = np.array([(int(a) * int(w)) % q for a, w in zip(d, twist)], dtype=np.uint64)
        return oracle.ntt_forward(plans, 0, t)

    rng = np.random.default_rng(1)
    d = rng.integers(0, q, n, dtype=np.uint64)
    e = evaluations(d)
    stored = np.array([e[bitrev(x, log_n)] for x in range(n)], dtype=np.uint64)  # bit-reversed storage
    for g in _galois_elements(log_n):
        es = evaluations(oracle.poly_automorphism(d, q, g))
        stored_s = np.array([es[bitrev(x, log_n)] for x in range(n)], dtype=np.uint64)
        assert all(stored_s[x] == stored[galois_source(x, g, log_n)] for x in range(n)), g
