"""Parity at the benchmark's own shapes: N = 2^16, 24 limbs of 50-bit primes, 2 aux primes, the reference's
base-2^30 gadget (40 digits at the top level), so the wide key product runs at its largest bound
(|S| <= 40 * 2^16 * 2^29 * q < 2^101 against four 29-bit internal primes).

* `mult_relinearized` (src/rns/context/ops.rs:124-133) through the batched entry point on two pairs and
  through the per-op entry point, each bit-exact against the oracle.
* The mixed-level relinearize + rescale batch (context/ops.rs:111-122 then 32-37) at 8, 16 and 24 limbs,
  captured in a CUDA graph and replayed, bit-exact against the oracle's relinearize and rescale.

The oracle takes about ten seconds per 24-limb operation on 16 host cores.
"""
import math
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # collected on CPU-only machines, never run there
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

from test_gpu_parity import rand_ct  # noqa: E402


@pytest.fixture(scope="module")
def env(pkg, oracle):
    pkg.lib()
    from rnsckks_gb300 import context as C
    oracle.set_threads(os.cpu_count() or 1)
    params = pkg.params.bench_params()
    ctx = C.RnsCkksContext(params)
    n = params.poly_degree
    qpl = oracle.Plans(n, params.primes)
    ppl = oracle.Plans(n, params.aux_primes)
    return C, ctx, params, qpl, ppl


def _key(rng, params, limbs):
    qm = params.q_moduli()[:limbs]
    allm = qm + params.p_moduli()
    D = math.ceil(math.prod(qm).bit_length() / 30)
    return np.stack([rand_ct(rng, allm, params.poly_degree) for _ in range(D)]), D


def test_headline_shape_batched_and_per_op_are_bit_exact(env, oracle):
    C, ctx, params, qpl, ppl = env
    n, q = params.poly_degree, params.q_moduli()
    assert n == 1 << 16 and len(q) == 24 and len(params.aux_primes) == 2
    rng = np.random.default_rng(0x24)
    key, D = _key(rng, params, 24)
    assert D == 40
    ksk = ctx.upload_keyswitch_key(key, 23, 2)
    pairs = [(rand_ct(rng, q, n), rand_ct(rng, q, n)) for _ in range(2)]
    lhs = [C.RnsCiphertext(C.to_device(a), 40) for a, _ in pairs]
    rhs = [C.RnsCiphertext(C.to_device(b), 40) for _, b in pairs]
    batched = [o.numpy() for o in ctx.mult_relinearized_batch(lhs, rhs, [ksk, ksk])]
    single = ctx.mult_relinearized(lhs[0], rhs[0], ksk).numpy()
    for (a, b), got in zip(pairs, batched):
        m0, m1 = oracle.mult_relinearized(qpl, ppl, a[0], a[1], b[0], b[1], key, D)
        assert np.array_equal(got[0], m0) and np.array_equal(got[1], m1)
    assert np.array_equal(single, batched[0])


def test_mixed_level_relinearize_rescale_graph_replay_is_bit_exact(env, oracle):
    C, ctx, params, qpl, ppl = env
    n, q = params.poly_degree, params.q_moduli()
    rng = np.random.default_rng(0xC)
    limbs_list = [24, 8, 16]
    keys, host = {}, {}
    for limbs in limbs_list:
        host[limbs] = _key(rng, params, limbs)
        keys[limbs] = ctx.upload_keyswitch_key(host[limbs][0], limbs - 1, 2)
    quads = [rand_ct(rng, q[:limbs], n, 3) for limbs in limbs_list]
    cts = [C.RnsQuadraticCiphertext(C.to_device(x), 80) for x in quads]
    ks = [keys[limbs] for limbs in limbs_list]
    side = torch.cuda.Stream()
    with torch.cuda.stream(side):
        ctx.reserve(23, len(cts))
        outs = [torch.zeros((2, limbs - 1, n), dtype=torch.int64, device="cuda") for limbs in limbs_list]
        graph = ctx.capture_graph(lambda: ctx.relinearize_rescale_batch(cts, ks, outs))
        graph.launch()
        side.synchronize()
        got = [C.to_host(o) for o in outs]
        for o in outs:
            o.zero_()
        graph.launch()  # a second replay gives the same residues
        side.synchronize()
        again = [C.to_host(o) for o in outs]
    torch.cuda.synchronize()
    for limbs, x, g, g2 in zip(limbs_list, quads, got, again):
        key, D = host[limbs]
        pl = qpl.prefix(limbs)
        r0, r1 = oracle.relinearize(pl, ppl, x[0], x[1], x[2], key, D)
        assert np.array_equal(g[0], oracle.rescale_poly(pl, r0)), limbs
        assert np.array_equal(g[1], oracle.rescale_poly(pl, r1)), limbs
        assert np.array_equal(g, g2)
