"""Autotuner for the library's launch-shape tunables.

The tunables (`rc_tune_set`: jobs per key-switch launch, jobs per CTA of the key product, the forward
butterfly mode, the fused tensor pass, the transforms' four-step split, CTAs per SM of their column pass and
polynomials per row block, jobs per stage and key-product groups of the host pipeline) change how work is
split into launches, never the results.  The tuner times each candidate on synthetic inputs of the caller's shape (ring degree, level,
batch), keeps the fastest, applies it to the context and caches the choice per (device, shape) in a JSON
file, so later runs apply it without measuring.
"""
from __future__ import annotations

import ctypes
import itertools
import json
import os
import time
from pathlib import Path
from typing import Callable, Dict, Iterable, List, Optional, Sequence

from ._lib import RcCiphertext, call

DEVICE_CANDIDATES: Dict[str, Sequence[int]] = {"ks_jobs": (8, 16, 32, 64), "mac_bc": (4, 8), "lazy_ntt": (0, 1),
                                               "fuse_tensor": (0, 1)}
# kernel shapes of the 64-bit transforms, tuned after the launch-shape tunables above (with their choice
# applied): CTAs per SM the column pass is compiled for (2 leaves it more registers), polynomials per row
# block (one twiddle staging each), and the four-step split (the column phase's log size; both phases must
# have 2^6..2^8 points, so at N = 2^16 only 8 x 8 exists); and the key product's form for job groups (one CTA
# per tile, or persistent CTAs taking (tile, limb) units with double-buffered digit tiles)
SHAPE_CANDIDATES: Dict[str, Sequence[int]] = {"col_ctas": (2, 3), "row_polys": (8, 16), "mac_persistent": (0, 1)}
# N = 2^16 only: the passes in the 16-residues-per-lane form (bits of "ntt_r16": 1 forward 64-bit columns, 8 the
# key product's dual-prime columns; 0 none)
R16_CANDIDATES: Sequence[int] = (9, 0)


def split_candidates(log_n: int) -> List[int]:
    """Column-phase log sizes of the four-step split for a ring of 2^log_n points (both phases 6..8)."""
    return [m for m in (6, 7, 8) if 6 <= log_n - m <= 8]
# host_edge: the first and last stages have chunk / host_edge jobs (a shorter fill and drain against one more
# stage's overhead)
# host_phased: 0 independent stages, 1 one key-product group, 2 two groups on two compute streams
HOST_CANDIDATES: Dict[str, Sequence[int]] = {"host_chunk": (2, 4, 8, 16), "host_phased": (0, 1, 2),
                                             "host_edge": (2, 4)}


def default_cache_path() -> Path:
    env = os.environ.get("RNSCKKS_TUNE_CACHE")
    if env:
        return Path(env)
    return Path(os.path.expanduser("~")) / ".cache" / "rnsckks_gb300" / "autotune.json"


def shape_key(device: str, n: int, limbs: int, aux: int, level: int, batch: int, what: str) -> str:
    return f"{what}|{device}|N={n}|L={limbs}|K={aux}|level={level}|batch={batch}"


def load_cache(path: Path) -> Dict[str, dict]:
    try:
        return json.loads(path.read_text())
    except (OSError, ValueError):
        return {}


def store_cache(path: Path, key: str, entry: dict) -> None:
    data = load_cache(path)
    data[key] = entry
    path.parent.mkdir(parents=True, exist_ok=True)
    tmp = path.with_suffix(".tmp")
    tmp.write_text(json.dumps(data, indent=1, sort_keys=True))
    tmp.replace(path)


def candidates(space: Dict[str, Sequence[int]]) -> List[Dict[str, int]]:
    names = sorted(space)
    return [dict(zip(names, vals)) for vals in itertools.product(*(space[n] for n in names))]


def choose(trials: Iterable[dict]) -> dict:
    """The fastest trial (ties: the first measured)."""
    best = None
    for t in trials:
        if t.get("ms") is None:
            continue
        if best is None or t["ms"] < best["ms"]:
            best = t
    if best is None:
        raise RuntimeError("no candidate ran")
    return best


def _valid(ctx, name: str, value: int) -> bool:
    if name == "lazy_ntt" and value:
        return all(q < (1 << 57) for q in ctx.q_moduli + ctx.p_moduli)
    return True


def apply(ctx, config: Dict[str, int]) -> None:
    for name, value in config.items():
        call("rc_tune_set", ctx.handle, name.encode(), int(value))


def current(ctx, names: Iterable[str]) -> Dict[str, int]:
    out = {}
    for n in names:
        v = ctypes.c_int32()
        call("rc_tune_get", ctx.handle, n.encode(), ctypes.byref(v))
        out[n] = v.value
    return out


def _measure(fn: Callable[[], None], reps: int, sync: Callable[[], None]) -> float:
    fn()
    sync()
    t0 = time.perf_counter()
    for _ in range(reps):
        fn()
    sync()
    return (time.perf_counter() - t0) * 1e3 / reps


def tune(ctx, what: str, run: Callable[[], None], level: int, batch: int,
         space: Dict[str, Sequence[int]], reps: int = 3, cache: Optional[Path] = None,
         use_cache: bool = True) -> dict:
    """Time `run` under every candidate of `space`, apply and cache the fastest."""
    import torch
    dev = torch.cuda.get_device_name()
    key = shape_key(dev, ctx.params.poly_degree, len(ctx.q_moduli), len(ctx.p_moduli), level, batch, what)
    path = cache or default_cache_path()
    if use_cache:
        hit = load_cache(path).get(key)
        if hit:
            apply(ctx, hit["choice"])
            return dict(hit, cached=True)
    before = current(ctx, space)
    trials = []
    for cand in candidates(space):
        if not all(_valid(ctx, n, v) for n, v in cand.items()):
            continue
        apply(ctx, cand)
        ms = _measure(run, reps, torch.cuda.synchronize)
        trials.append({"config": cand, "ms": round(ms, 4)})
    best = choose(trials)
    apply(ctx, best["config"])
    entry = {"choice": best["config"], "ms": best["ms"], "default": before, "trials": trials}
    store_cache(path, key, entry)
    return dict(entry, cached=False)


def tune_mult_relinearized(ctx, lhs, rhs, keys, outs, reps: int = 3, cache: Optional[Path] = None,
                           use_cache: bool = True) -> dict:
    """Device tunables for `rc_mult_relinearized_batch` on the given device-resident batch."""
    import torch
    n = len(lhs)
    L = (RcCiphertext * n)(*[a.raw() for a in lhs])
    R = (RcCiphertext * n)(*[b.raw() for b in rhs])
    O = (RcCiphertext * n)(*[RcCiphertext(o.data_ptr(), 0, 0) for o in outs])
    K = (ctypes.c_void_p * n)(*[k.handle for k in keys])
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    run = lambda: call("rc_mult_relinearized_batch", ctx.handle, n, L, R, K, O, s)
    launch = tune(ctx, "mult_relinearized_batch", run, lhs[0].level, n, DEVICE_CANDIDATES, reps, cache, use_cache)
    space = dict(SHAPE_CANDIDATES)
    splits = split_candidates(ctx.params.poly_degree.bit_length() - 1)
    if len(splits) > 1:
        space["ntt_split"] = splits
    if ctx.params.poly_degree == 1 << 16:  # which passes take the 16-residues-per-lane form (default, none)
        space["ntt_r16"] = R16_CANDIDATES
    shapes = tune(ctx, "mult_relinearized_batch_shapes", run, lhs[0].level, n, space, reps, cache, use_cache)
    return {"choice": dict(launch["choice"], **shapes["choice"]), "ms": shapes["ms"],
            "cached": launch["cached"] and shapes["cached"], "trials": launch.get("trials", []),
            "shape_trials": shapes.get("trials", [])}


def tune_host_pipeline(ctx, run: Callable[[], None], level: int, batch: int, reps: int = 2,
                       cache: Optional[Path] = None, use_cache: bool = True) -> dict:
    """`host_chunk` for the pipelined host-buffer entry; `run` makes one host-buffer batch call."""
    return tune(ctx, "mult_relinearized_batch_host", run, level, batch, HOST_CANDIDATES, reps, cache, use_cache)
