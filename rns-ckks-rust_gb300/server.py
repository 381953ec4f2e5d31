"""Continuous-batching request loop for homomorphic jobs on one GPU.

Jobs (relinearized Hadamard products, Halevi-Shoup dot products, Paterson-Stockmeyer polynomial evaluations)
arrive at any time with their ciphertexts and keys already resident on the device.  The scheduler keeps a
FIFO queue; whenever an execution slot is free it takes the oldest waiting job, gathers the waiting jobs that
can share its batched call (same routine, context and parameters), admits as many of them as the device
memory budget allows (each job declares its footprint: inputs, outputs, intermediates and scratch), and hands
the batch to the slot.  Slots run on their own CUDA streams, so batches overlap on the device; a job that
arrives while others run is admitted as soon as a slot and memory free up (continuous batching).  Each job
records arrival, admission and completion times; `stats()` gives throughput and p50/p99 latency.

Batched routines return the same residues as one-at-a-time calls (every kernel is an exact per-job function
of its inputs), so a job's result does not depend on what it was batched with.

The reference crate has no server; this module is the serving form the GPU build adds around the
`src/algorithms` routines and `mult_relinearized` (src/rns/context/ops.rs:124-133).
"""
from __future__ import annotations

import threading
import time
from collections import deque
from dataclasses import dataclass, field
from typing import Any, Callable, Dict, List, Optional, Sequence, Tuple

import numpy as np


@dataclass
class Job:
    """One request.  `batch_key` groups jobs that may share one batched call; `footprint` is the device memory
    (bytes) the job needs while it runs."""
    kind: str
    batch_key: Tuple
    footprint: int
    payload: Any = None
    arrival: float = 0.0
    admitted: float = 0.0
    done: float = 0.0
    result: Any = None
    error: Optional[BaseException] = None
    event: threading.Event = field(default_factory=threading.Event)

    @property
    def latency(self) -> float:
        return self.done - self.arrival

    def wait(self, timeout: Optional[float] = None) -> Any:
        if not self.event.wait(timeout):
            raise TimeoutError("job did not finish in time")
        if self.error is not None:
            raise self.error
        return self.result


class Scheduler:
    """Admission and batching policy (no GPU here).  `executor(slot, jobs)` runs a batch and returns the
    per-job results; it is called on the slot's worker thread."""

    def __init__(self, executor: Callable[[int, List[Job]], Sequence[Any]], slots: int = 3,
                 memory_budget: int = 1 << 34, max_batch: int = 16, clock: Callable[[], float] = time.perf_counter):
        if slots < 1:
            raise ValueError("at least one slot")
        self.executor = executor
        self.slots = slots
        self.budget = int(memory_budget)
        self.max_batch = max_batch
        self.clock = clock
        self.in_use = 0
        self.peak_in_use = 0
        self.queue: deque = deque()
        self.free_slots = list(range(slots))
        self.cv = threading.Condition()
        self.finished: List[Job] = []
        self.batches: List[Tuple[int, str, int]] = []  # (slot, kind, size)
        self._stop = False
        self._threads: List[threading.Thread] = []
        self._work: Dict[int, List[Job]] = {}

    # ---- client side ----
    def submit(self, job: Job) -> Job:
        if job.footprint > self.budget:
            raise ValueError(f"job needs {job.footprint} bytes of device memory, above the budget {self.budget}")
        with self.cv:
            job.arrival = self.clock()
            self.queue.append(job)
            self.cv.notify_all()
        return job

    def start(self) -> "Scheduler":
        self._stop = False
        t = threading.Thread(target=self._dispatch_loop, daemon=True)
        t.start()
        self._threads = [t]
        for s in range(self.slots):
            w = threading.Thread(target=self._worker_loop, args=(s,), daemon=True)
            w.start()
            self._threads.append(w)
        return self

    def drain(self, timeout: float = 600.0) -> None:
        """Wait until every submitted job has finished."""
        end = time.monotonic() + timeout
        with self.cv:
            while self.queue or self.in_use or len(self.free_slots) < self.slots:
                left = end - time.monotonic()
                if left <= 0:
                    raise TimeoutError("jobs still pending")
                self.cv.wait(min(left, 0.5))

    def stop(self) -> None:
        with self.cv:
            self._stop = True
            self.cv.notify_all()
        for t in self._threads:
            t.join(timeout=10)

    # ---- policy ----
    def _next_batch(self) -> Optional[List[Job]]:
        """Oldest waiting job plus the waiting jobs that share its batch key, in arrival order, as many as
        fit the memory still free (at least the oldest one, which always fits an empty device)."""
        if not self.queue:
            return None
        head = self.queue[0]
        if self.in_use + head.footprint > self.budget:
            return None  # wait for memory: keep FIFO order, no overtaking
        batch, used = [], self.in_use
        for job in list(self.queue):
            if len(batch) == self.max_batch:
                break
            if job.batch_key != head.batch_key:
                continue
            if used + job.footprint > self.budget:
                break
            batch.append(job)
            used += job.footprint
        for job in batch:
            self.queue.remove(job)
        return batch

    def _dispatch_loop(self) -> None:
        with self.cv:
            while not self._stop:
                if self.free_slots and self.queue:
                    batch = self._next_batch()
                    if batch:
                        slot = self.free_slots.pop(0)
                        now = self.clock()
                        for j in batch:
                            j.admitted = now
                        self.in_use += sum(j.footprint for j in batch)
                        self.peak_in_use = max(self.peak_in_use, self.in_use)
                        self.batches.append((slot, batch[0].kind, len(batch)))
                        self._work[slot] = batch
                        self.cv.notify_all()
                        continue
                self.cv.wait(0.05)

    def _worker_loop(self, slot: int) -> None:
        while True:
            with self.cv:
                while slot not in self._work and not self._stop:
                    self.cv.wait(0.05)
                if self._stop and slot not in self._work:
                    return
                batch = self._work.pop(slot)
            try:
                results = list(self.executor(slot, batch))
                err = None
            except BaseException as e:  # the jobs carry the error; the server keeps running
                results, err = [None] * len(batch), e
            now = self.clock()
            with self.cv:
                for j, r in zip(batch, results):
                    j.result, j.error, j.done = r, err, now
                    self.finished.append(j)
                self.in_use -= sum(j.footprint for j in batch)
                self.free_slots.append(slot)
                self.cv.notify_all()
            for j in batch:
                j.event.set()

    # ---- reporting ----
    def stats(self) -> Dict[str, Any]:
        done = [j for j in self.finished if j.error is None]
        if not done:
            return {"jobs": 0}
        lat = np.array([j.latency for j in done]) * 1e3
        span = max(j.done for j in done) - min(j.arrival for j in done)
        by_kind = {}
        for k in sorted({j.kind for j in done}):
            lk = np.array([j.latency for j in done if j.kind == k]) * 1e3
            by_kind[k] = {"jobs": int(lk.size), "p50_ms": round(float(np.percentile(lk, 50)), 3),
                          "p99_ms": round(float(np.percentile(lk, 99)), 3)}
        sizes = [b[2] for b in self.batches]
        return {"jobs": len(done), "throughput_jobs_per_s": round(len(done) / span, 2) if span > 0 else None,
                "p50_ms": round(float(np.percentile(lat, 50)), 3), "p99_ms": round(float(np.percentile(lat, 99)), 3),
                "mean_batch": round(float(np.mean(sizes)), 2) if sizes else 0,
                "peak_device_bytes": int(self.peak_in_use), "by_kind": by_kind}


# --------------------------------------------------------------------------------------------------------
# GPU executor: the three job kinds of the served workload
# --------------------------------------------------------------------------------------------------------

def ciphertext_bytes(n: int, limbs: int, comps: int = 2) -> int:
    return comps * limbs * n * 8


def keyswitch_scratch_bytes(n: int, limbs: int, aux: int, digits: int) -> int:
    """Per-job device scratch of one key switch on the wide path (digits, digit transforms, products) plus the
    quadratic ciphertext of a multiplication."""
    return digits * n * 4 + 2 * digits * 2 * n * 8 + 2 * (limbs + aux) * 2 * n * 8 + 3 * limbs * n * 8


class GpuExecutor:
    """Runs batches of jobs on per-slot CUDA streams through the batched routines of `algorithms` and the
    context.  Jobs carry (kind, ctx, inputs...); see `hadamard_job`, `halevi_shoup_job`,
    `paterson_stockmeyer_job`.  With `native` (the default) the Halevi-Shoup and Paterson-Stockmeyer batches
    run as one library call each (the native schedules, same residues)."""

    def __init__(self, slots: int, native: bool = True):
        import torch
        self.torch = torch
        self.native = native
        self.streams = [torch.cuda.Stream() for _ in range(slots)]

    def __call__(self, slot: int, jobs: List[Job]) -> List[Any]:
        from . import algorithms as A
        torch = self.torch
        with torch.cuda.stream(self.streams[slot]):
            kind = jobs[0].kind
            p0 = jobs[0].payload
            ctx = p0["ctx"]
            if kind == "hadamard":
                out = ctx.mult_relinearized_batch([j.payload["lhs"] for j in jobs], [j.payload["rhs"] for j in jobs],
                                                  [j.payload["key"] for j in jobs])
            elif kind == "halevi_shoup":
                hs = A.halevi_shoup_dot_product_native if self.native else A.halevi_shoup_dot_product_batch
                out = hs(ctx, [j.payload["ct"] for j in jobs], [j.payload["plain"] for j in jobs], p0["keys"])
            elif kind == "paterson_stockmeyer":
                if self.native:
                    out = A.paterson_stockmeyer_eval_native(ctx, [j.payload["ct"] for j in jobs], p0["coeffs"],
                                                            p0["keys"])
                else:
                    out = A.paterson_stockmeyer_eval_batch(ctx, [j.payload["ct"] for j in jobs], p0["coeffs"],
                                                           p0["keys"], p0.get("plains"))
            else:
                raise ValueError(f"unknown job kind {kind}")
            self.streams[slot].synchronize()
        return out


def hadamard_job(ctx, lhs, rhs, key) -> Job:
    n, limbs = ctx.params.poly_degree, lhs.level + 1
    aux = len(ctx.p_moduli)
    fp = 3 * ciphertext_bytes(n, limbs) + keyswitch_scratch_bytes(n, limbs, aux, ctx.decomp_digits(lhs.level))
    return Job("hadamard", ("hadamard", id(ctx), lhs.level, id(key)), fp,
               {"ctx": ctx, "lhs": lhs, "rhs": rhs, "key": key})


def halevi_shoup_job(ctx, ct, plain, keys) -> Job:
    n, limbs = ctx.params.poly_degree, ct.level + 1
    aux = len(ctx.p_moduli)
    fp = 4 * ciphertext_bytes(n, limbs) + keyswitch_scratch_bytes(n, limbs, aux, ctx.decomp_digits(ct.level))
    return Job("halevi_shoup", ("halevi_shoup", id(ctx), ct.level, len(plain), id(keys)), fp,
               {"ctx": ctx, "ct": ct, "plain": plain, "keys": keys})


def paterson_stockmeyer_job(ctx, ct, coeffs, keys, plains=None) -> Job:
    from . import algorithms as A
    n, limbs = ctx.params.poly_degree, ct.level + 1
    aux = len(ctx.p_moduli)
    b = A.paterson_stockmeyer_block_size(len(coeffs))
    blocks = -(-len(coeffs) // b)
    fp = (b + blocks + 3) * ciphertext_bytes(n, limbs) + keyswitch_scratch_bytes(n, limbs, aux,
                                                                                 ctx.decomp_digits(ct.level))
    return Job("paterson_stockmeyer", ("paterson_stockmeyer", id(ctx), ct.level, ct.scale_bits,
                                       tuple(float(c) for c in coeffs), id(keys)), fp,
               {"ctx": ctx, "ct": ct, "coeffs": list(coeffs), "keys": keys, "plains": plains})


class KeyStore:
    """Device-resident keys kept as serialised records in a directory, so a restarted server reloads them with
    one host->device copy each instead of generating and transforming them again.

    Keys are stored by name, singly (`put`) or as groups keyed by an integer (`put_group`: rotation keys by
    step, relinearization keys by level); `index.json` lists names, files and kinds.  `KeyStore.open` on a
    context with the same modulus chain reloads everything (a record made for another chain is refused by
    the library)."""

    INDEX = "index.json"

    def __init__(self, ctx, directory):
        import os
        self.ctx, self.dir = ctx, str(directory)
        os.makedirs(self.dir, exist_ok=True)
        self.index: Dict[str, Dict[str, Any]] = {}
        self.keys: Dict[str, Any] = {}

    def _path(self, fname: str) -> str:
        import os
        return os.path.join(self.dir, fname)

    def _write_index(self) -> None:
        import json
        import os
        tmp = self._path(self.INDEX + ".tmp")
        with open(tmp, "w") as f:
            json.dump(self.index, f, indent=1, sort_keys=True)
        os.replace(tmp, self._path(self.INDEX))

    @staticmethod
    def _switching_key(key):
        return getattr(key, "keyswitch_key", key)

    def _save_one(self, fname: str, key) -> None:
        self._switching_key(key).save(self._path(fname))

    def put(self, name: str, key) -> None:
        kind = "rotation" if hasattr(key, "keyswitch_key") else "keyswitch"
        fname = f"{name}.rcksk"
        self._save_one(fname, key)
        self.index[name] = {"kind": kind, "file": fname}
        self.keys[name] = key
        self._write_index()

    def put_group(self, name: str, keys: Dict[int, Any]) -> None:
        files, kind = {}, "keyswitch"
        for k, key in keys.items():
            kind = "rotation" if hasattr(key, "keyswitch_key") else "keyswitch"
            fname = f"{name}.{int(k)}.rcksk"
            self._save_one(fname, key)
            files[str(int(k))] = fname
        self.index[name] = {"kind": kind, "group": files}
        self.keys[name] = dict(keys)
        self._write_index()

    def get(self, name: str):
        return self.keys[name]

    def _load(self, kind: str, fname: str):
        if kind == "rotation":
            return self.ctx.load_rotation_key(self._path(fname))
        return self.ctx.load_keyswitch_key(self._path(fname))

    @classmethod
    def open(cls, ctx, directory) -> "KeyStore":
        """Reload every key listed in the directory's index onto `ctx`."""
        import json
        store = cls(ctx, directory)
        with open(store._path(cls.INDEX)) as f:
            store.index = json.load(f)
        for name, entry in store.index.items():
            if "group" in entry:
                store.keys[name] = {int(k): store._load(entry["kind"], fn) for k, fn in entry["group"].items()}
            else:
                store.keys[name] = store._load(entry["kind"], entry["file"])
        return store
