"""Scheduler of the continuous-batching server, on the CPU with a fake executor: admission by device-memory
footprint, FIFO order, batching of jobs that share a batch key, continuous admission while batches run,
error isolation, and the latency report."""
import threading
import time

import pytest


@pytest.fixture(scope="module")
def S(pkg):
    from rnsckks_gb300 import server
    return server


class FakeGpu:
    """Records the memory held by running batches whenever a batch starts."""

    def __init__(self, delay=0.01):
        self.delay = delay
        self.lock = threading.Lock()
        self.running = 0
        self.peak = 0
        self.calls = []

    def __call__(self, slot, jobs):
        fp = sum(j.footprint for j in jobs)
        with self.lock:
            self.running += fp
            self.peak = max(self.peak, self.running)
            self.calls.append((slot, [j.payload for j in jobs]))
        time.sleep(self.delay)
        with self.lock:
            self.running -= fp
        if any(j.payload == "boom" for j in jobs):
            raise RuntimeError("injected failure")
        return [("done", j.payload) for j in jobs]


def test_admission_never_exceeds_the_memory_budget(S):
    gpu = FakeGpu(0.005)
    sch = S.Scheduler(gpu, slots=4, memory_budget=1000, max_batch=8).start()
    try:
        jobs = [sch.submit(S.Job("k", ("k", i % 3), footprint=100 + 37 * (i % 7), payload=i)) for i in range(120)]
        sch.drain(60)
    finally:
        sch.stop()
    assert all(j.wait(1) == ("done", j.payload) for j in jobs)
    assert gpu.peak <= 1000 and sch.peak_in_use <= 1000
    assert sch.in_use == 0


def test_oversized_job_is_refused(S):
    sch = S.Scheduler(FakeGpu(), slots=1, memory_budget=100)
    with pytest.raises(ValueError, match="above the budget"):
        sch.submit(S.Job("k", ("k",), footprint=101))


def test_jobs_sharing_a_key_are_batched_and_fifo_is_kept(S):
    gate = threading.Event()

    def exec_(slot, jobs):
        gate.wait(5)
        return [j.payload for j in jobs]

    sch = S.Scheduler(exec_, slots=1, memory_budget=10 ** 9, max_batch=4).start()
    try:
        first = sch.submit(S.Job("a", ("a",), 1, payload=0))
        time.sleep(0.1)  # job 0 occupies the only slot
        rest = [sch.submit(S.Job("b" if i % 2 else "a", ("b",) if i % 2 else ("a",), 1, payload=i))
                for i in range(1, 11)]
        gate.set()
        sch.drain(10)
    finally:
        sch.stop()
    sizes = [b[2] for b in sch.batches]
    kinds = [b[1] for b in sch.batches]
    assert sizes[0] == 1 and max(sizes) == 4  # later batches gather the waiting jobs of one key
    # the oldest waiting job is always in the next batch: job 1 (b) goes before jobs 2, 4 (a)
    assert kinds[:3] == ["a", "b", "a"]
    assert [j.wait(1) for j in [first] + rest] == list(range(11))


def test_jobs_arriving_while_others_run_are_admitted(S):
    gpu = FakeGpu(0.02)
    sch = S.Scheduler(gpu, slots=2, memory_budget=10 ** 6, max_batch=16).start()
    try:
        jobs = []
        for i in range(30):
            jobs.append(sch.submit(S.Job("k", ("k",), 10, payload=i)))
            time.sleep(0.003)
        sch.drain(30)
    finally:
        sch.stop()
    assert all(j.done >= j.admitted >= j.arrival for j in jobs)
    assert len(sch.batches) < 30  # some batches held several jobs
    st = sch.stats()
    assert st["jobs"] == 30 and st["p99_ms"] >= st["p50_ms"] > 0 and st["throughput_jobs_per_s"] > 0


def test_a_failing_batch_does_not_stop_the_server(S):
    gpu = FakeGpu(0.001)
    sch = S.Scheduler(gpu, slots=1, memory_budget=10 ** 6, max_batch=1).start()
    try:
        bad = sch.submit(S.Job("k", ("k",), 1, payload="boom"))
        good = sch.submit(S.Job("k", ("k",), 1, payload="fine"))
        sch.drain(10)
    finally:
        sch.stop()
    with pytest.raises(RuntimeError, match="injected failure"):
        bad.wait(1)
    assert good.wait(1) == ("done", "fine")
