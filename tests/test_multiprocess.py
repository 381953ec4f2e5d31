"""The multi-GPU form of the bench (replicas only: one process per GPU, no collective on the data path, a
barrier around the timed region and the maximum time over ranks) on the CPU with the gloo backend and two
ranks, as torchrun launches it (RANK / WORLD_SIZE / MASTER_ADDR / MASTER_PORT from the environment).
"""
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent

CHILD = r"""
import json, os, sys, time
sys.path.insert(0, {root!r})
import bench
rank, world, local = bench.dist_setup(2)
assert (world, local) == (2, 0), (world, local)
# ranks time different amounts of work; every rank must see the maximum
t = 0.05 * (rank + 1)
time.sleep(t)
bench.barrier(world)
worst = bench.max_over_ranks(t, world)
# whole-job throughput of replicas: units of all ranks over the slowest rank's time
units_per_rank = 32
value = world * units_per_rank / worst
print(json.dumps({{"rank": rank, "worst": worst, "value": value}}), flush=True)
import torch.distributed as dist
dist.destroy_process_group()
"""


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_rank_gloo_barrier_and_max_over_ranks():
    pytest.importorskip("torch")
    port = _free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), WORLD_SIZE="2", LOCAL_RANK="0", MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES="")
        procs.append(subprocess.Popen([sys.executable, "-c", CHILD.format(root=str(ROOT))], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=120)
        assert p.returncode == 0, err[-2000:]
        outs.append(out.strip().splitlines()[-1])
    import json
    res = [json.loads(o) for o in outs]
    assert {r["rank"] for r in res} == {0, 1}
    for r in res:
        assert abs(r["worst"] - 0.10) < 1e-9  # the slower rank's time, on both ranks
        assert abs(r["value"] - 2 * 32 / 0.10) < 1e-6
