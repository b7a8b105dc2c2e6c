"""The multi-rank path of bench.py (replicas only: one cavity per GPU, no data-path collective)
on CPU with the gloo backend, world size 2: the barrier and the max-over-ranks step time, and the
reference arm's rank rule (rank 0 alone works and prints)."""
import os
import socket
import subprocess
import sys

import pytest

from conftest import REPO

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as td
    sys.path.insert(0, REPO)
    import bench
    td.init_process_group("gloo", rank=rank, world_size=world)
    bench._barrier(td)
    v = bench._max_over_ranks(torch, td, 10.0 * (rank + 1))
    q.put((rank, v))
    td.destroy_process_group()


def test_max_over_ranks_with_gloo():
    ctx = torch.multiprocessing.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == {0: 20.0, 1: 20.0}


def test_reference_arm_runs_on_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--impl", "reference", "--steps", "1"],
                       capture_output=True, text=True, env=env, timeout=300)
    assert r.returncode == 0 and r.stdout.strip() == ""
