"""The multi-GPU path is replicas only: each rank simulates its own seeded model and
the ranks meet only to combine the timing (max over ranks) and the molecule-steps
(sum). That combination runs here on CPU ranks over gloo (world size 2), as bench.py
runs it over NCCL; the reference arm leaves ranks other than 0 without work."""
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, str(ROOT))
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    # rank r: (r + 1) seconds, 1000 * (r + 1) molecule-steps
    t, n = bench.combine_ranks(rank + 1.0, 1000 * (rank + 1), world, "cpu")
    dist.destroy_process_group()
    out.put((rank, t, n))


def test_ranks_combine_max_time_and_summed_steps():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res == [(0, 2.0, 3000.0), (1, 2.0, 3000.0)]


def test_one_rank_needs_no_process_group():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.combine_ranks(1.5, 42, 1, "cpu") == (1.5, 42.0)


def test_reference_arm_leaves_other_ranks_idle():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1", "--warmup", "1"],
                       env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0
    assert r.stdout.strip() == ""  # rank 1 prints nothing and does no work
