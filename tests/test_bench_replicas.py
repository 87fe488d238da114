"""bench.py's N > 1 path on CPU: world_size-2 gloo ranks, the slowest rank's
time taken by every rank, the whole-job value, and the reference arm running
on rank 0 only."""
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws))
    import torch.distributed as dist
    sys.path.insert(0, str(ROOT))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    ms = [10.0, 25.0][rank]
    t_max = bench.max_over_ranks(ms, ws, "cpu")
    value = bench.job_value(1e9, ws, t_max)
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, t_max, value))


def test_max_over_ranks_and_job_value_gloo_world_size_2():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t_max, value in out:
        assert t_max == 25.0                       # the slowest rank
        assert value == pytest.approx(2 * 1e9 / 0.025 / 1e9)   # both ranks' units over it


def test_reference_arm_nonzero_rank_exits_without_work():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "3"], cwd=ROOT, env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0
    assert r.stdout.strip() == ""
