"""The replica bookkeeping of `bench.py --gpus N` on CPU: two gloo ranks
rendezvous on 127.0.0.1, agree on the slowest rank's time, and the whole-job
figure counts every rank's bytes; the reference arm runs on rank 0 only."""
import os
import pathlib
import socket
import subprocess
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

ROOT = pathlib.Path(__file__).resolve().parent.parent


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, times, q):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, str(ROOT))
    import bench
    import torch.distributed as dist
    r, w = bench.dist_init()
    assert dist.get_backend() == "gloo"
    bench.dist_barrier(w)
    ms = bench.dist_max(w, times[r])
    q.put((r, w, ms, bench.whole_job_gbs(w, 10 ** 9, ms)))
    bench.dist_barrier(w)
    dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time():
    if torch.cuda.is_available():
        pytest.skip("the CPU replica test runs where no GPU is visible")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    times = [2.0, 3.0]
    procs = [ctx.Process(target=_rank, args=(r, 2, port, times, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs)
    got = sorted(q.get(timeout=5) for _ in range(2))
    for r, w, ms, gbs in got:
        assert w == 2 and ms == 3.0
        assert abs(gbs - 2 * 1e9 / 3e-3 / 1e9) < 1e-9  # both ranks' bytes over the slowest time


def test_reference_arm_runs_on_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1", MASTER_ADDR="127.0.0.1")
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--gpus", "2"],
                       env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0
    assert r.stdout.strip() == ""
