"""bench.py's replica plumbing on CPU processes: two ranks over gloo on
127.0.0.1, a barrier on both sides of the timed region and the max over ranks
(no data-path collective), as `bench.py --gpus 2` runs under torchrun."""
import multiprocessing as mp
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE="2", LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    r, world, local = bench.dist_env()
    d = bench.Dist(world)
    d.barrier()
    worst = d.max(10.0 * (r + 1))            # rank 1 is the slower one
    d.barrier()
    d.close()
    q.put((r, world, local, worst))


def test_two_ranks_barrier_and_max_over_ranks():
    pytest.importorskip("torch.distributed")
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    try:
        got = sorted(q.get(timeout=120) for _ in procs)
    finally:
        for p in procs:
            p.join(timeout=60)
            if p.is_alive():
                p.kill()
    assert got == [(0, 2, 0, 20.0), (1, 2, 1, 20.0)]
    assert all(p.exitcode == 0 for p in procs)


def test_reference_arm_other_ranks_exit_without_work():
    """Under torchrun only rank 0 times and prints the reference arm; rank 1
    exits 0 at once with no output (no process group to wait on)."""
    import subprocess
    import time
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1", MASTER_ADDR="127.0.0.1",
               MASTER_PORT="29533")
    t0 = time.time()
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2",
                          "--steps", "1", "--warmup", "3"], capture_output=True, text=True, env=env, timeout=120)
    assert out.returncode == 0, out.stderr
    assert out.stdout.strip() == ""
    assert time.time() - t0 < 60
