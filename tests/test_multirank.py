"""The multi-GPU (replica) path of bench.py on CPU: two gloo ranks run the same aggregation the
GPU ranks run -- a barrier, the maximum over ranks of the step time, and the whole-job throughput
world x work / slowest time -- and the reference arm leaves ranks other than 0 without work."""
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch

    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    torch.distributed.init_process_group("gloo", rank=rank, world_size=world, init_method="env://")
    try:
        import bench

        torch.distributed.barrier()
        ms = bench.max_over_ranks(3.0 + rank, world)  # the ranks' own step times differ
        q.put((rank, ms, bench.replica_throughput(1.0e9, ms * 1e-3, world)))
        torch.distributed.barrier()
    finally:
        torch.distributed.destroy_process_group()


def test_replicas_take_the_slowest_rank():
    import torch.multiprocessing as tmp

    ctx = tmp.get_context("spawn")
    q = ctx.Queue()
    world, port = 2, _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[1] for o in out] == [4.0, 4.0]  # every rank sees the slowest time
    assert out[0][2] == pytest.approx(2 * 1.0e9 / 4.0e-3)


def test_reference_arm_other_ranks_exit_without_work():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2"],
                       cwd=ROOT, env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip() == ""
