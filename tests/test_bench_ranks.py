"""CPU: the multi-rank host logic of bench.py - max over ranks of the timed
region and the whole-job aggregate - on two gloo ranks, and the reference
arm's rank handling (ranks other than 0 do nothing)."""
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


def _worker(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    local = [12.5, 40.0][rank]  # this rank's timed-region milliseconds
    m = bench.reduce_step_ms(local, world)
    out[rank] = (m, bench.aggregate_gpairs(m, world, 10, 1000))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_two_gloo_ranks_and_aggregate():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    for r in range(2):
        m, v = out[r]
        assert m == 40.0
        # 2 replicas x 10 steps x 1000^2 pairs in 40 ms
        assert v == pytest.approx(2 * 10 * 1e6 / 0.040 / 1e9)


def test_reference_arm_other_ranks_exit_quietly():
    env = dict(os.environ, WORLD_SIZE="2", RANK="1", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2",
                        "--steps", "1", "--warmup", "1"], env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0
    assert r.stdout.strip() == ""


def test_single_rank_reduction_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.reduce_step_ms(7.25, 1) == 7.25
    assert bench.aggregate_gpairs(10.0, 1, 5, 2000) == pytest.approx(5 * 4e6 / 0.010 / 1e9)
