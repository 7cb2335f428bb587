"""The multi-GPU path of the benchmark is replicas only: every rank runs its
own suspension and the ranks exchange one scalar (the max step time).  This
checks that host logic with two gloo ranks on the CPU."""
import json
import os
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _worker(rank, world, port, times, out):
    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms, value = bench.replica_throughput(times[rank], world, device="cpu")
    out[rank] = (ms, value, bench.replica_seed(rank))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_throughput_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    with ctx.Manager() as mgr:
        out = mgr.dict()
        times = [1.25, 2.0]
        port = 29500 + os.getpid() % 1000
        procs = [ctx.Process(target=_worker, args=(r, 2, port, times, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        res = dict(out)
    for r in range(2):
        ms, value, seed = res[r]
        assert ms == 2.0                      # max over ranks
        assert value == pytest.approx(2 * 1e3 / 2.0)  # whole-job: both replicas
    assert res[0][2] != res[1][2]             # independent suspensions


def test_reference_arm_only_rank0_prints():
    """Under torchrun the reference arm runs on rank 0; other ranks exit 0
    without work or output."""
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference",
                        "--steps", "1", "--warmup", "0"], env=env, capture_output=True,
                       text=True, timeout=120)
    assert r.returncode == 0
    assert r.stdout.strip() == ""


def test_replica_throughput_single_rank_has_no_collective():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.replica_throughput(4.0, 1) == (4.0, 250.0)
