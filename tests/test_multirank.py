"""The replicas-only multi-GPU mode of bench.py, host side, as world-size-2 gloo ranks on the CPU: each
rank's timing is reduced to the maximum over ranks (the slowest replica sets the job's time), the
whole-job throughput counts every rank's units, and the reference arm runs on rank 0 alone (the
other ranks exit 0 without work or output)."""
import os
import subprocess
import sys
from pathlib import Path

import pytest
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, str(ROOT))
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ws, r, local = bench.dist_env()
    ms = bench.max_over_ranks(1.5 + rank, "cpu")  # rank 1 is slower
    out[rank] = (ws, r, local, ms, bench.replica_throughput(1_000_000, ws, ms))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_and_throughput_gloo():
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        port = 29500 + os.getpid() % 1000
        procs = [ctx.Process(target=_rank_main, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        res = dict(out)
    for rank in (0, 1):
        ws, r, local, ms, tput = res[rank]
        assert (ws, r, local) == (2, rank, rank)
        assert ms == 2.5  # every rank reports the slowest replica's time
        assert tput == pytest.approx(2_000_000 / 2.5e-3 / 1e6)


def test_single_rank_reduction_is_identity():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.max_over_ranks(3.25, "cpu") == 3.25
    assert bench.replica_throughput(5_772_303, 1, 2.0) == pytest.approx(2886.1515)


def test_reference_arm_runs_on_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1", "--warmup", "0"],
                       env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip() == ""
