"""Host side of the benchmark: the PCG32 stream behind the bounce rays equals the oracle's PCG32, the
batch is a pure function of the camera rays and their hits, and the reference arm builds that batch
and times the CPU ray cast without loading the GPU library."""
import json
import math
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

import bench
import oracle

ROOT = Path(__file__).resolve().parents[1]


@pytest.mark.parametrize("n,stream,lanes", [(1, 1, 4), (9, 3, 4), (10_000, 4, 64), (123_457, 5, 4096)])
def test_pcg32_fill_matches_oracle(n, stream, lanes):
    ref = np.zeros(n, np.uint32)
    oracle.orc().orc_pcg32_fill(0x5EED, stream, 0, n, oracle.ptr(ref))
    assert np.array_equal(bench.pcg32_fill(0x5EED, stream, n, lanes=lanes), ref)


def small_batch():
    sc = oracle.cornell_scene(0x5EED, 2, 8, 4)
    th = float(np.float32(math.tan(math.radians(45.0) / 2.0)))
    cam = oracle.camera((0, 0, 3.4), (0, 0, 0), (0, 1, 0), th, 64, 36)
    prim = oracle.camera_rays(cam, 0x5EED, 2, 2).view(np.float32).reshape(-1, 8)
    bvh = oracle.CpuBVH(sc["xyz"], sc["indices"], leaf_max=2)
    hits = bvh.closest_hit(prim).view(np.uint32).reshape(-1, 4)
    return sc, bvh, prim, hits


def test_bounce_batch_layout():
    sc, bvh, prim, hits = small_batch()
    b = bench.bounce_batch(prim, hits, 4)
    hit = hits[:, 0] != 0xFFFFFFFF
    assert b.dtype == np.float32 and b.shape == (len(prim) + hit.sum(), 8)
    assert np.array_equal(b[: len(prim)], prim)
    sec = b[len(prim):]
    t = hits[hit, 1].view(np.float32)
    assert np.array_equal(sec[:, 0:3], prim[hit, 0:3] + prim[hit, 4:7] * t[:, None])
    assert np.all(sec[:, 3] == np.float32(1e-4)) and np.all(sec[:, 7] == np.float32(1e4))
    assert np.allclose(np.linalg.norm(sec[:, 4:7], axis=1), 1.0, atol=1e-6)
    # deterministic: the same inputs give the same bytes and digest
    assert bench.batch_digest(bench.bounce_batch(prim, hits, 4)) == bench.batch_digest(b)
    assert bench.batch_digest(bench.bounce_batch(prim, hits, 5)) != bench.batch_digest(b)


def test_cpu_bvh_baseline_hits_equal_bruteforce():
    sc, bvh, prim, hits = small_batch()
    b = bench.bounce_batch(prim, hits, 4)
    kind, trace = bench.cpu_bvh_tracer(sc["xyz"], sc["indices"])
    got, used = trace(b)
    ref = oracle.closest_hit_bruteforce(sc["xyz"], sc["indices"], b.view(oracle.RAY_DTYPE).reshape(-1))
    assert got.tobytes() == ref.tobytes()
    assert used >= 1 and kind in ("reference", "port")
    if oracle.ref() is not None:
        assert kind == "reference"


def test_reference_arm_runs_without_the_gpu_library(tmp_path):
    code = ("import sys, runpy; sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '0', "
            "'--cpu-seconds', '1.5']; runpy.run_path('bench.py', run_name='__main__'); "
            "bad = sorted(m for m in sys.modules if m.startswith('vierkant_gb300') or m == 'torch'); "
            "print('LOADED', bad)")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = r.stdout.strip().splitlines()
    line = json.loads(lines[0])
    assert lines[-1] == "LOADED []"
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["config"]["rays_per_step"] == 5_772_303
    assert line["cpu_baseline"]["kind"] in ("reference", "port")
