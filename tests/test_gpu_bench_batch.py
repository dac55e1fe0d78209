"""The two benchmark arms trace the same bytes: the GPU arm's batch (GPU camera rays and GPU closest
hits, bounce rays on the host) equals the reference arm's (the oracle's camera rays and CPU BVH hits),
and the GPU's hits over the whole batch equal the CPU BVH traversal's with the reference's triangle
test."""
import math

import numpy as np
import pytest
import torch

import bench
import oracle
from vierkant_gb300 import geometry
from vierkant_gb300.raytracing import BVH

pytestmark = pytest.mark.gpu


def test_bench_batch_identical_in_both_arms(ctx):
    sc = geometry.cornell_scene(bench.SEED, 2, 64, 16)
    bvh = BVH(ctx, torch.from_numpy(sc["xyz"]).cuda(), torch.from_numpy(sc["indices"].astype(np.int32)).cuda())
    batch_dev, batch_np = bench.make_batch(ctx, bvh, 0)
    hits = bvh.closest_hit(batch_dev).cpu().numpy().view(np.uint32)
    bvh.close()

    osc = oracle.cornell_scene(bench.SEED, 2, 64, 16)
    th = float(np.float32(math.tan(math.radians(45.0) / 2.0)))
    cam = oracle.camera((0, 0, 3.4), (0, 0, 0), (0, 1, 0), th, bench.WIDTH, bench.HEIGHT)
    prim = oracle.camera_rays(cam, bench.SEED, 2, bench.SPP).view(np.float32).reshape(-1, 8)
    kind, trace = bench.cpu_bvh_tracer(osc["xyz"], osc["indices"])
    phits, _ = trace(prim)
    ref_batch = bench.bounce_batch(prim, phits.view(np.uint32).reshape(-1, 4), 4)
    assert batch_np.tobytes() == ref_batch.tobytes()
    assert bench.bench_config(196_618, batch_np) == bench.bench_config(196_618, ref_batch)
    cpu_hits, _ = trace(ref_batch)
    assert np.array_equal(hits, cpu_hits.view(np.uint32).reshape(-1, 4))
