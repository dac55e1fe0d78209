"""Path tracer with the neural radiance cache attached (vkg_tracer_attach_cache).

* bookkeeping: rendering paths end in the cache at their terminate_depth-th interaction, training
  paths produce records and optimiser steps, detaching restores the plain estimator bit for bit;
* what the trained network gains: the same estimator with the network's prediction replaced by zero
  (the path cut at its second bounce) is biased dark against the FP64 oracle; the trained cache
  removes most of that bias and lowers the RMSE at the same sample count.
"""
import math

import numpy as np
import pytest
import torch

from vierkant_gb300 import geometry
from vierkant_gb300.nrc import NeuralRadianceCache, cache_for_scene
from vierkant_gb300.pathtracer import PBRPathTracer, Scene, procedural_sky, sun_direction

pytestmark = pytest.mark.gpu

CROP = (576, 528, 128, 128)


@pytest.fixture(scope="module")
def world(ctx):
    sc = geometry.cornell_scene(0x5EED, 2, 64, 16)
    env = procedural_sky(ctx, 2048, 1024, sun_direction(), 5e4, 3.8e-5)
    scene = Scene(ctx, sc["xyz"], sc["indices"], sc["tri_material"], sc["materials"], env)
    cam = geometry.camera_lookat((0, 0, 3.4), (0, 0, 0), (0, 1, 0), 45.0, 1280, 720)
    yield {"scene": scene, "cam": cam}
    scene.close()


def settings(spp, crop):
    s = PBRPathTracer.default_settings()
    s.num_samples = spp
    s.max_trace_depth = 6
    s.rr_start_depth = 3
    for k in range(4):
        s.crop[k] = crop[k]
    return s


def lum(a):
    return 0.2126 * a[..., 0] + 0.7152 * a[..., 1] + 0.0722 * a[..., 2]


def test_cache_bookkeeping_and_detach(ctx, world):
    crop = (600, 500, 64, 64)
    cfg = NeuralRadianceCache.default_config()
    cfg.train_paths = 8192
    cache = cache_for_scene(ctx, world["scene"], cfg)
    lo, hi = world["scene"].bounds()
    assert all(cache.config.scene_min[a] < lo[a] and cache.config.scene_max[a] > hi[a] for a in range(3))
    pt = PBRPathTracer(ctx, seed=5, settings=settings(2, crop))
    plain_ref = PBRPathTracer(ctx, seed=5, settings=settings(2, crop))
    ref = plain_ref.render_scene(world["scene"], world["cam"]).clone()
    pt.attach_cache(cache)
    steps0 = cache.info().step
    for _ in range(3):
        img = pt.render_scene(world["scene"], world["cam"])
        st = pt.statistics()
        assert 0 < st.cache_queries <= 64 * 64 * 2
        assert 0 < st.train_records <= cfg.train_paths * cfg.train_depth
        assert st.train_ms > 0 and st.total_ms >= st.raytrace_ms
    assert torch.isfinite(img).all() and (img >= 0).all()
    # one optimiser step per non-empty window: 8192 x 4 records fit in one 65,536 window
    assert cache.info().step - steps0 == 3
    pt.attach_cache(None)
    pt.reset_accumulator()
    again = pt.render_scene(world["scene"], world["cam"])
    assert torch.equal(again, ref)
    pt.close()
    plain_ref.close()
    cache.close()


def _run(ctx, world, ref, mode, frames, warmup):
    pt = PBRPathTracer(ctx, seed=9, settings=settings(1, CROP))
    cfg = NeuralRadianceCache.default_config()
    if mode == "zero":
        cfg.train_paths = 0
    cache = cache_for_scene(ctx, world["scene"], cfg)
    if mode == "zero":
        cache.load_params(torch.zeros(cache.info().num_mlp_params, device="cuda"))
    pt.attach_cache(cache)
    for _ in range(warmup):
        pt.render_scene(world["scene"], world["cam"])
    pt.reset_accumulator()
    for _ in range(frames):
        img = pt.render_scene(world["scene"], world["cam"])
    img = img.cpu().numpy().astype(np.float64)
    pt.close()
    cache.close()
    bias = (img.sum() - ref.sum()) / ref.sum()
    rmse = math.sqrt(np.mean((lum(img) - lum(ref)) ** 2))
    return bias, rmse


def test_trained_cache_recovers_the_cut_paths(ctx, world, golden):
    g = golden("pt_oracle_crop")
    ref = g["mean"].astype(np.float64)
    assert tuple(g["crop"]) == CROP
    b0, r0 = _run(ctx, world, ref, "zero", 48, 8)
    b1, r1 = _run(ctx, world, ref, "nrc", 48, 8)
    print(f"without the network: bias {b0:+.4f} rmse {r0:.4f}   trained cache: bias {b1:+.4f} rmse {r1:.4f}")
    assert b0 < -0.04  # the second bounce onwards is missing
    assert abs(b1) < 0.4 * abs(b0)
    assert r1 < r0
