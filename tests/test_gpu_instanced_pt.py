"""Path tracing instanced (two-level) scenes.

* identity instances: the Cornell scene split into one mesh per wall quad and per sphere, every mesh
  instanced once with the identity transform, renders bit for bit like the single-level scene (the
  object-space rays equal the world rays, shading points and normals come out identical, and the
  instance order follows the triangle order so closest-hit ties resolve alike);
* a small stress scene (terrain + many transformed instances) renders finite radiance with paths on
  both the terrain and the instances.
"""
import numpy as np
import pytest
import torch

from vierkant_gb300 import geometry
from vierkant_gb300.pathtracer import InstancedScene, PBRPathTracer, Scene, procedural_sky, sun_direction

pytestmark = pytest.mark.gpu

from radiance_stats import check, compare, lum, render_batches, report
from scene_helpers import split_cornell


def settings(spp, crop):
    s = PBRPathTracer.default_settings()
    s.num_samples, s.max_trace_depth, s.rr_start_depth = spp, 6, 3
    for k in range(4):
        s.crop[k] = crop[k]
    return s


def test_identity_instances_render_like_the_flat_scene(ctx):
    sc = geometry.cornell_scene(0x5EED, 2, 64, 16)
    env = procedural_sky(ctx, 1024, 512, sun_direction(), 5e4, 3.8e-5)
    flat = Scene(ctx, sc["xyz"], sc["indices"], sc["tri_material"], sc["materials"], env)
    meshes, inst = split_cornell(sc)
    inst_scene = InstancedScene(ctx, meshes, inst, sc["materials"], env)
    cam = geometry.camera_lookat((0, 0, 3.4), (0, 0, 0), (0, 1, 0), 45.0, 1280, 720)
    for crop in ((560, 500, 48, 48), (0, 0, 64, 40)):
        a = PBRPathTracer(ctx, seed=21, settings=settings(4, crop))
        b = PBRPathTracer(ctx, seed=21, settings=settings(4, crop))
        ia = a.render_scene(flat, cam).clone()
        ib = b.render_scene(inst_scene, cam).clone()
        sa, sb = a.statistics(), b.statistics()
        assert torch.equal(ia, ib), (ia - ib).abs().max().item()
        assert sa.extension_rays == sb.extension_rays and sa.shadow_rays == sb.shadow_rays
        a.close()
        b.close()
    # the instance boxes are unions of quantised (outward-rounded) BLAS child boxes: they contain the
    # geometry and exceed it by little
    lo, hi = np.array(inst_scene.bounds()[0]), np.array(inst_scene.bounds()[1])
    glo, ghi = sc["xyz"].min(axis=0), sc["xyz"].max(axis=0)
    assert np.all(lo <= glo) and np.all(hi >= ghi)
    assert np.all(glo - lo < 0.05 * (ghi - glo)) and np.all(hi - ghi < 0.05 * (ghi - glo))
    flat.close()
    inst_scene.close()


def test_small_stress_scene_renders(ctx):
    st = geometry.stress_scene(terrain_n=129, num_instances=2000, num_meshes=4, num_materials=16)
    env = procedural_sky(ctx, 512, 256, sun_direction(), 5e4, 3.8e-5)
    scene = InstancedScene(ctx, st["meshes"], st["instances"], st["materials"], env)
    cam = geometry.camera_lookat((0, 120, 300), (0, 0, 0), (0, 1, 0), 40.0, 384, 216)
    s = PBRPathTracer.default_settings()
    s.resolution[0], s.resolution[1] = 384, 216
    s.num_samples, s.max_trace_depth, s.rr_start_depth = 4, 8, 3
    pt = PBRPathTracer(ctx, seed=3, settings=s)
    img = pt.render_scene(scene, cam)
    stt = pt.statistics()
    assert torch.isfinite(img).all() and (img >= 0).all()
    assert stt.extension_rays > stt.paths  # bounces happened
    # the sky is visible near the top of the frame and geometry below it
    assert img[:10].mean() > 0 and img[-10:].mean() > 0
    pt.close()
    scene.close()


def test_instanced_radiance_against_fp64_oracle(ctx):
    """a small stress scene (terrain + 2,000 transformed instances): the GPU image of a crop against
    the FP64 oracle's instanced path at the same sample count, bias and RMSE within Monte-Carlo noise"""
    import math
    import oracle
    st = geometry.stress_scene(terrain_n=129, num_instances=2000, num_meshes=4, num_materials=16)
    sun = sun_direction()
    env_gpu = procedural_sky(ctx, 512, 256, sun, 5e4, 3.8e-5)
    scene = InstancedScene(ctx, st["meshes"], st["instances"], st["materials"], env_gpu)
    W, H, crop, spp = 384, 216, (150, 90, 32, 32), 512
    cam = geometry.camera_lookat((0, 120, 300), (0, 0, 0), (0, 1, 0), 40.0, W, H)
    s = PBRPathTracer.default_settings()
    s.resolution[0], s.resolution[1] = W, H
    s.num_samples, s.max_trace_depth, s.rr_start_depth = spp, 8, 3
    for k in range(4):
        s.crop[k] = crop[k]
    s.num_samples = spp // 8
    imgs = render_batches(lambda seed: PBRPathTracer(ctx, seed=seed, settings=s), scene, cam, 8, seed0=17)
    scene.close()
    th = float(np.float32(math.tan(math.radians(40.0) / 2.0)))
    ocam = oracle.camera((0, 120, 300), (0, 0, 0), (0, 1, 0), th, W, H)
    inst = st["instances"]
    ref, sq, _ = oracle.pt_render_instanced(st["meshes"], inst["transform"], inst["blas"], inst["material"],
                                            st["materials"], env_gpu.cpu().numpy(), ocam, spp, seed=99, max_depth=8,
                                            rr_depth=3, crop=crop)
    var = np.maximum(sq - lum(ref) ** 2, 0.0)
    stats = compare(imgs, ref, var, spp)
    report("instanced stress crop vs FP64 oracle", stats)
    # the oracle runs here at 512 spp on a 32^2 crop: its noise sets the resolution
    check(stats, max_bound=0.03)
