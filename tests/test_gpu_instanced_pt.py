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
from vierkant_gb300.raytracing import INSTANCE_DTYPE

pytestmark = pytest.mark.gpu

IDENTITY = np.array([1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0], np.float32)


def split_cornell(sc, tess=16):
    """one mesh per wall quad (2 triangles) and per sphere (12 tess^2 triangles), in triangle order"""
    xyz, idx, tm, mats = sc["xyz"], sc["indices"], sc["tri_material"], sc["materials"]
    groups = [(2 * q, 2 * q + 2) for q in range(5)]
    per = 12 * tess * tess
    groups += [(10 + k * per, 10 + (k + 1) * per) for k in range((len(idx) - 10) // per)]
    meshes, inst = [], np.zeros(len(groups), INSTANCE_DTYPE)
    for k, (a, b) in enumerate(groups):
        used, local = np.unique(idx[a:b].reshape(-1), return_inverse=True)
        m = int(tm[a])
        assert np.all(tm[a:b] == m)
        meshes.append((xyz[used], local.reshape(-1, 3).astype(np.uint32), int(mats[m]["twosided"])))
        inst[k]["transform"] = IDENTITY
        inst[k]["blas"] = k
        inst[k]["material"] = m
    return meshes, inst


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
    lo, hi = inst_scene.bounds()
    assert np.allclose(lo, sc["xyz"].min(axis=0), atol=1e-3) and np.allclose(hi, sc["xyz"].max(axis=0), atol=1e-3)
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
