"""Analytic lights and the sun disc on the GPU.

* path-for-path twin: the FP32 CPU twin reproduces the GPU image of the Cornell box with the showcase
  materials, one light of every type and a sun disc (light NEE through glass included), with and
  without the refractive-caustic suppression;
* radiance: the GPU image has bias and RMSE against the committed FP64 oracle consistent with
  Monte-Carlo noise;
* a light body seen by a camera ray shows color x intensity (the hit-side MIS weight is 1 without an
  NEE competitor);
* MIS, NEE-only and BSDF-only converge to the same image when paths are long enough that the last
  vertex's untraced BSDF ray carries no light;
* invalid light records are rejected; the batch renderer renders lit jobs like the tracer.
"""
import math

import numpy as np
import pytest
import torch

import oracle
from radiance_stats import check, compare, render_batches, report
from vierkant_gb300 import _lib, geometry
from vierkant_gb300.pathtracer import (LIGHT_DISK, LIGHT_DTYPE, LIGHT_RECT, LIGHT_SPHERE, LIGHT_TUBE, PBRPathTracer,
                                       Scene, cornell_lights)
from test_gpu_pathtracer import d2h

pytestmark = pytest.mark.gpu

W, H = 256, 144
NUM_SPHERES = 16
ENV = 0.1
SUN = dict(color=(1.0, 0.95, 0.9), intensity=3.0, spherical_coords=(math.radians(30), math.radians(200)),
           angular_size=0.05)


def settings(spp, max_depth=8, rr=3, mis=0, res=(W, H), crop=(0, 0, 0, 0), sun=True, suppress=False):
    s = PBRPathTracer.default_settings()
    s.resolution[0], s.resolution[1] = res
    s.num_samples, s.max_trace_depth, s.rr_start_depth, s.mis_mode = spp, max_depth, rr, mis
    for k in range(4):
        s.crop[k] = crop[k]
    if sun:
        for c in range(3):
            s.sun_color[c] = SUN["color"][c]
        s.sun_intensity = SUN["intensity"]
        s.sun_spherical_coords[0], s.sun_spherical_coords[1] = SUN["spherical_coords"]
        s.sun_angular_size = SUN["angular_size"]
    s.suppress_refractive_caustics = int(suppress)
    return s


def oracle_lights():
    sun = oracle.sun_light(SUN["color"], SUN["intensity"], SUN["spherical_coords"], SUN["angular_size"])
    return np.concatenate([np.array([sun], oracle.LIGHT_DTYPE), cornell_lights().astype(oracle.LIGHT_DTYPE)])


@pytest.fixture(scope="module")
def lit(ctx):
    sc = geometry.cornell_scene(0x5EED, 2, NUM_SPHERES, 16)
    mats = geometry.showcase_materials(sc["materials"])
    env = torch.full((64, 128, 3), ENV, dtype=torch.float32, device="cuda")
    scene = Scene(ctx, sc["xyz"], sc["indices"], sc["tri_material"], mats, env)
    scene.set_lights(cornell_lights())
    cam = geometry.camera_lookat((0, 0, 3.4), (0, 0, 0), (0, 1, 0), 45.0, W, H)
    th = float(np.float32(math.tan(math.radians(45.0) / 2.0)))
    ocam = oracle.camera((0, 0, 3.4), (0, 0, 0), (0, 1, 0), th, W, H)
    yield {"sc": sc, "mats": mats, "env": env, "scene": scene, "cam": cam, "ocam": ocam}
    scene.close()


@pytest.mark.parametrize("suppress", [False, True])
def test_twin_parity_path_for_path(ctx, lit, suppress):
    spp = 8
    pt = PBRPathTracer(ctx, seed=0x5EED, settings=settings(spp, suppress=suppress))
    img = pt.render_scene(lit["scene"], lit["cam"]).cpu().numpy().astype(np.float64)
    st = pt.statistics()
    pt.close()
    wptr, aptr, EW, EH = lit["scene"].env_tables()
    n = EW * EH
    w = d2h(wptr, 4 * n, np.float32)
    tab = d2h(aptr, 8 * n, np.uint32).reshape(n, 2)
    prob = np.ascontiguousarray(tab[:, 0].view(np.float32))
    alias = np.ascontiguousarray(tab[:, 1])
    sc = lit["sc"]
    bvh = oracle.CpuBVH(sc["xyz"], sc["indices"], 4)
    twin, _, rays = oracle.pt_render(False, sc["xyz"], sc["indices"], sc["tri_material"], lit["mats"], bvh,
                                     lit["env"].cpu().numpy(), lit["ocam"], spp, seed=0x5EED, batch=0, max_depth=8,
                                     rr_depth=3, alias_prob=prob, alias=alias, weight=w, lights=oracle_lights(),
                                     suppress_caustics=suppress)
    rel = np.abs(img - twin) / np.maximum(np.abs(twin), 1e-2)
    close = np.mean(np.all(rel < 1e-3, axis=-1))
    print(f"suppress {suppress}: close {close:.4f} sum ratio {img.sum() / twin.sum():.5f} "
          f"rays {st.extension_rays}/{rays[0]} {st.shadow_rays}/{rays[1]}")
    assert close > 0.9, close
    assert abs(img.sum() / twin.sum() - 1.0) < 0.02
    assert abs(st.extension_rays / rays[0] - 1.0) < 0.01
    assert abs(st.shadow_rays / rays[1] - 1.0) < 0.01


def test_radiance_against_fp64_oracle(ctx, lit, golden):
    """64 independent 512-spp batches (32,768 spp) against the FP64 fixture (full frame, 16,384 spp): the
    luminance bias is within 3 standard errors of zero, with 3 standard errors below 0.5 % (the caustics
    through the glass spheres are heavy-tailed, so this scene needs the most samples), and the RMSE
    within 1.2x the noise of the two estimates (radiance_stats)"""
    g = golden("pt_oracle_lights")
    assert tuple(g["size"]) == (W, H) and int(g["max_depth"]) == 8 and int(g["num_spheres"]) == NUM_SPHERES
    imgs = render_batches(lambda seed: PBRPathTracer(ctx, seed=seed, settings=settings(512)), lit["scene"],
                          lit["cam"], 64)
    st = compare(imgs, g["mean"], g["lum_var"], int(g["spp"]))
    report("lit showcase vs FP64 oracle", st)
    check(st)


def _body(kind):
    L = np.zeros(1, LIGHT_DTYPE)
    L["type"], L["color"], L["intensity"], L["range"] = kind, (0.5, 0.7, 0.9), 4.0, np.inf
    L["position"] = (0.0, 0.0, 0.0)
    L["direction"] = (0.0, 0.0, 1.0)  # rect / disk emit toward the camera; the tube axis
    L["tangent"] = (1.0, 0.0, 0.0)
    L["size_x"], L["size_y"] = 0.5, 0.5
    if kind == LIGHT_TUBE:
        L["direction"] = (1.0, 0.0, 0.0)
    return L


@pytest.mark.parametrize("kind", [LIGHT_RECT, LIGHT_DISK, LIGHT_SPHERE, LIGHT_TUBE])
def test_light_body_seen_directly(ctx, kind):
    # one small triangle far behind the camera keeps the scene non-empty
    xyz = np.array([[0, 0, 50], [1, 0, 50], [0, 1, 50]], np.float32)
    idx = np.array([[0, 1, 2]], np.uint32)
    mats = geometry.default_materials(1)
    env = torch.zeros((8, 16, 3), dtype=torch.float32, device="cuda")
    scene = Scene(ctx, xyz, idx, np.zeros(1, np.uint32), mats, env)
    scene.set_lights(_body(kind))
    cam = geometry.camera_lookat((0, 0, 4), (0, 0, 0), (0, 1, 0), 30.0, 32, 32)
    pt = PBRPathTracer(ctx, seed=1, settings=settings(4, res=(32, 32), sun=False))
    img = pt.render_scene(scene, cam).cpu().numpy()
    pt.close()
    scene.close()
    centre = img[14:18, 14:18].reshape(-1, 3)
    assert np.allclose(centre, np.array([0.5, 0.7, 0.9], np.float32) * 4.0, rtol=1e-5), centre[0]
    assert np.all(img[0, 0] == 0.0)  # the corner ray misses the body


def test_mis_modes_converge(ctx, lit):
    """deep paths, the lower half of the box (no light body in view), opaque materials: the three
    estimators agree. (With glass they differ by design: light NEE passes glass with the reference's
    tint while BSDF paths refract, two estimates of different light transport.)"""
    sc = lit["sc"]
    scene = Scene(ctx, sc["xyz"], sc["indices"], sc["tri_material"], sc["materials"], lit["env"])
    scene.set_lights(cornell_lights())
    crop = (80, 80, 96, 48)
    means = []
    for mis in (0, 1, 2):
        pt = PBRPathTracer(ctx, seed=9, settings=settings(512, max_depth=24, mis=mis, crop=crop))
        means.append(pt.render_scene(scene, lit["cam"]).double().mean().item())
        pt.close()
    scene.close()
    print("MIS / NEE / BSDF", means)
    assert abs(means[1] / means[0] - 1.0) < 0.02
    assert abs(means[2] / means[0] - 1.0) < 0.03


@pytest.mark.parametrize("field,value", [("type", 3), ("type", 9), ("direction", (0, 0, 0)), ("size_x", 0.0),
                                         ("range", 0.0), ("intensity", -1.0)])
def test_invalid_lights_rejected(ctx, lit, field, value):
    L = cornell_lights()[:1].copy()  # a rect
    L[field] = value
    with pytest.raises(_lib.VkgError):
        lit["scene"].set_lights(L)
    lit["scene"].set_lights(cornell_lights())  # the scene keeps working


@pytest.mark.parametrize("extend,stack", [(1, 64), (2, 128)])
def test_batch_renders_lights_like_the_tracer(ctx, lit, extend, stack):
    """the batch renderer with lit jobs (scene lights, with and without the sun) next to an unlit one:
    the lit jobs' images equal the single-scene tracer's bit for bit, over two accumulated batches. A
    batch shades all its jobs with one kernel variant, here the full one, so the metal-rough job —
    which the tracer alone shades with the metal-roughness variant — agrees up to the rounding of
    the out-of-line BSDF evaluation (FMA contraction across the call)"""
    from vierkant_gb300.batch import BatchJob, BatchRenderer
    sc = lit["sc"]
    plain = Scene(ctx, sc["xyz"], sc["indices"], sc["tri_material"], sc["materials"], lit["env"])
    cam_s = geometry.camera_lookat((0, 0, 3.4), (0, 0, 0), (0, 1, 0), 45.0, 96, 64)
    jobs = [BatchJob(lit["scene"], cam_s, settings(3, res=(96, 64), sun=True), seed=1),
            BatchJob(plain, cam_s, settings(2, res=(96, 64), sun=False), seed=2),
            BatchJob(lit["scene"], cam_s, settings(4, res=(96, 64), sun=False, mis=1), seed=3)]
    t = BatchRenderer.default_tuning()
    t.extend_kernel, t.stack_depth = extend, stack
    br = BatchRenderer(ctx, jobs, t)
    for r in (1, 2):
        imgs = [i.clone() for i in br.render()]
        for k, job in enumerate(jobs):
            pt = PBRPathTracer(ctx, seed=job.seed, settings=job.settings)
            for _ in range(r):
                ref = pt.render_scene(job.scene, job.camera).clone()
            pt.close()
            if k == 1:
                assert torch.allclose(imgs[k], ref, rtol=1e-5, atol=1e-6), (k, r, (imgs[k] - ref).abs().max().item())
            else:
                assert torch.equal(imgs[k], ref), (k, r, (imgs[k] - ref).abs().max().item())
    br.close()
    plain.close()
