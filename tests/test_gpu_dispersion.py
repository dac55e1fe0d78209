"""Chromatic dispersion (KHR_materials_dispersion; raypipeline.slang:481-491, :651-659,
utils/bsdf.slang:46-91) on the GPU:

* the showcase scene with its transmissive spheres dispersive matches the FP32 twin path for path
  (one more uniform per segment, the wavelength; the Cauchy ior; the lock and tint at the first
  transmission, the locked wavelength kept at FP16);
* against the FP64 oracle fixture (256x144, 4096 spp) the image passes the statistical test of the
  other radiance tests (radiance_stats);
* a white furnace: a smooth dispersive glass sphere under a constant unit environment stays white on
  average (the white balance of the wavelength's colour);
* a dispersion of 0 renders bit for bit like the material without the field, and a negative value is
  rejected.
"""
import math

import numpy as np
import pytest
import torch

import oracle
from radiance_stats import check, compare, render_batches, report
from test_gpu_pathtracer import d2h
from vierkant_gb300 import _lib, geometry
from vierkant_gb300.pathtracer import PBRPathTracer, Scene, procedural_sky, sun_direction

pytestmark = pytest.mark.gpu

W, H = 256, 144
SUN_PEAK, SUN_WIDTH = 50.0, 0.02


def settings(spp, max_depth=8, rr=3, res=(W, H)):
    s = PBRPathTracer.default_settings()
    s.resolution[0], s.resolution[1] = res
    s.num_samples, s.max_trace_depth, s.rr_start_depth, s.mis_mode = spp, max_depth, rr, 0
    return s


@pytest.fixture(scope="module")
def prism(ctx):
    sc = geometry.cornell_scene(0x5EED, 2, 64, 16)
    mats = geometry.dispersive_materials(geometry.showcase_materials(sc["materials"]), 3.0)
    assert (mats["dispersion"] > 0).sum() > 0
    env = procedural_sky(ctx, 2048, 1024, sun_direction(), SUN_PEAK, SUN_WIDTH)
    scene = Scene(ctx, sc["xyz"], sc["indices"], sc["tri_material"], mats, env)
    cam = geometry.camera_lookat((0, 0, 3.4), (0, 0, 0), (0, 1, 0), 45.0, W, H)
    th = float(np.float32(math.tan(math.radians(45.0) / 2.0)))
    ocam = oracle.camera((0, 0, 3.4), (0, 0, 0), (0, 1, 0), th, W, H)
    yield {"sc": sc, "mats": mats, "env": env, "scene": scene, "cam": cam, "ocam": ocam}
    scene.close()


def test_twin_parity_path_for_path(ctx, prism):
    spp = 8
    pt = PBRPathTracer(ctx, seed=0x5EED, settings=settings(spp))
    img = pt.render_scene(prism["scene"], prism["cam"]).cpu().numpy().astype(np.float64)
    st = pt.statistics()
    pt.close()
    wptr, aptr, EW, EH = prism["scene"].env_tables()
    n = EW * EH
    w = d2h(wptr, 4 * n, np.float32)
    tab = d2h(aptr, 8 * n, np.uint32).reshape(n, 2)
    prob = np.ascontiguousarray(tab[:, 0].view(np.float32))
    alias = np.ascontiguousarray(tab[:, 1])
    sc = prism["sc"]
    bvh = oracle.CpuBVH(sc["xyz"], sc["indices"], 4)
    twin, _, rays = oracle.pt_render(False, sc["xyz"], sc["indices"], sc["tri_material"], prism["mats"], bvh,
                                     prism["env"].cpu().numpy(), prism["ocam"], spp, seed=0x5EED, batch=0,
                                     max_depth=8, rr_depth=3, alias_prob=prob, alias=alias, weight=w)
    rel = np.abs(img - twin) / np.maximum(np.abs(twin), 1e-2)
    close = np.mean(np.all(rel < 1e-3, axis=-1))
    print(f"close {close:.4f} sum ratio {img.sum() / twin.sum():.5f} rays {st.extension_rays}/{rays[0]} "
          f"{st.shadow_rays}/{rays[1]}")
    assert close > 0.9, close
    assert abs(img.sum() / twin.sum() - 1.0) < 0.02
    assert abs(st.extension_rays / rays[0] - 1.0) < 0.01
    assert abs(st.shadow_rays / rays[1] - 1.0) < 0.01


def test_radiance_against_fp64_oracle(ctx, prism, golden):
    g = golden("pt_oracle_dispersion")
    assert tuple(g["size"]) == (W, H) and int(g["max_depth"]) == 8 and float(g["dispersion"]) == 3.0
    imgs = render_batches(lambda seed: PBRPathTracer(ctx, seed=seed, settings=settings(256)), prism["scene"],
                          prism["cam"], 16)
    st = compare(imgs, g["mean"], g["lum_var"], int(g["spp"]))
    report("dispersive showcase vs FP64 oracle", st)
    check(st)


def test_dispersive_glass_white_furnace(ctx):
    xyz, idx = oracle.icosphere(1.0, 4)
    mats = geometry.default_materials(1)
    mats["transmission"][0] = 1.0
    mats["roughness"][0] = 0.0
    mats["dispersion"][0] = 3.0
    env = torch.ones((64, 128, 3), dtype=torch.float32, device="cuda")
    scene = Scene(ctx, xyz, idx, np.zeros(len(idx), np.uint32), mats, env)
    cam = geometry.camera_lookat((0, 0, 4.0), (0, 0, 0), (0, 1, 0), 40.0, 64, 64)
    pt = PBRPathTracer(ctx, seed=7, settings=settings(2048, max_depth=32, rr=0, res=(64, 64)))
    img = pt.render_scene(scene, cam).cpu().numpy().astype(np.float64)
    pt.close()
    scene.close()
    centre = img[24:40, 24:40].reshape(-1, 3).mean(axis=0)
    print("dispersive furnace centre", centre)
    assert np.all(np.abs(centre - 1.0) < 0.02), centre


def test_zero_dispersion_is_the_plain_material_and_negative_is_refused(ctx):
    sc = geometry.cornell_scene(0x5EED, 2, 16, 8)
    mats = geometry.showcase_materials(sc["materials"])
    env = procedural_sky(ctx, 256, 128, sun_direction(), SUN_PEAK, SUN_WIDTH)
    a_scene = Scene(ctx, sc["xyz"], sc["indices"], sc["tri_material"], mats, env)
    m0 = mats.copy()
    m0["dispersion"] = 0.0
    b_scene = Scene(ctx, sc["xyz"], sc["indices"], sc["tri_material"], m0, env)
    cam = geometry.camera_lookat((0, 0, 3.4), (0, 0, 0), (0, 1, 0), 45.0, 64, 36)
    a = PBRPathTracer(ctx, seed=3, settings=settings(4, res=(64, 36)))
    b = PBRPathTracer(ctx, seed=3, settings=settings(4, res=(64, 36)))
    assert torch.equal(a.render_scene(a_scene, cam), b.render_scene(b_scene, cam))
    bad = mats.copy()
    bad["dispersion"][0] = -1.0
    with pytest.raises(_lib.VkgError):
        Scene(ctx, sc["xyz"], sc["indices"], sc["tri_material"], bad, env)
    for o in (a, b, a_scene, b_scene):
        o.close()
