"""Alpha-masked and blended materials on the GPU (the reference's any-hit coverage test,
raypipeline.slang:686-720, visibility_test.slang:45-87 and :131-152):

* path for path against the FP32 twin, and in radiance against the FP64 fixture pt_oracle_alpha.npz
  (radiance_stats), on the Cornell scene with a masked wall and masked / blended spheres;
* masks of full coverage render bit for bit like the opaque scene, masks of zero coverage like the
  scene without that geometry;
* a blended emitter is seen by a fraction alpha of the paths, a blended occluder passes 1 - alpha of
  a light (the oracle's analytic cases);
* an instanced scene with masked instances renders like the single-level one.
"""
import math

import numpy as np
import pytest
import torch

import oracle
from alpha_scenes import CROP as QCROP
from alpha_scenes import EYE, FOVY, HEIGHT, TARGET, UP, WIDTH, blend_quads, blend_shadow, blend_stack, sun
from radiance_stats import check, compare, render_batches, report
from scene_helpers import split_cornell
from test_gpu_pathtracer import CROP, d2h, settings
from vierkant_gb300 import geometry
from vierkant_gb300._lib import BLEND_MASK
from vierkant_gb300.pathtracer import InstancedScene, PBRPathTracer, Scene, procedural_sky, sun_direction

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def world(ctx):
    sc = geometry.cornell_scene(0x5EED, 2, 64, 16)
    nrm = geometry.cornell_vertex_normals(sc)
    uv, tg = geometry.cornell_texcoords(sc)
    tex = geometry.alpha_textures()
    mats = geometry.alpha_materials(sc["materials"])
    env = procedural_sky(ctx, 2048, 1024, sun_direction(), 5e4, 3.8e-5)
    scene = Scene(ctx, sc["xyz"], sc["indices"], sc["tri_material"], mats, env)
    scene.set_normals(nrm)
    scene.set_texcoords(uv)
    scene.set_tangents(tg)
    scene.set_textures(tex)
    cam = geometry.camera_lookat((0, 0, 3.4), (0, 0, 0), (0, 1, 0), 45.0, 1280, 720)
    th = float(np.float32(math.tan(math.radians(45.0) / 2.0)))
    ocam = oracle.camera((0, 0, 3.4), (0, 0, 0), (0, 1, 0), th, 1280, 720)
    yield {"sc": sc, "nrm": nrm, "uv": uv, "tg": tg, "tex": tex, "mats": mats, "env": env, "scene": scene,
           "cam": cam, "ocam": ocam}
    scene.close()


@pytest.mark.parametrize("crop", [(600, 560, 48, 48), (330, 330, 48, 48), (700, 300, 48, 48)])
def test_twin_parity_alpha(ctx, world, crop):
    spp = 8
    pt = PBRPathTracer(ctx, seed=0x5EED, settings=settings(spp, crop))
    img = pt.render_scene(world["scene"], world["cam"]).cpu().numpy().astype(np.float64)
    st = pt.statistics()
    pt.close()
    wptr, aptr, W, H = world["scene"].env_tables()
    n = W * H
    w = d2h(wptr, 4 * n, np.float32)
    tab = d2h(aptr, 8 * n, np.uint32).reshape(n, 2)
    prob = np.ascontiguousarray(tab[:, 0].view(np.float32))
    alias = np.ascontiguousarray(tab[:, 1])
    sc = world["sc"]
    bvh = oracle.CpuBVH(sc["xyz"], sc["indices"], 4)
    twin, _, rays = oracle.pt_render(False, sc["xyz"], sc["indices"], sc["tri_material"], world["mats"], bvh,
                                     world["env"].cpu().numpy(), world["ocam"], spp, seed=0x5EED, batch=0,
                                     rr_depth=3, crop=crop, alias_prob=prob, alias=alias, weight=w,
                                     normals=world["nrm"], uv=world["uv"], tangents=world["tg"],
                                     textures=world["tex"])
    rel = np.abs(img - twin) / np.maximum(np.abs(twin), 1e-2)
    close = np.mean(np.all(rel < 1e-3, axis=-1))
    assert close > 0.97, close
    assert abs(img.sum() / twin.sum() - 1.0) < 0.02
    assert abs(st.extension_rays / rays[0] - 1.0) < 0.01
    assert rays[1] > 0 and abs(st.shadow_rays / rays[1] - 1.0) < 0.01


def test_radiance_alpha_against_fp64_oracle(ctx, world, golden):
    g = golden("pt_oracle_alpha")
    assert tuple(g["crop"]) == CROP
    imgs = render_batches(lambda seed: PBRPathTracer(ctx, seed=seed, settings=settings(64, CROP)),
                          world["scene"], world["cam"], 16)
    st = compare(imgs, g["mean"], g["lum_var"], int(g["spp"]))
    report("Cornell crop, alpha masks and blends, vs FP64 oracle", st)
    check(st)


def _render(ctx, scene, cam, crop, spp=4, seed=6, max_depth=6, resolution=(1280, 720)):
    s = settings(spp, crop, max_depth=max_depth)
    s.resolution[0], s.resolution[1] = resolution
    p = PBRPathTracer(ctx, seed=seed, settings=s)
    img = p.render_scene(scene, cam).clone()
    p.close()
    return img


def test_full_and_zero_coverage(ctx, world):
    sc = world["sc"]
    # opaque and untextured, so that a mask's coverage is its material alpha
    base = world["mats"].copy()
    base["blend_mode"] = 0
    base["tex_color"] = 0xFFFFFFFF
    crop = (520, 300, 96, 96)

    def scene(mats, idx=None, tm=None):
        s = Scene(ctx, sc["xyz"], sc["indices"] if idx is None else idx,
                  sc["tri_material"] if tm is None else tm, mats, world["env"])
        s.set_normals(world["nrm"])
        s.set_texcoords(world["uv"])
        s.set_tangents(world["tg"])
        s.set_textures(world["tex"])
        return s

    s = scene(base)
    plain = _render(ctx, s, world["cam"], crop)
    s.close()
    full = base.copy()
    full["blend_mode"] = BLEND_MASK
    full["alpha"] = 1.0  # >= the cut-off everywhere
    s = scene(full)
    masked = _render(ctx, s, world["cam"], crop)
    s.close()
    assert torch.equal(plain, masked)
    # the last 16 spheres masked at alpha 0.25 < 0.5: as if their triangles were gone (they end the list)
    gone = np.arange(3 + 48, 3 + 64)
    zero = base.copy()
    zero["blend_mode"][gone] = BLEND_MASK
    zero["alpha"][gone] = 0.25
    s = scene(zero)
    a = _render(ctx, s, world["cam"], crop)
    s.close()
    keep = int(np.argmax(np.isin(sc["tri_material"], gone)))
    assert np.all(np.isin(sc["tri_material"][keep:], gone))
    s = scene(base, sc["indices"][:keep], sc["tri_material"][:keep])
    b = _render(ctx, s, world["cam"], crop)
    s.close()
    assert torch.equal(a, b)
    assert not torch.equal(plain, b)


def _quad_scene(ctx, xyz, idx, tm, m):
    env = torch.full((32, 64, 3), 1e-4, dtype=torch.float32, device="cuda")
    return Scene(ctx, xyz, idx, tm, m, env)


@pytest.mark.parametrize("alpha", [0.3, 0.75])
def test_blended_emitter_is_seen_by_alpha_of_the_paths(ctx, alpha):
    s = _quad_scene(ctx, *blend_quads(alpha))
    cam = geometry.camera_lookat(EYE, TARGET, UP, FOVY, WIDTH, HEIGHT)
    spp = 256
    img = _render(ctx, s, cam, QCROP, spp=spp, max_depth=1, resolution=(WIDTH, HEIGHT)).cpu().numpy().astype(np.float64)
    s.close()
    mean = img[..., :3].mean(axis=(0, 1))
    n = QCROP[2] * QCROP[3] * spp
    tol = 5.0 * math.sqrt(alpha * (1 - alpha) / n) + 1e-3
    assert abs(mean[0] - alpha) < tol, mean
    assert abs(mean[2] - (1 - alpha)) < tol, mean


def test_blended_candidates_of_a_ray_share_one_uniform(ctx):
    alpha = 0.4
    s = _quad_scene(ctx, *blend_stack(alpha))
    cam = geometry.camera_lookat(EYE, TARGET, UP, FOVY, WIDTH, HEIGHT)
    spp = 256
    img = _render(ctx, s, cam, QCROP, spp=spp, max_depth=1, resolution=(WIDTH, HEIGHT)).cpu().numpy().astype(np.float64)
    s.close()
    mean = img[..., :3].mean(axis=(0, 1))
    n = QCROP[2] * QCROP[3] * spp
    tol = 5.0 * math.sqrt(alpha * (1 - alpha) / n) + 1e-3
    assert abs(mean[0] - alpha) < tol and abs(mean[2] - (1 - alpha)) < tol, mean
    assert mean[1] < 1e-3, mean  # independent uniforms would show green at a (1 - a) = 0.24


def test_blended_occluder_passes_one_minus_alpha_of_the_light(ctx):
    alpha = 0.35
    cam = geometry.camera_lookat(EYE, TARGET, UP, FOVY, WIDTH, HEIGHT)
    out = []
    for occ in (False, True):
        s = _quad_scene(ctx, *blend_shadow(alpha, occ))
        s.set_lights(sun())
        out.append(_render(ctx, s, cam, QCROP, spp=128, max_depth=1, resolution=(WIDTH, HEIGHT))[..., :3].double().mean().item())
        s.close()
    open_, shaded = out
    assert open_ > 0.05
    n = QCROP[2] * QCROP[3] * 128
    assert abs(shaded / open_ - (1 - alpha)) < 5.0 * math.sqrt(alpha * (1 - alpha) / n) + 2e-3, (open_, shaded)


def test_instanced_masks_match_single_level(ctx, world):
    sc = geometry.cornell_scene(0x5EED, 2, 8, 8)
    nrm = geometry.cornell_vertex_normals(sc)
    uv, tg = geometry.cornell_texcoords(sc)
    mats = geometry.alpha_materials(sc["materials"])
    # masks only: blended candidates draw their shadow-ray uniforms per (instance, triangle), which
    # differ between the two scenes' numbering
    mats["blend_mode"] = np.where(mats["blend_mode"] == BLEND_MASK, BLEND_MASK, 0)
    meshes, inst = split_cornell(sc, tess=8)
    idx = sc["indices"]
    groups = [(2 * q, 2 * q + 2) for q in range(5)] + [(10 + k * 768, 10 + (k + 1) * 768) for k in range(8)]
    used = [np.unique(idx[a:b].reshape(-1)) for a, b in groups]
    env = procedural_sky(ctx, 256, 128, sun_direction(), 50.0, 0.02)
    cam = geometry.camera_lookat((0, 0, 3.4), (0, 0, 0), (0, 1, 0), 45.0, 1280, 720)
    crop = (300, 200, 160, 160)
    inst_scene = InstancedScene(ctx, meshes, inst, mats, env)
    for m, u in enumerate(used):
        inst_scene.set_normals(nrm[u], mesh=m)
        inst_scene.set_texcoords(uv[u], mesh=m)
        inst_scene.set_tangents(tg[u], mesh=m)
    inst_scene.set_textures(world["tex"])
    single = Scene(ctx, sc["xyz"], sc["indices"], sc["tri_material"], mats, env)
    single.set_normals(nrm)
    single.set_texcoords(uv)
    single.set_tangents(tg)
    single.set_textures(world["tex"])
    a = _render(ctx, inst_scene, cam, crop, spp=64, seed=11).cpu().numpy().astype(np.float64)
    b = _render(ctx, single, cam, crop, spp=64, seed=11).cpu().numpy().astype(np.float64)
    plain = mats.copy()
    plain["blend_mode"] = 0
    opaque = Scene(ctx, sc["xyz"], sc["indices"], sc["tri_material"], plain, env)
    opaque.set_normals(nrm)
    opaque.set_texcoords(uv)
    opaque.set_tangents(tg)
    opaque.set_textures(world["tex"])
    c = _render(ctx, opaque, cam, crop, spp=64, seed=11).cpu().numpy().astype(np.float64)
    for s in (inst_scene, single, opaque):
        s.close()
    assert abs(a.sum() / b.sum() - 1.0) < 0.02
    assert np.mean(np.abs(a - b)) < 0.1 * np.mean(np.abs(b))
    # the masks matter in this window
    assert np.mean(np.abs(c - b)) > 0.05 * np.mean(np.abs(b))
