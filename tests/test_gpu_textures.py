"""Material textures on the GPU (vkg_scene_set_textures / _texcoords / _tangents; the reference's
closest-hit texture terms, raypipeline.slang:299-320, :526-608):

* path for path against the FP32 twin with the same texels (mip chains built alike), texture
  coordinates, tangents, normals and textured materials, and in radiance against the FP64 fixture
  pt_oracle_textured.npz (radiance_stats);
* removing the textures (or the texture coordinates) gives back the untextured image bit for bit;
* an instanced scene with per-mesh texture coordinates and tangents renders like the single-level one.
"""
import math

import numpy as np
import pytest
import torch

import oracle
from radiance_stats import check, compare, render_batches, report
from scene_helpers import split_cornell
from test_gpu_pathtracer import CROP, d2h, settings
from vierkant_gb300 import geometry
from vierkant_gb300.pathtracer import InstancedScene, PBRPathTracer, Scene, procedural_sky, sun_direction

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def world(ctx):
    sc = geometry.cornell_scene(0x5EED, 2, 64, 16)
    nrm = geometry.cornell_vertex_normals(sc)
    uv, tg = geometry.cornell_texcoords(sc)
    tex = geometry.test_textures()
    mats = geometry.textured_materials(sc["materials"])
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


@pytest.mark.parametrize("crop", [(600, 560, 48, 48), (620, 160, 48, 48)])
def test_twin_parity_textured(ctx, world, crop):
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


def test_radiance_textured_against_fp64_oracle(ctx, world, golden):
    g = golden("pt_oracle_textured")
    assert tuple(g["crop"]) == CROP
    imgs = render_batches(lambda seed: PBRPathTracer(ctx, seed=seed, settings=settings(64, CROP)),
                          world["scene"], world["cam"], 16)
    st = compare(imgs, g["mean"], g["lum_var"], int(g["spp"]))
    report("Cornell crop, textured, vs FP64 oracle", st)
    check(st)


def test_removing_textures_restores_the_untextured_image(ctx, world):
    sc = world["sc"]
    crop = (560, 300, 64, 64)
    s = Scene(ctx, sc["xyz"], sc["indices"], sc["tri_material"], world["mats"], world["env"])
    s.set_normals(world["nrm"])

    def render():
        p = PBRPathTracer(ctx, seed=6, settings=settings(4, crop))
        img = p.render_scene(s, world["cam"]).clone()
        p.close()
        return img

    plain = render()
    s.set_texcoords(world["uv"])
    s.set_tangents(world["tg"])
    s.set_textures(world["tex"])
    textured = render()
    s.set_texcoords(None)
    no_uv = render()
    s.set_texcoords(world["uv"])
    s.set_textures([])
    no_tex = render()
    s.close()
    assert not torch.equal(plain, textured)
    assert torch.equal(plain, no_tex)
    # without texture coordinates nothing is sampled: the untextured image, up to the rounding of the
    # shade kernel's textured build (a separate compilation of the same arithmetic)
    a_, b_ = plain.cpu().numpy().astype(np.float64), no_uv.cpu().numpy().astype(np.float64)
    close = np.mean(np.all(np.abs(a_ - b_) <= 1e-3 * np.maximum(np.abs(a_), 1e-2), axis=-1))
    assert close > 0.97, close


def test_instanced_textures_match_single_level(ctx, world):
    sc = geometry.cornell_scene(0x5EED, 2, 8, 8)
    nrm = geometry.cornell_vertex_normals(sc)
    uv, tg = geometry.cornell_texcoords(sc)
    mats = geometry.textured_materials(sc["materials"])
    meshes, inst = split_cornell(sc, tess=8)
    idx = sc["indices"]
    groups = [(2 * q, 2 * q + 2) for q in range(5)] + [(10 + k * 768, 10 + (k + 1) * 768) for k in range(8)]
    used = [np.unique(idx[a:b].reshape(-1)) for a, b in groups]
    env = procedural_sky(ctx, 256, 128, sun_direction(), 50.0, 0.02)
    cam = geometry.camera_lookat((0, 0, 3.4), (0, 0, 0), (0, 1, 0), 45.0, 1280, 720)
    crop = (400, 200, 96, 96)
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

    def render(scene):
        p = PBRPathTracer(ctx, seed=11, settings=settings(64, crop))
        img = p.render_scene(scene, cam).cpu().numpy().astype(np.float64)
        p.close()
        return img

    a, b = render(inst_scene), render(single)
    assert abs(a.sum() / b.sum() - 1.0) < 0.02
    assert np.mean(np.abs(a - b)) < 0.1 * np.mean(np.abs(b))
    inst_scene.close()
    single.close()


def test_gltf_textured_scene_renders_like_the_direct_one(ctx, world, tmp_path):
    """the textured Cornell scene written as a glTF asset (PNG images, TEXCOORD_0, TANGENT, NORMAL,
    texture slots) renders bit for bit like the same scene built directly"""
    from gltf_writer import png, write
    from vierkant_gb300.gltf import scene_from_gltf
    sc = geometry.cornell_scene(0x5EED, 2, 8, 8)
    nrm = geometry.cornell_vertex_normals(sc)
    uv, tg = geometry.cornell_texcoords(sc)
    mats = geometry.textured_materials(sc["materials"])
    meshes, inst = split_cornell(sc, tess=8)
    idx = sc["indices"]
    groups = [(2 * q, 2 * q + 2) for q in range(5)] + [(10 + k * 768, 10 + (k + 1) * 768) for k in range(8)]
    used = [np.unique(idx[a:b].reshape(-1)) for a, b in groups]
    tex = world["tex"]

    def tref(k):
        return {"index": int(k)} if k != 0xFFFFFFFF else None

    gmats = []
    for m in mats:
        g = {"pbrMetallicRoughness": {"baseColorFactor": [float(c) for c in m["base_color"]] + [1.0],
                                      "metallicFactor": float(m["metalness"]),
                                      "roughnessFactor": float(m["roughness"])},
             "doubleSided": bool(m["twosided"]), "emissiveFactor": [float(c) for c in m["emission"]]}
        for slot, key, where in (("tex_color", "baseColorTexture", "pbr"),
                                 ("tex_ao_rough_metal", "metallicRoughnessTexture", "pbr"),
                                 ("tex_normal", "normalTexture", "top"), ("tex_emission", "emissiveTexture", "top")):
            r = tref(m[slot])
            if r is not None:
                (g["pbrMetallicRoughness"] if where == "pbr" else g)[key] = r
        gmats.append(g)
    gm = [[(x, i, int(inst[k]["material"]), None, nrm[u], {"TEXCOORD_0": uv[u],
                                                             "TANGENT": np.c_[tg[u], np.ones(len(u), np.float32)]})]
          for k, ((x, i, _), u) in enumerate(zip(meshes, used))]
    path = tmp_path / "textured.glb"
    write(path, gm, [dict(mesh=k) for k in range(len(meshes))], list(range(len(meshes))), materials=gmats,
          mode="glb", images=[(png(t, 6, 8), 10497, 10497) for t in tex])
    env = procedural_sky(ctx, 256, 128, sun_direction(), 50.0, 0.02)
    loaded = scene_from_gltf(ctx, str(path), env)
    direct_mats = mats.copy()
    direct_mats["emission"] = np.where(mats["tex_emission"][:, None] != 0xFFFFFFFF, 0.0, mats["emission"])
    direct = InstancedScene(ctx, meshes, inst, direct_mats, env)
    for m, u in enumerate(used):
        direct.set_normals(nrm[u], mesh=m)
        direct.set_texcoords(uv[u], mesh=m)
        direct.set_tangents(tg[u], mesh=m)
    direct.set_textures(tex)
    cam = geometry.camera_lookat((0, 0, 3.4), (0, 0, 0), (0, 1, 0), 45.0, 1280, 720)
    for crop in ((560, 300, 64, 64), (600, 100, 64, 64)):
        p = PBRPathTracer(ctx, seed=4, settings=settings(4, crop))
        q_ = PBRPathTracer(ctx, seed=4, settings=settings(4, crop))
        ia = p.render_scene(loaded, cam).clone()
        ib = q_.render_scene(direct, cam).clone()
        assert torch.equal(ia, ib), (ia - ib).abs().max().item()
        p.close()
        q_.close()
    loaded.close()
    direct.close()


def test_uv_transform(ctx, world):
    """the texture-coordinate transform (raypipeline.slang:350): the identity renders bit for bit like
    none, scaling by 2 like texture coordinates scaled by 2 on primary hits (both read level 0), and a
    rotated transform matches the FP32 twin path for path"""
    sc = world["sc"]
    crop = (600, 560, 48, 48)

    def scene(mats, uv):
        s = Scene(ctx, sc["xyz"], sc["indices"], sc["tri_material"], mats, world["env"])
        s.set_normals(world["nrm"])
        s.set_texcoords(uv)
        s.set_tangents(world["tg"])
        s.set_textures(world["tex"])
        return s

    def render(mats, uv, depth=6, spp=4):
        s = scene(mats, uv)
        p = PBRPathTracer(ctx, seed=0x5EED, settings=settings(spp, crop, max_depth=depth))
        img = p.render_scene(s, world["cam"]).clone()
        p.close()
        s.close()
        return img

    base = world["mats"]
    plain = render(base, world["uv"])
    ident = base.copy()
    ident["has_uv_transform"] = 1
    ident["uv_transform"] = (1, 0, 0, 0, 1, 0)
    assert torch.equal(plain, render(ident, world["uv"]))
    twice = base.copy()
    twice["has_uv_transform"] = 1
    twice["uv_transform"] = (2, 0, 0, 0, 2, 0)
    a = render(twice, world["uv"], depth=1)
    assert torch.equal(a, render(base, world["uv"] * 2, depth=1))
    assert not torch.equal(a, render(base, world["uv"], depth=1))
    rot = base.copy()
    rot["has_uv_transform"] = 1
    c, s_ = math.cos(0.7), math.sin(0.7)
    rot["uv_transform"] = (c, s_, 0.1, -s_, c, 0.2)
    spp = 8
    img = render(rot, world["uv"], spp=spp).cpu().numpy().astype(np.float64)
    ref = plain.cpu().numpy().astype(np.float64)
    assert np.abs(img - ref).mean() > 1e-3 * np.abs(ref).mean()
    s = scene(rot, world["uv"])
    wptr, aptr, W, H = s.env_tables()
    n = W * H
    w = d2h(wptr, 4 * n, np.float32)
    tab = d2h(aptr, 8 * n, np.uint32).reshape(n, 2)
    s.close()
    bvh = oracle.CpuBVH(sc["xyz"], sc["indices"], 4)
    twin, _, _ = oracle.pt_render(False, sc["xyz"], sc["indices"], sc["tri_material"], rot, bvh,
                                  world["env"].cpu().numpy(), world["ocam"], spp, seed=0x5EED, batch=0, rr_depth=3,
                                  crop=crop, alias_prob=np.ascontiguousarray(tab[:, 0].view(np.float32)),
                                  alias=np.ascontiguousarray(tab[:, 1]), weight=w, normals=world["nrm"],
                                  uv=world["uv"], tangents=world["tg"], textures=world["tex"])
    rel = np.abs(img - twin) / np.maximum(np.abs(twin), 1e-2)
    assert np.mean(np.all(rel < 1e-3, axis=-1)) > 0.97
