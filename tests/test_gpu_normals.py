"""Smooth shading with vertex normals (vkg_scene_set_normals; interpolate_vertex,
raypipeline.slang:336-360) on the GPU:

* path for path against the FP32 twin with the same vertex normals, and in radiance against the FP64
  oracle fixture pt_oracle_smooth.npz (the Cornell crop with sphere normals; radiance_stats);
* removing the normals gives back the face-normal image bit for bit;
* instanced scenes: normals from a glTF NORMAL attribute equal the same normals set directly (bit for
  bit), the octahedral snorm16 words of packed_vertex_t records decode to the same shading, and an
  instance split from the single-level scene with its normals renders like it.
"""
import math

import numpy as np
import pytest
import torch

import oracle
from gltf_writer import write
from radiance_stats import check, compare, render_batches, report
from scene_helpers import split_cornell
from test_gpu_pathtracer import CROP, d2h, settings
from vierkant_gb300 import geometry
from vierkant_gb300.gltf import scene_from_gltf
from vierkant_gb300.pathtracer import (PACKED_VERTEX_DTYPE, InstancedScene, PBRPathTracer, Scene, procedural_sky,
                                       sun_direction)

pytestmark = pytest.mark.gpu


def oct_words(n):
    """octahedral snorm16 words of unit vectors (packed_vertex.slang's pack(), restated in numpy)"""
    n = np.asarray(n, np.float64)
    p = n[:, :2] / np.abs(n).sum(axis=1, keepdims=True)
    neg = n[:, 2] < 0
    s = np.where(p >= 0, 1.0, -1.0)
    q = np.stack([(1 - np.abs(p[:, 1])) * s[:, 0], (1 - np.abs(p[:, 0])) * s[:, 1]], axis=1)
    p = np.where(neg[:, None], q, p)
    iv = np.rint(np.clip(p, -1, 1) * 32767).astype(np.int64)
    return ((iv[:, 0] & 0xFFFF) | ((iv[:, 1] & 0xFFFF) << 16)).astype(np.uint32)


@pytest.fixture(scope="module")
def world(ctx):
    sc = geometry.cornell_scene(0x5EED, 2, 64, 16)
    nrm = geometry.cornell_vertex_normals(sc)
    env = procedural_sky(ctx, 2048, 1024, sun_direction(), 5e4, 3.8e-5)
    scene = Scene(ctx, sc["xyz"], sc["indices"], sc["tri_material"], sc["materials"], env)
    scene.set_normals(nrm)
    cam = geometry.camera_lookat((0, 0, 3.4), (0, 0, 0), (0, 1, 0), 45.0, 1280, 720)
    th = float(np.float32(math.tan(math.radians(45.0) / 2.0)))
    ocam = oracle.camera((0, 0, 3.4), (0, 0, 0), (0, 1, 0), th, 1280, 720)
    yield {"sc": sc, "nrm": nrm, "env": env, "scene": scene, "cam": cam, "ocam": ocam}
    scene.close()


def test_twin_parity_smooth_normals(ctx, world):
    crop = (600, 560, 48, 48)
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
    twin, _, rays = oracle.pt_render(False, sc["xyz"], sc["indices"], sc["tri_material"], sc["materials"], bvh,
                                     world["env"].cpu().numpy(), world["ocam"], spp, seed=0x5EED, batch=0,
                                     rr_depth=3, crop=crop, alias_prob=prob, alias=alias, weight=w,
                                     normals=world["nrm"])
    rel = np.abs(img - twin) / np.maximum(np.abs(twin), 1e-2)
    close = np.mean(np.all(rel < 1e-3, axis=-1))
    assert close > 0.97, close
    assert abs(img.sum() / twin.sum() - 1.0) < 0.02
    assert abs(st.extension_rays / rays[0] - 1.0) < 0.01
    assert abs(st.shadow_rays / rays[1] - 1.0) < 0.01


def test_radiance_smooth_normals_against_fp64_oracle(ctx, world, golden):
    g = golden("pt_oracle_smooth")
    assert tuple(g["crop"]) == CROP
    imgs = render_batches(lambda seed: PBRPathTracer(ctx, seed=seed, settings=settings(64, CROP)),
                          world["scene"], world["cam"], 16)
    st = compare(imgs, g["mean"], g["lum_var"], int(g["spp"]))
    report("Cornell crop, smooth normals, vs FP64 oracle", st)
    check(st)


def test_removing_normals_restores_face_shading(ctx, world):
    sc = world["sc"]
    crop = (600, 300, 64, 64)
    s = Scene(ctx, sc["xyz"], sc["indices"], sc["tri_material"], sc["materials"], world["env"])

    def render():
        p = PBRPathTracer(ctx, seed=3, settings=settings(4, crop))
        img = p.render_scene(s, world["cam"]).clone()
        p.close()
        return img

    flat = render()
    s.set_normals(world["nrm"])
    smooth = render()
    s.set_normals(None)
    again = render()
    s.close()
    assert not torch.equal(flat, smooth)
    assert torch.equal(flat, again)


def test_instanced_normals_gltf_packed_and_split(ctx, world, tmp_path):
    sc = geometry.cornell_scene(0x5EED, 2, 8, 8)
    nrm = geometry.cornell_vertex_normals(sc)
    meshes, inst = split_cornell(sc, tess=8)
    mats = sc["materials"]
    # per-mesh normals in the split meshes' vertex order
    idx = sc["indices"]
    groups = [(2 * q, 2 * q + 2) for q in range(5)] + [(10 + k * 768, 10 + (k + 1) * 768) for k in range(8)]
    mesh_nrm = [nrm[np.unique(idx[a:b].reshape(-1))] for a, b in groups]
    env = procedural_sky(ctx, 256, 128, sun_direction(), 50.0, 0.02)
    cam = geometry.camera_lookat((0, 0, 3.4), (0, 0, 0), (0, 1, 0), 45.0, 1280, 720)
    crop = (600, 300, 64, 64)

    def render(scene, seed=5):
        p = PBRPathTracer(ctx, seed=seed, settings=settings(8, crop))
        img = p.render_scene(scene, cam).clone()
        p.close()
        return img

    direct = InstancedScene(ctx, meshes, inst, mats, env)
    flat = render(direct)
    for m, n in enumerate(mesh_nrm):
        direct.set_normals(n, mesh=m)
    smooth = render(direct)
    assert not torch.equal(flat, smooth)
    # glTF NORMAL attributes
    gm = [[(x, i, int(inst[k]["material"]), None, mesh_nrm[k])] for k, (x, i, _) in enumerate(meshes)]
    gmats = [{"pbrMetallicRoughness": {"baseColorFactor": [float(c) for c in m["base_color"]] + [1.0],
                                       "metallicFactor": float(m["metalness"]),
                                       "roughnessFactor": float(m["roughness"])},
              "doubleSided": bool(m["twosided"])} for m in mats]
    path = tmp_path / "smooth.glb"
    write(path, gm, [dict(mesh=k) for k in range(len(meshes))], list(range(len(meshes))), materials=gmats,
          mode="glb")
    loaded = scene_from_gltf(ctx, str(path), env)
    assert torch.equal(render(loaded), smooth)
    # packed_vertex_t records: octahedral snorm16 normals decoded on the device
    packed_meshes = []
    for (x, i, t), n in zip(meshes, mesh_nrm):
        rec = np.zeros(len(x), PACKED_VERTEX_DTYPE)
        rec["position"] = x
        rec["normal"] = oct_words(n)
        packed_meshes.append((rec, i, t))
    packed = InstancedScene(ctx, packed_meshes, inst, mats, env)
    for m, (rec, _, _) in enumerate(packed_meshes):
        packed.set_normals(rec, mesh=m)
    a = render(packed, seed=9).cpu().numpy().astype(np.float64)
    b = render(direct, seed=9).cpu().numpy().astype(np.float64)
    assert abs(a.sum() / b.sum() - 1.0) < 0.02
    assert np.mean(np.all(np.abs(a - b) / np.maximum(np.abs(b), 1e-2) < 1e-2, axis=-1)) > 0.8
    # the single-level scene with the same normals: the same image up to the two-level traversal
    single = Scene(ctx, sc["xyz"], sc["indices"], sc["tri_material"], mats, env)
    single.set_normals(nrm)
    c = render(single, seed=9).cpu().numpy().astype(np.float64)
    assert abs(c.sum() / b.sum() - 1.0) < 0.02
    for s_ in (direct, loaded, packed, single):
        s_.close()
