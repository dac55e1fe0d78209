"""Homogeneous participating media on the GPU (the MEDIA variant of the shade kernel).

* path-for-path twin: the FP32 CPU twin reproduces the GPU image of the media showcase (Cornell box,
  16 overlapping spheres cycled through fog, absorbing glass, emissive gas and scattering glass, one
  analytic light of each type) pixel by pixel up to transcendental / FMA rounding, with the same ray
  counts;
* radiance: the GPU image has bias and RMSE against the committed FP64 oracle consistent with
  Monte-Carlo noise;
* analytic: Beer-Lambert transmittance of an absorbing null-surface box, the emission integral of an
  emissive one, and a white scattering furnace, each against its closed form over the exact chords;
* media with a radiance cache and media in a batch are refused; invalid media parameters are rejected.
"""
import math

import numpy as np
import pytest
import torch

import oracle
from radiance_stats import check, compare, lum, render_batches, report
from vierkant_gb300 import _lib, geometry
from vierkant_gb300.pathtracer import PBRPathTracer, Scene, cornell_lights
from test_gpu_pathtracer import d2h
from test_oracle_media import H as BOX_H, RES, box_mesh, chords, medium_of, null_box_material

pytestmark = pytest.mark.gpu

W, HT = 256, 144
NUM_SPHERES = 16
ENV = 0.2
MAX_DEPTH = 10


def settings(spp, max_depth=MAX_DEPTH, rr=3, mis=0, res=(W, HT)):
    s = PBRPathTracer.default_settings()
    s.resolution[0], s.resolution[1] = res
    s.num_samples, s.max_trace_depth, s.rr_start_depth, s.mis_mode = spp, max_depth, rr, mis
    return s


@pytest.fixture(scope="module")
def fogged(ctx):
    sc = geometry.cornell_scene(0x5EED, 2, NUM_SPHERES, 16)
    mats = geometry.media_materials(sc["materials"])
    env = torch.full((64, 128, 3), ENV, dtype=torch.float32, device="cuda")
    scene = Scene(ctx, sc["xyz"], sc["indices"], sc["tri_material"], mats, env)
    scene.set_lights(cornell_lights())
    cam = geometry.camera_lookat((0, 0, 3.4), (0, 0, 0), (0, 1, 0), 45.0, W, HT)
    th = float(np.float32(math.tan(math.radians(45.0) / 2.0)))
    ocam = oracle.camera((0, 0, 3.4), (0, 0, 0), (0, 1, 0), th, W, HT)
    yield {"sc": sc, "mats": mats, "env": env, "scene": scene, "cam": cam, "ocam": ocam}
    scene.close()


def test_twin_parity_path_for_path(ctx, fogged):
    spp = 8
    pt = PBRPathTracer(ctx, seed=0x5EED, settings=settings(spp))
    img = pt.render_scene(fogged["scene"], fogged["cam"]).cpu().numpy().astype(np.float64)
    st = pt.statistics()
    pt.close()
    wptr, aptr, EW, EH = fogged["scene"].env_tables()
    n = EW * EH
    w = d2h(wptr, 4 * n, np.float32)
    tab = d2h(aptr, 8 * n, np.uint32).reshape(n, 2)
    prob = np.ascontiguousarray(tab[:, 0].view(np.float32))
    alias = np.ascontiguousarray(tab[:, 1])
    sc = fogged["sc"]
    bvh = oracle.CpuBVH(sc["xyz"], sc["indices"], 4)
    twin, _, rays = oracle.pt_render(False, sc["xyz"], sc["indices"], sc["tri_material"], fogged["mats"], bvh,
                                     fogged["env"].cpu().numpy(), fogged["ocam"], spp, seed=0x5EED, batch=0,
                                     max_depth=MAX_DEPTH, rr_depth=3, alias_prob=prob, alias=alias, weight=w,
                                     lights=cornell_lights().astype(oracle.LIGHT_DTYPE))
    rel = np.abs(img - twin) / np.maximum(np.abs(twin), 1e-2)
    close = np.mean(np.all(rel < 1e-3, axis=-1))
    print(f"close {close:.4f} sum ratio {img.sum() / twin.sum():.5f} rays {st.extension_rays}/{rays[0]} "
          f"{st.shadow_rays}/{rays[1]}")
    assert close > 0.9, close
    assert abs(img.sum() / twin.sum() - 1.0) < 0.02
    assert abs(st.extension_rays / rays[0] - 1.0) < 0.01
    assert abs(st.shadow_rays / rays[1] - 1.0) < 0.01


def test_radiance_against_fp64_oracle(ctx, fogged, golden):
    """32 independent 512-spp batches (16,384 spp) against the FP64 fixture (full frame): the luminance
    bias is within 3 standard errors of zero, with 3 standard errors below 0.5 %, and the RMSE within 1.2x
    the noise of the two estimates (radiance_stats)"""
    g = golden("pt_oracle_media")
    assert tuple(g["size"]) == (W, HT) and int(g["max_depth"]) == MAX_DEPTH
    assert int(g["num_spheres"]) == NUM_SPHERES and float(g["env"]) == np.float32(ENV)
    imgs = render_batches(lambda seed: PBRPathTracer(ctx, seed=seed, settings=settings(512)), fogged["scene"],
                          fogged["cam"], 32)
    st = compare(imgs, g["mean"], g["lum_var"], int(g["spp"]))
    report("media showcase vs FP64 oracle", st)
    check(st)


def _box_render(ctx, mat, env_value, spp, mis=0, max_depth=8):
    xyz, idx = box_mesh(BOX_H)
    env = torch.full((32, 64, 3), env_value, dtype=torch.float32, device="cuda")
    scene = Scene(ctx, xyz, idx, np.zeros(len(idx), np.uint32), mat, env)
    # the oracle's box camera: eye (0.3, 0.2, 4), tan(fovy / 2) = 0.2679
    cam = geometry.camera_lookat((0.3, 0.2, 4.0), (0, 0, 0), (0, 1, 0), math.degrees(2 * math.atan(0.2679)), RES,
                                 RES)
    pt = PBRPathTracer(ctx, seed=3, settings=settings(spp, max_depth=max_depth, rr=64, mis=mis, res=(RES, RES)))
    img = pt.render_scene(scene, cam).cpu().numpy().astype(np.float64)
    pt.close()
    scene.close()
    return img


def test_beer_lambert_absorbing_box(ctx):
    mat = null_box_material(attenuation_color=(0.5, 0.25, 0.8), attenuation_distance=1.0)
    ss, sa = medium_of(mat)
    Lc = chords()
    expect = np.exp(-(ss + sa)[None, None, None, :] * Lc[..., None]).mean(axis=2)
    img = _box_render(ctx, mat, 1.0, 1024)
    inside = (Lc > 0).all(axis=2)
    outside = ~(Lc > 0).any(axis=2)
    assert np.all(img[outside] == 1.0)
    for c in range(3):
        rel = img[..., c][inside].mean() / expect[..., c][inside].mean() - 1
        assert abs(rel) < 0.01, (c, rel)


def test_emissive_box_matches_emission_integral(ctx):
    le = np.array([2.0, 1.0, 0.5])
    mat = null_box_material(attenuation_color=(0.3, 0.3, 0.3), attenuation_distance=1.0, emission=le)
    ss, sa = medium_of(mat)
    st = ss + sa
    Lc = chords()
    expect = ((sa * le / st)[None, None, None, :] * (1 - np.exp(-st[None, None, None, :] * Lc[..., None]))).mean(2)
    img = _box_render(ctx, mat, 0.0, 256)
    smooth = (Lc > 0).all(axis=2) & (Lc.std(axis=2) < 0.01 * Lc.mean(axis=2))
    assert smooth.sum() > 30
    assert np.allclose(img[smooth], expect[smooth], rtol=3e-3, atol=0), np.abs(img[smooth] / expect[smooth] - 1).max()
    assert abs(img.sum() / expect.sum() - 1) < 0.01


@pytest.mark.parametrize("g,mis", [(0.0, 2), (0.6, 2), (-0.4, 2), (0.3, 0), (0.3, 1)])
def test_white_scattering_furnace(ctx, g, mis):
    mat = null_box_material(attenuation_color=(0.3, 0.3, 0.3), attenuation_distance=1.0, scatter_factor=1.0,
                            scatter_color=(1, 1, 1), phase_g=g)
    img = _box_render(ctx, mat, 1.0, 1024, mis=mis, max_depth=64)
    assert abs(img.mean() - 1) < 0.005, img.mean()


def test_media_refuse_cache_and_batch(ctx):
    """a scene with media (and no lights) cannot render through the radiance cache or in a batch"""
    from vierkant_gb300.batch import BatchJob, BatchRenderer
    from vierkant_gb300.nrc import NeuralRadianceCache
    xyz, idx = box_mesh(BOX_H)
    env = torch.ones((8, 16, 3), dtype=torch.float32, device="cuda")
    mat = null_box_material(attenuation_color=(0.5, 0.5, 0.5), attenuation_distance=1.0)
    scene = Scene(ctx, xyz, idx, np.zeros(len(idx), np.uint32), mat, env)
    cam = geometry.camera_lookat((0.3, 0.2, 4.0), (0, 0, 0), (0, 1, 0), 30.0, RES, RES)
    cfg = NeuralRadianceCache.default_config()
    cfg.log2_table_size = 14
    cache = NeuralRadianceCache(ctx, cfg)
    pt = PBRPathTracer(ctx, seed=1, settings=settings(1, res=(RES, RES)))
    pt.render_scene(scene, cam)  # the plain estimator renders it
    pt.attach_cache(cache)
    with pytest.raises(_lib.VkgError):
        pt.render_scene(scene, cam)
    pt.close()
    cache.close()
    with pytest.raises(_lib.VkgError):
        BatchRenderer(ctx, [BatchJob(scene, cam, settings(1, res=(RES, RES)), seed=1)])
    scene.close()


@pytest.mark.parametrize("field,value", [("attenuation_color", (0.0, 0.5, 0.5)), ("attenuation_color", (1.5, 1, 1)),
                                         ("scatter_factor", 1.5), ("scatter_color", (-0.1, 0, 0)), ("phase_g", 1.0),
                                         ("phase_g", -1.2)])
def test_invalid_media_rejected(ctx, field, value):
    mat = null_box_material(attenuation_color=(0.5, 0.5, 0.5), attenuation_distance=1.0)
    mat[field][0] = value
    xyz, idx = box_mesh(BOX_H)
    env = torch.ones((8, 16, 3), dtype=torch.float32, device="cuda")
    with pytest.raises(_lib.VkgError):
        Scene(ctx, xyz, idx, np.zeros(len(idx), np.uint32), mat, env)


def test_camera_medium_given_twin(ctx):
    """a camera inside a scattering box whose medium is given in the settings: the FP32 twin with the
    same camera medium reproduces the GPU image path for path"""
    from vierkant_gb300.pathtracer import CAMERA_MEDIUM_GIVEN, medium_params
    fields = dict(attenuation_color=(0.5, 0.7, 0.9), attenuation_distance=4.0, scatter_factor=0.8,
                  scatter_color=(0.9, 0.8, 0.7), phase_g=0.3)
    xyz, idx = box_mesh(5.0)
    mat = null_box_material(**fields)
    env = torch.full((32, 64, 3), 0.8, dtype=torch.float32, device="cuda")
    scene = Scene(ctx, xyz, idx, np.zeros(len(idx), np.uint32), mat, env)
    tan_half = 0.2679
    cam = geometry.camera_lookat((0.3, 0.2, 4.0), (0, 0, 0), (0, 1, 0), math.degrees(2 * math.atan(tan_half)), 64, 64)
    s = settings(16, max_depth=8, res=(64, 64))
    s.camera_medium_mode = CAMERA_MEDIUM_GIVEN
    s.camera_medium = medium_params(**fields)
    pt = PBRPathTracer(ctx, seed=11, settings=s)
    img = pt.render_scene(scene, cam).cpu().numpy().astype(np.float64)
    st = pt.statistics()
    pt.close()
    wptr, aptr, EW, EH = scene.env_tables()
    n = EW * EH
    w = d2h(wptr, 4 * n, np.float32)
    tab = d2h(aptr, 8 * n, np.uint32).reshape(n, 2)
    ocam = oracle.camera((0.3, 0.2, 4.0), (0, 0, 0), (0, 1, 0), float(cam.tan_half_fovy), 64, 64)
    twin, _, rays = oracle.pt_render(False, xyz, idx, np.zeros(len(idx), np.uint32), mat, oracle.CpuBVH(xyz, idx, 4),
                                     env.cpu().numpy(), ocam, 16, seed=11, max_depth=8, rr_depth=3,
                                     alias_prob=np.ascontiguousarray(tab[:, 0].view(np.float32)),
                                     alias=np.ascontiguousarray(tab[:, 1]), weight=w,
                                     camera_medium=oracle.medium_params(**fields))
    scene.close()
    rel = np.abs(img - twin) / np.maximum(np.abs(twin), 1e-2)
    close = np.mean(np.all(rel < 1e-3, axis=-1))
    print(f"close {close:.4f} sum ratio {img.sum() / twin.sum():.5f} rays {st.extension_rays}/{rays[0]}")
    assert close > 0.9 and abs(img.sum() / twin.sum() - 1) < 0.02
    assert abs(st.extension_rays / rays[0] - 1.0) < 0.01
    assert img.mean() < 0.8  # the medium's absorption dims the environment


def test_camera_medium_detected_in_instanced_scene(ctx):
    """PBRPathTracer.cpp:471-525: of the instances whose oriented world box contains the eye and whose
    material has a finite attenuation distance, the smallest; a render that detects it equals one given
    the same medium"""
    from vierkant_gb300.pathtracer import CAMERA_MEDIUM_GIVEN, InstancedScene, medium_params
    from vierkant_gb300.raytracing import INSTANCE_DTYPE
    fields = dict(attenuation_color=(0.6, 0.7, 0.8), attenuation_distance=3.0, scatter_factor=0.5,
                  scatter_color=(0.9, 0.9, 0.9), phase_g=0.2)
    mats = np.concatenate([null_box_material(), null_box_material(attenuation_color=(0.9, 0.9, 0.9),
                                                                  attenuation_distance=20.0),
                           null_box_material(attenuation_color=(0.5, 0.5, 0.5), attenuation_distance=2.0),
                           null_box_material(attenuation_color=(0.5, 0.5, 0.5), attenuation_distance=1.0),
                           null_box_material(**fields)])
    xyz, idx = box_mesh(1.0)

    def place(scale, t=(0, 0, 0), rot_z=False):
        M = np.diag(np.asarray(scale, np.float64))
        if rot_z:
            M = np.array([[0, -1, 0], [1, 0, 0], [0, 0, 1]], np.float64) @ M
        return np.concatenate([M, np.asarray(t, np.float64)[:, None]], axis=1).reshape(-1)

    inst = np.zeros(5, INSTANCE_DTYPE)
    rows = [(place((10, 10, 10)), 1),            # a large volume around the eye
            (place((3, 3, 3)), 2),               # a smaller one
            (place((2, 2, 2)), 0),               # smaller still, but no volume: skipped
            (place((1.5, 1.5, 1.5), (10, 0, 0)), 3),  # a volume away from the eye
            (place((4, 0.5, 4), rot_z=True), 4)]  # rotated: world half extents (0.5, 4, 4), the smallest
    for k, (T, m) in enumerate(rows):
        inst["transform"][k], inst["blas"][k], inst["material"][k] = T, 0, m
    env = torch.full((16, 32, 3), 0.8, dtype=torch.float32, device="cuda")
    scene = InstancedScene(ctx, [(xyz, idx, 0)], inst, mats, env)
    eye = (0.3, 0.2, 2.5)
    assert scene.camera_medium(eye) == 4
    assert scene.camera_medium((1.0, 0.0, 0.0)) == 2   # outside the rotated box, inside the 3-box
    assert scene.camera_medium((30.0, 0.0, 0.0)) is None
    cam = geometry.camera_lookat(eye, (0, 0, 0), (0, 1, 0), 40.0, 32, 32)
    images = []
    for given in (False, True):
        s = settings(8, max_depth=8, res=(32, 32))
        if given:
            s.camera_medium_mode = CAMERA_MEDIUM_GIVEN
            s.camera_medium = medium_params(**fields)
        pt = PBRPathTracer(ctx, seed=5, settings=s)
        images.append(pt.render_scene(scene, cam).clone())
        pt.close()
    scene.close()
    assert torch.equal(images[0], images[1])


def test_camera_medium_validated(ctx):
    from vierkant_gb300.pathtracer import CAMERA_MEDIUM_GIVEN, medium_params
    xyz, idx = box_mesh(1.0)
    env = torch.ones((8, 16, 3), dtype=torch.float32, device="cuda")
    scene = Scene(ctx, xyz, idx, np.zeros(len(idx), np.uint32), null_box_material(), env)
    cam = geometry.camera_lookat((0, 0, 4), (0, 0, 0), (0, 1, 0), 30.0, 8, 8)
    for bad in (dict(attenuation_color=(0, 1, 1)), dict(attenuation_distance=0.0), dict(phase_g=1.0),
                dict(scatter_factor=2.0), dict(ior=-1.0)):
        s = settings(1, res=(8, 8))
        s.camera_medium_mode = CAMERA_MEDIUM_GIVEN
        s.camera_medium = medium_params(**bad)
        pt = PBRPathTracer(ctx, seed=1, settings=s)
        with pytest.raises(_lib.VkgError):
            pt.render_scene(scene, cam)
        pt.close()
    s = settings(1, res=(8, 8))
    s.camera_medium_mode = 7
    pt = PBRPathTracer(ctx, seed=1, settings=s)
    with pytest.raises(_lib.VkgError):
        pt.render_scene(scene, cam)
    pt.close()
    scene.close()


def test_instanced_media_against_fp64_oracle(ctx):
    """the media showcase as a two-level scene (one identity instance per wall quad and sphere, its
    material per instance) against the instanced FP64 oracle on a crop: media, null surfaces and the
    media stack through the two-level traversal, and light shadow rays that take the optical depth of
    absorbing glass instances crossing by crossing"""
    from scene_helpers import split_cornell
    from vierkant_gb300.pathtracer import InstancedScene
    sc = geometry.cornell_scene(0x5EED, 2, NUM_SPHERES, 16)
    sc["materials"] = geometry.media_materials(sc["materials"])
    meshes, inst = split_cornell(sc)
    env = torch.full((64, 128, 3), ENV, dtype=torch.float32, device="cuda")
    scene = InstancedScene(ctx, meshes, inst, sc["materials"], env)
    scene.set_lights(cornell_lights())
    cam = geometry.camera_lookat((0, 0, 3.4), (0, 0, 0), (0, 1, 0), 45.0, W, HT)
    crop = (96, 40, 64, 64)
    s = settings(256)
    for k in range(4):
        s.crop[k] = crop[k]
    imgs = render_batches(lambda seed: PBRPathTracer(ctx, seed=seed, settings=s), scene, cam, 8)
    scene.close()
    th = float(np.float32(math.tan(math.radians(45.0) / 2.0)))
    ocam = oracle.camera((0, 0, 3.4), (0, 0, 0), (0, 1, 0), th, W, HT)
    spp = 512
    ref, sq, _ = oracle.pt_render_instanced(meshes, inst["transform"], inst["blas"], inst["material"],
                                            sc["materials"], env.cpu().numpy(), ocam, spp, seed=77,
                                            max_depth=MAX_DEPTH, rr_depth=3, crop=crop,
                                            lights=cornell_lights().astype(oracle.LIGHT_DTYPE))
    var = np.maximum(sq - lum(ref) ** 2, 0.0)
    st = compare(imgs, ref, var, spp)
    report("instanced media vs FP64 oracle", st)
    # the oracle runs here at 512 spp on a 64^2 crop: its noise sets the resolution (3 se ~ 2 %)
    check(st, max_bound=0.03)
