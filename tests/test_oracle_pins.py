"""The CPU oracle is pinned before it is trusted: against the reference's own compiled code
(oracle/_ref, when present), the committed golden fixtures made from it, and published
known-answer vectors."""
import ctypes as C
import hashlib
import math

import numpy as np
import pytest

import oracle
from oracle import ptr


def test_pcg32_published_known_answer():
    # pcg32_srandom_r(42, 54): the first six outputs of O'Neill's reference demo
    out = np.zeros(6, np.uint32)
    oracle.orc().orc_pcg32_fill(42, 54, 0, 6, ptr(out))
    assert [int(x) for x in out] == [0xa15c02b7, 0x7b47f409, 0xba1d3330, 0x83d2f293, 0xbfa4784b, 0xcbed606e]


def test_pcg32_jump_ahead_matches_sequential():
    seq = np.zeros(1000, np.uint32)
    oracle.orc().orc_pcg32_fill(0x5EED, 7, 0, 1000, ptr(seq))
    for skip in (1, 17, 500, 999):
        one = np.zeros(1, np.uint32)
        oracle.orc().orc_pcg32_fill(0x5EED, 7, skip, 1, ptr(one))
        assert one[0] == seq[skip]


def test_rng_tables_match_golden(golden):
    g = golden("rng")
    pcg = np.zeros(4096, np.uint32)
    oracle.orc().orc_pcg32_fill(0x5EED, 1, 0, 4096, ptr(pcg))
    assert np.array_equal(pcg, g["pcg32_5eed_1"])
    xx = [oracle.orc().orc_xxhash32(int(a), int(b)) for a, b in zip(g["xx_lhs"], g["xx_rhs"])]
    assert np.array_equal(np.array(xx, np.uint32), g["xxhash32"])


def test_ray_triangle_matches_reference_fixture(golden):
    g = golden("ray_triangle")
    L = oracle.orc()
    for i in range(len(g["type"])):
        out = np.zeros(3, np.float32)
        t = L.orc_intersect_ray_triangle(ptr(g["o"][i]), ptr(g["d"][i]), ptr(g["tri"][i]), ptr(out))
        assert t == g["type"][i]
        if t:
            assert out.tobytes() == g["tuv"][i].tobytes(), i


def test_ray_aabb_matches_reference_fixture(golden):
    g = golden("ray_aabb")
    L = oracle.orc()
    for i in range(len(g["type"])):
        tt = C.c_float()
        t = L.orc_intersect_ray_aabb(ptr(g["o"][i]), ptr(g["d"][i]), ptr(g["lo"][i]), ptr(g["hi"][i]), C.byref(tt))
        assert t == g["type"][i]
        if t:
            assert np.float32(tt.value).tobytes() == g["t"][i].tobytes()


def test_oracle_against_live_reference_random():
    R = oracle.ref()
    if R is None:
        pytest.skip("reference checkout not present here (fixtures cover this case)")
    rng = np.random.default_rng(5)
    L = oracle.orc()
    for _ in range(20000):
        o, d, tri = (rng.normal(size=k).astype(np.float32) for k in (3, 3, 9))
        a, b = np.zeros(3, np.float32), np.zeros(3, np.float32)
        ra = L.orc_intersect_ray_triangle(ptr(o), ptr(d), ptr(tri), ptr(a))
        rb = R.vkref_intersect_ray_triangle(ptr(o), ptr(d), ptr(tri), ptr(b))
        assert ra == rb and (not ra or a.tobytes() == b.tobytes())


def test_icosphere_counts_and_fixture(golden):
    xyz, idx = oracle.icosphere(1.0, 5)
    assert xyz.shape == (20472, 3) and idx.shape == (20480, 3)
    g = golden("config1_hits")
    assert hashlib.sha256(xyz.tobytes()).hexdigest() == str(g["sha_xyz"])
    assert hashlib.sha256(idx.tobytes()).hexdigest() == str(g["sha_idx"])
    r = np.linalg.norm(xyz.astype(np.float64), axis=1)
    assert np.all(np.abs(r - 1.0) < 1e-6)


def test_config1_bruteforce_matches_reference_fixture(golden):
    g = golden("config1_hits")
    xyz, idx = oracle.icosphere(1.0, 5)
    th = float(np.float32(math.tan(math.radians(60.0) / 2.0)))
    assert np.float32(th) == g["tan_half_fovy"]
    cam = oracle.camera((0, 0, 3), (0, 0, 0), (0, 1, 0), th, 1024, 1024)
    rays = oracle.camera_rays(cam, 0x5EED, 1, 1)
    assert hashlib.sha256(rays.tobytes()).hexdigest() == str(g["sha_rays"])
    sub = np.ascontiguousarray(rays[g["ray_index"]][:2048])
    hits = oracle.closest_hit_bruteforce(xyz, idx, sub)
    assert np.array_equal(hits.view(np.uint32).reshape(-1, 4), g["hits"][:2048])


def test_known_answers_from_reference_source():
    xyz, idx = oracle.icosphere(1.0, 5)
    r = np.zeros(1, oracle.RAY_DTYPE)
    r["o"] = (0, 0, 3)
    r["d"] = (0, 0, -1)
    r["tmin"], r["tmax"] = 1e-4, 1e4
    h = oracle.closest_hit_bruteforce(xyz, idx, r)
    assert h["prim"][0] != 0xFFFFFFFF and 2.0 <= h["t"][0] < 2.01
    # grazing ray: |det| < 1e-9 is rejected (intersection.cpp:119-120)
    out = np.zeros(3, np.float32)
    tri = np.array([0, 0, 0, 1, 0, 0, 0, 1, 0], np.float32)
    assert oracle.orc().orc_intersect_ray_triangle(ptr(np.float32([0.2, 0.2, 0])), ptr(np.float32([1, 0, 0])),
                                                   ptr(tri), ptr(out)) == 0
    # origin inside the box returns t_max (intersection.cpp:179-183)
    tt = C.c_float()
    assert oracle.orc().orc_intersect_ray_aabb(ptr(np.float32([0, 0, 0])), ptr(np.float32([1, 0, 0])),
                                               ptr(np.float32([-1, -1, -1])), ptr(np.float32([2, 1, 1])),
                                               C.byref(tt)) == 1
    assert tt.value == 2.0
    # back-face culling: the outward face is front-facing for a ray from outside, a ray from the
    # centre passes through when culling is on
    r2 = np.zeros(1, oracle.RAY_DTYPE)
    r2["o"] = (0, 0, 0)
    r2["d"] = (0, 0, 1)
    r2["tmin"], r2["tmax"] = 1e-4, 1e4
    assert oracle.closest_hit_bruteforce(xyz, idx, r, cull=True)["prim"][0] != 0xFFFFFFFF
    assert oracle.closest_hit_bruteforce(xyz, idx, r2, cull=True)["prim"][0] == 0xFFFFFFFF
    assert oracle.closest_hit_bruteforce(xyz, idx, r2, cull=False)["prim"][0] != 0xFFFFFFFF


def _random_mesh(rng, nt, spread=1.0):
    xyz = (rng.normal(size=(3 * nt, 3)) * spread).astype(np.float32)
    base = rng.normal(size=(nt, 1, 3)).astype(np.float32) * 2
    xyz = (xyz.reshape(nt, 3, 3) * 0.2 + base).reshape(-1, 3).astype(np.float32)
    idx = np.arange(3 * nt, dtype=np.uint32).reshape(nt, 3)
    return xyz, idx


def _random_rays(rng, n, spread=3.0):
    rays = np.zeros(n, oracle.RAY_DTYPE)
    o = (rng.normal(size=(n, 3)) * spread).astype(np.float32)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True).astype(np.float32)
    rays["o"], rays["d"], rays["tmin"], rays["tmax"] = o, d, 1e-4, 1e4
    return rays


@pytest.mark.parametrize("leaf_max", [1, 4, 16])
@pytest.mark.parametrize("nt", [1, 2, 3, 37, 1000])
def test_oracle_bvh_equals_bruteforce(nt, leaf_max):
    rng = np.random.default_rng(nt * 31 + leaf_max)
    xyz, idx = _random_mesh(rng, nt)
    rays = _random_rays(rng, 3000)
    b = oracle.CpuBVH(xyz, idx, leaf_max)
    for cull in (False, True):
        assert b.closest_hit(rays, cull=cull).tobytes() == oracle.closest_hit_bruteforce(xyz, idx, rays,
                                                                                         cull=cull).tobytes()
        assert np.array_equal(b.any_hit(rays, cull=cull), oracle.any_hit_bruteforce(xyz, idx, rays, cull=cull))


def test_oracle_bvh_ties_and_degenerates():
    # duplicated triangles (exact t ties -> smaller id wins), degenerate and zero-area triangles
    rng = np.random.default_rng(3)
    xyz, idx = _random_mesh(rng, 200)
    idx = np.concatenate([idx, idx[:50], idx[10:20][:, [0, 0, 1]]]).astype(np.uint32)
    xyz = xyz.copy()
    rays = _random_rays(rng, 5000)
    rays["d"][::11, 1] = 0.0  # zero direction components
    b = oracle.CpuBVH(xyz, idx, 4)
    bf = oracle.closest_hit_bruteforce(xyz, idx, rays)
    assert b.closest_hit(rays).tobytes() == bf.tobytes()
    assert np.all(bf["prim"][bf["prim"] != 0xFFFFFFFF] < len(idx))


def test_oracle_bvh_empty_mesh():
    b = oracle.CpuBVH(np.zeros((0, 3), np.float32), np.zeros((0, 3), np.uint32))
    rays = _random_rays(np.random.default_rng(0), 10)
    assert np.all(b.closest_hit(rays)["prim"] == 0xFFFFFFFF)


def test_instanced_fp64_oracle_equals_flat_oracle():
    """the FP64 oracle's instanced path (instance BVH, object-space traversal, transformed shading),
    given the Cornell scene split into identity-instanced meshes, reproduces the flat FP64 oracle"""
    import math
    from scene_helpers import split_cornell
    sc = oracle.cornell_scene(0x5EED, 2, 64, 16)
    mats = oracle.cornell_materials(0x5EED, 2, 64)
    meshes, inst = split_cornell(dict(sc, materials=mats))
    th = float(np.float32(math.tan(math.radians(45.0) / 2.0)))
    cam = oracle.camera((0, 0, 3.4), (0, 0, 0), (0, 1, 0), th, 1280, 720)
    sun = np.array([0.2961981, 0.5, 0.8137977], np.float32)
    env = oracle.env_procedural(256, 128, sun)
    bvh = oracle.CpuBVH(sc["xyz"], sc["indices"], 4)
    crop = (600, 500, 24, 24)
    a, _, ra = oracle.pt_render(True, sc["xyz"], sc["indices"], sc["tri_material"], mats, bvh, env, cam, 8, crop=crop)
    b, _, rb = oracle.pt_render_instanced(meshes, inst["transform"], inst["blas"], inst["material"], mats, env, cam, 8,
                                          crop=crop)
    assert ra == rb
    assert np.array_equal(a, b)


def test_instanced_fp64_oracle_equals_flat_oracle_with_transmission():
    """the same with the showcase materials: transmissive sphere meshes, not flagged two-sided, are
    traced from both sides in the instanced path as in the flat one"""
    from scene_helpers import split_cornell
    from vierkant_gb300.geometry import showcase_materials
    sc = oracle.cornell_scene(0x5EED, 2, 64, 16)
    mats = showcase_materials(oracle.cornell_materials(0x5EED, 2, 64))
    meshes, inst = split_cornell(dict(sc, materials=mats))
    th = float(np.float32(math.tan(math.radians(45.0) / 2.0)))
    cam = oracle.camera((0, 0, 3.4), (0, 0, 0), (0, 1, 0), th, 256, 144)
    env = oracle.env_procedural(256, 128, np.array([0.2961981, 0.5, 0.8137977], np.float32), 50.0, 0.02)
    bvh = oracle.CpuBVH(sc["xyz"], sc["indices"], 4)
    crop = (96, 40, 48, 48)
    a, _, ra = oracle.pt_render(True, sc["xyz"], sc["indices"], sc["tri_material"], mats, bvh, env, cam, 4,
                                crop=crop, max_depth=8)
    b, _, rb = oracle.pt_render_instanced(meshes, inst["transform"], inst["blas"], inst["material"], mats, env, cam, 4,
                                          crop=crop, max_depth=8)
    assert ra == rb
    assert np.array_equal(a, b)


def _sphere_in_constant_env(material, spp=256, res=16):
    xyz, idx = oracle.icosphere(1.0, 4)
    cam = oracle.camera((0, 0, 4.0), (0, 0, 0), (0, 1, 0), 0.2679, res, res)
    env = np.ones((64, 128, 3), np.float32)
    img, _, _ = oracle.pt_render(True, xyz, idx, np.zeros(len(idx), np.uint32), material, oracle.CpuBVH(xyz, idx, 4),
                                 env, cam, spp, max_depth=32, rr_depth=0)
    return img.mean(axis=-1)


def test_fp64_oracle_glass_white_furnace():
    """energy conservation of the dielectric lobe (bsdf_disney.slang:44-95): a smooth glass sphere of
    white colour under a constant unit environment reflects or refracts every path, so radiance 1
    comes back at every pixel; a rough one (roughness 0.35) loses only a little at grazing angles"""
    from vierkant_gb300.geometry import MATERIAL_DTYPE
    m = np.zeros(1, MATERIAL_DTYPE)
    m["base_color"][0] = 1.0
    m["transmission"][0] = 1.0
    m["ior"][0] = 1.5
    smooth = _sphere_in_constant_env(m)
    assert abs(smooth[5:11, 5:11].mean() - 1.0) < 2e-3, smooth[5:11, 5:11].mean()
    assert abs(smooth.mean() - 1.0) < 0.01
    m["roughness"][0] = 0.35
    rough = _sphere_in_constant_env(m)
    assert abs(rough[5:11, 5:11].mean() - 1.0) < 0.01
    assert 0.9 < rough.mean() < 1.0


@pytest.mark.parametrize("kind", ["diffuse", "sheen", "metal", "plastic", "diffuse_transmission", "clearcoat",
                                  "iridescent_metal"])
def test_fp64_bsdf_sampling_matches_evaluation(kind):
    """sample_disney and eval_disney describe the same BSDF (bsdf_disney.slang:162-381): the albedo
    integral of f |cos| estimated from the sampler's f / pdf equals the one integrated over uniform
    directions with the evaluator, lobe choice from one rescaled uniform included. (The dielectric
    lobes are pinned by the white-furnace test instead: their near-delta shapes need far more uniform
    samples, and the reference's refraction value and pdf share an extra eta^2 that the sampler's
    f / pdf cancels.)"""
    from vierkant_gb300.geometry import MATERIAL_DTYPE
    m = np.zeros(1, MATERIAL_DTYPE)
    m["base_color"][0] = (0.8, 0.6, 0.4)
    m["ior"][0] = 1.5
    m["roughness"][0] = 0.5
    if kind == "diffuse":
        m["roughness"][0] = 1.0
    elif kind == "sheen":
        m["sheen_color"][0], m["sheen_roughness"][0] = (1, 1, 1), 0.5
    elif kind == "metal":
        m["metalness"][0] = 1.0
    elif kind == "diffuse_transmission":
        m["diffuse_transmission"][0], m["diffuse_transmission_color"][0] = 0.6, (0.5, 0.7, 0.9)
    elif kind == "clearcoat":
        m["clearcoat"][0], m["clearcoat_roughness"][0] = 1.0, 0.3
    elif kind == "iridescent_metal":
        m["iridescence"][0], m["iridescence_ior"][0], m["iridescence_thickness"][0] = 0.7, 1.3, 400.0
        m["metalness"][0] = 1.0
    rng = np.random.default_rng(1)
    n_ = np.array([0.0, 0.0, 1.0])
    th = math.radians(40)
    v = np.array([math.sin(th), 0.0, math.cos(th)])
    count = 30000
    a = np.zeros(3)
    for _ in range(count):
        d, pdf, f, _ = oracle.bsdf_sample(m, n_, v, 1.0, rng.random(3))
        if pdf > 0:
            a += f * abs(d[2]) / max(pdf, 1e-3)
    # the reference picks the thin-film or the plain specular lobe with probability s / 1 - s and puts
    # it into the pdf but leaves the lobe's value unweighted (bsdf_disney.slang:195-206, :266-277), while
    # eval_disney weights the values by s / 1 - s: for a metal the sampled albedo is therefore
    # eval(s) + eval(1 - s). Restated as written.
    flips = [m]
    if kind == "iridescent_metal":
        m2 = m.copy()
        m2["iridescence"][0] = 1.0 - m["iridescence"][0]
        flips.append(m2)
    b = np.zeros(3)
    for _ in range(count):
        z, p = 2 * rng.random() - 1, 2 * math.pi * rng.random()
        r = math.sqrt(max(0.0, 1 - z * z))
        for mm in flips:
            f, _ = oracle.bsdf_eval(mm, np.array([r * math.cos(p), r * math.sin(p), z]), n_, v, 1.0)
            b += f * abs(z) * 4 * math.pi
    ratio = a / b
    assert np.all(np.abs(ratio - 1.0) < 0.03), ratio


def test_fp64_lights_mis_modes_converge():
    """analytic lights in the FP64 oracle: MIS, NEE-only and BSDF-only estimate the same image of the
    lit Cornell box once paths are long (at a finite depth the last vertex's NEE has no traced BSDF
    counterpart, as in the reference's loop, so the modes differ there); delta lights (spot, omni) are
    reached by NEE alone in every mode"""
    from vierkant_gb300.pathtracer import cornell_lights
    sc = oracle.cornell_scene(0x5EED, 2, 16, 8)
    mats = oracle.cornell_materials(0x5EED, 2, 16)
    th = float(np.float32(math.tan(math.radians(45.0) / 2.0)))
    cam = oracle.camera((0, 0, 3.4), (0, 0, 0), (0, 1, 0), th, 160, 90)
    env = np.full((16, 32, 3), 0.02, np.float32)
    bvh = oracle.CpuBVH(sc["xyz"], sc["indices"], 4)
    sun = oracle.sun_light((1, 1, 0.9), 3.0, (math.radians(30), math.radians(200)), 0.2)
    lights = np.concatenate([np.array([sun], oracle.LIGHT_DTYPE), cornell_lights().astype(oracle.LIGHT_DTYPE)])
    crop = (40, 50, 80, 40)  # the lower part of the box: no light body in view
    means = []
    for mode in (0, 1, 2):
        img, _, _ = oracle.pt_render(True, sc["xyz"], sc["indices"], sc["tri_material"], mats, bvh, env, cam, 256,
                                     mis_mode=mode, crop=crop, lights=lights, max_depth=16, rr_depth=3)
        means.append(img.mean())
    assert abs(means[1] / means[0] - 1.0) < 0.02, means
    assert abs(means[2] / means[0] - 1.0) < 0.04, means


def test_sun_light_direction():
    """the settings' sun: +z rotated by the quaternion of (elevation, azimuth, 0)
    (PBRPathTracer.cpp:617-620), i.e. (cos e sin a, -sin e, cos e cos a)"""
    s = oracle.sun_light((1, 1, 1), 2.0, (math.radians(30), math.radians(20)), 0.01)
    e, a = math.radians(30), math.radians(20)
    assert np.allclose(s["direction"], (math.cos(e) * math.sin(a), -math.sin(e), math.cos(e) * math.cos(a)), atol=1e-6)
    assert s["type"] == 2 and s["intensity"] == 2.0 and np.isinf(s["range"])


def test_pixel_record_packing():
    """octahedral snorm16 normals and RGBA8 colours (octahedral_map.slang:9-55, color.slang:6-18)"""
    rng = np.random.default_rng(3)
    v = rng.normal(size=(2000, 3)).astype(np.float32)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    L = oracle.orc()
    L.orc_oct_encode.argtypes = [C.c_void_p, C.c_void_p]
    L.orc_oct_decode.argtypes = [C.c_void_p, C.c_void_p]
    L.orc_pack_snorm_2x16.argtypes = [C.c_float, C.c_float]
    L.orc_pack_snorm_2x16.restype = C.c_uint32
    L.orc_unpack_snorm_2x16.argtypes = [C.c_uint32, C.c_void_p]
    L.orc_pack_rgba8.argtypes = [C.c_float] * 4
    L.orc_pack_rgba8.restype = C.c_uint32
    worst = 0.0
    for n in v:
        p = np.zeros(2, np.float32)
        L.orc_oct_encode(ptr(np.ascontiguousarray(n)), ptr(p))
        q = np.zeros(2, np.float32)
        L.orc_unpack_snorm_2x16(L.orc_pack_snorm_2x16(float(p[0]), float(p[1])), ptr(q))
        d = np.zeros(3, np.float32)
        L.orc_oct_decode(ptr(q), ptr(d))
        worst = max(worst, float(np.linalg.norm(d - n)))
    assert worst < 1e-4, worst
    assert L.orc_pack_snorm_2x16(float("nan"), 0.0) == 0
    assert L.orc_pack_rgba8(1.0, 0.5, 0.0, 1.0) == 0xFF007FFF
    assert L.orc_pack_rgba8(2.0, -1.0, 0.25, 0.0) == 0x003F00FF


def test_denoise_restatement_properties():
    """the a-trous restatement keeps a constant image constant (the weights are normalised), and
    with the reference's albedo demodulation a flat image of any albedo too"""
    h, w = 23, 31
    px = np.zeros((h, w), oracle.PIXEL_DTYPE)
    px["radiance"] = (0.3, 0.5, 0.7)
    px["depth"] = np.linspace(0.01, 0.05, w, dtype=np.float32)[None, :]
    px["albedo"] = 0xFF804020
    out = oracle.denoise(px)
    assert np.allclose(out[..., :3], (0.3, 0.5, 0.7), rtol=1e-5)
    assert np.all(out[..., 3] == 0)
    # low-amplitude noise is smoothed (its spread shrinks, its mean stays); an isolated bright pixel
    # is an edge for the luminance weight and survives, as the filter intends
    rng = np.random.default_rng(5)
    px["radiance"] = (0.5 + 0.05 * rng.standard_normal((h, w, 1))).astype(np.float32)
    out = oracle.denoise(px)
    assert out[..., 0].std() < 0.3 * px["radiance"][..., 0].std()
    assert abs(out[..., 0].mean() - px["radiance"][..., 0].mean()) < 0.01
    px["radiance"][11, 15] = (10.0, 10.0, 10.0)
    out = oracle.denoise(px)
    assert out[11, 15, 0] > 9.0



def _iridescent_fresnel_numpy(outside, film, f0, thickness, cos1):
    """an independent transcription of utils/bsdf.slang:83-150 (thin film over a base of reflectance f0)"""
    xyz_to_rgb = np.array([[3.2404542, -0.9692660, 0.0556434], [-1.5371385, 1.8760108, -0.2040259],
                           [-0.4985314, 0.0415560, 1.0572252]])  # rows: the shader's float3x3 rows

    def sensitivity(opd, shift):
        phase = 2 * math.pi * opd * 1e-9
        val = np.array([5.4856e-13, 4.4201e-13, 5.2481e-13])
        pos = np.array([1.6810e+06, 1.7953e+06, 2.2084e+06])
        var = np.array([4.3278e+09, 9.3046e+09, 6.6121e+09])
        xyz = val * np.sqrt(2 * math.pi * var) * np.cos(pos * phase + shift) * np.exp(-phase ** 2 * var)
        xyz[0] += 9.7470e-14 * math.sqrt(2 * math.pi * 4.5282e+09) * math.cos(2.2399e+06 * phase + shift[0]) * \
            math.exp(-4.5282e+09 * phase ** 2)
        return (xyz / 1.0685e-7) @ xyz_to_rgb

    schlick = lambda c, r0: r0 + (1 - r0) * (1 - c) ** 5
    R12 = schlick(cos1, ((film - outside) / (film + outside)) ** 2)
    T121 = 1 - R12
    cos2sq = 1 - (outside / film) ** 2 * (1 - cos1 ** 2)
    if cos2sq < 0:
        return np.ones(3)
    cos2 = math.sqrt(cos2sq)
    q = np.sqrt(np.clip(f0, 0, 0.9999) + 0.0001)
    base = (1 + q) / (1 - q)
    R23 = schlick(cos2, ((base - film) / (base + film)) ** 2)
    phi = (math.pi - (math.pi if film < outside else 0.0)) + np.where(base < film, math.pi, 0.0)
    opd = 2 * film * thickness * cos2
    R123 = np.clip(R12 * R23, 1e-5, 0.9999)
    Rs = T121 ** 2 * R23 / (1 - R123)
    I = R12 + Rs
    Cm = Rs - T121
    for k in (1, 2):
        Cm = Cm * np.sqrt(R123)
        I = I + Cm * 2 * sensitivity(k * opd, k * phi)
    return np.maximum(I, 0)


def test_iridescent_fresnel_against_independent_transcription():
    """the oracle's thin-film Fresnel (pt_core.inc, double) equals a second transcription of the
    reference's formula in numpy over films, bases, thicknesses and angles (total internal
    reflection in the film included)"""
    L = oracle.orc()
    L.orc_iridescent_fresnel.argtypes = [C.c_double, C.c_double, C.c_void_p, C.c_double, C.c_double, C.c_void_p]
    rng = np.random.default_rng(8)
    for _ in range(300):
        film = rng.uniform(1.0, 2.2)
        outside = 1.0 if rng.random() < 0.8 else rng.uniform(1.0, 2.5)
        f0 = rng.uniform(0.0, 1.0, 3)
        thick = rng.uniform(0.0, 1200.0)
        cos1 = rng.uniform(0.0, 1.0)
        out = np.zeros(3)
        L.orc_iridescent_fresnel(outside, film, ptr(np.ascontiguousarray(f0)), thick, cos1, ptr(out))
        ref = _iridescent_fresnel_numpy(outside, film, f0, thick, cos1)
        # the oracle keeps the shader's single-precision constants (as the GPU does): ~1e-7 of the O(1) terms
        assert np.allclose(out, ref, rtol=2e-6, atol=1e-6), (out, ref)


def test_dispersion_cauchy_and_white_balance():
    """chromatic dispersion (utils/bsdf.slang:46-91): the Cauchy ior equals the material's ior at the
    sodium d-line and spreads (ior - 1) dispersion / 20 between the F and C lines (the
    KHR_materials_dispersion definition, dispersion = 20 / Abbe number); the white balance makes a
    uniform wavelength in [400, 700] nm average to white"""
    for ior, disp in ((1.5, 1.0), (1.33, 3.0), (2.4, 0.5)):
        assert abs(oracle.cauchy_ior(ior, disp, 587.6) - ior) < 1e-6
        spread = oracle.cauchy_ior(ior, disp, 486.1) - oracle.cauchy_ior(ior, disp, 656.3)
        assert abs(spread - (ior - 1) * disp / 20) < 1e-6 * max(1.0, spread)
        # shorter wavelengths refract more
        assert oracle.cauchy_ior(ior, disp, 420.0) > ior > oracle.cauchy_ior(ior, disp, 680.0)
    lam = np.linspace(400.0, 700.0, 3001)
    rgb = np.array([oracle.lambda_rgb(x) for x in lam])
    assert np.all(rgb >= 0)
    mean = np.trapezoid(rgb, lam, axis=0) / 300.0 * np.array([1.703734, 2.601105, 2.757475])
    assert np.allclose(mean, 1.0, atol=2e-3), mean
    # red at 650 nm, green at 540 nm, blue at 450 nm dominate
    assert np.argmax(oracle.lambda_rgb(650.0)) == 0 and np.argmax(oracle.lambda_rgb(540.0)) == 1
    assert np.argmax(oracle.lambda_rgb(450.0)) == 2
