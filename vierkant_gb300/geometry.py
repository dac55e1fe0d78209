"""Geometry generators (host, deterministic), mirroring vierkant::Geometry and the benchmark scenes.

- icosphere(radius, tess): Geometry::IcoSphere (src/Geometry.cpp:566-613), unshared vertices
- cornell_scene(seed, stream, num_spheres, n): 5-quad Cornell box + PCG32-placed cube-spheres
- camera_lookat(...): pinhole camera basis for the ray generators
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from ._lib import check, lib, vkg_camera, vkg_material

MATERIAL_DTYPE = np.dtype([("base_color", "<f4", 3), ("roughness", "<f4"), ("metalness", "<f4"),
                           ("emission", "<f4", 3), ("twosided", "<u4"), ("transmission", "<f4"), ("ior", "<f4"),
                           ("clearcoat", "<f4"), ("clearcoat_roughness", "<f4"), ("sheen_color", "<f4", 3),
                           ("sheen_roughness", "<f4"), ("diffuse_transmission", "<f4"),
                           ("diffuse_transmission_color", "<f4", 3), ("iridescence", "<f4"),
                           ("iridescence_ior", "<f4"), ("iridescence_thickness", "<f4"), ("attenuation_color", "<f4", 3),
                           ("attenuation_distance", "<f4"), ("scatter_color", "<f4", 3), ("scatter_factor", "<f4"),
                           ("phase_g", "<f4"), ("null_surface", "<u4"), ("dispersion", "<f4"),
                           ("tex_color", "<u4"), ("tex_normal", "<u4"), ("tex_emission", "<u4"),
                           ("tex_ao_rough_metal", "<u4"), ("tex_transmission", "<u4"),
                           ("tex_diffuse_transmission", "<u4"), ("tex_diffuse_transmission_color", "<u4"),
                           ("alpha", "<f4"), ("blend_mode", "<u4"), ("alpha_cutoff", "<f4"),
                           ("has_uv_transform", "<u4"), ("uv_transform", "<f4", 6)])
assert MATERIAL_DTYPE.itemsize == C.sizeof(vkg_material)


def default_materials(n: int) -> np.ndarray:
    """n material records with the reference's defaults (base colour 1, roughness 1, ior 1.5,
    diffuse-transmission colour 1, alpha 1, alpha cutoff 0.5, no textures, everything else 0), filled
    by the library."""
    m = vkg_material()
    check(lib().vkg_material_defaults(C.byref(m)))
    one = np.frombuffer(bytes(m), MATERIAL_DTYPE, count=1)
    return np.repeat(one, n).copy()


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def icosphere(radius: float = 1.0, tess: int = 5):
    L = lib()
    nv, nt = C.c_uint32(), C.c_uint32()
    check(L.vkg_geometry_icosphere_counts(tess, C.byref(nv), C.byref(nt)))
    xyz = np.zeros((nv.value, 3), np.float32)
    idx = np.zeros((nt.value, 3), np.uint32)
    check(L.vkg_geometry_icosphere(C.c_float(radius), tess, _p(xyz), _p(idx)))
    return xyz, idx


def cornell_scene(seed: int = 0x5EED, stream: int = 2, num_spheres: int = 64, n: int = 16):
    """Returns dict(xyz [V,3] f32, indices [T,3] u32, tri_material [T] u32, materials structured array)."""
    L = lib()
    nv, nt, nm = C.c_uint32(), C.c_uint32(), C.c_uint32()
    check(L.vkg_scene_cornell_counts(num_spheres, n, C.byref(nv), C.byref(nt), C.byref(nm)))
    xyz = np.zeros((nv.value, 3), np.float32)
    idx = np.zeros((nt.value, 3), np.uint32)
    tm = np.zeros(nt.value, np.uint32)
    mats = np.zeros(nm.value, MATERIAL_DTYPE)
    check(L.vkg_scene_cornell(seed, stream, num_spheres, n, _p(xyz), _p(idx), _p(tm), _p(mats)))
    return {"xyz": xyz, "indices": idx, "tri_material": tm, "materials": mats}


def cornell_vertex_normals(sc) -> np.ndarray:
    """Vertex normals for smooth shading of a cornell_scene(): a sphere's vertices point away from its
    centre (the mean of its vertices), the walls' vertices carry their face normal. float32 [V, 3]."""
    xyz = np.asarray(sc["xyz"], np.float64)
    idx = np.asarray(sc["indices"], np.int64)
    tm = np.asarray(sc["tri_material"])
    n = np.zeros_like(xyz)
    fn = np.cross(xyz[idx[:, 1]] - xyz[idx[:, 0]], xyz[idx[:, 2]] - xyz[idx[:, 0]])
    fn /= np.linalg.norm(fn, axis=1, keepdims=True)
    wall = tm < 3
    n[idx[wall].ravel()] = np.repeat(fn[wall], 3, axis=0)
    for m in np.unique(tm[~wall]):
        v = np.unique(idx[tm == m].ravel())
        d = xyz[v] - xyz[v].mean(axis=0)
        n[v] = d / np.linalg.norm(d, axis=1, keepdims=True)
    return n.astype(np.float32)


def cornell_texcoords(sc, repeat: float = 2.0):
    """Texture coordinates and tangents for a cornell_scene(): each wall quad maps its four corners to
    (0, 0), (r, 0), (r, r), (0, r) (r = repeat), its tangent along the first edge; a sphere's vertices
    get longitude / latitude about its centre (u = 0.5 + atan2(z, x) / 2 pi, v = acos(y) / pi) and
    the tangent of growing longitude. Returns (uv float32 [V, 2], tangents float32 [V, 3])."""
    xyz = np.asarray(sc["xyz"], np.float64)
    idx = np.asarray(sc["indices"], np.int64)
    tm = np.asarray(sc["tri_material"])
    uv = np.zeros((len(xyz), 2))
    tg = np.zeros((len(xyz), 3))
    corners = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float64) * repeat
    for q in range(5):
        v = np.arange(4 * q, 4 * q + 4)
        uv[v] = corners
        e = xyz[v[1]] - xyz[v[0]]
        tg[v] = e / np.linalg.norm(e)
    for m in np.unique(tm[tm >= 3]):
        v = np.unique(idx[tm == m].ravel())
        d = xyz[v] - xyz[v].mean(axis=0)
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        uv[v, 0] = 0.5 + np.arctan2(d[:, 2], d[:, 0]) / (2 * np.pi)
        uv[v, 1] = np.arccos(np.clip(d[:, 1], -1, 1)) / np.pi
        t = np.stack([-d[:, 2], np.zeros(len(v)), d[:, 0]], axis=1)
        n = np.linalg.norm(t, axis=1, keepdims=True)
        tg[v] = np.where(n > 1e-6, t / np.maximum(n, 1e-12), np.array([1.0, 0.0, 0.0]))
    return uv.astype(np.float32), tg.astype(np.float32)


def test_textures(size: int = 64):
    """Procedural RGBA8 textures for the textured test scenes: [0] a two-colour checker, [1] an
    ao-rough-metal map (g: roughness stripes, b: metal checker), [2] a tangent-space normal map of
    bumps, [3] an emission pattern. uint8 [size, size, 4] each."""
    y, x = np.mgrid[0:size, 0:size].astype(np.float64)
    u, v = (x + 0.5) / size, (y + 0.5) / size
    chk = ((x // 8 + y // 8) % 2).astype(bool)
    color = np.zeros((size, size, 4), np.uint8)
    color[chk] = (230, 200, 60, 255)
    color[~chk] = (40, 90, 200, 255)
    arm = np.zeros((size, size, 4), np.uint8)
    arm[..., 0] = 255
    arm[..., 1] = (64 + 191 * (0.5 + 0.5 * np.sin(2 * np.pi * 4 * u))).astype(np.uint8)
    arm[..., 2] = np.where(((x // 16 + y // 16) % 2) == 0, 255, 0).astype(np.uint8)
    arm[..., 3] = 255
    bx, by = np.sin(2 * np.pi * 4 * u), np.sin(2 * np.pi * 4 * v)
    nx, ny = 0.4 * bx, 0.4 * by
    nz = np.sqrt(np.maximum(0.0, 1 - nx * nx - ny * ny))
    nrm = np.stack([(nx * 0.5 + 0.5) * 255, (ny * 0.5 + 0.5) * 255, nz * 255, np.full_like(nx, 255)], axis=-1)
    nrm = np.rint(nrm).astype(np.uint8)
    em = np.zeros((size, size, 4), np.uint8)
    ring = np.abs(np.hypot(u - 0.5, v - 0.5) - 0.3) < 0.08
    em[ring] = (255, 160, 40, 255)
    em[~ring] = (0, 0, 0, 255)
    return [color, arm, nrm, em]


def textured_materials(materials: np.ndarray) -> np.ndarray:
    """The Cornell materials with textures (indices into test_textures()): the back and floor walls
    checkered, spheres in turn checkered, ao-rough-metal mapped, normal mapped, with an emission
    pattern, or untextured."""
    m = np.array(materials, MATERIAL_DTYPE, copy=True)
    NO = 0xFFFFFFFF
    for f in ("tex_color", "tex_normal", "tex_emission", "tex_ao_rough_metal", "tex_transmission",
              "tex_diffuse_transmission", "tex_diffuse_transmission_color"):
        m[f] = NO
    m["tex_color"][0] = 0
    for s in range(len(m) - 3):
        i, kind = 3 + s, s % 5
        if kind == 0:
            m["tex_color"][i] = 0
        elif kind == 1:
            m["tex_ao_rough_metal"][i] = 1
        elif kind == 2:
            m["tex_normal"][i] = 2
        elif kind == 3:
            m["tex_emission"][i] = 3
            m["emission"][i] = (2.0, 2.0, 2.0)
    return m


def alpha_textures(size: int = 64):
    """test_textures() plus two colour textures with coverage in alpha: [4] a cut-out (an orange
    checker whose other squares have alpha 0), [5] a teal colour whose alpha ramps from 0 to 1 along u.
    uint8 [size, size, 4] each."""
    y, x = np.mgrid[0:size, 0:size].astype(np.float64)
    chk = ((x // 8 + y // 8) % 2).astype(bool)
    cut = np.zeros((size, size, 4), np.uint8)
    cut[..., :3] = (240, 140, 40)
    cut[..., 3] = np.where(chk, 255, 0).astype(np.uint8)
    ramp = np.zeros((size, size, 4), np.uint8)
    ramp[..., :3] = (40, 200, 190)
    ramp[..., 3] = np.rint(255 * (x + 0.5) / size).astype(np.uint8)
    return test_textures(size) + [cut, ramp]


ALPHA_KINDS = ("mask, cut-out texture", "blend, ramp texture", "blend, alpha 0.4", "opaque")


def alpha_materials(materials: np.ndarray) -> np.ndarray:
    """The Cornell materials with coverage (textures from alpha_textures()): the left wall
    (material 1) masked by the cut-out texture, so that light comes in through its holes; sphere s
    (material 3 + s) becomes ALPHA_KINDS[s % 4]. Alpha 1 and cut-off 0.5 unless stated."""
    from ._lib import BLEND_BLEND, BLEND_MASK
    m = np.array(materials, MATERIAL_DTYPE, copy=True)
    NO = 0xFFFFFFFF
    for f in ("tex_color", "tex_normal", "tex_emission", "tex_ao_rough_metal", "tex_transmission",
              "tex_diffuse_transmission", "tex_diffuse_transmission_color"):
        m[f] = NO
    m["alpha"] = 1.0
    m["alpha_cutoff"] = 0.5
    m["blend_mode"][1] = BLEND_MASK
    m["tex_color"][1] = 4
    for s in range(len(m) - 3):
        i, kind = 3 + s, s % 4
        if kind == 0:
            m["blend_mode"][i] = BLEND_MASK
            m["tex_color"][i] = 4
        elif kind == 1:
            m["blend_mode"][i] = BLEND_BLEND
            m["tex_color"][i] = 5
        elif kind == 2:
            m["blend_mode"][i] = BLEND_BLEND
            m["alpha"][i] = 0.4
    return m


SHOWCASE_KINDS = ("metal-rough", "glass", "rough glass", "clearcoat", "sheen", "diffuse transmission", "iridescent")


def showcase_materials(materials: np.ndarray) -> np.ndarray:
    """The Cornell-box material table with its spheres cycled through the Disney lobes: sphere s
    (material 3 + s) becomes SHOWCASE_KINDS[s % 7] and keeps its generated colour (lightened for glass;
    iridescent spheres alternate between dielectric and metal); the walls and the metal-rough spheres
    are unchanged."""
    m = np.array(materials, MATERIAL_DTYPE, copy=True)
    for s in range(len(m) - 3):
        i, kind = 3 + s, s % len(SHOWCASE_KINDS)
        c = m["base_color"][i].copy()
        if kind == 0:
            continue
        m["metalness"][i] = 0.0
        if kind in (1, 2):
            m["transmission"][i] = 1.0
            m["ior"][i] = 1.5 if kind == 1 else 1.33
            m["roughness"][i] = 0.0 if kind == 1 else 0.35
            m["base_color"][i] = 0.75 + 0.25 * c
        elif kind == 3:
            m["clearcoat"][i] = 1.0
            m["clearcoat_roughness"][i] = 0.05
            m["roughness"][i] = 0.6
        elif kind == 4:
            m["sheen_color"][i] = (0.9, 0.9, 0.9)
            m["sheen_roughness"][i] = 0.5
            m["roughness"][i] = 0.9
        elif kind == 5:
            m["diffuse_transmission"][i] = 0.6
            m["diffuse_transmission_color"][i] = c
            m["roughness"][i] = 0.7
        else:
            m["iridescence"][i] = 1.0
            m["iridescence_ior"][i] = 1.3
            m["iridescence_thickness"][i] = 400.0
            m["roughness"][i] = 0.25
            m["metalness"][i] = 1.0 if s % 2 else 0.0
    return m


MEDIA_KINDS = ("metal-rough", "fog", "absorbing glass", "emissive gas", "scattering glass")


def dispersive_materials(materials: np.ndarray, dispersion: float = 3.0) -> np.ndarray:
    """a copy of `materials` whose transmissive materials disperse (KHR_materials_dispersion value;
    3.0 is an Abbe number of about 6.7, strongly coloured)"""
    m = materials.copy()
    m["dispersion"][m["transmission"] > 0] = np.float32(dispersion)
    return m


def media_materials(materials: np.ndarray) -> np.ndarray:
    """The Cornell-box material table with its spheres cycled through homogeneous media: sphere s
    (material 3 + s) becomes MEDIA_KINDS[s % 5] with its generated colour c as the medium's tint —
    fog (a null surface around a forward-scattering medium), absorbing glass (Beer-Lambert inside a
    smooth dielectric), emissive gas (a null surface around an absorbing medium that emits 4 c) and
    scattering glass (a rough dielectric around a scattering medium). Attenuation distances are 0.25,
    about one sphere radius. Overlapping spheres nest their media on the per-path stack."""
    m = np.array(materials, MATERIAL_DTYPE, copy=True)
    for s in range(len(m) - 3):
        i, kind = 3 + s, s % len(MEDIA_KINDS)
        c = m["base_color"][i].copy()
        if kind == 0:
            continue
        m["metalness"][i] = 0.0
        m["attenuation_distance"][i] = 0.25
        if kind == 1:
            m["null_surface"][i] = 1
            m["attenuation_color"][i] = 0.35 + 0.5 * c
            m["scatter_factor"][i] = 1.0
            m["scatter_color"][i] = 0.6 + 0.4 * c
            m["phase_g"][i] = 0.5
        elif kind == 2:
            m["transmission"][i] = 1.0
            m["ior"][i] = 1.5
            m["roughness"][i] = 0.0
            m["base_color"][i] = 1.0
            m["attenuation_color"][i] = 0.2 + 0.8 * c
        elif kind == 3:
            m["null_surface"][i] = 1
            m["attenuation_color"][i] = (0.5, 0.5, 0.5)
            m["emission"][i] = 4.0 * c
        else:
            m["transmission"][i] = 1.0
            m["ior"][i] = 1.33
            m["roughness"][i] = 0.2
            m["base_color"][i] = 1.0
            m["attenuation_color"][i] = 0.3 + 0.6 * c
            m["scatter_factor"][i] = 1.0
            m["scatter_color"][i] = 0.5 + 0.5 * c
            m["phase_g"][i] = -0.2
    return m


def camera_lookat(eye, target, up, fovy_deg: float, width: int, height: int) -> vkg_camera:
    """tan(fovy/2) is evaluated here in double precision and passed to the library as a float."""
    L = lib()
    e = np.asarray(eye, np.float32)
    t = np.asarray(target, np.float32)
    u = np.asarray(up, np.float32)
    cam = vkg_camera()
    tan_half = float(np.float32(math.tan(math.radians(fovy_deg) / 2.0)))
    check(L.vkg_camera_lookat(_p(e), _p(t), _p(u), C.c_float(tan_half), width, height, C.byref(cam)))
    return cam


class _Pcg32:
    """PCG32 (XSH-RR, O'Neill 2014) for host-side workload parameters; the same generator as the kernels'."""
    MULT = 6364136223846793005
    MASK = (1 << 64) - 1

    def __init__(self, initstate: int, initseq: int):
        self.state = 0
        self.inc = ((initseq << 1) | 1) & self.MASK
        self.next()
        self.state = (self.state + initstate) & self.MASK
        self.next()

    def next(self) -> int:
        old = self.state
        self.state = (old * self.MULT + self.inc) & self.MASK
        xorshifted = (((old >> 18) ^ old) >> 27) & 0xFFFFFFFF
        rot = old >> 59
        return ((xorshifted >> rot) | (xorshifted << ((-rot) & 31))) & 0xFFFFFFFF

    def uniform(self) -> float:
        return (self.next() >> 8) * (1.0 / (1 << 24))


BATCH_RESOLUTIONS = (256, 512, 768, 1024)
BATCH_SPP = (4, 16, 64)


def batch_scene_params(index: int, seed: int = 0x5EED, min_tris: int = 5_000, max_tris: int = 2_000_000):
    """Parameters of scene `index` of the batched uneven workload (PCG32 seed 0x5EED, stream 3 + index):
    triangle count log-uniform in [min_tris, max_tris] (a Cornell box plus that many 3,072-triangle
    cube-spheres as fit, at least one), square resolution from {256, 512, 768, 1024}, spp from {4, 16, 64}.
    Returns dict(stream, spheres, triangles, resolution, spp)."""
    g = _Pcg32(seed, 3 + index)
    u_tris, u_res, u_spp = g.uniform(), g.uniform(), g.uniform()
    target = math.exp(math.log(min_tris) + u_tris * (math.log(max_tris) - math.log(min_tris)))
    spheres = max(1, int(round((target - 10) / 3072)))
    return {"stream": 3 + index, "spheres": spheres, "triangles": 10 + 3072 * spheres,
            "resolution": BATCH_RESOLUTIONS[min(3, int(u_res * 4))], "spp": BATCH_SPP[min(2, int(u_spp * 3))]}


def cubesphere(n: int, radius: float = 1.0):
    """cube-sphere of n x n quads per face: (xyz [6(n+1)^2, 3] f32, indices [12 n^2, 3] u32)"""
    xyz = np.zeros((6 * (n + 1) ** 2, 3), np.float32)
    idx = np.zeros((12 * n * n, 3), np.uint32)
    check(lib().vkg_geometry_cubesphere(n, C.c_float(radius), _p(xyz), _p(idx)))
    return xyz, idx


def terrain(n: int = 2048, extent: float = 512.0, height: float = 40.0, frequency: float = 1.0 / 128.0,
            octaves: int = 8, seed: int = 0x5EED):
    """fBm-over-simplex heightfield: (xyz [n^2, 3] f32, indices [2 (n-1)^2, 3] u32)"""
    xyz = np.zeros((n * n, 3), np.float32)
    idx = np.zeros((2 * (n - 1) ** 2, 3), np.uint32)
    check(lib().vkg_geometry_terrain(n, C.c_float(extent), C.c_float(height), C.c_float(frequency), octaves, seed,
                                     _p(xyz), _p(idx)))
    return xyz, idx


def random_instances(n: int, num_meshes: int, lo, hi, *, seed: int = 0x5EED, stream: int = 5, mat_base: int = 0,
                     num_mats: int = 1, smin: float = 0.5, smax: float = 2.0):
    """n instances (vierkant_gb300.raytracing.INSTANCE_DTYPE) with uniform translation in [lo, hi],
    uniform rotation, scale U[smin, smax], uniform mesh and material (PCG32(seed, stream))"""
    from .raytracing import INSTANCE_DTYPE
    out = np.zeros(n, INSTANCE_DTYPE)
    lo = np.asarray(lo, np.float32)
    hi = np.asarray(hi, np.float32)
    check(lib().vkg_instances_random(seed, stream, n, num_meshes, mat_base, num_mats, _p(lo), _p(hi), C.c_float(smin),
                                     C.c_float(smax), _p(out)))
    return out


def stress_scene(*, terrain_n: int = 2048, num_instances: int = 100_000, num_meshes: int = 20,
                 num_materials: int = 256, seed: int = 0x5EED):
    """The stress workload: a terrain_n^2-vertex fBm terrain (8 octaves, 512 x 512 units, +-40 height)
    and num_instances instances of num_meshes cube-spheres (n = 21 .. 65 quads per face, i.e. 5,292 to
    50,700 triangles) with uniform translation over the terrain's box, uniform rotation, scale U[0.5, 2]
    and one of num_materials random metal-rough materials (PCG32(seed, stream 5)).
    Returns dict(meshes=[(xyz, idx, twosided)], instances, materials)."""
    tx, ti = terrain(terrain_n, seed=seed)
    meshes = [(tx, ti, 1)]
    for k in range(num_meshes):
        n = 21 + int(round(44 * k / max(1, num_meshes - 1)))
        x, i = cubesphere(n, 1.0)
        meshes.append((x, i, 0))
    lo = tx.min(axis=0)
    hi = tx.max(axis=0)
    inst = random_instances(num_instances, num_meshes, lo, hi, seed=seed, stream=5, mat_base=1,
                            num_mats=num_materials)
    inst["blas"] += 1  # mesh 0 is the terrain
    from .raytracing import INSTANCE_DTYPE
    ground = np.zeros(1, INSTANCE_DTYPE)
    ground[0]["transform"] = np.array([1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0], np.float32)
    ground[0]["blas"] = 0
    ground[0]["material"] = 0
    mats = np.zeros(1 + num_materials, MATERIAL_DTYPE)
    mats[0]["base_color"] = (0.35, 0.45, 0.30)
    mats[0]["roughness"] = 0.9
    g = _Pcg32(seed, 6)
    for m in range(1, 1 + num_materials):
        mats[m]["base_color"] = [0.1 + 0.8 * g.uniform() for _ in range(3)]
        mats[m]["roughness"] = 0.05 + 0.95 * g.uniform()
        mats[m]["metalness"] = 1.0 if g.uniform() < 0.3 else 0.0
    return {"meshes": meshes, "instances": np.concatenate([ground, inst]), "materials": mats}
