"""CPU oracle loader. TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this package, and only as
the checker / the timed CPU reference. The product (vierkant_gb300, libvkg.so) never imports it.

- ``orc()``  -> liboracle.so: C restatement of the reference's algorithms (see oracle.h)
- ``ref()``  -> _ref/libvkref.so: the reference's own src/intersection.cpp compiled unmodified
               against the project-written shim from the copy in baseline/_ref (None if that copy
               is absent)
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
# the reference's files this oracle compiles, copied unmodified into baseline/_ref by `make -C oracle stage`
REF_ROOT = Path(os.environ.get("VKG_REFERENCE_ROOT", str(HERE.parent / "baseline" / "_ref")))

RAY_DTYPE = np.dtype([("o", "<f4", 3), ("tmin", "<f4"), ("d", "<f4", 3), ("tmax", "<f4")])
HIT_DTYPE = np.dtype([("prim", "<u4"), ("t", "<f4"), ("u", "<f4"), ("v", "<f4")])


class orc_bvh(C.Structure):
    _fields_ = [("num_tris", C.c_uint32), ("num_nodes", C.c_uint32), ("depth", C.c_uint32), ("leaf_max", C.c_uint32),
                ("scene_min", C.c_float * 3), ("scene_max", C.c_float * 3), ("margin", C.c_float),
                ("morton", C.POINTER(C.c_uint32)), ("sorted_prim", C.POINTER(C.c_uint32)),
                ("bvh2_left", C.POINTER(C.c_uint32)), ("bvh2_right", C.POINTER(C.c_uint32)),
                ("nodes", C.c_void_p), ("tris", C.c_void_p)]


class orc_camera(C.Structure):
    _fields_ = [("eye", C.c_float * 3), ("right", C.c_float * 3), ("up", C.c_float * 3), ("back", C.c_float * 3),
                ("tan_half_fovy", C.c_float), ("aspect", C.c_float), ("width", C.c_uint32), ("height", C.c_uint32)]


class orc_sphere_params(C.Structure):
    _fields_ = [("radius", C.c_float), ("center", C.c_float * 3), ("roughness", C.c_float),
                ("metalness", C.c_float), ("base", C.c_float * 3)]


def build(ref: bool | None = None, quiet: bool = True) -> None:
    """make liboracle.so (always) and _ref/libvkref.so (when the reference checkout is present)."""
    out = subprocess.DEVNULL if quiet else None
    subprocess.run(["make", "-s", "-C", str(HERE), "liboracle.so"], check=True, stdout=out)
    if ref is None:
        ref = (REF_ROOT / "src" / "intersection.cpp").exists()
    if ref:
        subprocess.run(["make", "-s", "-C", str(HERE), "ref", f"REF_ROOT={REF_ROOT}"], check=True, stdout=out)


_orc = None
_ref = None


def orc() -> C.CDLL:
    global _orc
    if _orc is None:
        p = HERE / "liboracle.so"
        if not p.exists():
            build(ref=False)
        L = C.CDLL(str(p))
        vp, u32, u64, i32, f32 = C.c_void_p, C.c_uint32, C.c_uint64, C.c_int, C.c_float
        sig = {
            "orc_pcg32_fill": (None, [u64, u64, u64, u32, vp]),
            "orc_xxhash32": (u32, [u32, u32]),
            "orc_rnd": (f32, [C.POINTER(u32)]),
            "orc_intersect_ray_triangle": (i32, [vp, vp, vp, vp]),
            "orc_intersect_ray_triangle_cull": (i32, [vp, vp, vp, i32, vp]),
            "orc_intersect_ray_aabb": (i32, [vp, vp, vp, vp, C.POINTER(f32)]),
            "orc_closest_hit_bruteforce": (i32, [vp, vp, u32, vp, u32, vp, i32, i32]),
            "orc_any_hit_bruteforce": (i32, [vp, vp, u32, vp, u32, vp, i32, i32]),
            "orc_bvh_closest_hit_fn": (i32, [vp, vp, u32, vp, i32, vp, vp, vp]),
            "orc_icosphere_counts": (u32, [u32, C.POINTER(u32)]),
            "orc_icosphere": (None, [f32, u32, vp, vp]),
            "orc_cornell_sphere_params": (None, [u64, u64, u32, vp]),
            "orc_cornell_scene": (None, [u64, u64, u32, u32, vp, vp, vp]),
            "orc_camera_lookat": (None, [vp, vp, vp, f32, u32, u32, C.POINTER(orc_camera)]),
            "orc_camera_rays_pcg": (None, [C.POINTER(orc_camera), u64, u64, u32, vp]),
            "orc_bvh_build": (i32, [vp, vp, u32, u32, C.POINTER(orc_bvh)]),
            "orc_bvh_free": (None, [C.POINTER(orc_bvh)]),
            "orc_bvh_closest_hit": (i32, [C.POINTER(orc_bvh), vp, u32, vp, i32, i32, vp]),
            "orc_bvh_any_hit": (i32, [C.POINTER(orc_bvh), vp, u32, vp, i32, i32]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        L.orc_pt_material_size.restype = u32
        if L.orc_pt_material_size() != MATERIAL_DTYPE.itemsize:
            raise RuntimeError("liboracle.so's material record does not match MATERIAL_DTYPE: rebuild the oracle")
        _orc = L
    return _orc


def ref() -> C.CDLL | None:
    global _ref
    if _ref is None:
        p = HERE / "_ref" / "libvkref.so"
        if not p.exists():
            return None
        L = C.CDLL(str(p))
        vp, u32, i32, f32 = C.c_void_p, C.c_uint32, C.c_int, C.c_float
        sig = {
            "vkref_intersect_ray_triangle": (i32, [vp, vp, vp, vp]),
            "vkref_intersect_ray_aabb": (i32, [vp, vp, vp, vp, C.POINTER(f32)]),
            "vkref_intersect_ray_sphere": (i32, [vp, vp, vp, f32, C.POINTER(f32)]),
            "vkref_intersect_ray_plane": (i32, [vp, vp, vp, C.POINTER(f32)]),
            "vkref_triangle_aabb_overlap": (u32, [vp, vp, vp]),
            "vkref_triangle_triangle_overlap": (u32, [vp, vp]),
            "vkref_closest_hit_bruteforce": (i32, [vp, vp, u32, vp, u32, vp, i32, i32]),
            "vkref_mesh_create": (vp, [vp, vp, u32]),
            "vkref_mesh_destroy": (None, [vp]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _ref = L
    return _ref


def ptr(a: np.ndarray) -> C.c_void_p:
    return a.ctypes.data_as(C.c_void_p)


# ---- convenience wrappers ----------------------------------------------------------------------
def icosphere(radius=1.0, tess=5):
    L = orc()
    nt = C.c_uint32()
    nv = L.orc_icosphere_counts(tess, C.byref(nt))
    xyz = np.zeros((nv, 3), np.float32)
    idx = np.zeros((nt.value, 3), np.uint32)
    L.orc_icosphere(radius, tess, ptr(xyz), ptr(idx))
    return xyz, idx


def cornell_scene(seed=0x5EED, stream=2, num_spheres=64, n=16):
    L = orc()
    nv = 20 + num_spheres * 6 * (n + 1) ** 2
    nt = 10 + num_spheres * 12 * n * n
    xyz = np.zeros((nv, 3), np.float32)
    idx = np.zeros((nt, 3), np.uint32)
    tm = np.zeros(nt, np.uint32)
    L.orc_cornell_scene(seed, stream, num_spheres, n, ptr(xyz), ptr(idx), ptr(tm))
    params = (orc_sphere_params * max(1, num_spheres))()
    L.orc_cornell_sphere_params(seed, stream, num_spheres, C.cast(params, C.c_void_p))
    return {"xyz": xyz, "indices": idx, "tri_material": tm, "spheres": params}


def camera(eye, target, up, tan_half_fovy, width, height) -> orc_camera:
    cam = orc_camera()
    e, t, u = (np.asarray(x, np.float32) for x in (eye, target, up))
    orc().orc_camera_lookat(ptr(e), ptr(t), ptr(u), tan_half_fovy, width, height, C.byref(cam))
    return cam


def camera_rays(cam: orc_camera, seed: int, stream: int, spp: int = 1) -> np.ndarray:
    rays = np.zeros(cam.width * cam.height * spp, RAY_DTYPE)
    orc().orc_camera_rays_pcg(C.byref(cam), seed, stream, spp, ptr(rays))
    return rays


def closest_hit_bruteforce(xyz, idx, rays, nthreads=0, cull=False):
    hits = np.zeros(len(rays), HIT_DTYPE)
    orc().orc_closest_hit_bruteforce(ptr(xyz), ptr(idx), idx.shape[0], ptr(rays), len(rays), ptr(hits), nthreads,
                                     int(cull))
    return hits


def any_hit_bruteforce(xyz, idx, rays, nthreads=0, cull=False):
    occ = np.zeros(len(rays), np.uint32)
    orc().orc_any_hit_bruteforce(ptr(xyz), ptr(idx), idx.shape[0], ptr(rays), len(rays), ptr(occ), nthreads,
                                 int(cull))
    return occ


NODE_BYTES = 96
TRI_BYTES = 48


class CpuBVH:
    """The oracle's LBVH -> 8-wide BVH (same algorithm as the GPU build), with CPU traversal."""

    def __init__(self, xyz, idx, leaf_max=4):
        self.xyz, self.idx = np.ascontiguousarray(xyz, np.float32), np.ascontiguousarray(idx, np.uint32)
        self.b = orc_bvh()
        rc = orc().orc_bvh_build(ptr(self.xyz), ptr(self.idx), self.idx.shape[0], leaf_max, C.byref(self.b))
        if rc != 0:
            raise RuntimeError(f"orc_bvh_build failed ({rc})")

    def __del__(self):
        try:
            orc().orc_bvh_free(C.byref(self.b))
        except Exception:
            pass

    @property
    def morton(self):
        return np.ctypeslib.as_array(self.b.morton, (self.b.num_tris,)).copy() if self.b.num_tris else np.zeros(0)

    @property
    def sorted_prim(self):
        return np.ctypeslib.as_array(self.b.sorted_prim, (self.b.num_tris,)).copy() if self.b.num_tris else np.zeros(0)

    def node_bytes(self) -> bytes:
        return C.string_at(self.b.nodes, self.b.num_nodes * NODE_BYTES) if self.b.num_nodes else b""

    def tri_bytes(self) -> bytes:
        return C.string_at(self.b.tris, self.b.num_tris * TRI_BYTES) if self.b.num_tris else b""

    def closest_hit(self, rays, nthreads=0, cull=False, stats=False):
        hits = np.zeros(len(rays), HIT_DTYPE)
        st = np.zeros(2, np.uint64)
        orc().orc_bvh_closest_hit(C.byref(self.b), ptr(rays), len(rays), ptr(hits), nthreads, int(cull), ptr(st))
        return (hits, (int(st[0]), int(st[1]))) if stats else hits

    def any_hit(self, rays, nthreads=0, cull=False):
        occ = np.zeros(len(rays), np.uint32)
        orc().orc_bvh_any_hit(C.byref(self.b), ptr(rays), len(rays), ptr(occ), nthreads, int(cull))
        return occ

    def closest_hit_ref(self, mesh: "RefMesh", rays, nthreads=0, stats=False):
        """Closest hit over this BVH with every triangle test done by the reference's own
        vierkant::intersect (intersection.cpp:114-129) on the original triangle; no culling. Returns
        (hits, threads used) or (hits, threads, (visits, tests)) with stats."""
        hits = np.zeros(len(rays), HIT_DTYPE)
        st = np.zeros(2, np.uint64)
        used = orc().orc_bvh_closest_hit_fn(C.byref(self.b), ptr(rays), len(rays), ptr(hits), nthreads, mesh.fn,
                                            mesh.handle, ptr(st))
        return (hits, used, (int(st[0]), int(st[1]))) if stats else (hits, used)


class RefMesh:
    """The reference's vierkant::Triangle array of an indexed mesh (needs oracle/_ref)."""

    def __init__(self, xyz, idx):
        R = ref()
        if R is None:
            raise RuntimeError("oracle/_ref/libvkref.so was not built")
        xyz, idx = np.ascontiguousarray(xyz, np.float32), np.ascontiguousarray(idx, np.uint32)
        self.handle = R.vkref_mesh_create(ptr(xyz), ptr(idx), idx.shape[0])
        self.fn = C.cast(R.vkref_mesh_intersect, C.c_void_p)

    def __del__(self):
        try:
            ref().vkref_mesh_destroy(self.handle)
        except Exception:
            pass


INST_HIT_DTYPE = np.dtype([("prim", "<u4"), ("inst", "<u4"), ("t", "<f4"), ("u", "<f4"), ("v", "<f4"),
                           ("pad", "<u4", 3)])


def tlas_closest_hit(blas: list, w2o, inst_blas, rays, cull=False, nthreads=0):
    """two-level closest hit (oracle/tlas.c): instances in input order, w2o [N, 12] world -> object"""
    w2o = np.ascontiguousarray(w2o, np.float32)
    ib = np.ascontiguousarray(inst_blas, np.uint32)
    arr = (C.POINTER(orc_bvh) * len(blas))(*[C.pointer(b.b) for b in blas])
    hits = np.zeros(len(rays), INST_HIT_DTYPE)
    orc().orc_tlas_closest_hit(arr, ptr(w2o), ptr(ib), len(ib), ptr(rays), len(rays), int(cull), ptr(hits), nthreads)
    return hits


def tlas_any_hit(blas: list, w2o, inst_blas, rays, cull=False, nthreads=0):
    w2o = np.ascontiguousarray(w2o, np.float32)
    ib = np.ascontiguousarray(inst_blas, np.uint32)
    arr = (C.POINTER(orc_bvh) * len(blas))(*[C.pointer(b.b) for b in blas])
    occ = np.zeros(len(rays), np.uint32)
    orc().orc_tlas_any_hit(arr, ptr(w2o), ptr(ib), len(ib), ptr(rays), len(rays), int(cull), ptr(occ), nthreads)
    return occ


# ---- path tracer (FP32 twin / FP64 oracle) ---------------------------------------------------------
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


class orc_pt_scene(C.Structure):
    _fields_ = [("xyz", C.c_void_p), ("idx", C.c_void_p), ("tri_mat", C.c_void_p), ("mats", C.c_void_p),
                ("ntri", C.c_uint32), ("nmat", C.c_uint32), ("nrm", C.c_void_p), ("uv", C.c_void_p),
                ("tng", C.c_void_p), ("tex", C.c_void_p), ("texels", C.c_void_p), ("ntex", C.c_uint32)]


TEX_REC_DTYPE = np.dtype([("width", "<u4"), ("height", "<u4"), ("levels", "<u4"), ("wrap", "<u4"),
                          ("offset", "<u4", 16)])


def texture_pool(textures):
    """Texture records (TEX_REC_DTYPE) and the RGBA8 texel array (uint32) of every level, as
    vkg_scene_set_textures builds them: level k + 1 is the rounded mean (sum + 2) >> 2 of 2 x 2 texels
    of level k, the last row / column repeated for odd sizes. textures: uint8 [H, W, 4] arrays or
    (array, wrap_s, wrap_t) tuples."""
    recs = np.zeros(len(textures), TEX_REC_DTYPE)
    pool, total = [], 0
    for k, t in enumerate(textures):
        img, ws, wt = t if isinstance(t, tuple) else (t, 0, 0)
        lvl = np.ascontiguousarray(img, np.uint8).astype(np.uint32)
        h, w = lvl.shape[:2]
        recs[k]["width"], recs[k]["height"], recs[k]["wrap"] = w, h, ws | (wt << 8)
        n = 0
        while True:
            recs[k]["offset"][n] = total
            words = lvl[..., 0] | (lvl[..., 1] << 8) | (lvl[..., 2] << 16) | (lvl[..., 3] << 24)
            pool.append(words.reshape(-1).astype(np.uint32))
            total += words.size
            n += 1
            if (w == 1 and h == 1) or n == 16:
                break
            pw, ph = w, h
            w, h = max(1, w // 2), max(1, h // 2)
            xs0 = np.minimum(2 * np.arange(w), pw - 1)
            xs1 = np.minimum(2 * np.arange(w) + 1, pw - 1)
            ys0 = np.minimum(2 * np.arange(h), ph - 1)
            ys1 = np.minimum(2 * np.arange(h) + 1, ph - 1)
            s = (lvl[ys0][:, xs0] + lvl[ys0][:, xs1] + lvl[ys1][:, xs0] + lvl[ys1][:, xs1] + 2) >> 2
            lvl = s.astype(np.uint32)
        recs[k]["levels"] = n
    texels = np.concatenate(pool) if pool else np.zeros(1, np.uint32)
    return recs, texels


def tex_sample(recs, texels, k, u, v, lam):
    """texture k sampled at (u, v), level lambda, by the oracle (FP64): RGBA floats"""
    L = orc()
    L.orc_tex_sample.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_double, C.c_void_p]
    out = np.zeros(4, np.float64)
    L.orc_tex_sample(recs[k:k + 1].ctypes.data, texels.ctypes.data, u, v, lam, out.ctypes.data)
    return out


def _normals(normals):
    """unit vertex normals as the tracers store them: float32 [V, 3], each normalised in float32"""
    n = np.ascontiguousarray(normals, np.float32).reshape(-1, 3)
    return np.ascontiguousarray(n / np.sqrt((n * n).sum(axis=1, dtype=np.float32))[:, None], np.float32)


class orc_pt_env(C.Structure):
    _fields_ = [("rgb", C.c_void_p), ("weight", C.c_void_p), ("alias_prob", C.c_void_p), ("alias", C.c_void_p),
                ("cdf", C.c_void_p), ("w", C.c_uint32), ("h", C.c_uint32)]


class orc_pt_settings(C.Structure):
    _fields_ = [("seed", C.c_uint32), ("batch", C.c_uint32), ("spp", C.c_uint32), ("max_depth", C.c_uint32),
                ("rr_depth", C.c_uint32), ("mis_mode", C.c_uint32), ("disable_material", C.c_uint32),
                ("draw_skybox", C.c_uint32), ("max_path_beta", C.c_float), ("environment", C.c_float),
                ("crop", C.c_uint32 * 4), ("num_lights", C.c_uint32), ("suppress_caustics", C.c_uint32),
                ("lights", C.c_void_p), ("pixels", C.c_void_p), ("clip_near", C.c_float),
                ("camera_medium", C.c_void_p), ("camera_material", C.c_uint32)]


# per-pixel record (32 bytes, the layout of vkg_pixel_data)
PIXEL_DTYPE = np.dtype([("radiance", "<f4", 3), ("alpha", "<f4"), ("depth", "<f4"), ("normal", "<u4"),
                        ("object_id", "<u4"), ("albedo", "<u4")])


def post_fx(hdr_rgba, tonemap=True, bloom=True, exposure=2.0, gamma=1.0, brightness_thresh=(0.95, 1.1),
            iterations=3):
    """bloom + tonemap composition of an HDR image [h, w, 4] float32 (oracle/postfx.c)"""
    src = np.ascontiguousarray(hdr_rgba, np.float32)
    h, w = src.shape[:2]
    out = np.zeros_like(src)
    orc().orc_post_fx.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_int, C.c_int, C.c_float, C.c_float,
                                  C.c_float, C.c_float, C.c_uint32, C.c_void_p]
    orc().orc_post_fx(ptr(src), w, h, int(tonemap), int(bloom), exposure, gamma, brightness_thresh[0],
                      brightness_thresh[1], iterations, ptr(out))
    return out


def denoise(pixels):
    """the a-trous denoise pass over pixel records [h, w] (PIXEL_DTYPE); returns rgba [h, w, 4] float32"""
    px = np.ascontiguousarray(pixels, PIXEL_DTYPE)
    h, w = px.shape
    out = np.zeros((h, w, 4), np.float32)
    orc().orc_denoise.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p]
    orc().orc_denoise(ptr(px), w, h, ptr(out))
    return out


# analytic light record (80 bytes, the layout of vkg_light)
LIGHT_DTYPE = np.dtype([("position", "<f4", 3), ("type", "<u4"), ("color", "<f4", 3), ("intensity", "<f4"),
                        ("direction", "<f4", 3), ("range", "<f4"), ("spot_angle_scale", "<f4"),
                        ("spot_angle_offset", "<f4"), ("angular_size", "<f4"), ("size_y", "<f4"),
                        ("tangent", "<f4", 3), ("size_x", "<f4")])


def sun_light(color, intensity, spherical_coords, angular_size):
    """the tracer settings' sun as a directional light record (oracle restatement)"""
    out = np.zeros(1, LIGHT_DTYPE)
    orc().orc_sun_light.argtypes = [C.c_void_p, C.c_float, C.c_void_p, C.c_float, C.c_void_p]
    orc().orc_sun_light(ptr(np.asarray(color, np.float32)), intensity, ptr(np.asarray(spherical_coords, np.float32)),
                        angular_size, ptr(out))
    return out[0]


MEDIUM_PARAMS = ("attenuation_color", "attenuation_distance", "scatter_factor", "scatter_color", "phase_g", "ior",
                 "emission_color", "emission_intensity")
MEDIUM_DEFAULTS = dict(attenuation_color=(0.7, 0.7, 0.7), attenuation_distance=1.0, scatter_factor=0.0,
                       scatter_color=(1, 1, 1), phase_g=0.0, ior=1.0, emission_color=(1, 1, 1),
                       emission_intensity=0.0)


def medium_params(**kw):
    """the 14 floats of a camera medium (medium_params_t order) from keyword fields over the defaults"""
    d = dict(MEDIUM_DEFAULTS, **kw)
    return np.concatenate([np.atleast_1d(np.asarray(d[k], np.float32)) for k in MEDIUM_PARAMS]).astype(np.float32)


def _settings(seed, batch, spp, max_depth, rr_depth, mis_mode, draw_skybox, max_path_beta, environment, crop, lights,
              suppress_caustics, pixels=None, clip_near=0.1, camera_medium=None, camera_material=None):
    arr = np.ascontiguousarray(np.asarray(lights if lights is not None else [], LIGHT_DTYPE).reshape(-1))
    cm = np.ascontiguousarray(camera_medium, np.float32) if camera_medium is not None else None
    assert cm is None or cm.shape == (14,)
    st = orc_pt_settings(seed, batch, spp, max_depth, rr_depth, mis_mode, 0, draw_skybox, max_path_beta, environment,
                         (C.c_uint32 * 4)(*crop), len(arr), int(suppress_caustics),
                         arr.ctypes.data_as(C.c_void_p) if len(arr) else None,
                         pixels.ctypes.data_as(C.c_void_p) if pixels is not None else None, clip_near,
                         cm.ctypes.data_as(C.c_void_p) if cm is not None else None,
                         0xFFFFFFFF if camera_material is None else int(camera_material))
    return st, (arr, cm)


def cornell_materials(seed=0x5EED, stream=2, num_spheres=64):
    """Material table of the Cornell benchmark scene (walls two-sided, spheres one-sided)."""
    sc = cornell_scene(seed, stream, num_spheres, 1)
    mats = np.zeros(3 + num_spheres, MATERIAL_DTYPE)
    mats["base_color"][0] = (0.73, 0.73, 0.73)
    mats["base_color"][1] = (0.65, 0.05, 0.05)
    mats["base_color"][2] = (0.12, 0.45, 0.15)
    mats["roughness"][:3] = 1.0
    mats["twosided"][:3] = 1
    for s in range(num_spheres):
        p = sc["spheres"][s]
        mats["base_color"][3 + s] = tuple(p.base)
        mats["roughness"][3 + s] = p.roughness
        mats["metalness"][3 + s] = p.metalness
    return mats


def env_procedural(w, h, sun_dir, peak=5e4, width=3.8e-5):
    rgb = np.zeros((h, w, 3), np.float32)
    sd = np.ascontiguousarray(sun_dir, np.float32)
    orc().orc_pt_env_procedural.argtypes = [C.c_uint32, C.c_uint32, C.c_void_p, C.c_double, C.c_double, C.c_void_p]
    orc().orc_pt_env_procedural(w, h, ptr(sd), peak, width, ptr(rgb))
    return rgb


def env_tables_fp64(rgb):
    h, w = rgb.shape[:2]
    weight = np.zeros(w * h, np.float32)
    cdf = np.zeros(w * h + 1, np.float64)
    L = orc()
    L.orc_pt_env_tables.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p]
    L.orc_pt_env_tables(ptr(np.ascontiguousarray(rgb, np.float32)), w, h, ptr(weight), ptr(cdf))
    return weight, cdf


def pt_render(fp64, xyz, idx, tri_mat, mats, bvh: "CpuBVH", env_rgb, cam, spp, *, seed=0x5EED, batch=0, max_depth=6,
              rr_depth=3, mis_mode=0, crop=(0, 0, 0, 0), environment=1.0, draw_skybox=1, max_path_beta=0.0,
              alias_prob=None, alias=None, weight=None, cdf=None, nthreads=0, lights=None, suppress_caustics=False,
              pixels=None, clip_near=0.1, camera_medium=None, camera_material=None, normals=None, uv=None,
              tangents=None, textures=None):
    """Mean radiance per crop pixel ([h, w, 3] float64), mean squared luminance per pixel, (ext, shadow) rays.
    pixels: optional PIXEL_DTYPE array [h, w] of the crop, filled with the pixel records (radiance left 0)
    the tracer writes. normals / tangents / uv: optional vertex normals [V, 3] (smooth shading),
    tangents [V, 3] and texture coordinates [V, 2]; textures: as texture_pool takes them."""
    L = orc()
    L.orc_pt_render.argtypes = [C.c_int, C.POINTER(orc_pt_scene), C.POINTER(orc_bvh), C.POINTER(orc_pt_env),
                                C.POINTER(orc_camera), C.POINTER(orc_pt_settings), C.c_void_p, C.c_void_p, C.c_void_p,
                                C.c_int]
    if np.asarray(mats).dtype.itemsize != MATERIAL_DTYPE.itemsize:
        raise ValueError("materials must be 208-byte material records")
    keep = [np.ascontiguousarray(a) for a in (xyz, idx, tri_mat, mats)]
    nrm = _normals(normals) if normals is not None else None
    tng = _normals(tangents) if tangents is not None else None
    tuv = np.ascontiguousarray(uv, np.float32) if uv is not None else None
    recs, texels = texture_pool(textures) if textures else (None, None)
    keep += [a for a in (nrm, tng, tuv, recs, texels) if a is not None]
    scene = orc_pt_scene(ptr(keep[0]), ptr(keep[1]), ptr(keep[2]), ptr(keep[3]), keep[1].shape[0], len(mats),
                         ptr(nrm) if nrm is not None else None, ptr(tuv) if tuv is not None else None,
                         ptr(tng) if tng is not None else None, ptr(recs) if recs is not None else None,
                         ptr(texels) if texels is not None else None, len(recs) if recs is not None else 0)
    rgb = np.ascontiguousarray(env_rgb, np.float32)
    h, w = rgb.shape[:2]
    if fp64 and (weight is None or cdf is None):
        weight, cdf = env_tables_fp64(rgb)
    env = orc_pt_env(ptr(rgb), ptr(np.ascontiguousarray(weight, np.float32)),
                     ptr(alias_prob) if alias_prob is not None else None,
                     ptr(alias) if alias is not None else None, ptr(cdf) if cdf is not None else None, w, h)
    cw = crop[2] or cam.width
    ch = crop[3] or cam.height
    st, _keep = _settings(seed, batch, spp, max_depth, rr_depth, mis_mode, draw_skybox, max_path_beta, environment,
                          crop, lights, suppress_caustics, pixels, clip_near, camera_medium, camera_material)
    out = np.zeros((ch, cw, 3), np.float64)
    sq = np.zeros((ch, cw), np.float64)
    stats = np.zeros(2, np.uint64)
    L.orc_pt_render(int(fp64), C.byref(scene), C.byref(bvh.b), C.byref(env), C.byref(cam), C.byref(st), ptr(out),
                    ptr(sq), ptr(stats), nthreads)
    return out, sq, (int(stats[0]), int(stats[1]))


def pt_variance_split(xyz, idx, tri_mat, mats, bvh: "CpuBVH", env_rgb, cam, spp, fork_depth, *, seed=0x5EED,
                      max_depth=6, rr_depth=3, mis_mode=0, crop=(0, 0, 0, 0), nthreads=0):
    """FP64 variance split at the surface reached by segment fork_depth (orc_pt_variance_split):
    [h, w, 4] float64 {mean luminance, per-sample variance of the plain estimator, the tail variance an
    exact cache there would remove, fraction of samples reaching it}, and (extension, shadow) rays of
    one trace per sample."""
    L = orc()
    L.orc_pt_variance_split.argtypes = [C.POINTER(orc_pt_scene), C.POINTER(orc_bvh), C.POINTER(orc_pt_env),
                                        C.POINTER(orc_camera), C.POINTER(orc_pt_settings), C.c_uint32, C.c_void_p,
                                        C.c_void_p, C.c_int]
    keep = [np.ascontiguousarray(a) for a in (xyz, idx, tri_mat, mats)]
    scene = orc_pt_scene(ptr(keep[0]), ptr(keep[1]), ptr(keep[2]), ptr(keep[3]), keep[1].shape[0], len(mats))
    rgb = np.ascontiguousarray(env_rgb, np.float32)
    h, w = rgb.shape[:2]
    weight, cdf = env_tables_fp64(rgb)
    env = orc_pt_env(ptr(rgb), ptr(np.ascontiguousarray(weight, np.float32)), None, None, ptr(cdf), w, h)
    cw = crop[2] or cam.width
    ch = crop[3] or cam.height
    st, _keep = _settings(seed, 0, spp, max_depth, rr_depth, mis_mode, 1, 0.0, 1.0, crop, None, False, None, 0.1,
                          None, None)
    out = np.zeros((ch, cw, 4), np.float64)
    stats = np.zeros(2, np.uint64)
    L.orc_pt_variance_split(C.byref(scene), C.byref(bvh.b), C.byref(env), C.byref(cam), C.byref(st), fork_depth,
                            ptr(out), ptr(stats), nthreads)
    return out, (int(stats[0]), int(stats[1]))


class orc_pt_instances(C.Structure):
    _fields_ = [("mesh_bvh", C.c_void_p), ("mesh_xyz", C.c_void_p), ("mesh_idx", C.c_void_p),
                ("mesh_nvert", C.c_void_p), ("mesh_twosided", C.c_void_p), ("num_meshes", C.c_uint32),
                ("o2w", C.c_void_p), ("inst_mesh", C.c_void_p), ("inst_mat", C.c_void_p),
                ("num_instances", C.c_uint32), ("mesh_nrm", C.c_void_p), ("mesh_uv", C.c_void_p),
                ("mesh_tng", C.c_void_p)]


def pt_render_instanced(meshes, o2w, inst_mesh, inst_mat, mats, env_rgb, cam, spp, *, seed=0x5EED, batch=0,
                        max_depth=6, rr_depth=3, mis_mode=0, crop=(0, 0, 0, 0), environment=1.0, draw_skybox=1,
                        nthreads=0, mesh_bvhs=None, lights=None, suppress_caustics=False, camera_medium=None,
                        camera_material=None, mesh_normals=None):
    """FP64 oracle of an instanced scene: meshes [(xyz, idx, twosided)], o2w [N, 12] object -> world,
    mesh and material index per instance; mesh_normals: optional per-mesh vertex normals (or None). Returns (mean radiance [h, w, 3], mean squared luminance,
    (ext, shadow) rays). camera_medium: medium_params(...) floats; camera_material: the material whose
    medium the camera sits in."""
    L = orc()
    L.orc_pt_render_instanced.argtypes = [C.POINTER(orc_pt_scene), C.POINTER(orc_pt_instances),
                                          C.POINTER(orc_pt_env), C.POINTER(orc_camera),
                                          C.POINTER(orc_pt_settings), C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
    keep = []
    bvhs = mesh_bvhs if mesh_bvhs is not None else [CpuBVH(x, i, 4) for x, i, _ in meshes]
    xyzs = [np.ascontiguousarray(x, np.float32) for x, _, _ in meshes]
    idxs = [np.ascontiguousarray(i, np.uint32) for _, i, _ in meshes]
    keep += xyzs + idxs
    bvh_arr = (C.POINTER(orc_bvh) * len(meshes))(*[C.pointer(b.b) for b in bvhs])
    xyz_arr = (C.c_void_p * len(meshes))(*[x.ctypes.data for x in xyzs])
    idx_arr = (C.c_void_p * len(meshes))(*[i.ctypes.data for i in idxs])
    nvert = np.array([len(x) for x in xyzs], np.uint32)
    twos = np.array([int(t) for _, _, t in meshes], np.uint8)
    o2w = np.ascontiguousarray(o2w, np.float32)
    im = np.ascontiguousarray(inst_mesh, np.uint32)
    imat = np.ascontiguousarray(inst_mat, np.uint32)
    mats = np.ascontiguousarray(mats)
    if mats.dtype.itemsize != MATERIAL_DTYPE.itemsize:
        raise ValueError("materials must be 208-byte material records")
    keep += [nvert, twos, o2w, im, imat, mats]
    nrm_arr = None
    if mesh_normals is not None:
        nrms = [_normals(n) if n is not None else None for n in mesh_normals]
        keep += [n for n in nrms if n is not None]
        nrm_arr = (C.c_void_p * len(meshes))(*[n.ctypes.data if n is not None else None for n in nrms])
    inst = orc_pt_instances(C.cast(bvh_arr, C.c_void_p), C.cast(xyz_arr, C.c_void_p), C.cast(idx_arr, C.c_void_p),
                            ptr(nvert), ptr(twos), len(meshes), ptr(o2w), ptr(im), ptr(imat), len(im),
                            C.cast(nrm_arr, C.c_void_p) if nrm_arr is not None else None)
    scene = orc_pt_scene(None, None, None, ptr(mats), 0, len(mats))
    rgb = np.ascontiguousarray(env_rgb, np.float32)
    h, w = rgb.shape[:2]
    weight, cdf = env_tables_fp64(rgb)
    env = orc_pt_env(ptr(rgb), ptr(np.ascontiguousarray(weight, np.float32)), None, None, ptr(cdf), w, h)
    cw = crop[2] or cam.width
    ch = crop[3] or cam.height
    st, _keep = _settings(seed, batch, spp, max_depth, rr_depth, mis_mode, draw_skybox, 0.0, environment, crop,
                          lights, suppress_caustics, None, 0.1, camera_medium, camera_material)
    out = np.zeros((ch, cw, 3), np.float64)
    sq = np.zeros((ch, cw), np.float64)
    stats = np.zeros(2, np.uint64)
    L.orc_pt_render_instanced(C.byref(scene), C.byref(inst), C.byref(env), C.byref(cam), C.byref(st), ptr(out),
                              ptr(sq), ptr(stats), nthreads)
    return out, sq, (int(stats[0]), int(stats[1]))


def cauchy_ior(ior, dispersion, lam):
    L = orc()
    L.orc_cauchy_ior.restype = C.c_double
    L.orc_cauchy_ior.argtypes = [C.c_double, C.c_double, C.c_double]
    return L.orc_cauchy_ior(ior, dispersion, lam)


def lambda_rgb(lam):
    L = orc()
    L.orc_lambda_rgb.argtypes = [C.c_double, C.c_void_p]
    out = np.zeros(3)
    L.orc_lambda_rgb(lam, ptr(out))
    return out


def phase_hg(cos_theta, g):
    """FP64 Henyey-Greenstein phase function value (phase_function.slang:10-14)"""
    L = orc()
    L.orc_phase_hg.argtypes = [C.c_double, C.c_double]
    L.orc_phase_hg.restype = C.c_double
    return L.orc_phase_hg(float(cos_theta), float(g))


def phase_hg_sample(x, y, g):
    """one FP64 phase-function sample around +z: (direction, pdf)"""
    L = orc()
    L.orc_phase_hg_sample.argtypes = [C.c_double, C.c_double, C.c_double, C.c_void_p, C.c_void_p]
    d = np.zeros(3)
    pdf = C.c_double()
    L.orc_phase_hg_sample(float(x), float(y), float(g), ptr(d), C.byref(pdf))
    return d, pdf.value


def bsdf_sample(material, n, v, eta, u):
    """one FP64 sample_disney: (direction, pdf, f, transmission)"""
    L = orc()
    L.orc_bsdf_sample.argtypes = [C.c_void_p] * 3 + [C.c_double] + [C.c_void_p] * 5
    m = np.ascontiguousarray(material)
    d = np.zeros(3)
    f = np.zeros(3)
    pdf = C.c_double()
    tr = C.c_int()
    L.orc_bsdf_sample(ptr(m), ptr(np.asarray(n, np.float64)), ptr(np.asarray(v, np.float64)), eta,
                      ptr(np.asarray(u, np.float64)), ptr(d), C.byref(pdf), ptr(f), C.byref(tr))
    return d, pdf.value, f, bool(tr.value)


def bsdf_eval(material, l, n, v, eta):
    """one FP64 eval_disney: (f, mixture pdf)"""
    L = orc()
    L.orc_bsdf_eval.argtypes = [C.c_void_p] * 4 + [C.c_double, C.c_void_p]
    L.orc_bsdf_eval.restype = C.c_double
    m = np.ascontiguousarray(material)
    f = np.zeros(3)
    pdf = L.orc_bsdf_eval(ptr(m), ptr(np.asarray(l, np.float64)), ptr(np.asarray(n, np.float64)),
                          ptr(np.asarray(v, np.float64)), eta, ptr(f))
    return f, pdf
