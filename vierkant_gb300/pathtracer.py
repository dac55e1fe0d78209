"""Path tracer API mirroring vierkant's PBRPathTracer (include/vierkant/PBRPathTracer.hpp:37-386).

    ctx = Context(0)
    scene = Scene(ctx, xyz, indices, tri_material, materials, env_rgb)   # BVH + env sampling tables
    pt = PBRPathTracer(ctx, seed=0x5EED, settings=PBRPathTracer.default_settings())
    pt.settings.num_samples = 64
    image = pt.render_scene(scene, camera)      # running mean over batches, [H, W, 3] fp32 on the GPU
    pt.current_batch(); pt.reset_accumulator(); pt.statistics()

All work runs in libvkg's kernels; torch only provides device memory and the stream.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np
import torch

from ._lib import (check, lib, vkg_bvh_info, vkg_camera, vkg_light, vkg_light_source, vkg_medium_params,
                   vkg_pixel_data, vkg_post_fx_settings, vkg_scene_desc, vkg_settings, vkg_tracer_create_info,
                   vkg_tracer_stats)
from .raytracing import Context

# the benchmark sky's sun: 30 deg elevation, 20 deg azimuth (measured from +z toward +x), 5e4 peak, width 3.8e-5
SUN_ELEVATION_DEG = 30.0
SUN_AZIMUTH_DEG = 20.0


def sun_direction(elevation_deg=SUN_ELEVATION_DEG, azimuth_deg=SUN_AZIMUTH_DEG):
    e, a = math.radians(elevation_deg), math.radians(azimuth_deg)
    return np.array([math.sin(a) * math.cos(e), math.sin(e), math.cos(a) * math.cos(e)], np.float32)


def procedural_sky(ctx: Context, width=2048, height=1024, sun_dir=None, sun_peak=5e4, sun_width=3.8e-5):
    """environment_white gradient + sun lobe, as a [height, width, 3] fp32 CUDA tensor."""
    if sun_dir is None:
        sun_dir = sun_direction()
    out = torch.empty((height, width, 3), dtype=torch.float32, device=f"cuda:{ctx.device}")
    sd = np.ascontiguousarray(sun_dir, np.float32)
    check(lib().vkg_env_procedural_sky(ctx.handle, width, height, sd.ctypes.data_as(C.c_void_p), C.c_float(sun_peak),
                                       C.c_float(sun_width), C.c_void_p(out.data_ptr()), C.c_void_p(ctx.stream())),
          ctx.handle, "vkg_env_procedural_sky")
    return out


# analytic lights: the reference's LightType values and the 80-byte light record
LIGHT_OMNI, LIGHT_SPOT, LIGHT_DIRECTIONAL, LIGHT_RECT, LIGHT_SPHERE, LIGHT_TUBE, LIGHT_DISK = 0, 1, 2, 4, 5, 6, 7
LIGHT_DTYPE = np.dtype([("position", "<f4", 3), ("type", "<u4"), ("color", "<f4", 3), ("intensity", "<f4"),
                        ("direction", "<f4", 3), ("range", "<f4"), ("spot_angle_scale", "<f4"),
                        ("spot_angle_offset", "<f4"), ("angular_size", "<f4"), ("size_y", "<f4"),
                        ("tangent", "<f4", 3), ("size_x", "<f4")])
assert LIGHT_DTYPE.itemsize == C.sizeof(vkg_light)


def convert_light(type, color=(1.0, 1.0, 1.0), intensity=1.0, range=math.inf, inner_cone_angle=0.0,
                  outer_cone_angle=math.pi / 4, size=(1.0, 1.0), rotation=None, translation=(0.0, 0.0, 0.0)):
    """A light record from a light-source asset placed by an object transform (row-major 3x3 rotation,
    translation), as the reference's convert_light does; returns one LIGHT_DTYPE element."""
    src = vkg_light_source(type, (C.c_float * 3)(*color), intensity, range, inner_cone_angle, outer_cone_angle,
                           (C.c_float * 2)(*size))
    rot = np.ascontiguousarray(np.eye(3) if rotation is None else rotation, np.float32).reshape(9)
    tr = np.ascontiguousarray(translation, np.float32)
    out = vkg_light()
    check(lib().vkg_light_convert(C.byref(src), rot.ctypes.data_as(C.c_void_p), tr.ctypes.data_as(C.c_void_p),
                                  C.byref(out)))
    return np.frombuffer(bytes(out), LIGHT_DTYPE, count=1)[0]


def cornell_lights(intensity_scale: float = 1.0) -> np.ndarray:
    """One light of every analytic type inside the Cornell box ([-1, 1]^3, open toward +z): a rect on
    the ceiling facing down, a sphere, a spot, a tube along x, a disk on the back wall and an omni."""
    L = np.zeros(6, LIGHT_DTYPE)
    rows = [
        dict(type=LIGHT_RECT, position=(0.0, 0.98, 0.0), direction=(0, -1, 0), tangent=(1, 0, 0), size_x=0.25,
             size_y=0.25, color=(1.0, 0.9, 0.8), intensity=8.0),
        dict(type=LIGHT_SPHERE, position=(-0.6, 0.6, -0.5), size_x=0.15, color=(0.9, 0.9, 1.0), intensity=6.0),
        dict(type=LIGHT_SPOT, position=(0.6, 0.9, 0.3), direction=(-0.2, -1, 0), color=(1.0, 1.0, 0.9),
             intensity=3.0),
        dict(type=LIGHT_TUBE, position=(0.3, 0.2, -0.8), direction=(1, 0, 0), size_x=0.06, size_y=0.3,
             color=(0.8, 1.0, 0.8), intensity=5.0),
        dict(type=LIGHT_DISK, position=(0.0, 0.5, -0.99), direction=(0, 0, 1), size_x=0.15, color=(1.0, 0.8, 0.8),
             intensity=6.0),
        dict(type=LIGHT_OMNI, position=(-0.7, -0.5, 0.5), color=(1.0, 1.0, 1.0), intensity=0.5),
    ]
    for i, r in enumerate(rows):
        L[i]["range"] = np.inf
        L[i]["spot_angle_scale"], L[i]["spot_angle_offset"] = 1.0, 0.0
        for k, v in r.items():
            L[i][k] = v
        d = np.asarray(L[i]["direction"], np.float64)
        if np.any(d):
            L[i]["direction"] = d / np.linalg.norm(d)
        L[i]["intensity"] *= intensity_scale
    # the spot cone: inner 0.3 rad, outer 0.6 rad (convert_light's scale / offset)
    sc = 1.0 / max(0.001, math.cos(0.3) - math.cos(0.6))
    L[2]["spot_angle_scale"], L[2]["spot_angle_offset"] = sc, -math.cos(0.6) * sc
    return L


# the per-pixel record (pixel_data_t layout): radiance, coverage, depth, octahedral normal, object id, RGBA8 albedo
PIXEL_DTYPE = np.dtype([("radiance", "<f4", 3), ("alpha", "<f4"), ("depth", "<f4"), ("normal", "<u4"),
                        ("object_id", "<u4"), ("albedo", "<u4")])
assert PIXEL_DTYPE.itemsize == C.sizeof(vkg_pixel_data)


def denoise(ctx: Context, pixels: torch.Tensor, width: int, height: int, with_depth: bool = False):
    """The reference's a-trous denoise pass over pixel records (a uint8 CUDA tensor of width x height
    x 32 bytes, e.g. PBRPathTracer.pixel_data()); returns the rgba image (and the depth)."""
    out = torch.empty((height, width, 4), dtype=torch.float32, device=pixels.device)
    dep = torch.empty((height, width), dtype=torch.float32, device=pixels.device) if with_depth else None
    check(lib().vkg_denoise(ctx.handle, C.c_void_p(pixels.data_ptr()), width, height, C.c_void_p(out.data_ptr()),
                            C.c_void_p(dep.data_ptr()) if dep is not None else None, C.c_void_p(ctx.stream())),
          ctx.handle, "vkg_denoise")
    return (out, dep) if with_depth else out


def post_fx_settings(**kw) -> vkg_post_fx_settings:
    """the reference's post-FX defaults (tonemap and bloom on, exposure 2, gamma 1, brightness threshold
    (0.95, 1.1), 3 blur iterations), with keyword overrides"""
    s = vkg_post_fx_settings()
    check(lib().vkg_post_fx_default(C.byref(s)))
    for k, v in kw.items():
        if k == "brightness_thresh":
            s.brightness_thresh[0], s.brightness_thresh[1] = v
        else:
            setattr(s, k, v)
    return s


def post_fx(ctx: Context, hdr_rgba: torch.Tensor, settings: vkg_post_fx_settings | None = None) -> torch.Tensor:
    """Bloom + tonemap composition of an HDR [h, w, 4] float32 CUDA image."""
    h, w = hdr_rgba.shape[:2]
    src = hdr_rgba.contiguous()
    out = torch.empty_like(src)
    s = settings if settings is not None else post_fx_settings()
    check(lib().vkg_post_fx(ctx.handle, C.c_void_p(src.data_ptr()), w, h, C.byref(s), C.c_void_p(out.data_ptr()),
                            C.c_void_p(ctx.stream())), ctx.handle, "vkg_post_fx")
    return out


CAMERA_MEDIUM_DETECT, CAMERA_MEDIUM_GIVEN = 0, 1


def medium_params(**kw) -> vkg_medium_params:
    """A vkg_medium_params with the reference's defaults (medium_params_t) and the given fields."""
    p = vkg_medium_params()
    check(lib().vkg_medium_params_default(C.byref(p)))
    for k, v in kw.items():
        f = getattr(p, k)
        if isinstance(f, C.Array):
            for i, x in enumerate(v):
                f[i] = x
        else:
            setattr(p, k, v)
    return p


class _Lights:
    def camera_medium(self, eye) -> int | None:
        """The material of the medium a render from `eye` starts in (camera_medium_mode DETECT), or None."""
        e = (C.c_float * 3)(*[float(x) for x in eye])
        m = C.c_uint32()
        check(lib().vkg_scene_camera_medium(self.handle, e, C.byref(m)))
        return None if m.value == 0xFFFFFFFF else m.value

    def set_lights(self, lights):
        """Analytic lights of the scene (LIGHT_DTYPE records; empty removes them)."""
        arr = np.ascontiguousarray(np.asarray(lights, LIGHT_DTYPE).reshape(-1))
        check(lib().vkg_scene_set_lights(self.ctx.handle, self.handle,
                                         arr.ctypes.data_as(C.c_void_p) if len(arr) else None, len(arr)),
              self.ctx.handle, "vkg_scene_set_lights")


    def set_normals(self, normals, mesh: int = 0):
        """Vertex normals for smooth shading (the interpolated vertex normal, turned to the side the
        ray hit, becomes the shading normal): float [V, 3] (normalised on upload), PACKED_VERTEX_DTYPE
        records (their octahedral normal words), or None for face normals. mesh: the mesh of an
        instanced scene."""
        from ._lib import NORMALS_FLOAT3, NORMALS_OCT_SNORM16
        dev = f"cuda:{self.ctx.device}"
        if normals is None:
            src, stride, fmt = None, 0, NORMALS_FLOAT3
        elif isinstance(normals, np.ndarray) and normals.dtype == PACKED_VERTEX_DTYPE:
            buf = torch.from_numpy(np.ascontiguousarray(normals).view(np.uint8).copy()).to(dev)
            src, stride, fmt = buf.data_ptr() + 12, PACKED_VERTEX_DTYPE.itemsize, NORMALS_OCT_SNORM16
        else:
            a = normals if isinstance(normals, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(normals, np.float32))
            buf = a.to(dev, torch.float32).contiguous()
            src, stride, fmt = buf.data_ptr(), 12, NORMALS_FLOAT3
        check(lib().vkg_scene_set_normals(self.ctx.handle, self.handle, mesh, C.c_void_p(src), stride, fmt,
                                          C.c_void_p(self.ctx.stream())), self.ctx.handle, "vkg_scene_set_normals")

    def set_tangents(self, tangents, mesh: int = 0):
        """Vertex tangents for normal maps: float [V, 3] (normalised on upload), PACKED_VERTEX_DTYPE
        records (their octahedral tangent words), or None."""
        from ._lib import NORMALS_FLOAT3, NORMALS_OCT_SNORM16
        src, stride, fmt, _keep = self._attr(tangents, 3, "tangent", 16, NORMALS_FLOAT3, NORMALS_OCT_SNORM16)
        check(lib().vkg_scene_set_tangents(self.ctx.handle, self.handle, mesh, C.c_void_p(src), stride, fmt,
                                           C.c_void_p(self.ctx.stream())), self.ctx.handle, "vkg_scene_set_tangents")

    def set_texcoords(self, uv, mesh: int = 0):
        """Texture coordinates: float [V, 2], PACKED_VERTEX_DTYPE records (their fp16 texcoords), or None."""
        from ._lib import TEXCOORD_FLOAT2, TEXCOORD_HALF2
        src, stride, fmt, _keep = self._attr(uv, 2, "texcoord", 20, TEXCOORD_FLOAT2, TEXCOORD_HALF2)
        check(lib().vkg_scene_set_texcoords(self.ctx.handle, self.handle, mesh, C.c_void_p(src), stride, fmt,
                                            C.c_void_p(self.ctx.stream())), self.ctx.handle, "vkg_scene_set_texcoords")

    def _attr(self, a, comps, packed_field, packed_offset, fmt_float, fmt_packed):
        dev = f"cuda:{self.ctx.device}"
        if a is None:
            return None, 0, fmt_float, None
        if isinstance(a, np.ndarray) and a.dtype == PACKED_VERTEX_DTYPE:
            buf = torch.from_numpy(np.ascontiguousarray(a).view(np.uint8).copy()).to(dev)
            return buf.data_ptr() + packed_offset, PACKED_VERTEX_DTYPE.itemsize, fmt_packed, buf
        t = a if isinstance(a, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(a, np.float32))
        buf = t.to(dev, torch.float32).contiguous()
        assert buf.numel() % comps == 0
        return buf.data_ptr(), 4 * comps, fmt_float, buf

    def set_textures(self, textures):
        """The scene's textures: a list of uint8 [H, W, 4] RGBA arrays (UNORM) or (array, wrap_s, wrap_t)
        tuples (pathtracer.WRAP_*; REPEAT by default); an empty list removes them."""
        from ._lib import vkg_texture_desc
        descs = (vkg_texture_desc * max(1, len(textures)))()
        keep = []
        for k, t in enumerate(textures):
            img, ws, wt = (t if isinstance(t, tuple) else (t, 0, 0))
            img = np.ascontiguousarray(img, np.uint8)
            assert img.ndim == 3 and img.shape[2] == 4, "RGBA8 [H, W, 4]"
            keep.append(img)
            descs[k] = vkg_texture_desc(img.ctypes.data, img.shape[1], img.shape[0], ws, wt)
        check(lib().vkg_scene_set_textures(self.ctx.handle, self.handle, descs, len(textures),
                                           C.c_void_p(self.ctx.stream())), self.ctx.handle, "vkg_scene_set_textures")

class Scene(_Lights):
    def __init__(self, ctx: Context, xyz, indices, tri_material, materials, env_rgb, leaf_max=2):
        dev = f"cuda:{ctx.device}"

        def t(a, dt):
            if isinstance(a, np.ndarray):
                a = torch.from_numpy(np.ascontiguousarray(a))
            return a.to(dev).contiguous().view(dt) if a.dtype.itemsize == dt.itemsize else a.to(dev, dt).contiguous()

        self.ctx = ctx
        xyz = t(xyz, torch.float32)
        idx = torch.from_numpy(np.ascontiguousarray(indices, np.uint32).view(np.int32)).to(dev) \
            if isinstance(indices, np.ndarray) else indices.to(dev).contiguous()
        tm = torch.from_numpy(np.ascontiguousarray(tri_material, np.uint32).view(np.int32)).to(dev) \
            if isinstance(tri_material, np.ndarray) else tri_material.to(dev).contiguous()
        mats = torch.from_numpy(np.frombuffer(np.ascontiguousarray(materials).tobytes(), np.uint8).copy()).to(dev)
        env = env_rgb.to(dev, torch.float32).contiguous()
        d = vkg_scene_desc(xyz.data_ptr(), xyz.numel() // 3, idx.data_ptr(), idx.numel() // 3, tm.data_ptr(),
                           mats.data_ptr(), len(materials), env.data_ptr(), env.shape[1], env.shape[0], leaf_max)
        h = C.c_void_p()
        check(lib().vkg_scene_create(ctx.handle, C.byref(d), C.byref(h), C.c_void_p(ctx.stream())), ctx.handle,
              "vkg_scene_create")
        self.handle = h
        self.num_tris = idx.numel() // 3
        ctx.adopt(self)

    def bounds(self):
        """(min xyz, max xyz) of the scene's geometry, as the BVH build saw them"""
        b = C.c_void_p()
        check(lib().vkg_scene_bvh(self.handle, C.byref(b)))
        inf = vkg_bvh_info()
        check(lib().vkg_bvh_info_get(b, C.byref(inf)))
        return tuple(inf.scene_min), tuple(inf.scene_max)

    def env_tables(self):
        w, a = C.c_void_p(), C.c_void_p()
        W, H = C.c_uint32(), C.c_uint32()
        check(lib().vkg_scene_env_tables(self.handle, C.byref(w), C.byref(a), C.byref(W), C.byref(H)))
        return w.value, a.value, W.value, H.value

    def close(self):
        if getattr(self, "handle", None) and getattr(self.ctx, "handle", None):
            lib().vkg_scene_destroy(self.ctx.handle, self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# the reference's packed_vertex_t (packed_vertex.slang:17-23): position, octahedral normal and tangent,
# fp16 texture coordinates; 24 bytes
PACKED_VERTEX_DTYPE = np.dtype([("position", "<f4", 3), ("normal", "<u4"), ("tangent", "<u4"),
                                ("texcoord", "<f2", 2)])


class InstancedScene(_Lights):
    """A two-level scene: meshes [(xyz, indices, twosided)] each with its own BVH (xyz: float [V, 3] or
    PACKED_VERTEX_DTYPE records), instances
    (raytracing.INSTANCE_DTYPE: object -> world transform, mesh, material) under a top-level BVH,
    materials (MATERIAL_DTYPE) and the environment map. Renders with PBRPathTracer like Scene."""

    def __init__(self, ctx: Context, meshes, instances, materials, env_rgb, leaf_max=2):
        from ._lib import vkg_instanced_scene_desc, vkg_mesh_desc
        from .raytracing import INSTANCE_DTYPE
        dev = f"cuda:{ctx.device}"
        self.ctx = ctx
        self._keep = []
        descs = (vkg_mesh_desc * max(1, len(meshes)))()
        for k, (xyz, idx, twosided) in enumerate(meshes):
            if xyz.dtype == PACKED_VERTEX_DTYPE:
                # the reference's packed_vertex_t records: positions read with a 24-byte stride
                x = torch.from_numpy(np.ascontiguousarray(xyz).view(np.uint8).copy()).to(dev)
                nv, stride = len(xyz), PACKED_VERTEX_DTYPE.itemsize
            else:
                x = torch.from_numpy(np.ascontiguousarray(xyz, np.float32)).to(dev)
                nv, stride = x.shape[0], 0
            i = torch.from_numpy(np.ascontiguousarray(idx, np.uint32).view(np.int32)).to(dev)
            self._keep += [x, i]
            descs[k] = vkg_mesh_desc(x.data_ptr(), nv, i.data_ptr(), i.shape[0], int(twosided), stride)
        inst = torch.from_numpy(np.ascontiguousarray(instances, INSTANCE_DTYPE).view(np.uint8).copy()).to(dev)
        mats = torch.from_numpy(np.frombuffer(np.ascontiguousarray(materials).tobytes(), np.uint8).copy()).to(dev)
        env = env_rgb.to(dev, torch.float32).contiguous()
        self._keep += [inst, mats, env]
        d = vkg_instanced_scene_desc(descs, len(meshes), inst.data_ptr(), len(instances), mats.data_ptr(),
                                     len(materials), env.data_ptr(), env.shape[1], env.shape[0], leaf_max)
        h = C.c_void_p()
        check(lib().vkg_scene_create_instanced(ctx.handle, C.byref(d), C.byref(h), C.c_void_p(ctx.stream())),
              ctx.handle, "vkg_scene_create_instanced")
        self.handle = h
        self._keep = []  # the scene copied everything it needs
        self.num_instances = len(instances)
        ctx.adopt(self)

    def bounds(self):
        from ._lib import vkg_tlas_info
        t = C.c_void_p()
        check(lib().vkg_scene_tlas(self.handle, C.byref(t)))
        inf = vkg_tlas_info()
        check(lib().vkg_tlas_info_get(t, C.byref(inf)))
        return tuple(inf.scene_min), tuple(inf.scene_max)

    def close(self):
        if getattr(self, "handle", None) and getattr(self.ctx, "handle", None):
            lib().vkg_scene_destroy(self.ctx.handle, self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class PBRPathTracer:
    """PBRPathTracer::create / settings / render_scene / reset_accumulator / current_batch / statistics."""

    @staticmethod
    def default_settings() -> vkg_settings:
        s = vkg_settings()
        check(lib().vkg_settings_default(C.byref(s)))
        return s

    def __init__(self, ctx: Context, seed: int = 0, settings: vkg_settings | None = None):
        self.ctx = ctx
        self.settings = settings if settings is not None else self.default_settings()
        info = vkg_tracer_create_info(seed, self.settings)
        h = C.c_void_p()
        check(lib().vkg_tracer_create(ctx.handle, C.byref(info), C.byref(h)), ctx.handle, "vkg_tracer_create")
        self.handle = h
        self.cache = None
        ctx.adopt(self)

    def attach_cache(self, cache):
        """render through a NeuralRadianceCache (None: plain estimator again); see vkg_tracer_attach_cache"""
        check(lib().vkg_tracer_attach_cache(self.handle, cache.handle if cache is not None else None), self.ctx.handle,
              "vkg_tracer_attach_cache")
        self.cache = cache

    def _crop(self):
        s = self.settings
        if s.crop[2] and s.crop[3]:
            return s.crop[2], s.crop[3]
        return s.resolution[0], s.resolution[1]

    def render_scene(self, scene: Scene, camera: vkg_camera, out: torch.Tensor | None = None) -> torch.Tensor:
        check(lib().vkg_tracer_set_settings(self.handle, C.byref(self.settings)), self.ctx.handle, "settings")
        w, h = self._crop()
        if out is None:
            out = torch.empty((h, w, 3), dtype=torch.float32, device=f"cuda:{self.ctx.device}")
        check(lib().vkg_tracer_render(self.handle, scene.handle, C.byref(camera), C.c_void_p(out.data_ptr()),
                                      C.c_void_p(self.ctx.stream())), self.ctx.handle, "vkg_tracer_render")
        return out

    def pixel_data(self) -> torch.Tensor:
        """The pixel records of the traced window after the last render (uint8 [h, w, 32]; view the
        host copy with PIXEL_DTYPE)."""
        w, h = self._crop()
        out = torch.empty((h, w, 32), dtype=torch.uint8, device=f"cuda:{self.ctx.device}")
        check(lib().vkg_tracer_pixel_data(self.handle, C.c_void_p(out.data_ptr()), C.c_void_p(self.ctx.stream())),
              self.ctx.handle, "vkg_tracer_pixel_data")
        return out

    def reset_accumulator(self):
        check(lib().vkg_tracer_reset_accumulator(self.handle))

    def current_batch(self) -> int:
        b = C.c_uint32()
        check(lib().vkg_tracer_current_batch(self.handle, C.byref(b)))
        return b.value

    def statistics(self) -> vkg_tracer_stats:
        st = vkg_tracer_stats()
        check(lib().vkg_tracer_statistics(self.handle, C.byref(st)), self.ctx.handle, "vkg_tracer_statistics")
        return st

    def close(self):
        if getattr(self, "handle", None) and getattr(self.ctx, "handle", None):
            lib().vkg_tracer_destroy(self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
