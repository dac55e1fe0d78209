"""glTF 2.0 scenes for the path tracer: the C loader (vkg_gltf_*) into numpy arrays, and an
InstancedScene with the asset's lights."""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import check, lib, vkg_gltf_counts
from .geometry import MATERIAL_DTYPE
from .raytracing import INSTANCE_DTYPE


def load_gltf(path: str) -> dict:
    """Reads a .gltf / .glb file. Returns dict(meshes=[(xyz [V,3] f32, indices [T,3] u32, twosided)],
    normals / texcoords / tangents (per mesh: [V,3] / [V,2] / [V,3] f32 or None), instances
    (INSTANCE_DTYPE: object -> world, mesh index in "blas", material), materials (MATERIAL_DTYPE, texture
    slots indexing `textures`), textures ((uint8 [H, W, 4], wrap_s, wrap_t) per glTF texture), lights
    (pathtracer.LIGHT_DTYPE), skipped_primitives, skipped_textures)."""
    from .pathtracer import LIGHT_DTYPE
    L = lib()
    h = C.c_void_p()
    err = C.create_string_buffer(512)
    st = L.vkg_gltf_load(str(path).encode(), C.byref(h), err, len(err))
    if st != 0:
        raise ValueError(f"vkg_gltf_load({path}): {err.value.decode(errors='replace')}")
    try:
        n = vkg_gltf_counts()
        check(L.vkg_gltf_counts_get(h, C.byref(n)))
        meshes, normals, texcoords, tangents = [], [], [], []
        for i in range(n.num_meshes):
            xp, ip = C.POINTER(C.c_float)(), C.POINTER(C.c_uint32)()
            nv, nt = C.c_uint32(), C.c_uint32()
            check(L.vkg_gltf_mesh(h, i, C.byref(xp), C.byref(nv), C.byref(ip), C.byref(nt)))
            xyz = np.ctypeslib.as_array(xp, (nv.value, 3)).copy() if nv.value else np.zeros((0, 3), np.float32)
            idx = np.ctypeslib.as_array(ip, (nt.value, 3)).copy() if nt.value else np.zeros((0, 3), np.uint32)
            meshes.append((xyz, idx, 0))
            npp = C.POINTER(C.c_float)()
            check(L.vkg_gltf_mesh_normals(h, i, C.byref(npp)))
            normals.append(np.ctypeslib.as_array(npp, (nv.value, 3)).copy() if npp and nv.value else None)
            upp, tpp = C.POINTER(C.c_float)(), C.POINTER(C.c_float)()
            check(L.vkg_gltf_mesh_texcoords(h, i, C.byref(upp)))
            check(L.vkg_gltf_mesh_tangents(h, i, C.byref(tpp)))
            texcoords.append(np.ctypeslib.as_array(upp, (nv.value, 2)).copy() if upp and nv.value else None)
            tangents.append(np.ctypeslib.as_array(tpp, (nv.value, 3)).copy() if tpp and nv.value else None)
        inst = np.zeros(n.num_instances, INSTANCE_DTYPE)
        check(L.vkg_gltf_instances(h, inst.ctypes.data_as(C.c_void_p) if n.num_instances else None))
        mats = np.zeros(n.num_materials, MATERIAL_DTYPE)
        check(L.vkg_gltf_materials(h, mats.ctypes.data_as(C.c_void_p)))
        lights = np.zeros(n.num_lights, LIGHT_DTYPE)
        check(L.vkg_gltf_lights(h, lights.ctypes.data_as(C.c_void_p) if n.num_lights else None))
        from ._lib import vkg_texture_desc
        descs = (vkg_texture_desc * max(1, n.num_textures))()
        check(L.vkg_gltf_textures(h, descs if n.num_textures else None))
        textures = []
        for k in range(n.num_textures):
            d = descs[k]
            buf = (C.c_uint8 * (d.width * d.height * 4)).from_address(d.h_rgba8)
            textures.append((np.frombuffer(buf, np.uint8).reshape(d.height, d.width, 4).copy(), d.wrap_s, d.wrap_t))
        return {"meshes": meshes, "normals": normals, "texcoords": texcoords, "tangents": tangents,
                "textures": textures, "skipped_textures": n.skipped_textures,
                "instances": inst, "materials": mats, "lights": lights,
                "skipped_primitives": n.skipped_primitives}
    finally:
        L.vkg_gltf_destroy(h)


def scene_from_gltf(ctx, path: str, env_rgb):
    """An InstancedScene of a glTF asset with its KHR_lights_punctual lights, its meshes' vertex
    normals, texture coordinates and tangents, and its textures set."""
    from .pathtracer import InstancedScene
    a = load_gltf(path)
    scene = InstancedScene(ctx, a["meshes"], a["instances"], a["materials"], env_rgb)
    for m, nrm in enumerate(a["normals"]):
        if nrm is not None:
            scene.set_normals(nrm, mesh=m)
    for m, (uv, tg) in enumerate(zip(a["texcoords"], a["tangents"])):
        if uv is not None:
            scene.set_texcoords(uv, mesh=m)
        if tg is not None:
            scene.set_tangents(tg, mesh=m)
    if a["textures"]:
        scene.set_textures(a["textures"])
    if len(a["lights"]):
        scene.set_lights(a["lights"])
    return scene
