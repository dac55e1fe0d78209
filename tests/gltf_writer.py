"""Writes small glTF 2.0 assets for the loader tests (no GPU, no third-party code): meshes of float
positions + uint32 / uint16 indices, a node hierarchy with matrix or TRS transforms, materials with
the KHR extensions the loader reads, KHR_lights_punctual lights; as .gltf with embedded base64 or an
external .bin, or as .glb."""
import base64
import json
import struct

import numpy as np


def _pad4(b: bytes, fill=b"\x00") -> bytes:
    return b + fill * ((4 - len(b) % 4) % 4)


def write(path, meshes, nodes, scene_roots, materials=None, lights=None, mode="embedded", index_type=np.uint32,
          extra=None):
    """meshes: [[(xyz [V,3], indices [T,3] or None, material or None, prim_mode or None[, normals [V,3]]),
    ...], ...];
    nodes: [dict(mesh=, children=, matrix=[16] | translation=, rotation=(x,y,z,w), scale=, light=)]"""
    blob = b""
    views, accessors = [], []

    def add(arr: np.ndarray, target, comps_type, ctype):
        nonlocal blob
        data = np.ascontiguousarray(arr).tobytes()
        off = len(blob)
        blob = _pad4(blob + data)
        views.append({"buffer": 0, "byteOffset": off, "byteLength": len(data), "target": target})
        a = {"bufferView": len(views) - 1, "componentType": ctype, "count": int(arr.shape[0]), "type": comps_type}
        if comps_type == "VEC3":
            a["min"] = [float(v) for v in arr.min(axis=0)]
            a["max"] = [float(v) for v in arr.max(axis=0)]
        accessors.append(a)
        return len(accessors) - 1

    gm = []
    for prims in meshes:
        ps = []
        for prim in prims:
            xyz, idx, mat, pmode = prim[:4]
            p = {"attributes": {"POSITION": add(np.asarray(xyz, np.float32), 34962, "VEC3", 5126)}}
            if len(prim) > 4 and prim[4] is not None:
                nrm = np.asarray(prim[4], np.float32)
                p["attributes"]["NORMAL"] = add(nrm, 34962, "VEC3" if nrm.shape[1] == 3 else "VEC2", 5126)
            if idx is not None:
                ct = {np.uint32: 5125, np.uint16: 5123, np.uint8: 5121}[index_type]
                p["indices"] = add(np.asarray(idx, index_type).reshape(-1), 34963, "SCALAR", ct)
            if mat is not None:
                p["material"] = mat
            if pmode is not None:
                p["mode"] = pmode
            ps.append(p)
        gm.append({"primitives": ps})
    doc = {"asset": {"version": "2.0", "generator": "tests/gltf_writer.py"}, "scene": 0,
           "scenes": [{"nodes": list(scene_roots)}], "nodes": [], "meshes": gm, "accessors": accessors,
           "bufferViews": views}
    for n in nodes:
        d = {k: v for k, v in n.items() if k != "light"}
        if "light" in n:
            d["extensions"] = {"KHR_lights_punctual": {"light": n["light"]}}
        doc["nodes"].append(d)
    if materials:
        doc["materials"] = materials
    used = set()
    for m in materials or []:
        used.update((m.get("extensions") or {}).keys())
    if lights:
        doc.setdefault("extensions", {})["KHR_lights_punctual"] = {"lights": lights}
        used.add("KHR_lights_punctual")
    if used:
        doc["extensionsUsed"] = sorted(used)
    if extra:
        doc.update(extra)
    if mode == "embedded":
        doc["buffers"] = [{"byteLength": len(blob),
                           "uri": "data:application/octet-stream;base64," + base64.b64encode(blob).decode()}]
        open(path, "w").write(json.dumps(doc))
    elif mode == "external":
        binname = str(path).rsplit("/", 1)[-1].rsplit(".", 1)[0] + ".bin"
        open(str(path).rsplit("/", 1)[0] + "/" + binname, "wb").write(blob)
        doc["buffers"] = [{"byteLength": len(blob), "uri": binname}]
        open(path, "w").write(json.dumps(doc))
    else:  # glb
        doc["buffers"] = [{"byteLength": len(blob)}]
        js = _pad4(json.dumps(doc).encode(), b" ")
        bn = _pad4(blob)
        total = 12 + 8 + len(js) + 8 + len(bn)
        with open(path, "wb") as f:
            f.write(struct.pack("<4sII", b"glTF", 2, total))
            f.write(struct.pack("<II", len(js), 0x4E4F534A) + js)
            f.write(struct.pack("<II", len(bn), 0x004E4942) + bn)
