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
          extra=None, images=None):
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
            if len(prim) > 5 and prim[5]:
                # more attributes: name -> float array, or (array, componentType) for normalised integers
                for name, arr in prim[5].items():
                    ctype = 5126
                    if isinstance(arr, tuple):
                        arr, ctype = arr
                    a_ = np.asarray(arr)
                    kind = {1: "SCALAR", 2: "VEC2", 3: "VEC3", 4: "VEC4"}[a_.shape[1]]
                    p["attributes"][name] = add(a_, 34962, kind, ctype)
                    if ctype != 5126:
                        accessors[-1]["normalized"] = True
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
    if images:
        # images: PNG (or any) file images as bytes, embedded as buffer views (glb / external) or data URIs
        doc["images"], doc["textures"], doc["samplers"] = [], [], []
        for k, (data, ws, wt) in enumerate(images):
            if mode == "embedded":
                doc["images"].append({"uri": "data:image/png;base64," + base64.b64encode(data).decode()})
            else:
                off = len(blob)
                blob = _pad4(blob + data)
                views.append({"buffer": 0, "byteOffset": off, "byteLength": len(data)})
                doc["images"].append({"bufferView": len(views) - 1, "mimeType": "image/png"})
            doc["samplers"].append({"wrapS": ws, "wrapT": wt})
            doc["textures"].append({"source": k, "sampler": k})
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


def png(rgba, color_type=6, depth=8, filters=(0, 1, 2, 3, 4), palette=None, trns=None, level=9, strategy=None):
    """A PNG file of image data (uint8 / uint16 [H, W, C] or palette indices [H, W]) with the given
    colour type and bit depth, the rows filtered with the filter types in turn, zlib level / strategy
    as asked (level 0: stored blocks; strategy zlib.Z_FIXED: fixed Huffman codes)."""
    import zlib
    img = np.asarray(rgba)
    h, w = img.shape[:2]
    ch = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[color_type]
    if depth < 8:
        per = 8 // depth
        rows = []
        for y in range(h):
            bits = img[y].reshape(-1).astype(np.uint32)
            packed = bytearray((w + per - 1) // per)
            for x in range(w):
                packed[x // per] |= int(bits[x]) << (8 - depth * (x % per + 1))
            rows.append(bytes(packed))
        bpp = 1
    else:
        dt = ">u2" if depth == 16 else "u1"
        rows = [np.ascontiguousarray(img[y].reshape(w * ch).astype(dt)).tobytes() for y in range(h)]
        bpp = ch * depth // 8
    raw, prev = bytearray(), bytes(len(rows[0]))
    for y, row in enumerate(rows):
        f = filters[y % len(filters)]
        out = bytearray(len(row))
        for x in range(len(row)):
            a = row[x - bpp] if x >= bpp else 0
            b = prev[x]
            c = prev[x - bpp] if x >= bpp else 0
            if f == 0:
                pred = 0
            elif f == 1:
                pred = a
            elif f == 2:
                pred = b
            elif f == 3:
                pred = (a + b) >> 1
            else:
                p_ = a + b - c
                pa, pb, pc = abs(p_ - a), abs(p_ - b), abs(p_ - c)
                pred = a if pa <= pb and pa <= pc else (b if pb <= pc else c)
            out[x] = (row[x] - pred) & 0xFF
        raw += bytes([f]) + out
        prev = row
    if strategy is None:
        comp = zlib.compress(bytes(raw), level)
    else:
        co = zlib.compressobj(level, zlib.DEFLATED, 15, 9, strategy)
        comp = co.compress(bytes(raw)) + co.flush()

    def chunk(t, d):
        return struct.pack(">I", len(d)) + t + d + struct.pack(">I", zlib.crc32(t + d) & 0xFFFFFFFF)

    outb = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, color_type, 0, 0, 0))
    if palette is not None:
        outb += chunk(b"PLTE", bytes(np.asarray(palette, np.uint8).reshape(-1)))
    if trns is not None:
        outb += chunk(b"tRNS", bytes(np.asarray(trns, np.uint8)))
    outb += chunk(b"IDAT", comp) + chunk(b"IEND", b"")
    return outb
