"""RayBuilder's wire records read as they are (vkg_materials_from_wire / vkg_instances_from_wire):
byte images of RayBuilder::material_struct_t (208 B) and RayBuilder::entry_t (192 B) into the
library's material and instance records."""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import check, lib, vkg_wire_entry_info
from .geometry import MATERIAL_DTYPE
from .raytracing import INSTANCE_DTYPE

WIRE_MATERIAL_BYTES = 208
WIRE_ENTRY_BYTES = 192
ENTRY_INFO_DTYPE = np.dtype([("buffer_index", "<u4"), ("base_index", "<u4"), ("vertex_offset", "<i4"),
                             ("aabb_min", "<f4", 3), ("aabb_max", "<f4", 3), ("has_uv_transform", "<u4"),
                             ("uv_transform", "<f4", 6)])
assert ENTRY_INFO_DTYPE.itemsize == C.sizeof(vkg_wire_entry_info)


def _bytes(records, size):
    b = np.ascontiguousarray(np.frombuffer(records, np.uint8) if isinstance(records, (bytes, bytearray))
                             else np.asarray(records).view(np.uint8).reshape(-1))
    if b.size % size:
        raise ValueError(f"wire records: {b.size} bytes is not a multiple of {size}")
    return b, b.size // size


def materials_from_wire(records) -> tuple[np.ndarray, int]:
    """material_struct_t records (bytes or any array of them) -> (MATERIAL_DTYPE array, number of
    records that use textures or a blend mode, which are dropped)"""
    b, n = _bytes(records, WIRE_MATERIAL_BYTES)
    out = np.zeros(n, MATERIAL_DTYPE)
    dropped = C.c_uint32()
    check(lib().vkg_materials_from_wire(b.ctypes.data_as(C.c_void_p) if n else None, n,
                                        out.ctypes.data_as(C.c_void_p) if n else None, C.byref(dropped)))
    return out, dropped.value


def instances_from_wire(records) -> tuple[np.ndarray, np.ndarray]:
    """entry_t records -> (INSTANCE_DTYPE array: object -> world T R S, mesh = buffer_index, material;
    ENTRY_INFO_DTYPE array: buffer / base index, vertex offset, object-space box)"""
    b, n = _bytes(records, WIRE_ENTRY_BYTES)
    out = np.zeros(n, INSTANCE_DTYPE)
    info = np.zeros(n, ENTRY_INFO_DTYPE)
    check(lib().vkg_instances_from_wire(b.ctypes.data_as(C.c_void_p) if n else None, n,
                                        out.ctypes.data_as(C.c_void_p) if n else None,
                                        info.ctypes.data_as(C.c_void_p) if n else None))
    return out, info
