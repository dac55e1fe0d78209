"""Scene helpers shared by the tests (no GPU needed)."""
import numpy as np

from vierkant_gb300.raytracing import INSTANCE_DTYPE

IDENTITY = np.array([1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0], np.float32)


def split_cornell(sc, tess=16):
    """one mesh per wall quad (2 triangles) and per sphere (12 tess^2 triangles), in triangle order"""
    xyz, idx, tm, mats = sc["xyz"], sc["indices"], sc["tri_material"], sc["materials"]
    groups = [(2 * q, 2 * q + 2) for q in range(5)]
    per = 12 * tess * tess
    groups += [(10 + k * per, 10 + (k + 1) * per) for k in range((len(idx) - 10) // per)]
    meshes, inst = [], np.zeros(len(groups), INSTANCE_DTYPE)
    for k, (a, b) in enumerate(groups):
        used, local = np.unique(idx[a:b].reshape(-1), return_inverse=True)
        m = int(tm[a])
        assert np.all(tm[a:b] == m)
        meshes.append((xyz[used], local.reshape(-1, 3).astype(np.uint32), int(mats[m]["twosided"])))
        inst[k]["transform"] = IDENTITY
        inst[k]["blas"] = k
        inst[k]["material"] = m
    return meshes, inst
