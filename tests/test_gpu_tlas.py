"""Two-level BVH (vkg_tlas_*): closest-hit and any-hit records of rays through instanced meshes equal
the CPU two-level oracle (oracle/tlas.c: every instance in input order, the same separately rounded
world -> object move, the instance's mesh traced by the oracle's traversal) bit for bit; instance
records hold the inverse transforms; edge cases return misses or errors."""
import numpy as np
import pytest
import torch

import oracle
from vierkant_gb300 import _lib, geometry
from vierkant_gb300.raytracing import BVH, INSTANCE_DTYPE, RAY_CULL_BACK_FACES, TLAS

pytestmark = pytest.mark.gpu


def random_rotation(rng):
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def make_instances(rng, n, nblas):
    inst = np.zeros(n, INSTANCE_DTYPE)
    for i in range(n):
        m = random_rotation(rng) * rng.uniform(0.5, 2.0)
        t = rng.uniform(-3, 3, size=3)
        inst[i]["transform"] = np.concatenate([m, t[:, None]], axis=1).astype(np.float32).reshape(12)
        inst[i]["blas"] = rng.integers(0, nblas)
        inst[i]["material"] = i
    return inst


def rays_between(rng, n):
    o = rng.uniform(-7, 7, size=(n, 3)).astype(np.float32)
    target = rng.uniform(-3, 3, size=(n, 3)).astype(np.float32)
    d = target - o
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r = np.zeros((n, 8), np.float32)
    r[:, 0:3], r[:, 3], r[:, 4:7], r[:, 7] = o, 1e-4, d.astype(np.float32), 1e4
    return r


@pytest.fixture(scope="module")
def meshes():
    ico = geometry.icosphere(1.0, 2)
    box = geometry.cornell_scene(0x5EED, 9, 1, 4)
    return [(ico["xyz"] if isinstance(ico, dict) else ico[0], ico["indices"] if isinstance(ico, dict) else ico[1]),
            (box["xyz"], box["indices"]),
            (np.zeros((3, 3), np.float32), np.zeros((0, 3), np.uint32))]


def build(ctx, meshes, inst):
    blas = [BVH(ctx, torch.from_numpy(x), torch.from_numpy(i.astype(np.int32))) for x, i in meshes]
    cpu = [oracle.CpuBVH(x, i, 4) for x, i in meshes]
    return blas, cpu, TLAS(ctx, blas, inst)


@pytest.mark.parametrize("n_inst,cull", [(1, False), (37, False), (37, True), (300, False)])
def test_two_level_hits_equal_oracle(ctx, meshes, n_inst, cull):
    rng = np.random.default_rng(n_inst + 10 * cull)
    inst = make_instances(rng, n_inst, len(meshes))
    blas, cpu, tl = build(ctx, meshes, inst)
    rec = tl.instance_records()
    # the device's inverses are the inverses of the given transforms
    for i in range(n_inst):
        o2w = np.vstack([inst[i]["transform"].reshape(3, 4).astype(np.float64), [0, 0, 0, 1]])
        w2o = np.vstack([rec[i, 0:12].reshape(3, 4).astype(np.float64), [0, 0, 0, 1]])
        assert np.allclose(w2o @ o2w, np.eye(4), atol=2e-5), i
        assert np.array_equal(rec[i, 12:24], inst[i]["transform"])
    rays = rays_between(rng, 20_000)
    flags = RAY_CULL_BACK_FACES if cull else 0
    g = tl.closest_hit(torch.from_numpy(rays).cuda(), flags=flags).cpu().numpy()
    ref = oracle.tlas_closest_hit(cpu, rec[:, 0:12], inst["blas"], rays, cull=cull)
    gv = g.view(np.uint32)
    assert np.array_equal(gv[:, 0], ref["prim"]) and np.array_equal(gv[:, 1], ref["inst"])
    hit = ref["prim"] != 0xFFFFFFFF
    assert hit.mean() > (0.05 if n_inst == 1 else 0.2)
    for k, name in ((2, "t"), (3, "u"), (4, "v")):
        assert np.array_equal(g[:, k].view(np.float32)[hit], ref[name][hit]), name
    occ = tl.any_hit(torch.from_numpy(rays).cuda(), flags=flags).cpu().numpy()
    assert np.array_equal(occ.astype(np.uint32), oracle.tlas_any_hit(cpu, rec[:, 0:12], inst["blas"], rays, cull=cull))
    assert np.array_equal(occ.astype(bool), hit)
    info = tl.info()
    assert info.num_instances == n_inst and info.num_blas == len(meshes) and info.depth >= 1
    tl.close()


def test_two_level_edge_cases(ctx, meshes):
    rng = np.random.default_rng(5)
    blas = [BVH(ctx, torch.from_numpy(x), torch.from_numpy(i.astype(np.int32))) for x, i in meshes]
    rays = torch.from_numpy(rays_between(rng, 1000)).cuda()
    empty = TLAS(ctx, blas, np.zeros(0, INSTANCE_DTYPE))
    h = empty.closest_hit(rays).cpu().numpy().view(np.uint32)
    assert np.all(h[:, 0] == 0xFFFFFFFF) and np.all(h[:, 1] == 0xFFFFFFFF)
    assert not empty.any_hit(rays).cpu().numpy().any()
    empty.close()
    bad = make_instances(rng, 4, len(meshes))
    bad[2]["transform"] = 0
    with pytest.raises(_lib.VkgError):
        TLAS(ctx, blas, bad)
    bad = make_instances(rng, 4, len(meshes))
    bad[1]["blas"] = 7
    with pytest.raises(_lib.VkgError):
        TLAS(ctx, blas, bad)
    # only the empty mesh: every ray misses
    only_empty = make_instances(rng, 5, 1)
    only_empty["blas"] = 2
    t2 = TLAS(ctx, blas, only_empty)
    assert np.all(t2.closest_hit(rays).cpu().numpy().view(np.uint32)[:, 0] == 0xFFFFFFFF)
    t2.close()
