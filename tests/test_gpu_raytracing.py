"""GPU parity of the closest-hit / any-hit path through the C ABI: camera rays, the LBVH build
(Morton codes, sorted order, 8-wide nodes, triangle records) and the traversal are bit-identical to
the CPU oracle, and hit ids / t / u / v are bit-identical to brute force over the reference's
ray-triangle test (the committed fixture made from the reference's own code)."""
import hashlib
import math

import numpy as np
import pytest
import torch

import oracle
from vierkant_gb300 import geometry
from vierkant_gb300._lib import RAY_COUNT_STATS, RAY_CULL_BACK_FACES, RAY_KEEP_ORDER, VkgError
from vierkant_gb300.raytracing import BVH

pytestmark = pytest.mark.gpu


def to_dev(a, dtype=None):
    t = torch.from_numpy(np.ascontiguousarray(a))
    if dtype is not None:
        t = t.view(dtype)
    return t.cuda()


def rays_dev(rays_np):
    return to_dev(rays_np.view(np.float32).reshape(-1, 8))


def hits_np(h):
    return h.cpu().numpy().view(np.uint32).reshape(-1, 4)


def config1_scene():
    xyz, idx = geometry.icosphere(1.0, 5)
    th = float(np.float32(math.tan(math.radians(60.0) / 2.0)))
    cam_o = oracle.camera((0, 0, 3), (0, 0, 0), (0, 1, 0), th, 1024, 1024)
    cam_p = geometry.camera_lookat((0, 0, 3), (0, 0, 0), (0, 1, 0), 60.0, 1024, 1024)
    return xyz, idx, cam_o, cam_p


def test_camera_rays_bit_exact(ctx, golden):
    xyz, idx, cam_o, cam_p = config1_scene()
    g = ctx.camera_rays(cam_p, 0x5EED, 1, 1)
    torch.cuda.synchronize()
    ref = oracle.camera_rays(cam_o, 0x5EED, 1, 1)
    got = g.cpu().numpy()
    assert got.tobytes() == ref.tobytes()
    assert hashlib.sha256(got.tobytes()).hexdigest() == str(golden("config1_hits")["sha_rays"])
    # multi-sample batches continue the same stream
    g4 = ctx.camera_rays(cam_p, 0x5EED, 3, 2)
    ref4 = oracle.camera_rays(cam_o, 0x5EED, 3, 2)
    assert g4.cpu().numpy().tobytes() == ref4.tobytes()


@pytest.mark.parametrize("leaf_max", [1, 4, 8])
def test_bvh_build_bit_exact_icosphere(ctx, leaf_max):
    xyz, idx, _, _ = config1_scene()
    b = BVH(ctx, to_dev(xyz), to_dev(idx.astype(np.int32)), leaf_max=leaf_max)
    cb = oracle.CpuBVH(xyz, idx, leaf_max)
    inf = b.info()
    assert inf.num_nodes == cb.b.num_nodes and inf.depth == cb.b.depth
    assert np.float32(inf.margin) == np.float32(cb.b.margin)
    n = inf.num_tris
    morton = torch.empty(n, dtype=torch.int32, device="cuda")
    sorted_ = torch.empty(n, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    cudart_copy(morton, inf.d_morton, 4 * n)
    cudart_copy(sorted_, inf.d_sorted, 4 * n)
    assert np.array_equal(morton.cpu().numpy().view(np.uint32), cb.morton)
    assert np.array_equal(sorted_.cpu().numpy().view(np.uint32), cb.sorted_prim)
    nodes = torch.empty(inf.num_nodes * 96, dtype=torch.uint8, device="cuda")
    cudart_copy(nodes, inf.d_nodes, inf.num_nodes * 96)
    assert nodes.cpu().numpy().tobytes() == cb.node_bytes()
    tris = torch.empty(n * 48, dtype=torch.uint8, device="cuda")
    cudart_copy(tris, inf.d_tris, n * 48)
    assert tris.cpu().numpy().tobytes() == cb.tri_bytes()
    b.close()


def cudart_copy(dst: torch.Tensor, src_ptr: int, nbytes: int):
    """device-to-device copy of a library-owned buffer into a torch tensor (test helper)."""
    import ctypes as C
    C.memmove  # noqa: B018
    cudart = _cudart()
    rc = cudart.cudaMemcpy(C.c_void_p(dst.data_ptr()), C.c_void_p(src_ptr), C.c_size_t(nbytes), 3)
    assert rc == 0


def _cudart():
    import ctypes as C
    import glob
    for cand in ["libcudart.so.13", "libcudart.so"] + sorted(glob.glob("/usr/local/cuda/lib64/libcudart.so*")):
        try:
            lib = C.CDLL(cand)
            lib.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
            return lib
        except OSError:
            continue
    raise RuntimeError("libcudart not found")


def test_config1_closest_hit_full(ctx, golden):
    """All 1,048,576 config-1 rays: GPU hits == oracle BVH traversal (bit-exact), the fixture subset
    == the reference's brute-force hits, and the per-ray work counters match the oracle's."""
    xyz, idx, cam_o, cam_p = config1_scene()
    b = BVH(ctx, to_dev(xyz), to_dev(idx.astype(np.int32)))
    rays = ctx.camera_rays(cam_p, 0x5EED, 1, 1)
    ctx.stats(reset=True)
    hits = b.closest_hit(rays, flags=RAY_COUNT_STATS)
    visits, tests = ctx.stats(reset=True)
    h = hits_np(hits)
    cb = oracle.CpuBVH(xyz, idx, DEFAULT_LEAF)
    ref_rays = oracle.camera_rays(cam_o, 0x5EED, 1, 1)
    ch, st = cb.closest_hit(ref_rays, stats=True)
    assert h.tobytes() == ch.tobytes()
    assert (visits, tests) == st
    g = golden("config1_hits")
    assert np.array_equal(h[g["ray_index"]], g["hits"])
    # the plain (non-counting) kernel gives the same bytes
    h2 = hits_np(b.closest_hit(rays))
    assert h2.tobytes() == h.tobytes()
    b.close()


DEFAULT_LEAF = 2  # the library's default BVH leaf size


def cornell(ctx):
    sc = geometry.cornell_scene(0x5EED, 2, 64, 16)
    b = BVH(ctx, to_dev(sc["xyz"]), to_dev(sc["indices"].astype(np.int32)))
    return sc, b


def secondary_rays(rng, hits_np_arr, rays_np, n):
    """rays leaving the primary hit points in random directions (incoherent bounce rays)."""
    hit = hits_np_arr[:, 0] != 0xFFFFFFFF
    sel = np.nonzero(hit)[0][:n]
    t = hits_np_arr[sel, 1].view(np.float32)
    o = rays_np["o"][sel] + rays_np["d"][sel] * t[:, None]
    d = rng.normal(size=(len(sel), 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True).astype(np.float32)
    out = np.zeros(len(sel), oracle.RAY_DTYPE)
    out["o"], out["d"], out["tmin"], out["tmax"] = o.astype(np.float32), d, 1e-4, 1e4
    return out


def test_cornell_primary_and_secondary_bit_exact(ctx):
    sc, b = cornell(ctx)
    th = float(np.float32(math.tan(math.radians(45.0) / 2.0)))
    cam_o = oracle.camera((0, 0, 3.4), (0, 0, 0), (0, 1, 0), th, 1280, 720)
    cam_p = geometry.camera_lookat((0, 0, 3.4), (0, 0, 0), (0, 1, 0), 45.0, 1280, 720)
    rays = ctx.camera_rays(cam_p, 0x5EED, 2, 1)
    ref_rays = oracle.camera_rays(cam_o, 0x5EED, 2, 1)
    assert rays.cpu().numpy().tobytes() == ref_rays.tobytes()
    cb = oracle.CpuBVH(sc["xyz"], sc["indices"], DEFAULT_LEAF)
    assert b.info().num_nodes == cb.b.num_nodes
    h = hits_np(b.closest_hit(rays))
    assert h.tobytes() == cb.closest_hit(ref_rays).tobytes()
    # brute force over the reference's triangle test on a subset
    sub = np.ascontiguousarray(ref_rays[::997])
    bf = oracle.closest_hit_bruteforce(sc["xyz"], sc["indices"], sub)
    assert np.ascontiguousarray(h[::997]).tobytes() == bf.tobytes()
    # incoherent secondary rays
    rng = np.random.default_rng(9)
    sec = secondary_rays(rng, h, ref_rays, 200000)
    hs = hits_np(b.closest_hit(rays_dev(sec)))
    assert hs.tobytes() == cb.closest_hit(sec).tobytes()
    sub2 = np.ascontiguousarray(sec[::211])
    assert np.ascontiguousarray(hs[::211]).tobytes() == oracle.closest_hit_bruteforce(
        sc["xyz"], sc["indices"], sub2).tobytes()
    # culling and any-hit
    for cull in (0, RAY_CULL_BACK_FACES):
        hc = hits_np(b.closest_hit(rays_dev(sec), flags=cull))
        assert hc.tobytes() == cb.closest_hit(sec, cull=bool(cull)).tobytes()
        occ = b.any_hit(rays_dev(sec), flags=cull).cpu().numpy().view(np.uint32)
        assert np.array_equal(occ, cb.any_hit(sec, cull=bool(cull)))
    b.close()


def test_binned_batches_equal_given_order(ctx):
    """Batches of 2^19 rays or more are traced in bins (origin cell x direction). On a ragged mixed
    batch (921,600 camera rays + 500,000 incoherent bounce rays): hits, any-hit flags and the work
    counters equal tracing in the given order (VKG_RAY_KEEP_ORDER), with and without culling, the
    bounce rays equal the CPU traversal bit for bit, and a call captured into a CUDA graph (traced
    in the given order) replays to the same hits."""
    sc, b = cornell(ctx)
    cb = oracle.CpuBVH(sc["xyz"], sc["indices"], DEFAULT_LEAF)
    th = float(np.float32(math.tan(math.radians(45.0) / 2.0)))
    cam_o = oracle.camera((0, 0, 3.4), (0, 0, 0), (0, 1, 0), th, 1280, 720)
    ref_rays = oracle.camera_rays(cam_o, 0x5EED, 2, 1)
    h0 = np.ascontiguousarray(cb.closest_hit(ref_rays)).view(np.uint32).reshape(-1, 4)
    sec = secondary_rays(np.random.default_rng(21), h0, ref_rays, 500000)
    assert sec.shape[0] == 500000
    batch = np.concatenate([ref_rays, sec])
    assert batch.shape[0] % 256 != 0
    d = rays_dev(batch)
    for cull in (0, RAY_CULL_BACK_FACES):
        ctx.stats(reset=True)
        hb = hits_np(b.closest_hit(d, flags=cull | RAY_COUNT_STATS))
        sb = ctx.stats(reset=True)
        hk = hits_np(b.closest_hit(d, flags=cull | RAY_COUNT_STATS | RAY_KEEP_ORDER))
        sk = ctx.stats(reset=True)
        assert hb.tobytes() == hk.tobytes()
        assert sb == sk
        assert hits_np(b.closest_hit(d, flags=cull)).tobytes() == hb.tobytes()
        if cull == 0:
            h_plain = hb
        assert hb[ref_rays.shape[0]:].tobytes() == cb.closest_hit(sec, cull=bool(cull)).tobytes()
        ob = b.any_hit(d, flags=cull).cpu().numpy()
        ok = b.any_hit(d, flags=cull | RAY_KEEP_ORDER).cpu().numpy()
        assert np.array_equal(ob, ok)
    # inside a stream capture the call traces in the given order
    out = torch.empty((batch.shape[0], 4), dtype=torch.int32, device="cuda")
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        b.closest_hit(d, out)
    torch.cuda.current_stream().wait_stream(side)
    out.zero_()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        b.closest_hit(d, out)
    g.replay()
    torch.cuda.synchronize()
    assert hits_np(out).tobytes() == h_plain.tobytes()
    b.close()


@pytest.mark.parametrize("w,h,spp", [(320, 180, 1), (1280, 720, 3)])
def test_host_buffer_variant_equals_device(ctx, w, h, spp):
    """one chunk, and 2.76 M rays: three chunks of the two-stream copy / trace pipeline, the last ragged"""
    sc, b = cornell(ctx)
    cam_p = geometry.camera_lookat((0, 0, 3.4), (0, 0, 0), (0, 1, 0), 45.0, w, h)
    rays = ctx.camera_rays(cam_p, 0x5EED, 2, spp)
    dev = hits_np(b.closest_hit(rays))
    rh = rays.cpu().pin_memory()
    hh = torch.empty((rays.shape[0], 4), dtype=torch.int32).pin_memory()
    b.closest_hit_host(rh, hh)
    assert hh.numpy().tobytes() == dev.tobytes()
    # pageable buffers too
    hp = torch.empty((rays.shape[0], 4), dtype=torch.int32)
    b.closest_hit_host(rays.cpu(), hp)
    assert hp.numpy().tobytes() == dev.tobytes()
    b.close()


@pytest.mark.parametrize("nt", [1, 2, 5, 100, 5000])
def test_small_meshes_and_edge_rays(ctx, nt):
    rng = np.random.default_rng(nt)
    xyz = (rng.normal(size=(3 * nt, 3)) * 0.3 + np.repeat(rng.normal(size=(nt, 3)), 3, axis=0)).astype(np.float32)
    idx = np.arange(3 * nt, dtype=np.uint32).reshape(nt, 3)
    if nt >= 5:
        idx = np.concatenate([idx, idx[:3], idx[:2][:, [0, 0, 1]]]).astype(np.uint32)  # duplicates, degenerate
    b = BVH(ctx, to_dev(xyz), to_dev(idx.astype(np.int32)), leaf_max=2)
    rays = np.zeros(4096, oracle.RAY_DTYPE)
    rays["o"] = (rng.normal(size=(4096, 3)) * 2).astype(np.float32)
    d = rng.normal(size=(4096, 3)).astype(np.float32)
    d[::7, 0] = 0.0
    d[::13, 2] = 0.0
    d /= np.linalg.norm(d, axis=1, keepdims=True).astype(np.float32)
    rays["d"] = d
    rays["tmin"] = 1e-4
    rays["tmax"] = np.where(np.arange(4096) % 3 == 0, 2.0, 1e4).astype(np.float32)  # short rays too
    h = hits_np(b.closest_hit(rays_dev(rays)))
    bf = oracle.closest_hit_bruteforce(xyz, idx, rays)
    assert h.tobytes() == bf.tobytes()
    occ = b.any_hit(rays_dev(rays)).cpu().numpy().view(np.uint32)
    assert np.array_equal(occ, oracle.any_hit_bruteforce(xyz, idx, rays))
    b.close()


def test_empty_bvh_and_errors(ctx):
    b = BVH(ctx, torch.zeros((0, 3), device="cuda"), torch.zeros((0, 3), dtype=torch.int32, device="cuda"))
    rays = torch.zeros((100, 8), device="cuda")
    rays[:, 5] = -1.0
    rays[:, 7] = 1e4
    h = hits_np(b.closest_hit(rays))
    assert np.all(h[:, 0] == 0xFFFFFFFF)
    assert np.all(b.any_hit(rays).cpu().numpy() == 0)
    b.close()
    # an index outside the vertex buffer is rejected by the build
    xyz = torch.zeros((3, 3), device="cuda")
    idx = torch.tensor([[0, 1, 7]], dtype=torch.int32, device="cuda")
    with pytest.raises(VkgError) as e:
        BVH(ctx, xyz, idx)
    assert e.value.status == 1
    # misaligned ray buffers are rejected
    xyz, idx, _, _ = config1_scene()
    b = BVH(ctx, to_dev(xyz), to_dev(idx.astype(np.int32)))
    buf = torch.zeros(8 * 10 + 1, device="cuda")
    with pytest.raises(VkgError):
        b.closest_hit(buf[1:].view(10, 8))
    b.close()


def test_deterministic_reruns(ctx):
    sc, b = cornell(ctx)
    cam_p = geometry.camera_lookat((0, 0, 3.4), (0, 0, 0), (0, 1, 0), 45.0, 640, 360)
    rays = ctx.camera_rays(cam_p, 7, 5, 2)
    a = hits_np(b.closest_hit(rays))
    for _ in range(3):
        assert hits_np(b.closest_hit(rays)).tobytes() == a.tobytes()
    # rebuilding gives identical nodes
    b2 = BVH(ctx, to_dev(sc["xyz"]), to_dev(sc["indices"].astype(np.int32)))
    assert hits_np(b2.closest_hit(rays)).tobytes() == a.tobytes()
    b.close()
    b2.close()
