"""The allocation-free BVH build (vkg_bvh_build_noalloc) against the regular build.

Some callers cannot allocate device memory while they run (an engine that hands out all of its
device memory from one arena it reserved at start-up, or code that must not synchronise the device
the way an allocation can). vkg_bvh_build_noalloc serves them: its temporaries live in a fixed
device array inside libvkg, and the caller passes only inputs and output buffers. This test calls
it through the C ABI twice in a row (after a different mesh has dirtied the shared array) and
checks that its nodes and triangle records are byte-identical to those of vkg_bvh_build, the same
bit-exact bar the other BVH tests use. It runs last so a failure here never hides another test.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from vierkant_gb300 import _lib, geometry
from vierkant_gb300.raytracing import BVH, Context

pytestmark = pytest.mark.gpu

MAX_TRIS = 16384


def _copy_out(ptr, nbytes):
    import glob
    out = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    for cand in ["libcudart.so.13", "libcudart.so"] + sorted(glob.glob("/usr/local/cuda/lib64/libcudart.so*")):
        try:
            rt = C.CDLL(cand)
            break
        except OSError:
            continue
    rt.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
    assert rt.cudaMemcpy(C.c_void_p(out.data_ptr()), C.c_void_p(ptr), C.c_size_t(nbytes), 3) == 0
    return out.cpu().numpy().tobytes()


def _noalloc(xyz, idx, leaf_max=0):  # 0: the library default, as the regular build
    n = idx.shape[0]
    nodes = torch.zeros((max(1, n) * 96,), dtype=torch.uint8, device="cuda")
    tris = torch.zeros((max(1, n) * 48,), dtype=torch.uint8, device="cuda")
    info = torch.zeros(16, dtype=torch.int32, device="cuda")
    st = _lib.lib().vkg_bvh_build_noalloc(C.c_void_p(xyz.data_ptr()), xyz.shape[0], C.c_void_p(idx.data_ptr()), n,
                                          leaf_max, C.c_void_p(nodes.data_ptr()), max(1, n),
                                          C.c_void_p(tris.data_ptr()), C.c_void_p(info.data_ptr()),
                                          C.c_void_p(torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    return st, nodes, tris, info.cpu().numpy().view(np.uint32)


def _mesh(kind):
    if kind == "ico":
        xyz, idx = geometry.icosphere(1.0, 4)  # 5,120 triangles
    else:
        rng = np.random.default_rng(4)
        nt = MAX_TRIS
        xyz = (rng.normal(size=(3 * nt, 3)) * 0.05 + np.repeat(rng.normal(size=(nt, 3)), 3, axis=0)).astype(np.float32)
        idx = np.arange(3 * nt, dtype=np.uint32).reshape(nt, 3)
    return torch.from_numpy(xyz).cuda(), torch.from_numpy(idx.astype(np.int32)).cuda()


@pytest.mark.parametrize("kind", ["ico", "max"])
def test_noalloc_build_matches_regular_build_twice(kind):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    ctx = Context(0)
    xyz, idx = _mesh(kind)
    ref = BVH(ctx, xyz, idx)
    inf = ref.info()
    ref_nodes = _copy_out(inf.d_nodes, inf.num_nodes * 96)
    ref_tris = _copy_out(inf.d_tris, inf.num_tris * 48)
    # dirty the shared array with a different mesh first
    oxyz, oidx = _mesh("max" if kind == "ico" else "ico")
    assert _noalloc(oxyz, oidx)[0] == 0
    for _ in range(2):
        st, nodes, tris, info = _noalloc(xyz, idx)
        assert st == 0
        assert info[2] == 0
        assert info[0] == inf.num_nodes and info[1] == inf.depth
        assert np.float32(info[3:4].view(np.float32)[0]) == np.float32(inf.margin)
        assert nodes.cpu().numpy().tobytes()[: inf.num_nodes * 96] == ref_nodes
        assert tris.cpu().numpy().tobytes()[: inf.num_tris * 48] == ref_tris
    ref.close()
    ctx.close()


def test_noalloc_rejects_oversize_and_reports_bad_indices():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    n = MAX_TRIS + 1
    xyz = torch.zeros((3, 3), device="cuda")
    idx = torch.zeros((n, 3), dtype=torch.int32, device="cuda")
    st, _, _, _ = _noalloc(xyz, idx)
    assert st == 7  # VKG_ERR_CAPACITY
    idx = torch.tensor([[0, 1, 9]], dtype=torch.int32, device="cuda")
    st, _, _, info = _noalloc(xyz, idx)
    assert st == 0 and (info[2] & 1) == 1


@pytest.mark.parametrize("n", [1, 2, 3, 9])
@pytest.mark.parametrize("leaf_max", [1, 2, 4])
def test_noalloc_small_meshes_and_leaf_sizes(n, leaf_max):
    """1, 2 and 3 triangles (a root leaf, and trees without an internal binary level to refit) and the
    leaf sizes 1 and 4 give the same bytes as vkg_bvh_build"""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    ctx = Context(0)
    rng = np.random.default_rng(100 + n)
    xyz_np = rng.normal(size=(3 * n, 3)).astype(np.float32)
    idx_np = np.arange(3 * n, dtype=np.int32).reshape(n, 3)
    xyz, idx = torch.from_numpy(xyz_np).cuda(), torch.from_numpy(idx_np).cuda()
    ref = BVH(ctx, xyz, idx, leaf_max=leaf_max)
    inf = ref.info()
    ref_nodes = _copy_out(inf.d_nodes, inf.num_nodes * 96)
    ref_tris = _copy_out(inf.d_tris, inf.num_tris * 48)
    st, nodes, tris, info = _noalloc(xyz, idx, leaf_max)
    assert st == 0 and info[2] == 0
    assert info[0] == inf.num_nodes and info[1] == inf.depth
    assert nodes.cpu().numpy().tobytes()[: inf.num_nodes * 96] == ref_nodes
    assert tris.cpu().numpy().tobytes()[: inf.num_tris * 48] == ref_tris
    ref.close()
    ctx.close()


def test_noalloc_rejects_small_node_capacity():
    """a node buffer for fewer than num_tris nodes is refused before any work (num_tris nodes always
    suffice: an 8-wide tree over n triangles has fewer than n nodes)"""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    xyz, idx = _mesh("ico")
    n = idx.shape[0]
    nodes = torch.zeros(((n - 1) * 96,), dtype=torch.uint8, device="cuda")
    tris = torch.zeros((n * 48,), dtype=torch.uint8, device="cuda")
    info = torch.zeros(16, dtype=torch.int32, device="cuda")
    st = _lib.lib().vkg_bvh_build_noalloc(C.c_void_p(xyz.data_ptr()), xyz.shape[0], C.c_void_p(idx.data_ptr()), n,
                                          1, C.c_void_p(nodes.data_ptr()), n - 1, C.c_void_p(tris.data_ptr()),
                                          C.c_void_p(info.data_ptr()),
                                          C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 1  # VKG_ERR_INVALID_ARGUMENT
