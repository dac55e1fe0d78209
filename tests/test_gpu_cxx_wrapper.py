"""The C++20 wrapper's owning classes (include/vierkant_gb/raytracing.hpp, PBRPathTracer.hpp) on the
GPU: a program built with g++ -std=c++20 against libvkg traces the icosphere through
vierkant::gb::bvh with hits equal to the oracle's brute force over the reference's ray-triangle test,
renders two batches through vierkant::gb::PBRPathTracer, and gets a failing call as a C++ exception."""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

import oracle
from vierkant_gb300 import _lib

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parents[1]


def test_cxx_wrapper_on_the_gpu(tmp_path):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    libdir = Path(_lib.lib()._name).parent
    cuda = Path("/usr/local/cuda")
    exe = tmp_path / "wrapper_gpu"
    cmd = ["g++", "-std=c++20", "-O2", f"-I{ROOT / 'include'}", f"-I{cuda / 'include'}",
           str(ROOT / "tests" / "cxx" / "wrapper_gpu.cpp"), f"-L{libdir}", "-lvkg", f"-Wl,-rpath,{libdir}",
           f"-L{cuda / 'lib64'}", "-lcudart", f"-Wl,-rpath,{cuda / 'lib64'}", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    r = subprocess.run([str(exe), str(tmp_path)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    assert "batches 2 " in r.stdout and "error caught: 1" in r.stdout, r.stdout
    hits = np.fromfile(tmp_path / "hits.bin", oracle.HIT_DTYPE)
    rays = np.fromfile(tmp_path / "rays.bin", oracle.RAY_DTYPE)
    th = float(np.fromfile(tmp_path / "tan.bin", np.float32)[0])
    xyz, idx = oracle.icosphere(1.0, 5)
    cam = oracle.camera((0, 0, 3), (0, 0, 0), (0, 1, 0), th, 256, 256)
    assert rays.tobytes() == oracle.camera_rays(cam, 0x5EED, 1, 1).tobytes()
    ref = oracle.closest_hit_bruteforce(xyz, idx, rays)
    assert (ref["prim"] != 0xFFFFFFFF).sum() > 1000
    assert hits.tobytes() == ref.tobytes()
    img = np.fromfile(tmp_path / "image.bin", np.float32)
    assert img.size == 64 * 64 * 3 and np.all(np.isfinite(img)) and img.sum() > 0
