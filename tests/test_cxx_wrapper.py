"""The C++20 wrapper headers (include/vierkant_gb/*.hpp) compile with g++ -std=c++20 next to the
reference's own include/vierkant/intersection.hpp, and vierkant::gb::intersect returns what the
reference's vierkant::intersect returns, bit for bit, on every golden case and on 200,000 seeded random
ray-triangle / ray-box cases (tests/cxx/wrapper_parity.cpp, linked with the reference's unmodified
src/intersection.cpp and libvkg.so)."""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

import oracle
from vierkant_gb300 import _lib

ROOT = Path(__file__).resolve().parents[1]
ROW = np.dtype([("type", "<i4"), ("t", "<f4"), ("u", "<f4"), ("v", "<f4")])


@pytest.fixture(scope="module")
def wrapper_bin(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    ref = oracle.REF_ROOT
    if not (ref / "src" / "intersection.cpp").exists():
        pytest.skip("the reference's intersection code is not staged (make -C oracle stage)")
    libdir = Path(_lib.lib()._name).parent
    out = tmp_path_factory.mktemp("cxx") / "wrapper_parity"
    cmd = ["g++", "-std=c++20", "-O2", "-ffp-contract=off", "-w",
           f"-I{ROOT / 'oracle' / 'ref_shim'}", f"-I{ref / 'include'}", f"-I{ROOT / 'include'}",
           str(ROOT / "tests" / "cxx" / "wrapper_parity.cpp"), str(ref / "src" / "intersection.cpp"),
           f"-L{libdir}", "-lvkg", f"-Wl,-rpath,{libdir}", "-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return out


def test_wrapper_equals_reference(wrapper_bin, tmp_path, golden):
    inputs = {
        "ray_triangle": ("o", "d", "tri"),
        "ray_aabb": ("o", "d", "lo", "hi"),
        "ray_sphere": ("o", "d", "c", "r"),
        "ray_plane": ("o", "d", "plane"),
        "tri_box": ("tri", "lo", "hi"),
        "tri_tri": ("a", "b"),
    }
    for kind, keys in inputs.items():
        g = golden(kind)
        cols = [np.asarray(g[k], np.float32).reshape(len(g[keys[0]]), -1) for k in keys]
        np.ascontiguousarray(np.concatenate(cols, axis=1)).tofile(tmp_path / f"{kind}.in")
    r = subprocess.run([str(wrapper_bin), str(tmp_path)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert "random mismatches: 0" in r.stdout and "throws: 1" in r.stdout, r.stdout
    for kind in inputs:
        gb = np.fromfile(tmp_path / f"{kind}.gb", ROW)
        ref = np.fromfile(tmp_path / f"{kind}.ref", ROW)
        assert len(gb) == len(golden(kind)[inputs[kind][0]])
        assert np.array_equal(gb["type"], ref["type"]), kind
        hit = ref["type"] != 0
        assert gb[hit].tobytes() == ref[hit].tobytes(), kind
        g = golden(kind)
        if kind == "ray_triangle":
            assert np.array_equal(gb["type"], g["type"])
            assert np.stack([gb["t"], gb["u"], gb["v"]], 1)[hit].tobytes() == g["tuv"][hit].tobytes()
        elif kind in ("tri_box", "tri_tri"):
            assert np.array_equal(gb["type"].astype(np.uint32), g["overlap"])
        else:
            assert np.array_equal(gb["type"], g["type"])
            assert gb["t"][hit].tobytes() == g["t"][hit].tobytes()
