"""Build libvkg.so in-tree: every CUDA translation unit for sm_103a plus the C++20 host code.

Usage: ``python -m vierkant_gb300.build`` (or ``__graft_entry__.build()``). Translation units
compile in parallel; a unit is rebuilt only when a source or header is newer than its object.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
INCLUDE = PKG.parent / "include"
OBJDIR = PKG / "_build"
LIB = PKG / "libvkg.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = shutil.which("nvcc") or os.path.join(CUDA_HOME, "bin", "nvcc")
CXX = os.environ.get("CXX", "g++")

NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++20", "--expt-relaxed-constexpr",
                     "-Xcompiler", "-fPIC,-ffp-contract=off", "-diag-suppress", "550"]
CXX_FLAGS = ["-O2", "-std=c++20", "-fPIC", "-ffp-contract=off", "-Wall", "-Wextra",
             "-Wno-unused-parameter", f"-I{CUDA_HOME}/include"]


def _sources():
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))


def _headers():
    return list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.hpp")) + list(INCLUDE.glob("*.h"))


def _stale(obj: Path, src: Path, hdr_mtime: float) -> bool:
    if not obj.exists():
        return True
    m = obj.stat().st_mtime
    return m < src.stat().st_mtime or m < hdr_mtime


def _compile(src: Path, obj: Path, verbose: bool) -> None:
    if src.suffix == ".cu":
        cmd = [NVCC, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)]
    else:
        cmd = [CXX, *CXX_FLAGS, "-c", str(src), "-o", str(obj)]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {src.name}\n{r.stdout}\n{r.stderr}")


def build(verbose: bool = False, force: bool = False) -> Path:
    """Compile (incrementally) and link vierkant_gb300/libvkg.so; returns its path."""
    OBJDIR.mkdir(exist_ok=True)
    hdr_mtime = max((h.stat().st_mtime for h in _headers()), default=0.0)
    srcs = _sources()
    jobs = []
    objs = []
    for s in srcs:
        o = OBJDIR / (s.name + ".o")
        objs.append(o)
        if force or _stale(o, s, hdr_mtime):
            jobs.append((s, o))
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            futs = [ex.submit(_compile, s, o, verbose) for s, o in jobs]
            for f in futs:
                f.result()
    if jobs or not LIB.exists() or LIB.stat().st_mtime < max(o.stat().st_mtime for o in objs):
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [NVCC, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    p = build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    print(p)
