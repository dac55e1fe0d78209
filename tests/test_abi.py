"""The C ABI library loads and exports every entry point declared in include/vkg.h (no GPU calls)."""
import re
from pathlib import Path

from vierkant_gb300 import _lib

HEADER = Path(__file__).resolve().parents[1] / "include" / "vkg.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(vkg_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_entry_points():
    names = declared_functions()
    assert "vkg_closest_hit" in names and "vkg_bvh_build" in names and "vkg_intersect_ray_triangle" in names


def test_library_exports_every_declared_symbol():
    L = _lib.lib()
    missing = [n for n in declared_functions() if not hasattr(L, n)]
    assert not missing, f"declared in vkg.h but not exported: {missing}"


def test_bindings_cover_header():
    # every declared function has a ctypes signature in the Python binding
    missing = [n for n in declared_functions() if n not in _lib.SIGNATURES]
    assert not missing, missing


def test_version_string():
    assert _lib.lib().vkg_version().decode().startswith("vkg ")
