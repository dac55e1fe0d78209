"""The C ABI library loads and exports every entry point declared in include/*.h (the drop-in vkg.h and
the test-only vkg_diag.h), with no GPU calls."""
import re
from pathlib import Path

from vierkant_gb300 import _lib

HEADERS = sorted((Path(__file__).resolve().parents[1] / "include").glob("*.h"))


def declared_functions():
    names = set()
    for h in HEADERS:
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names |= set(re.findall(r"\b(vkg_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_functions()
    assert "vkg_closest_hit" in names and "vkg_bvh_build" in names and "vkg_intersect_ray_triangle" in names
    assert "vkg_diag_wait_timeout" in names and len(HEADERS) >= 2


def test_library_exports_every_declared_symbol():
    L = _lib.lib()
    missing = [n for n in declared_functions() if not hasattr(L, n)]
    assert not missing, f"declared in include/*.h but not exported: {missing}"


def test_bindings_cover_header():
    # every declared function has a ctypes signature in the Python binding
    missing = [n for n in declared_functions() if n not in _lib.SIGNATURES]
    assert not missing, missing


def test_version_string():
    assert _lib.lib().vkg_version().decode().startswith("vkg ")
