"""vierkant_gb300: GB300-native path-tracing hot path of vierkant (closest-hit BVH queries and the
PBRPathTracer radiance estimator) behind a C ABI (include/vkg.h, libvkg.so)."""
from ._lib import INSIDE, INTERSECT, REJECT, VKG_MISS, VkgError, lib  # noqa: F401
from .intersection import AABB, OBB, Plane, Ray, Sphere, Triangle, intersect  # noqa: F401

__all__ = ["lib", "VkgError", "REJECT", "INTERSECT", "INSIDE", "VKG_MISS", "Ray", "Triangle", "AABB", "OBB",
           "Sphere", "Plane", "intersect"]
