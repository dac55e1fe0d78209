// Host side of libvkg: context / error plumbing, the scalar intersection API (drop-in for
// vierkant::intersect, src/intersection.cpp), geometry generators (Geometry::IcoSphere and the
// Cornell-box benchmark scene) and the camera helper.
//
// Compiled with -ffp-contract=off: every float operation rounds separately, matching the
// reference's x86-64 build, so the scalar results are bit-identical to vierkant's.
#include "internal.hpp"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <limits>
#include <vector>

namespace vkg
{

vkg_status set_error(vkg_ctx *ctx, vkg_status status, const char *fmt, ...)
{
    if(ctx)
    {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        std::vsnprintf(buf, sizeof(buf), fmt, ap);
        va_end(ap);
        ctx->last_error = buf;
    }
    return status;
}

vkg_status cuda_check(vkg_ctx *ctx, cudaError_t err, const char *what)
{
    if(err == cudaSuccess) return VKG_OK;
    vkg_status s = (err == cudaErrorMemoryAllocation) ? VKG_ERR_OUT_OF_MEMORY : VKG_ERR_CUDA;
    return set_error(ctx, s, "%s: %s (%s)", what, cudaGetErrorName(err), cudaGetErrorString(err));
}

vkg_status bind_device(vkg_ctx *ctx)
{
    int cur = -1;
    if(cudaGetDevice(&cur) == cudaSuccess && cur == ctx->device) return VKG_OK;
    return cuda_check(ctx, cudaSetDevice(ctx->device), "cudaSetDevice");
}

}// namespace vkg

using namespace vkg;

extern "C" {

const char *vkg_version(void) { return "vkg 0.1 sm_103a"; }

vkg_status vkg_ctx_create(int device, vkg_ctx **out)
{
    if(!out) return VKG_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    int count = 0;
    if(cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count) return VKG_ERR_CUDA;
    auto *ctx = new vkg_ctx();
    ctx->device = device;
    if(cudaSetDevice(device) != cudaSuccess ||
       cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
       cudaMalloc(&ctx->d_counters, 4 * sizeof(unsigned long long)) != cudaSuccess ||
       cudaMemset(ctx->d_counters, 0, 4 * sizeof(unsigned long long)) != cudaSuccess ||
       cudaMalloc(&ctx->d_work, sizeof(uint32_t)) != cudaSuccess)
    {
        delete ctx;
        return VKG_ERR_CUDA;
    }
    *out = ctx;
    return VKG_OK;
}

vkg_status vkg_ctx_destroy(vkg_ctx *ctx)
{
    if(!ctx) return VKG_OK;
    bind_device(ctx);
    cudaFree(ctx->d_counters);
    cudaFree(ctx->d_work);
    cudaFree(ctx->d_stage_rays);
    cudaFree(ctx->d_stage_hits);
    for(cudaStream_t s: ctx->pipe)
        if(s) cudaStreamDestroy(s);
    for(cudaEvent_t e: ctx->pipe_ev)
        if(e) cudaEventDestroy(e);
    cudaFree(ctx->bins.keys);
    cudaFree(ctx->bins.perm);
    cudaFree(ctx->bins.tile_counts);
    cudaFree(ctx->bins.bin_totals);
    if(ctx->bins.done) cudaEventDestroy(ctx->bins.done);
    delete ctx;
    return VKG_OK;
}

const char *vkg_last_error(const vkg_ctx *ctx) { return ctx ? ctx->last_error.c_str() : "invalid context"; }

// ---- scalar intersection API ----------------------------------------------------------------

// intersection.cpp:114-129
vkg_status vkg_intersect_ray_triangle(const float o[3], const float d[3], const float tri[9],
                                      vkg_ray_triangle_intersection *out)
{
    if(!o || !d || !tri || !out) return VKG_ERR_INVALID_ARGUMENT;
    float e1[3], e2[3];
    for(int a = 0; a < 3; ++a)
    {
        e1[a] = tri[3 + a] - tri[a];
        e2[a] = tri[6 + a] - tri[a];
    }
    float t = 0.f, u = 0.f, v = 0.f;
    int r = tri_test(tri[0], tri[1], tri[2], e1[0], e1[1], e1[2], e2[0], e2[1], e2[2], o[0], o[1], o[2], d[0], d[1],
                     d[2], 0, t, u, v);
    *out = r ? vkg_ray_triangle_intersection{VKG_INTERSECT, t, u, v} : vkg_ray_triangle_intersection{VKG_REJECT, 0, 0, 0};
    return VKG_OK;
}

static inline float dot3h(const float a[3], const float b[3]) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

// intersection.cpp:152-184 (axes given as three unit column vectors)
static vkg_ray_intersection obb_slab(const float o[3], const float d[3], const float center[3], const float axes[9],
                                     const float half[3])
{
    const float epsilon = 1e-10f;
    float t_min = -FLT_MAX, t_max = FLT_MAX;
    float p[3] = {center[0] - o[0], center[1] - o[1], center[2] - o[2]};
    for(int i = 0; i < 3; i++)
    {
        float e = dot3h(axes + 3 * i, p);
        float f = dot3h(axes + 3 * i, d);
        if(std::fabs(f) > epsilon)
        {
            float t1 = (e + half[i]) / f;
            float t2 = (e - half[i]) / f;
            if(t1 > t2) std::swap(t1, t2);
            if(t1 > t_min) t_min = t1;
            if(t2 < t_max) t_max = t2;
            if(t_min > t_max) return {VKG_REJECT, 0.f};
            if(t_max < 0) return {VKG_REJECT, 0.f};
        }
        else if((-e - half[i]) > 0 || (-e + half[i]) < 0) { return {VKG_REJECT, 0.f}; }
    }
    return {VKG_INTERSECT, t_min > 0 ? t_min : t_max};
}

vkg_status vkg_intersect_ray_obb(const float o[3], const float d[3], const float center[3], const float axes[9],
                                 const float half_lengths[3], vkg_ray_intersection *out)
{
    if(!o || !d || !center || !axes || !half_lengths || !out) return VKG_ERR_INVALID_ARGUMENT;
    *out = obb_slab(o, d, center, axes, half_lengths);
    return VKG_OK;
}

// AABB::intersect -> OBB(aabb, identity) (intersection.cpp:219-227, :308-312)
vkg_status vkg_intersect_ray_aabb(const float o[3], const float d[3], const float bmin[3], const float bmax[3],
                                  vkg_ray_intersection *out)
{
    if(!o || !d || !bmin || !bmax || !out) return VKG_ERR_INVALID_ARGUMENT;
    float c[3], center[3], half[3];
    for(int a = 0; a < 3; ++a)
    {
        c[a] = (bmax[a] + bmin[a]) / 2.f;
        half[a] = ((bmax[a] - bmin[a]) / 2.f) * 1.0f;
    }
    // identity-matrix transform of the centre, evaluated the way a 4x4 matrix-vector product sums
    const float I[4][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {0, 0, 0}};
    for(int r = 0; r < 3; ++r) center[r] = I[0][r] * c[0] + I[1][r] * c[1] + I[2][r] * c[2] + I[3][r] * 1.0f;
    const float axes[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    *out = obb_slab(o, d, center, axes, half);
    return VKG_OK;
}

// intersection.cpp:133-148
vkg_status vkg_intersect_ray_sphere(const float o[3], const float d[3], const float center[3], float radius,
                                    vkg_ray_intersection *out)
{
    if(!o || !d || !center || !out) return VKG_ERR_INVALID_ARGUMENT;
    float l[3] = {center[0] - o[0], center[1] - o[1], center[2] - o[2]};
    float s = dot3h(l, d);
    float l2 = dot3h(l, l);
    float r2 = radius * radius;
    *out = {VKG_REJECT, 0.f};
    if(s < 0 && l2 > r2) return VKG_OK;
    float m2 = l2 - s * s;
    if(m2 > r2) return VKG_OK;
    float q = std::sqrt(r2 - m2);
    *out = {VKG_INTERSECT, l2 > r2 ? s - q : s + q};
    return VKG_OK;
}

// Plane(a, b, c, d) (intersection.cpp:196-201) + intersect(Plane, Ray) (intersection.cpp:10-21)
vkg_status vkg_intersect_ray_plane(const float o[3], const float d[3], const float plane[4], vkg_ray_intersection *out)
{
    if(!o || !d || !plane || !out) return VKG_ERR_INVALID_ARGUMENT;
    float len = std::sqrt(plane[0] * plane[0] + plane[1] * plane[1] + plane[2] * plane[2]);
    float c[4] = {plane[0] / len, plane[1] / len, plane[2] / len, plane[3] / len};
    float nn[3] = {-c[0], -c[1], -c[2]};
    float denom = dot3h(nn, d);
    *out = {VKG_REJECT, 0.f};
    if(static_cast<double>(std::fabs(denom)) > 1e-6)
    {
        float dist = (c[3] - dot3h(o, nn)) / denom;
        if(dist >= 0) *out = {VKG_INTERSECT, dist};
    }
    return VKG_OK;
}

// Triangle-box overlap by separating axes (Akenine-Moeller 2001): the 9 edge x axis directions,
// the box faces (triangle bounds) and the triangle plane; box given as min/max like
// intersect(const Triangle&, const AABB&) (intersection.cpp:364-370, centre + half extents).
vkg_status vkg_intersect_triangle_aabb(const float tri[9], const float bmin[3], const float bmax[3], uint32_t *out)
{
    if(!tri || !bmin || !bmax || !out) return VKG_ERR_INVALID_ARGUMENT;
    float c[3], h[3], v[3][3], e[3][3];
    for(int a = 0; a < 3; ++a)
    {
        c[a] = (bmax[a] + bmin[a]) / 2.f;
        h[a] = (bmax[a] - bmin[a]) / 2.f;
    }
    for(int k = 0; k < 3; ++k)
        for(int a = 0; a < 3; ++a) v[k][a] = tri[3 * k + a] - c[a];
    for(int a = 0; a < 3; ++a)
    {
        e[0][a] = v[1][a] - v[0][a];
        e[1][a] = v[2][a] - v[1][a];
        e[2][a] = v[0][a] - v[2][a];
    }
    *out = 0;
    // projection of vertex p onto (unit axis `ax`) x (edge E); two vertices suffice because the
    // edge's own endpoints project to the same value. pair[edge][axis] = the vertices used.
    static const int pair[3][3][2] = {{{0, 2}, {0, 2}, {1, 2}}, {{0, 2}, {0, 2}, {0, 1}}, {{0, 1}, {0, 1}, {1, 2}}};
    for(int j = 0; j < 3; ++j)
    {
        const float *E = e[j];
        const float fx = std::fabs(E[0]), fy = std::fabs(E[1]), fz = std::fabs(E[2]);
        for(int ax = 0; ax < 3; ++ax)
        {
            float p[2], rad;
            for(int q = 0; q < 2; ++q)
            {
                const float *P = v[pair[j][ax][q]];
                if(ax == 0) p[q] = E[2] * P[1] - E[1] * P[2];
                else if(ax == 1) p[q] = E[0] * P[2] - E[2] * P[0];
                else p[q] = E[1] * P[0] - E[0] * P[1];
            }
            if(ax == 0) rad = fz * h[1] + fy * h[2];
            else if(ax == 1) rad = fz * h[0] + fx * h[2];
            else rad = fy * h[0] + fx * h[1];
            float mn = std::min(p[0], p[1]), mx = std::max(p[0], p[1]);
            if(mn > rad || mx < -rad) return VKG_OK;
        }
    }
    for(int a = 0; a < 3; ++a)
    {
        float mn = v[0][a], mx = v[0][a];
        for(int k = 1; k < 3; ++k)
        {
            if(v[k][a] < mn) mn = v[k][a];
            if(v[k][a] > mx) mx = v[k][a];
        }
        if(mn > h[a] || mx < -h[a]) return VKG_OK;
    }
    // plane of the triangle against the box: nearest / farthest box corner along the normal
    float n[3] = {e[0][1] * e[1][2] - e[0][2] * e[1][1], e[0][2] * e[1][0] - e[0][0] * e[1][2],
                  e[0][0] * e[1][1] - e[0][1] * e[1][0]};
    float vmin[3], vmax[3];
    for(int a = 0; a < 3; ++a)
    {
        if(n[a] > 0.0f)
        {
            vmin[a] = -h[a] - v[0][a];
            vmax[a] = h[a] - v[0][a];
        }
        else
        {
            vmin[a] = h[a] - v[0][a];
            vmax[a] = -h[a] - v[0][a];
        }
    }
    if(dot3h(n, vmin) > 0.0f) return VKG_OK;
    *out = dot3h(n, vmax) >= 0.0f ? 1u : 0u;
    return VKG_OK;
}


// ---- triangle-triangle overlap (Guigue & Devillers 2003, orientation predicates) -------------
// intersect(const Triangle&, const Triangle&) (intersection.cpp:374-378). Same predicates and the
// same separately-rounded arithmetic as the reference's variant: signed distances are clamped to
// zero within 1e-12, interval tests use ">= -1e-12", coplanar pairs fall back to a 2D test in the
// projection plane that maximises the triangle area.
namespace tt
{
using P3 = const float *;
using P2 = const float *;
constexpr float EPS = 1e-12f;

inline void sub(P3 a, P3 b, float *r)
{
    r[0] = a[0] - b[0];
    r[1] = a[1] - b[1];
    r[2] = a[2] - b[2];
}
inline void cross(const float *a, const float *b, float *r)
{
    r[0] = a[1] * b[2] - a[2] * b[1];
    r[1] = a[2] * b[0] - a[0] * b[2];
    r[2] = a[0] * b[1] - a[1] * b[0];
}
inline float dot(const float *a, const float *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

// T1 = (a1, b1, c1) has a1 alone on the positive side of T2's plane and T2 = (a2, b2, c2) has a2
// alone on the positive side of T1's plane: the triangles overlap iff both line intervals meet
inline int interval_test(P3 a1, P3 b1, P3 c1, P3 a2, P3 b2, P3 c2)
{
    float u[3], w[3], n[3], d[3];
    sub(a2, b1, u);
    sub(a1, b1, w);
    cross(u, w, n);
    sub(b2, b1, d);
    if(dot(d, n) >= -EPS) return 0;
    sub(a2, a1, u);
    sub(c1, a1, w);
    cross(u, w, n);
    sub(c2, a1, d);
    if(dot(d, n) >= -EPS) return 0;
    return 1;
}

inline float orient2(P2 a, P2 b, P2 c) { return (a[0] - c[0]) * (b[1] - c[1]) - (a[1] - c[1]) * (b[0] - c[0]); }

// vertex of T1 (p1) lies in a vertex region of T2
inline int vertex_region(P2 p1, P2 q1, P2 r1, P2 p2, P2 q2, P2 r2)
{
    if(orient2(r2, p2, q1) >= 0.f)
    {
        if(orient2(r2, q2, q1) <= 0.f)
        {
            if(orient2(p1, p2, q1) > 0.f) return orient2(p1, q2, q1) <= 0.f;
            if(orient2(p1, p2, r1) >= 0.f) return orient2(q1, r1, p2) >= 0.f;
            return 0;
        }
        if(orient2(p1, q2, q1) <= 0.f && orient2(r2, q2, r1) <= 0.f) return orient2(q1, r1, q2) >= 0.f;
        return 0;
    }
    if(orient2(r2, p2, r1) >= 0.f)
    {
        if(orient2(q1, r1, r2) >= 0.f) return orient2(p1, p2, r1) >= 0.f;
        if(orient2(q1, r1, q2) >= 0.f) return orient2(r2, r1, q2) >= 0.f;
    }
    return 0;
}

// vertex of T1 (p1) lies in an edge region of T2
inline int edge_region(P2 p1, P2 q1, P2 r1, P2 p2, P2 q2, P2 r2)
{
    if(orient2(r2, p2, q1) >= 0.f)
    {
        if(orient2(p1, p2, q1) >= 0.f) return orient2(p1, q1, r2) >= 0.f;
        if(orient2(q1, r1, p2) >= 0.f) return orient2(r1, p1, p2) >= 0.f;
        return 0;
    }
    if(orient2(r2, p2, r1) >= 0.f && orient2(p1, p2, r1) >= 0.f)
        return orient2(p1, r1, r2) >= 0.f || orient2(q1, r1, r2) >= 0.f;
    return 0;
}

// both triangles counter-clockwise
inline int ccw_overlap_2d(P2 p1, P2 q1, P2 r1, P2 p2, P2 q2, P2 r2)
{
    const bool s0 = orient2(p2, q2, p1) >= 0.f;
    const bool s1 = orient2(q2, r2, p1) >= 0.f;
    if(s0)
    {
        if(s1)
        {
            if(orient2(r2, p2, p1) >= 0.f) return 1;
            return edge_region(p1, q1, r1, p2, q2, r2);
        }
        if(orient2(r2, p2, p1) >= 0.f) return edge_region(p1, q1, r1, r2, p2, q2);
        return vertex_region(p1, q1, r1, p2, q2, r2);
    }
    if(s1)
    {
        if(orient2(r2, p2, p1) >= 0.f) return edge_region(p1, q1, r1, q2, r2, p2);
        return vertex_region(p1, q1, r1, q2, r2, p2);
    }
    return vertex_region(p1, q1, r1, r2, p2, q2);
}

inline int overlap_2d(P2 p1, P2 q1, P2 r1, P2 p2, P2 q2, P2 r2)
{
    const bool cw1 = orient2(p1, q1, r1) < 0.f, cw2 = orient2(p2, q2, r2) < 0.f;
    P2 b1 = cw1 ? r1 : q1, c1 = cw1 ? q1 : r1;
    P2 b2 = cw2 ? r2 : q2, c2 = cw2 ? q2 : r2;
    return ccw_overlap_2d(p1, b1, c1, p2, b2, c2);
}

inline int coplanar(P3 p1, P3 q1, P3 r1, P3 p2, P3 q2, P3 r2, const float n1[3])
{
    const float nx = n1[0] < 0.f ? -n1[0] : n1[0];
    const float ny = n1[1] < 0.f ? -n1[1] : n1[1];
    const float nz = n1[2] < 0.f ? -n1[2] : n1[2];
    float P[6][2];
    P3 src[6] = {p1, q1, r1, p2, q2, r2};
    // projection onto the plane of largest area; the first two vertices swap for the YZ / XZ cases
    int ax0, ax1;
    bool swap_pq;
    if(nx > nz && nx >= ny) { ax0 = 2; ax1 = 1; swap_pq = true; }
    else if(ny > nz && ny >= nx) { ax0 = 0; ax1 = 2; swap_pq = true; }
    else { ax0 = 0; ax1 = 1; swap_pq = false; }
    for(int t = 0; t < 2; ++t)
    {
        P3 a = src[3 * t], b = src[3 * t + 1], c = src[3 * t + 2];
        if(swap_pq) std::swap(a, b);
        P[3 * t][0] = a[ax0]; P[3 * t][1] = a[ax1];
        P[3 * t + 1][0] = b[ax0]; P[3 * t + 1][1] = b[ax1];
        P[3 * t + 2][0] = c[ax0]; P[3 * t + 2][1] = c[ax1];
    }
    return overlap_2d(P[0], P[1], P[2], P[3], P[4], P[5]);
}

// permute T2 into the canonical form for a T1 triple already canonical (a1 positive side)
inline int place_t2(P3 a1, P3 b1, P3 c1, P3 p2, P3 q2, P3 r2, float dp, float dq, float dr, const float n1[3])
{
    if(dp > 0.f)
    {
        if(dq > 0.f) return interval_test(a1, c1, b1, r2, p2, q2);
        if(dr > 0.f) return interval_test(a1, c1, b1, q2, r2, p2);
        return interval_test(a1, b1, c1, p2, q2, r2);
    }
    if(dp < 0.f)
    {
        if(dq < 0.f) return interval_test(a1, b1, c1, r2, p2, q2);
        if(dr < 0.f) return interval_test(a1, b1, c1, q2, r2, p2);
        return interval_test(a1, c1, b1, p2, q2, r2);
    }
    if(dq < 0.f)
    {
        if(dr >= 0.f) return interval_test(a1, c1, b1, q2, r2, p2);
        return interval_test(a1, b1, c1, p2, q2, r2);
    }
    if(dq > 0.f)
    {
        if(dr > 0.f) return interval_test(a1, c1, b1, p2, q2, r2);
        return interval_test(a1, b1, c1, q2, r2, p2);
    }
    if(dr > 0.f) return interval_test(a1, b1, c1, r2, p2, q2);
    if(dr < 0.f) return interval_test(a1, c1, b1, r2, p2, q2);
    return coplanar(a1, b1, c1, p2, q2, r2, n1);
}

inline int overlap_3d(P3 p1, P3 q1, P3 r1, P3 p2, P3 q2, P3 r2)
{
    float u[3], w[3], n1[3], n2[3];
    sub(p2, r2, u);
    sub(q2, r2, w);
    cross(u, w, n2);
    sub(p1, r2, u);
    float dp1 = dot(u, n2);
    sub(q1, r2, u);
    float dq1 = dot(u, n2);
    sub(r1, r2, u);
    float dr1 = dot(u, n2);
    if(dp1 * dq1 > 0.f && dp1 * dr1 > 0.f) return 0;
    sub(q1, p1, u);
    sub(r1, p1, w);
    cross(u, w, n1);
    sub(p2, r1, u);
    float dp2 = dot(u, n1);
    sub(q2, r1, u);
    float dq2 = dot(u, n1);
    sub(r2, r1, u);
    float dr2 = dot(u, n1);
    if(dp2 * dq2 > 0.f && dp2 * dr2 > 0.f) return 0;
    auto clamp0 = [](float &x) {
        if(std::fabs(x) <= EPS) x = 0.f;
    };
    clamp0(dp1); clamp0(dq1); clamp0(dr1);
    clamp0(dp2); clamp0(dq2); clamp0(dr2);
    // permute T1 so its lone vertex comes first; T2 orientation flips with T1's side
    if(dp1 > 0.f)
    {
        if(dq1 > 0.f) return place_t2(r1, p1, q1, p2, r2, q2, dp2, dr2, dq2, n1);
        if(dr1 > 0.f) return place_t2(q1, r1, p1, p2, r2, q2, dp2, dr2, dq2, n1);
        return place_t2(p1, q1, r1, p2, q2, r2, dp2, dq2, dr2, n1);
    }
    if(dp1 < 0.f)
    {
        if(dq1 < 0.f) return place_t2(r1, p1, q1, p2, q2, r2, dp2, dq2, dr2, n1);
        if(dr1 < 0.f) return place_t2(q1, r1, p1, p2, q2, r2, dp2, dq2, dr2, n1);
        return place_t2(p1, q1, r1, p2, r2, q2, dp2, dr2, dq2, n1);
    }
    if(dq1 < 0.f)
    {
        if(dr1 >= 0.f) return place_t2(q1, r1, p1, p2, r2, q2, dp2, dr2, dq2, n1);
        return place_t2(p1, q1, r1, p2, q2, r2, dp2, dq2, dr2, n1);
    }
    if(dq1 > 0.f)
    {
        if(dr1 > 0.f) return place_t2(p1, q1, r1, p2, r2, q2, dp2, dr2, dq2, n1);
        return place_t2(q1, r1, p1, p2, q2, r2, dp2, dq2, dr2, n1);
    }
    if(dr1 > 0.f) return place_t2(r1, p1, q1, p2, q2, r2, dp2, dq2, dr2, n1);
    if(dr1 < 0.f) return place_t2(r1, p1, q1, p2, r2, q2, dp2, dr2, dq2, n1);
    return coplanar(p1, q1, r1, p2, q2, r2, n1);
}
}// namespace tt

vkg_status vkg_intersect_triangle_triangle(const float a[9], const float b[9], uint32_t *out)
{
    if(!a || !b || !out) return VKG_ERR_INVALID_ARGUMENT;
    *out = static_cast<uint32_t>(tt::overlap_3d(a, a + 3, a + 6, b, b + 3, b + 6));
    return VKG_OK;
}

// ---- geometry ----------------------------------------------------------------------------------

static inline void radius_normalize(const float v[3], float radius, float *out)
{
    float inv = 1.0f / std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    for(int i = 0; i < 3; ++i) out[i] = radius * (v[i] * inv);
}

vkg_status vkg_geometry_icosphere_counts(uint32_t tess, uint32_t *num_vertices, uint32_t *num_tris)
{
    if(tess > 12) return VKG_ERR_CAPACITY;
    uint64_t nv = 12, nt = 20;
    for(uint32_t i = 0; i < tess; ++i)
    {
        nv += 3 * nt;
        nt *= 4;
    }
    if(num_vertices) *num_vertices = static_cast<uint32_t>(nv);
    if(num_tris) *num_tris = static_cast<uint32_t>(nt);
    return VKG_OK;
}

// Geometry.cpp:566-613 with tessellate() (Geometry.cpp:141-192): each subdivided triangle appends
// three new vertices (ac, ab, bc) = (k, k+1, k+2) placed at radius * normalize(sum of endpoints).
vkg_status vkg_geometry_icosphere(float radius, uint32_t tess, float *xyz, uint32_t *indices)
{
    if(!xyz || !indices) return VKG_ERR_INVALID_ARGUMENT;
    uint32_t nv_final, nt_final;
    if(vkg_geometry_icosphere_counts(tess, &nv_final, &nt_final) != VKG_OK) return VKG_ERR_CAPACITY;
    const float phi = 1.61803398874989484820f;
    const float e1 = radius / std::sqrt(1.f + phi * phi);
    const float e2 = phi * e1;
    const float base[12][3] = {{-e1, e2, 0},  {e1, e2, 0},  {-e1, -e2, 0}, {e1, -e2, 0}, {0, -e1, e2},  {0, e1, e2},
                               {0, -e1, -e2}, {0, e1, -e2}, {e2, 0, -e1},  {e2, 0, e1},  {-e2, 0, -e1}, {-e2, 0, e1}};
    std::vector<uint32_t> idx = {0, 11, 5, 0, 5,  1,  0,  1, 7, 0, 7,  10, 0, 10, 11, 1, 5, 9, 5, 11,
                                 4, 11, 10, 2, 10, 7,  6,  7, 1, 8, 3,  9,  4, 3,  4, 2, 3, 2, 6,  3,
                                 6, 8,  3,  8, 9,  4,  9,  5, 2, 4, 11, 6,  2, 10, 8, 6, 7, 9, 8,  1};
    std::memcpy(xyz, base, sizeof(base));
    uint32_t nv = 12;
    for(uint32_t it = 0; it < tess; ++it)
    {
        std::vector<uint32_t> next;
        next.reserve(idx.size() * 4);
        for(size_t j = 0; j < idx.size(); j += 3)
        {
            const uint32_t a = idx[j], b = idx[j + 1], c = idx[j + 2], k = nv;
            next.insert(next.end(), {a, k + 1, k, k + 1, b, k + 2, k, k + 2, c, k, k + 1, k + 2});
            float s[3];
            for(int q = 0; q < 3; ++q) s[q] = xyz[3 * a + q] + xyz[3 * b + q];
            radius_normalize(s, radius, xyz + 3 * (k + 1));
            for(int q = 0; q < 3; ++q) s[q] = xyz[3 * a + q] + xyz[3 * c + q];
            radius_normalize(s, radius, xyz + 3 * k);
            for(int q = 0; q < 3; ++q) s[q] = xyz[3 * b + q] + xyz[3 * c + q];
            radius_normalize(s, radius, xyz + 3 * (k + 2));
            nv += 3;
        }
        idx.swap(next);
    }
    std::memcpy(indices, idx.data(), idx.size() * sizeof(uint32_t));
    return VKG_OK;
}

// Cube-sphere: 6 faces of n x n quads, each quad two counter-clockwise (outward) triangles.
static const float CS_N[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
static const float CS_U[6][3] = {{0, 0, -1}, {0, 0, 1}, {1, 0, 0}, {1, 0, 0}, {1, 0, 0}, {-1, 0, 0}};

static void cubesphere(float radius, const float center[3], uint32_t n, float *xyz, uint32_t *idx, uint32_t vbase)
{
    const uint32_t vpf = (n + 1) * (n + 1);
    for(uint32_t f = 0; f < 6; ++f)
    {
        const float *N = CS_N[f], *U = CS_U[f];
        const float V[3] = {N[1] * U[2] - U[1] * N[2], N[2] * U[0] - U[2] * N[0], N[0] * U[1] - U[0] * N[1]};
        for(uint32_t j = 0; j <= n; ++j)
            for(uint32_t i = 0; i <= n; ++i)
            {
                const float a = static_cast<float>(2 * i) / static_cast<float>(n) - 1.0f;
                const float b = static_cast<float>(2 * j) / static_cast<float>(n) - 1.0f;
                float q[3], p[3];
                for(int c = 0; c < 3; ++c) q[c] = (N[c] + a * U[c]) + b * V[c];
                radius_normalize(q, radius, p);
                float *dst = xyz + 3 * static_cast<size_t>(f * vpf + j * (n + 1) + i);
                for(int c = 0; c < 3; ++c) dst[c] = p[c] + center[c];
            }
        for(uint32_t j = 0; j < n; ++j)
            for(uint32_t i = 0; i < n; ++i)
            {
                const uint32_t v00 = vbase + f * vpf + j * (n + 1) + i, v10 = v00 + 1, v01 = v00 + (n + 1),
                               v11 = v01 + 1;
                uint32_t *t = idx + 6 * static_cast<size_t>((f * n + j) * n + i);
                const uint32_t tt[6] = {v00, v10, v11, v00, v11, v01};
                std::memcpy(t, tt, sizeof(tt));
            }
    }
}

vkg_status vkg_scene_cornell_counts(uint32_t num_spheres, uint32_t n, uint32_t *num_vertices, uint32_t *num_tris,
                                    uint32_t *num_materials)
{
    if(n == 0 || n > 1024 || num_spheres > 100000) return VKG_ERR_CAPACITY;
    const uint64_t nv = 20 + (uint64_t)num_spheres * 6 * (n + 1) * (n + 1);
    const uint64_t nt = 10 + (uint64_t)num_spheres * 12 * n * n;
    if(nv >= (1ull << 32) || nt >= MAX_TRIS) return VKG_ERR_CAPACITY;
    if(num_vertices) *num_vertices = static_cast<uint32_t>(nv);
    if(num_tris) *num_tris = static_cast<uint32_t>(nt);
    if(num_materials) *num_materials = 3 + num_spheres;
    return VKG_OK;
}

// Cornell box: back (z=-1), floor (y=-1), ceiling (y=+1) white 0.73; left (x=-1) red; right (x=+1)
// green; roughness 1, metalness 0, two-sided; faces point into the box; open toward +z. Spheres are
// closed one-sided meshes (back faces culled for path rays). Spheres: PCG32
// (seed, stream) draws per sphere, in order: radius U[0.1,0.4]; centre U[-1+r, 1-r]^3;
// roughness U[0.05, 1]; metalness Bernoulli(0.3); base colour U[0.1, 0.9]^3.
vkg_status vkg_scene_cornell(uint64_t seed, uint64_t stream, uint32_t num_spheres, uint32_t n, float *xyz,
                             uint32_t *indices, uint32_t *tri_material, vkg_material *materials)
{
    uint32_t nv, nt, nm;
    if(vkg_scene_cornell_counts(num_spheres, n, &nv, &nt, &nm) != VKG_OK) return VKG_ERR_CAPACITY;
    if(!xyz || !indices) return VKG_ERR_INVALID_ARGUMENT;
    static const float CB[20][3] = {{-1, -1, -1}, {1, -1, -1},  {1, 1, -1},   {-1, 1, -1}, {-1, -1, 1},
                                    {1, -1, 1},   {1, -1, -1},  {-1, -1, -1}, {-1, 1, -1}, {1, 1, -1},
                                    {1, 1, 1},    {-1, 1, 1},   {-1, -1, 1},  {-1, -1, -1}, {-1, 1, -1},
                                    {-1, 1, 1},   {1, -1, -1},  {1, -1, 1},   {1, 1, 1},   {1, 1, -1}};
    static const uint32_t CBM[5] = {0, 0, 0, 1, 2};
    std::memcpy(xyz, CB, sizeof(CB));
    for(uint32_t q = 0; q < 5; ++q)
    {
        const uint32_t a = 4 * q;
        const uint32_t t[6] = {a, a + 1, a + 2, a, a + 2, a + 3};
        std::memcpy(indices + 6 * q, t, sizeof(t));
        if(tri_material) tri_material[2 * q] = tri_material[2 * q + 1] = CBM[q];
    }
    if(materials)
    {
        const float cols[3][3] = {{0.73f, 0.73f, 0.73f}, {0.65f, 0.05f, 0.05f}, {0.12f, 0.45f, 0.15f}};
        for(int m = 0; m < 3; ++m)
        {
            vkg_material mat;
            vkg_material_defaults(&mat);
            std::memcpy(mat.base_color, cols[m], sizeof(cols[m]));
            mat.roughness = 1.f;
            mat.metalness = 0.f;
            mat.twosided = 1u; // walls block light from both sides (closed box)
            materials[m] = mat;
        }
    }
    pcg32 g = pcg32_seed(seed, stream);
    const uint32_t vps = 6 * (n + 1) * (n + 1), tps = 12 * n * n;
    for(uint32_t s = 0; s < num_spheres; ++s)
    {
        const float radius = 0.1f + 0.3f * u01(pcg32_next(g));
        const float lo = -1.0f + radius, hi = 1.0f - radius;
        float center[3];
        for(int c = 0; c < 3; ++c) center[c] = lo + (hi - lo) * u01(pcg32_next(g));
        const float rough = 0.05f + 0.95f * u01(pcg32_next(g));
        const float metal = u01(pcg32_next(g)) < 0.3f ? 1.0f : 0.0f;
        float base[3];
        for(int c = 0; c < 3; ++c) base[c] = 0.1f + 0.8f * u01(pcg32_next(g));
        const uint32_t vb = 20 + s * vps;
        cubesphere(radius, center, n, xyz + 3 * static_cast<size_t>(vb),
                   indices + 3 * static_cast<size_t>(10 + s * tps), vb);
        if(tri_material)
            for(uint32_t t = 0; t < tps; ++t) tri_material[10 + s * tps + t] = 3 + s;
        if(materials)
        {
            vkg_material mat;
            vkg_material_defaults(&mat);
            std::memcpy(mat.base_color, base, sizeof(base));
            mat.roughness = rough;
            mat.metalness = metal;
            materials[3 + s] = mat;
        }
    }
    return VKG_OK;
}

vkg_status vkg_light_convert(const vkg_light_source *src, const float rotation[9], const float translation[3],
                             vkg_light *out)
{
    if(!src || !rotation || !translation || !out) return VKG_ERR_INVALID_ARGUMENT;
    // convert_light (punctual_light.hpp:92-111): position from the translation, direction = R (0,0,-1),
    // tangent = R (1,0,0), the spot cone as scale / offset of the cosine
    vkg_light l{};
    for(int c = 0; c < 3; ++c)
    {
        l.position[c] = translation[c];
        l.color[c] = src->color[c];
        l.direction[c] = -rotation[3 * c + 2];
        l.tangent[c] = rotation[3 * c];
    }
    l.type = src->type;
    l.intensity = src->intensity;
    l.range = src->range > 0.f ? src->range : std::numeric_limits<float>::infinity();
    l.spot_angle_scale = 1.f / std::max(0.001f, std::cos(src->inner_cone_angle) - std::cos(src->outer_cone_angle));
    l.spot_angle_offset = -std::cos(src->outer_cone_angle) * l.spot_angle_scale;
    l.size_x = src->size[0];
    l.size_y = src->size[1];
    *out = l;
    return VKG_OK;
}

vkg_status vkg_material_defaults(vkg_material *m)
{
    if(!m) return VKG_ERR_INVALID_ARGUMENT;
    // the reference's material_struct_t defaults (RayBuilder.hpp:42-66, Material.hpp:125-129)
    *m = vkg_material{};
    for(int c = 0; c < 3; ++c) m->base_color[c] = m->diffuse_transmission_color[c] = 1.f;
    m->roughness = 1.f;
    m->ior = 1.5f;
    m->iridescence_ior = 1.3f;
    m->iridescence_thickness = 400.f;
    for(int c = 0; c < 3; ++c) m->attenuation_color[c] = m->scatter_color[c] = 1.f;
    m->attenuation_distance = std::numeric_limits<float>::infinity();
    m->tex_color = m->tex_normal = m->tex_emission = m->tex_ao_rough_metal = m->tex_transmission = VKG_NO_TEXTURE;
    m->tex_diffuse_transmission = m->tex_diffuse_transmission_color = VKG_NO_TEXTURE;
    m->alpha = 1.f;
    m->blend_mode = VKG_BLEND_OPAQUE;
    m->alpha_cutoff = 0.5f;
    m->has_uv_transform = 0u;
    m->uv_transform[0] = m->uv_transform[4] = 1.f;
    return VKG_OK;
}

vkg_status vkg_camera_lookat(const float eye[3], const float target[3], const float up[3], float tan_half_fovy,
                             uint32_t width, uint32_t height, vkg_camera *out)
{
    if(!eye || !target || !up || !out || width == 0 || height == 0) return VKG_ERR_INVALID_ARGUMENT;
    auto norm = [](const float v[3], float r[3]) {
        float inv = 1.0f / std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        for(int i = 0; i < 3; ++i) r[i] = v[i] * inv;
    };
    float f[3] = {target[0] - eye[0], target[1] - eye[1], target[2] - eye[2]}, fw[3], r[3], rr[3], u[3];
    norm(f, fw);
    r[0] = fw[1] * up[2] - up[1] * fw[2];
    r[1] = fw[2] * up[0] - up[2] * fw[0];
    r[2] = fw[0] * up[1] - up[0] * fw[1];
    norm(r, rr);
    u[0] = rr[1] * fw[2] - fw[1] * rr[2];
    u[1] = rr[2] * fw[0] - fw[2] * rr[0];
    u[2] = rr[0] * fw[1] - fw[0] * rr[1];
    for(int i = 0; i < 3; ++i)
    {
        out->eye[i] = eye[i];
        out->right[i] = rr[i];
        out->up[i] = u[i];
        out->back[i] = -fw[i];
    }
    out->tan_half_fovy = tan_half_fovy;
    out->aspect = static_cast<float>(width) / static_cast<float>(height);
    out->width = width;
    out->height = height;
    return VKG_OK;
}

}// extern "C"
