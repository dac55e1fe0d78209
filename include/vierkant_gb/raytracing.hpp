// vierkant_gb/raytracing.hpp -- C++20 owners of the C ABI's context and BVH handles.
//
// The reference traces rays through the Vulkan driver's acceleration structures (RayBuilder builds
// them, src/RayBuilder.cpp:98-300; TraceRay / RayQuery query them, shaders/slang/raypipeline.slang:182,
// shaders/slang/ray/visibility_test.slang:45-87). Here a context owns a vkg_ctx and a bvh owns a
// vkg_bvh built on the GPU; both release their handle when the last shared owner goes. Buffers are
// caller-owned device memory (prefix d_), work is asynchronous on the caller's cudaStream_t (passed
// as void*), and a failed call throws vierkant::gb::error with the context's message.
#pragma once

#include <memory>
#include <string>

#include "intersection.hpp"

namespace vierkant::gb
{

class context;
using ContextPtr = std::shared_ptr<context>;

class context
{
public:
    //! a context bound to CUDA device `device` (vkg_ctx_create)
    static ContextPtr create(int device = 0) { return ContextPtr(new context(device)); }

    context(const context &) = delete;

    context &operator=(const context &) = delete;

    ~context() { vkg_ctx_destroy(m_ctx); }

    [[nodiscard]] vkg_ctx *handle() const { return m_ctx; }

    //! vkg_last_error of this context
    [[nodiscard]] std::string last_error() const { return vkg_last_error(m_ctx); }

    //! throws vierkant::gb::error with the context's message if status is not VKG_OK
    void check(vkg_status status, const char *what) const
    {
        if(status != VKG_OK) { throw error(status, std::string(what) + ": " + last_error()); }
    }

    //! node visits and triangle tests counted by launches with VKG_RAY_COUNT_STATS
    void ray_stats(uint64_t &node_visits, uint64_t &tri_tests, bool reset = true) const
    {
        check(vkg_ray_stats_get(m_ctx, &node_visits, &tri_tests, reset ? 1 : 0), "vkg_ray_stats_get");
    }

private:
    explicit context(int device) { vierkant::gb::check(vkg_ctx_create(device, &m_ctx), "vkg_ctx_create"); }

    vkg_ctx *m_ctx = nullptr;
};

class bvh;
using BVHPtr = std::shared_ptr<bvh>;

class bvh
{
public:
    //! builds an 8-wide BVH over an indexed triangle mesh in device memory (fp32 xyz, uint32
    //! indices); synchronises `stream` (vkg_bvh_build)
    static BVHPtr build(const ContextPtr &ctx, const float *d_xyz, uint32_t num_vertices, const uint32_t *d_indices,
                        uint32_t num_tris, uint32_t leaf_max = 0, void *stream = nullptr)
    {
        vkg_bvh_build_options opt{leaf_max};
        vkg_bvh *b = nullptr;
        ctx->check(vkg_bvh_build(ctx->handle(), d_xyz, num_vertices, d_indices, num_tris, &opt, &b, stream),
                   "vkg_bvh_build");
        return BVHPtr(new bvh(ctx, b));
    }

    bvh(const bvh &) = delete;

    bvh &operator=(const bvh &) = delete;

    ~bvh() { vkg_bvh_destroy(m_ctx->handle(), m_bvh); }

    [[nodiscard]] const vkg_bvh *handle() const { return m_bvh; }

    [[nodiscard]] vkg_bvh_info info() const
    {
        vkg_bvh_info i{};
        m_ctx->check(vkg_bvh_info_get(m_bvh, &i), "vkg_bvh_info_get");
        return i;
    }

    //! closest hit per ray: INTERSECT with tmin < t < tmax, smallest t, ties to the smaller triangle id
    void closest_hit(const vkg_ray *d_rays, uint32_t num_rays, vkg_hit *d_hits, uint32_t flags = 0,
                     void *stream = nullptr) const
    {
        m_ctx->check(vkg_closest_hit(m_ctx->handle(), m_bvh, d_rays, num_rays, d_hits, flags, stream),
                     "vkg_closest_hit");
    }

    //! d_occluded[i] = 1 if ray i has any hit with tmin < t < tmax
    void any_hit(const vkg_ray *d_rays, uint32_t num_rays, uint32_t *d_occluded, uint32_t flags = 0,
                 void *stream = nullptr) const
    {
        m_ctx->check(vkg_any_hit(m_ctx->handle(), m_bvh, d_rays, num_rays, d_occluded, flags, stream),
                     "vkg_any_hit");
    }

    //! host buffers in and out; synchronises
    void closest_hit_host(const vkg_ray *h_rays, uint32_t num_rays, vkg_hit *h_hits, uint32_t flags = 0,
                          void *stream = nullptr) const
    {
        m_ctx->check(vkg_closest_hit_host(m_ctx->handle(), m_bvh, h_rays, num_rays, h_hits, flags, stream),
                     "vkg_closest_hit_host");
    }

private:
    bvh(ContextPtr ctx, vkg_bvh *b) : m_ctx(std::move(ctx)), m_bvh(b) {}

    ContextPtr m_ctx;
    vkg_bvh *m_bvh = nullptr;
};

//! pinhole camera looking from eye at target (vkg_camera_lookat); fovy in radians
inline vkg_camera camera_lookat(const vec3 &eye, const vec3 &target, const vec3 &up, float fovy, uint32_t width,
                                uint32_t height)
{
    vkg_camera cam{};
    check(vkg_camera_lookat(eye.data(), target.data(), up.data(), std::tan(fovy / 2.f), width, height, &cam),
          "vkg_camera_lookat");
    return cam;
}

}// namespace vierkant::gb
