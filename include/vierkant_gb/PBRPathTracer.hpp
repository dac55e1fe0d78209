// vierkant_gb/PBRPathTracer.hpp -- C++20 counterpart of vierkant::PBRPathTracer over the C ABI.
//
// Mirrors include/vierkant/PBRPathTracer.hpp:35-182: PBRPathTracerPtr (shared ownership), create(...)
// with a create_info_t holding the seed and the settings, a public `settings` member, render_scene,
// current_batch, reset_accumulator and statistics; non-copyable and non-movable. The Vulkan parts are
// replaced: the Rasterizer and the output images by a caller-owned device buffer (crop width x height x
// 3 fp32), the Scene by vierkant::gb::scene (geometry, materials and environment already in device
// memory), the camera object by a vkg_camera. Rendering is asynchronous on the caller's stream.
#pragma once

#include <memory>

#include "raytracing.hpp"

namespace vierkant::gb
{

class scene;
using ScenePtr = std::shared_ptr<scene>;

//! a path-tracer scene (vkg_scene): one mesh with per-triangle materials and an equirect environment
class scene
{
public:
    static ScenePtr create(const ContextPtr &ctx, const vkg_scene_desc &desc, void *stream = nullptr)
    {
        vkg_scene *s = nullptr;
        ctx->check(vkg_scene_create(ctx->handle(), &desc, &s, stream), "vkg_scene_create");
        return ScenePtr(new scene(ctx, s));
    }

    //! instanced scene: one BVH per mesh under a two-level BVH over the instances
    static ScenePtr create(const ContextPtr &ctx, const vkg_instanced_scene_desc &desc, void *stream = nullptr)
    {
        vkg_scene *s = nullptr;
        ctx->check(vkg_scene_create_instanced(ctx->handle(), &desc, &s, stream), "vkg_scene_create_instanced");
        return ScenePtr(new scene(ctx, s));
    }

    scene(const scene &) = delete;

    scene &operator=(const scene &) = delete;

    ~scene() { vkg_scene_destroy(m_ctx->handle(), m_scene); }

    [[nodiscard]] const vkg_scene *handle() const { return m_scene; }

    [[nodiscard]] vkg_scene *handle() { return m_scene; }

private:
    scene(ContextPtr ctx, vkg_scene *s) : m_ctx(std::move(ctx)), m_scene(s) {}

    ContextPtr m_ctx;
    vkg_scene *m_scene = nullptr;
};

class PBRPathTracer;
using PBRPathTracerPtr = std::shared_ptr<PBRPathTracer>;

class PBRPathTracer
{
public:
    //! settings_t, PBRPathTracer.hpp:42-110 (same field names)
    using settings_t = vkg_settings;

    //! statistics_t / timings_t, PBRPathTracer.hpp:112-127, of the last render
    using statistics_t = vkg_tracer_stats;

    //! create_info_t, PBRPathTracer.hpp:129-141: the seed and the initial settings
    struct create_info_t
    {
        uint32_t seed = 0;
        settings_t settings = default_settings();
    };

    //! what one render_scene call did
    struct render_result_t
    {
        uint32_t num_samples = 0; //!< paths per pixel traced by this call (0 once max_num_batches is reached)
        uint32_t batch = 0;       //!< the accumulator's batch index after the call
    };

    static settings_t default_settings()
    {
        settings_t s{};
        check(vkg_settings_default(&s), "vkg_settings_default");
        return s;
    }

    //! PBRPathTracer::create, PBRPathTracer.hpp:144
    static PBRPathTracerPtr create(const ContextPtr &ctx, const create_info_t &create_info)
    {
        vkg_tracer_create_info info{create_info.seed, create_info.settings};
        vkg_tracer *t = nullptr;
        ctx->check(vkg_tracer_create(ctx->handle(), &info, &t), "vkg_tracer_create");
        return PBRPathTracerPtr(new PBRPathTracer(ctx, t, create_info.settings));
    }

    PBRPathTracer(const PBRPathTracer &) = delete;

    PBRPathTracer(PBRPathTracer &&) = delete;

    PBRPathTracer &operator=(PBRPathTracer other) = delete;

    ~PBRPathTracer() { vkg_tracer_destroy(m_tracer); }

    //! PBRPathTracer::render_scene, PBRPathTracer.hpp:161-162: applies `settings`, traces one batch
    //! of settings.num_samples paths per pixel and blends it into the running mean; d_rgb_out (may be
    //! null) receives the accumulated image
    render_result_t render_scene(const ScenePtr &scene, const vkg_camera &cam, float *d_rgb_out,
                                 void *stream = nullptr)
    {
        m_ctx->check(vkg_tracer_set_settings(m_tracer, &settings), "vkg_tracer_set_settings");
        uint32_t before = current_batch();
        m_ctx->check(vkg_tracer_render(m_tracer, scene->handle(), &cam, d_rgb_out, stream), "vkg_tracer_render");
        uint32_t after = current_batch();
        return {after != before ? settings.num_samples : 0u, after};
    }

    //! PBRPathTracer::current_batch, PBRPathTracer.hpp:169
    [[nodiscard]] size_t current_batch() const
    {
        uint32_t b = 0;
        m_ctx->check(vkg_tracer_current_batch(m_tracer, &b), "vkg_tracer_current_batch");
        return b;
    }

    //! PBRPathTracer::reset_accumulator, PBRPathTracer.hpp:174
    void reset_accumulator() { m_ctx->check(vkg_tracer_reset_accumulator(m_tracer), "vkg_tracer_reset_accumulator"); }

    //! PBRPathTracer::statistics, PBRPathTracer.hpp:179 (the last render's; waits for it)
    [[nodiscard]] statistics_t statistics() const
    {
        statistics_t s{};
        m_ctx->check(vkg_tracer_statistics(m_tracer, &s), "vkg_tracer_statistics");
        return s;
    }

    //! the pixel records (pixel_data_t) of the traced window after the last render
    void pixel_data(vkg_pixel_data *d_out, void *stream = nullptr) const
    {
        m_ctx->check(vkg_tracer_pixel_data(m_tracer, d_out, stream), "vkg_tracer_pixel_data");
    }

    //! access to global settings, PBRPathTracer.hpp:182
    settings_t settings;

private:
    PBRPathTracer(ContextPtr ctx, vkg_tracer *t, const settings_t &s) : settings(s), m_ctx(std::move(ctx)), m_tracer(t)
    {}

    ContextPtr m_ctx;
    vkg_tracer *m_tracer = nullptr;
};

}// namespace vierkant::gb
