// Material textures of the path tracer (the reference's closest-hit texture terms,
// shaders/slang/raypipeline.slang:299-320, :526-606).
//
// Storage: RGBA8 texels (UNORM, as the reference's R8G8B8A8_UNORM textures, model_loading.cpp:12-24),
// every level of every texture in one array; a texture's record holds its size, level count, wrap
// modes and the first texel of each level. Levels are made on the host (vkg_scene_set_textures):
// level k + 1 is the rounded mean of 2 x 2 texels of level k, the last row / column repeated for odd
// sizes.
//
// Sampling (Sampler2D.SampleLevel with linear min / mag / mip filters): lambda clamped to
// [0, levels - 1], bilinear at floor(lambda) and the next level, blended by the fraction; texel
// centres at (i + 0.5) / size; REPEAT, CLAMP_TO_EDGE or MIRRORED_REPEAT per axis.
#pragma once

#include "pathtrace.cuh"

namespace vkg
{

constexpr uint32_t TEX_MAX_LEVELS = 16;

struct alignas(16) tex_rec
{
    uint32_t width, height, levels, wrap; // wrap: s in bits 0-7, t in bits 8-15 (VKG_WRAP_*)
    uint32_t offset[TEX_MAX_LEVELS];      // first texel of each level
};
static_assert(sizeof(tex_rec) == 80, "tex_rec layout");

__device__ __forceinline__ int tex_wrap(int x, int n, uint32_t mode)
{
    if(mode == VKG_WRAP_CLAMP_TO_EDGE) return min(max(x, 0), n - 1);
    if(mode == VKG_WRAP_MIRRORED_REPEAT)
    {
        const int p = 2 * n;
        int m = x % p;
        if(m < 0) m += p;
        return m < n ? m : p - 1 - m;
    }
    int m = x % n;
    return m < 0 ? m + n : m;
}

__device__ __forceinline__ float4 tex_fetch(const uint32_t *__restrict__ texels, uint32_t base, int w, int x, int y)
{
    const uint32_t c = __ldg(&texels[base + (uint32_t)(y * w + x)]);
    constexpr float k = 1.f / 255.f;
    return make_float4((float)(c & 0xFFu) * k, (float)((c >> 8) & 0xFFu) * k, (float)((c >> 16) & 0xFFu) * k,
                       (float)(c >> 24) * k);
}

__device__ __forceinline__ float4 lerp4(float4 a, float4 b, float t)
{
    return make_float4(a.x + (b.x - a.x) * t, a.y + (b.y - a.y) * t, a.z + (b.z - a.z) * t, a.w + (b.w - a.w) * t);
}

__device__ __forceinline__ float4 tex_bilinear(const tex_rec &T, const uint32_t *__restrict__ texels, uint32_t level,
                                               float u, float v)
{
    const int w = max((int)(T.width >> level), 1), h = max((int)(T.height >> level), 1);
    float fx = u * (float)w - 0.5f, fy = v * (float)h - 0.5f;
    if(!(fabsf(fx) < 1e8f)) fx = 0.f; // NaN / huge coordinates: any texel is as good
    if(!(fabsf(fy) < 1e8f)) fy = 0.f;
    const float x0f = floorf(fx), y0f = floorf(fy);
    const float ax = fx - x0f, ay = fy - y0f;
    const int x0 = (int)x0f, y0 = (int)y0f;
    const uint32_t ws = T.wrap & 0xFFu, wt = (T.wrap >> 8) & 0xFFu;
    const int xa = tex_wrap(x0, w, ws), xb = tex_wrap(x0 + 1, w, ws);
    const int ya = tex_wrap(y0, h, wt), yb = tex_wrap(y0 + 1, h, wt);
    const uint32_t base = T.offset[level];
    const float4 top = lerp4(tex_fetch(texels, base, w, xa, ya), tex_fetch(texels, base, w, xb, ya), ax);
    const float4 bot = lerp4(tex_fetch(texels, base, w, xa, yb), tex_fetch(texels, base, w, xb, yb), ax);
    return lerp4(top, bot, ay);
}

// SampleLevel(uv, lambda)
__device__ __forceinline__ float4 tex_sample(const tex_rec &T, const uint32_t *__restrict__ texels, float u, float v,
                                             float lambda)
{
    const float top = (float)(T.levels - 1);
    float l = lambda > 0.f ? lambda : 0.f; // NaN -> level 0
    l = l < top ? l : top;
    const uint32_t l0 = (uint32_t)l;
    const float f = l - (float)l0;
    const float4 a = tex_bilinear(T, texels, l0, u, v);
    if(f > 0.f && l0 + 1 < T.levels) return lerp4(a, tex_bilinear(T, texels, l0 + 1, u, v), f);
    return a;
}

}// namespace vkg
