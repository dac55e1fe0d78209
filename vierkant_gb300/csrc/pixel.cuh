// Per-pixel record helpers: octahedral normal encoding with two snorm16 values and RGBA8 colours,
// as the reference packs its pixel_data_t.
//   normalized_vector_to_octahedral_mapping / octahedral_mapping_to_normalized_vector,
//   pack_snorm_2x16 / unpack_snorm_2x16   shaders/slang/utils/octahedral_map.slang:9-55
//   color_cast                           shaders/slang/utils/color.slang:6-18
#pragma once

#include "internal.hpp"

#include <cmath>

namespace vkg
{

#if defined(__CUDACC__)
#define VKG_HD __host__ __device__ __forceinline__
#else
#define VKG_HD inline
#endif

VKG_HD float2 oct_encode(float x, float y, float z)
{
    const float s = 1.f / (fabsf(x) + fabsf(y) + fabsf(z));
    float px = x * s, py = y * s;
    if(z < 0.f)
    {
        const float qx = (1.f - fabsf(py)) * (px >= 0.f ? 1.f : -1.f);
        const float qy = (1.f - fabsf(px)) * (py >= 0.f ? 1.f : -1.f);
        px = qx;
        py = qy;
    }
    return make_float2(px, py);
}

VKG_HD float3 oct_decode(float px, float py)
{
    float nx = px, ny = py;
    const float nz = 1.f - fabsf(px) - fabsf(py);
    if(nz < 0.f)
    {
        nx = (1.f - fabsf(py)) * (px >= 0.f ? 1.f : -1.f);
        ny = (1.f - fabsf(px)) * (py >= 0.f ? 1.f : -1.f);
    }
    const float inv = 1.f / sqrtf(nx * nx + ny * ny + nz * nz);
    return make_float3(nx * inv, ny * inv, nz * inv);
}

// two snorm16 in the low / high half of a word (round to nearest even, NaN -> 0)
VKG_HD uint32_t pack_snorm_2x16(float x, float y)
{
    if(x != x || y != y) return 0u;
    x = fminf(fmaxf(x, -1.f), 1.f);
    y = fminf(fmaxf(y, -1.f), 1.f);
    const int ix = (int)rintf(x * 32767.f), iy = (int)rintf(y * 32767.f);
    return ((uint32_t)ix & 0xFFFFu) | ((uint32_t)iy << 16);
}

VKG_HD float2 unpack_snorm_2x16(uint32_t p)
{
    const int ix = (int)(int16_t)(p & 0xFFFFu), iy = (int)(int16_t)(p >> 16);
    return make_float2(fmaxf((float)ix / 32767.f, -1.f), fmaxf((float)iy / 32767.f, -1.f));
}

// RGBA8: each channel clamped to [0, 1], times 255, truncated
VKG_HD uint32_t pack_rgba8(float r, float g, float b, float a)
{
    auto q = [](float v) { return (uint32_t)(fminf(fmaxf(v, 0.f), 1.f) * 255.f); };
    return q(r) | (q(g) << 8) | (q(b) << 16) | (q(a) << 24);
}

VKG_HD float3 unpack_rgb8(uint32_t c)
{
    return make_float3((float)(c & 0xFFu) / 255.f, (float)((c >> 8) & 0xFFu) / 255.f,
                       (float)((c >> 16) & 0xFFu) / 255.f);
}

#undef VKG_HD

}// namespace vkg
