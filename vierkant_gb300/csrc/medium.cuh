// Homogeneous participating media of the path tracer: the per-material medium record, the
// Henyey-Greenstein phase function and the per-path medium stack.
//
// Restated from the reference:
//   medium of a boundary material   shaders/slang/raypipeline.slang:493-511 (sigma_t = -log(attenuation
//                                   colour) / distance, Kulla-Conty single-scattering albedo from the
//                                   multi-scatter albedo, emission of null surfaces)
//   free-flight sampling, emission  raypipeline.slang:388-474 (homogeneous branch)
//   media stack Enter / Leave       raypipeline.slang:189-194, :516-523, :656-664 (4 entries, entry 0 vacuum)
//   phase_hg / sample_phase_hg      shaders/slang/utils/phase_function.slang:10-31
#pragma once

#include "pathtrace.cuh"

namespace vkg
{

constexpr uint32_t MEDIUM_VOLUME = 1u; // finite attenuation distance
constexpr uint32_t MEDIUM_NULL = 2u;   // null surface
constexpr uint32_t MEDIA_STACK = 3u;   // pushable entries above vacuum (the reference's MAX_MEDIA_STACK_SIZE 4)

// the medium a material bounds (host-computed table, one record per material)
struct medium_rec
{
    float sigma_s[3], g;
    float sigma_a[3], ior;
    float emission[3];
    uint32_t flags;
};

inline bool material_has_volume(const vkg_material &m)
{
    return m.attenuation_distance > 0.f && m.attenuation_distance < 3.0e38f;
}

// raypipeline.slang:493-511 for a front-face hit of material m
inline medium_rec medium_from_material(const vkg_material &m)
{
    medium_rec r{};
    const bool vol = material_has_volume(m);
    for(int c = 0; c < 3; ++c)
    {
        const float st = vol ? -std::log(m.attenuation_color[c]) / m.attenuation_distance : 0.f;
        const float ms = m.scatter_factor * m.scatter_color[c];
        const float kc = 4.09712f + 4.20863f * ms - std::sqrt(9.59217f + 41.6808f * ms + 17.7126f * ms * ms);
        const float ss = 1.f - kc * kc;
        r.sigma_s[c] = ss * st;
        r.sigma_a[c] = (1.f - ss) * st;
        r.emission[c] = m.null_surface ? m.emission[c] : 0.f;
    }
    r.g = m.phase_g;
    r.ior = m.ior;
    r.flags = (vol ? MEDIUM_VOLUME : 0u) | (m.null_surface ? MEDIUM_NULL : 0u);
    return r;
}

// a medium given directly (media.hpp:26-49 converted as to_media, media.cpp:6-23): always a volume,
// emission colour x intensity
inline medium_rec medium_from_params(const vkg_medium_params &p)
{
    medium_rec r{};
    for(int c = 0; c < 3; ++c)
    {
        const float st = -std::log(p.attenuation_color[c]) / p.attenuation_distance;
        const float ms = p.scatter_factor * p.scatter_color[c];
        const float kc = 4.09712f + 4.20863f * ms - std::sqrt(9.59217f + 41.6808f * ms + 17.7126f * ms * ms);
        const float ss = 1.f - kc * kc;
        r.sigma_s[c] = ss * st;
        r.sigma_a[c] = (1.f - ss) * st;
        r.emission[c] = p.emission_color[c] * p.emission_intensity;
    }
    r.g = p.phase_g;
    r.ior = p.ior;
    r.flags = MEDIUM_VOLUME;
    return r;
}

inline bool medium_params_valid(const vkg_medium_params &p)
{
    auto unit = [](float x) { return x >= 0.f && x <= 1.f; };
    for(int c = 0; c < 3; ++c)
        if(!(p.attenuation_color[c] > 0.f && p.attenuation_color[c] <= 1.f) || !unit(p.scatter_color[c]) ||
           !(p.emission_color[c] >= 0.f) || !std::isfinite(p.emission_color[c]))
            return false;
    return p.attenuation_distance > 0.f && std::isfinite(p.attenuation_distance) && unit(p.scatter_factor) &&
           p.phase_g > -1.f && p.phase_g < 1.f && p.ior > 0.f && std::isfinite(p.ior) &&
           p.emission_intensity >= 0.f && std::isfinite(p.emission_intensity);
}

#if defined(__CUDACC__)

constexpr float PT_ONE_OVER_FOUR_PI = 0.07957747154594766788f;

// Henyey-Greenstein phase function (phase_function.slang:10-14)
__device__ __forceinline__ float phase_hg(float cos_theta, float g)
{
    const float denom = 1.f + g * g - 2.f * g * cos_theta;
    return PT_ONE_OVER_FOUR_PI * (1.f - g * g) / (denom * sqrtf(denom));
}

// a phase-function sample around +z (phase_function.slang:17-31)
__device__ __forceinline__ float3 sample_phase_hg(float x, float y, float g, float &pdf)
{
    const float phi = y * 2.f * PT_PI;
    float ct;
    if(fabsf(g) < 1e-3f) ct = 1.f - 2.f * x;
    else
    {
        const float sq = (1.f - g * g) / (1.f - g + 2.f * g * x);
        ct = (1.f + g * g - sq * sq) / (2.f * g);
    }
    const float st = fminf(fmaxf(sqrtf(1.f - ct * ct), 0.f), 1.f);
    pdf = phase_hg(ct, g);
    return f3(st * cosf(phi), st * sinf(phi), ct);
}

// per-path stack (x: entries above vacuum, y..w: material ids bottom to top)
__device__ __forceinline__ uint32_t stack_top(const uint4 &s)
{
    return s.x == 0 ? 0xFFFFFFFFu : (s.x == 1 ? s.y : (s.x == 2 ? s.z : s.w));
}
__device__ __forceinline__ uint32_t stack_at(const uint4 &s, uint32_t k) // k = 1..x
{
    return k == 1 ? s.y : (k == 2 ? s.z : s.w);
}
// ior of stack entry k (0: vacuum); a null surface keeps the ior of the medium it was entered from
__device__ __forceinline__ float stack_ior(const medium_rec *M, const uint4 &s, uint32_t k)
{
    float ior = 1.f;
    for(uint32_t i = 1; i <= k && i <= s.x; ++i)
    {
        const medium_rec &r = M[stack_at(s, i)];
        if(!(r.flags & MEDIUM_NULL)) ior = r.ior;
    }
    return ior;
}
__device__ __forceinline__ void stack_push(uint4 &s, uint32_t id)
{
    // a full stack overwrites its top entry (the reference: min(index + 1, MAX - 1))
    const uint32_t k = s.x < MEDIA_STACK ? s.x + 1 : MEDIA_STACK;
    s.x = k;
    if(k == 1) s.y = id;
    else if(k == 2) s.z = id;
    else s.w = id;
}
__device__ __forceinline__ void stack_pop(uint4 &s)
{
    if(s.x > 0) s.x -= 1;
}

#endif // __CUDACC__

}// namespace vkg
