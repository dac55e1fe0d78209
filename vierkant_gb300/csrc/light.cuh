// Analytic lights of the path tracer: sampling for next-event estimation, closed-form hits of the
// light bodies by BSDF-sampled rays, the matching solid-angle pdfs and the MIS weights.
//
// Restated from the reference shaders:
//   sample_light                 shaders/slang/ray/direct_lighting.slang:32-137
//   bsdf_reachable, intersect_light  direct_lighting.slang:148-236
//   mis_weight_nee / mis_weight_hit  direct_lighting.slang:239-252
//   light_pdf                    direct_lighting.slang:256-293
//   nee_surface                  direct_lighting.slang:297-332
//   sample_unit_disc / sample_unit_sphere_cap  shaders/slang/utils/sampling.slang:31-40, :55-64
// Lights are emitters only: their bodies never block or terminate a path (the reference's
// "ghost-light" pass, raypipeline.slang:196-224).
#pragma once

#include "pathtrace.cuh"

namespace vkg
{

#if defined(__CUDACC__)

__device__ __forceinline__ float3 lv3(const float *p) { return f3(p[0], p[1], p[2]); }

// spherical cap of half-angle sigma around +z, uniform in solid angle
__device__ __forceinline__ float3 sample_unit_sphere_cap(float x, float y, float sigma)
{
    float phi = 2.f * PT_PI * y;
    float cs = cosf(sigma);
    float ct = x * (1.f - cs) + cs;
    float st = sqrtf(1.f - ct * ct);
    return f3(st * cosf(phi), st * sinf(phi), ct);
}

struct light_sample
{
    float3 dir;   // unit direction from the shading point toward the light
    float dist;   // shadow-ray tmax
    float pdf;    // solid-angle pdf (1 for delta lights)
    float3 radiance; // unshadowed incident radiance (0: no sample)
};

__device__ __forceinline__ light_sample sample_light(const vkg_light &l, float3 P, float x, float y)
{
    light_sample r;
    r.pdf = 1.f;
    r.radiance = lv3(l.color) * l.intensity;
    const float3 ldir = lv3(l.direction);
    if(l.type == VKG_LIGHT_DIRECTIONAL)
    {
        // direction stores the propagation direction
        r.dir = -ldir;
        r.dist = PT_TMAX;
        if(l.angular_size > 0.f)
        {
            // sun disc: a direction in its cone
            r.dir = to_world(local_frame(r.dir), sample_unit_sphere_cap(x, y, l.angular_size));
            r.pdf = 1.f / (2.f * PT_PI * (1.f - cosf(l.angular_size)));
        }
    }
    else if(l.type == VKG_LIGHT_SPHERE)
    {
        const float3 tc = lv3(l.position) - P;
        const float d2 = dot(tc, tc), r2 = l.size_x * l.size_x;
        if(d2 <= r2)
        {
            r.radiance = f3(0.f, 0.f, 0.f);
            r.dir = f3(0.f, 0.f, 1.f);
            r.dist = PT_EPS;
        }
        else
        {
            // the cone the sphere subtends, sampled uniformly (sin sigma = r / d)
            const float sin2 = r2 / d2, cos_s = sqrtf(1.f - sin2);
            r.dir = to_world(local_frame(tc * rsqrtf(d2)), sample_unit_sphere_cap(x, y, asinf(sqrtf(sin2))));
            r.pdf = (1.f + cos_s) / (2.f * PT_PI * sin2);
            const float b = dot(r.dir, tc);
            r.dist = b - sqrtf(fmaxf(b * b - d2 + r2, 0.f));
        }
    }
    else if(l.type == VKG_LIGHT_RECT || l.type == VKG_LIGHT_DISK || l.type == VKG_LIGHT_TUBE)
    {
        // a uniform point Q of the emitting surface with normal n; area pdf -> solid angle
        float3 Q, n;
        const float3 pos = lv3(l.position);
        if(l.type == VKG_LIGHT_RECT)
        {
            const float3 tg = lv3(l.tangent), bt = cross(ldir, tg);
            Q = pos + tg * ((2.f * x - 1.f) * l.size_x) + bt * ((2.f * y - 1.f) * l.size_y);
            n = ldir;
            r.pdf = 1.f / (4.f * l.size_x * l.size_y);
        }
        else if(l.type == VKG_LIGHT_DISK)
        {
            const float rr = sqrtf(x), th = 2.f * PT_PI * y;
            Q = pos + to_world(local_frame(ldir), f3(l.size_x * rr * cosf(th), l.size_x * rr * sinf(th), 0.f));
            n = ldir;
            r.pdf = 1.f / (PT_PI * l.size_x * l.size_x);
        }
        else
        {
            // open cylinder mantle around the axis, emitting radially
            const float phi = 2.f * PT_PI * x;
            n = to_world(local_frame(ldir), f3(cosf(phi), sinf(phi), 0.f));
            Q = pos + ldir * ((2.f * y - 1.f) * l.size_y) + n * l.size_x;
            r.pdf = 1.f / (4.f * PT_PI * l.size_x * l.size_y);
        }
        const float3 tq = Q - P;
        const float d2 = dot(tq, tq);
        r.dist = fmaxf(sqrtf(d2), PT_EPS);
        r.dir = tq * (1.f / r.dist);
        const float cos_l = dot(n, -r.dir);
        r.pdf *= d2 / fmaxf(cos_l, PT_EPS);
        if(cos_l <= 0.f) r.radiance = f3(0.f, 0.f, 0.f); // back side: black, no shadow ray
    }
    else
    {
        // omni / spot: inverse-square falloff with the range window
        const float3 tl = lv3(l.position) - P;
        r.dist = fmaxf(sqrtf(dot(tl, tl)), PT_EPS);
        r.dir = tl * (1.f / r.dist);
        float w = r.dist / l.range;
        w *= w;
        float att = fminf(fmaxf(1.f - w * w, 0.f), 1.f) / (r.dist * r.dist);
        if(l.type == VKG_LIGHT_SPOT)
        {
            const float cd = dot(ldir, -r.dir);
            const float a = fminf(fmaxf(cd * l.spot_angle_scale + l.spot_angle_offset, 0.f), 1.f);
            att *= a * a;
        }
        r.radiance = r.radiance * att;
    }
    return r;
}

// light types that BSDF-sampled rays can reach: sun discs (on miss) and the area bodies
__device__ __forceinline__ bool bsdf_reachable(const vkg_light &l)
{
    return (l.type == VKG_LIGHT_DIRECTIONAL && l.angular_size > 0.f) || l.type == VKG_LIGHT_RECT ||
           l.type == VKG_LIGHT_SPHERE || l.type == VKG_LIGHT_TUBE || l.type == VKG_LIGHT_DISK;
}

// front-facing hit of a light body: (t, cosine at the light); t <= 0 is a miss
__device__ __forceinline__ float2 intersect_light(const vkg_light &l, float3 P, float3 dir)
{
    const float3 pos = lv3(l.position), ldir = lv3(l.direction);
    if(l.type == VKG_LIGHT_SPHERE)
    {
        const float3 tc = pos - P;
        const float d2 = dot(tc, tc), r2 = l.size_x * l.size_x;
        if(d2 <= r2) return make_float2(0.f, 0.f);
        const float b = dot(dir, tc), disc = b * b - d2 + r2;
        if(disc <= 0.f) return make_float2(0.f, 0.f);
        const float t = b - sqrtf(disc);
        if(t <= 0.f) return make_float2(0.f, 0.f);
        return make_float2(t, dot((P + dir * t - pos) * (1.f / l.size_x), -dir));
    }
    if(l.type == VKG_LIGHT_RECT || l.type == VKG_LIGHT_DISK)
    {
        const float cos_l = dot(ldir, -dir);
        if(cos_l <= 0.f) return make_float2(0.f, 0.f);
        const float t = dot(pos - P, ldir) / -cos_l;
        if(t <= 0.f) return make_float2(0.f, 0.f);
        const float3 q = P + dir * t - pos;
        if(l.type == VKG_LIGHT_RECT)
        {
            const float3 tg = lv3(l.tangent), bt = cross(ldir, tg);
            if(fabsf(dot(q, tg)) > l.size_x || fabsf(dot(q, bt)) > l.size_y) return make_float2(0.f, 0.f);
        }
        else if(dot(q, q) > l.size_x * l.size_x)
            return make_float2(0.f, 0.f);
        return make_float2(t, cos_l);
    }
    if(l.type == VKG_LIGHT_TUBE)
    {
        const float3 o = P - pos;
        const float3 dp = dir - ldir * dot(dir, ldir), op = o - ldir * dot(o, ldir);
        const float A = dot(dp, dp), B = dot(op, dp), Cc = dot(op, op) - l.size_x * l.size_x;
        const float disc = B * B - A * Cc;
        if(A <= PT_EPS || disc <= 0.f || Cc <= 0.f) return make_float2(0.f, 0.f);
        const float t = (-B - sqrtf(disc)) / A;
        if(t <= 0.f || fabsf(dot(o + dir * t, ldir)) > l.size_y) return make_float2(0.f, 0.f);
        const float cos_l = dot((op + dp * t) * (1.f / l.size_x), -dir);
        if(cos_l <= 0.f) return make_float2(0.f, 0.f);
        return make_float2(t, cos_l);
    }
    return make_float2(0.f, 0.f);
}

// solid-angle pdf with which sample_light produces direction dir from P
__device__ __forceinline__ float light_pdf(const vkg_light &l, float3 P, float3 dir)
{
    const float3 ldir = lv3(l.direction);
    if(l.type == VKG_LIGHT_DIRECTIONAL)
    {
        if(l.angular_size <= 0.f) return 0.f;
        const float cs = cosf(l.angular_size);
        return dot(dir, -ldir) < cs ? 0.f : 1.f / (2.f * PT_PI * (1.f - cs));
    }
    if(l.type == VKG_LIGHT_SPHERE)
    {
        const float3 tc = lv3(l.position) - P;
        const float d2 = dot(tc, tc), r2 = l.size_x * l.size_x;
        if(d2 <= r2) return 0.f;
        const float sin2 = r2 / d2, cos_s = sqrtf(1.f - sin2);
        return dot(dir, tc * rsqrtf(d2)) < cos_s ? 0.f : (1.f + cos_s) / (2.f * PT_PI * sin2);
    }
    if(l.type == VKG_LIGHT_RECT || l.type == VKG_LIGHT_DISK || l.type == VKG_LIGHT_TUBE)
    {
        const float2 h = intersect_light(l, P, dir);
        if(h.x <= 0.f) return 0.f;
        const float area = l.type == VKG_LIGHT_RECT ? 4.f * l.size_x * l.size_y
                           : l.type == VKG_LIGHT_DISK ? PT_PI * l.size_x * l.size_x
                                                      : 4.f * PT_PI * l.size_x * l.size_y;
        return h.x * h.x / (area * h.y);
    }
    return 0.f;
}

// MIS weights with the estimator switch (mis_mode 0 MIS, 1 NEE only, 2 BSDF only)
__device__ __forceinline__ float mis_weight_nee(uint32_t mode, float p_nee, float p_bsdf)
{
    if(mode == 1) return 1.f;
    if(mode == 2) return 0.f;
    return power_heuristic(p_nee, p_bsdf);
}
__device__ __forceinline__ float mis_weight_hit(uint32_t mode, float prev_pdf, float p_nee)
{
    if(mode == 1) return 0.f;
    if(mode == 2 || prev_pdf <= 0.f) return 1.f;
    return power_heuristic(prev_pdf, p_nee);
}

#endif // __CUDACC__

}// namespace vkg
