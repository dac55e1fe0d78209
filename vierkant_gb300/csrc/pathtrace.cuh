// Device math of the path tracer: environment lookup / importance sampling, the metal-roughness
// subset of vierkant's Disney BSDF, sampling helpers and MIS weights.
//
// Restated from the reference shaders (transmission = clearcoat = sheen = iridescence =
// diffuse transmission = 0, the material model of the benchmark scenes):
//   sample_disney / eval_disney   shaders/slang/ray/bsdf_disney.slang:162-296, :298-381
//   EvalDiffuse / EvalSpecular    bsdf_disney.slang:142-160, :97-110
//   GTR2, SmithGGX, SchlickFresnel shaders/slang/utils/bsdf.slang:9-13, :160-172
//   local_frame, sample_GGX_VNDF, sample_hemisphere_cosine  shaders/slang/utils/sampling.slang:16-22, :79-118
//   power_heuristic               shaders/slang/ray/direct_lighting.slang:140-144
//   environment_white             shaders/slang/utils/procedural_environment.slang:7-11
//   panorama mapping              shaders/slang/unlit/panorama.slang:12-15
#pragma once

#include "internal.hpp"

namespace vkg
{

constexpr float PT_PI = 3.14159265358979323846f;
constexpr float PT_ONE_OVER_PI = 0.31830988618379067154f;
constexpr float PT_EPS = 1e-4f;     // ray::EPS (ray_common.slang:12)
constexpr float PT_PDF_EPS = 1e-3f; // ray::PDF_EPS (ray_common.slang:13)
constexpr float PT_TMAX = 1e4f;     // ray::DEFAULT_TMAX (ray_common.slang:15)

struct env_alias
{
    float prob;
    uint32_t alias;
};

struct env_tables
{
    float *rgb = nullptr;      // W*H*3 radiance
    float *pdf_w = nullptr;    // W*H normalised weights (mean 1)
    env_alias *alias = nullptr; // W*H buckets
    uint32_t w = 0, h = 0;
};

vkg_status env_build(vkg_ctx *ctx, const float *d_rgb_in, uint32_t w, uint32_t h, env_tables &out, cudaStream_t st);
void env_free(env_tables &t);

#if defined(__CUDACC__)

__device__ __forceinline__ float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
__device__ __forceinline__ float3 operator+(float3 a, float3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 operator-(float3 a, float3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 operator*(float3 a, float3 b) { return f3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ float3 operator*(float3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float3 operator*(float s, float3 a) { return f3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float3 operator-(float3 a) { return f3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float3 cross(float3 a, float3 b)
{
    return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float3 normalize(float3 v) { return v * (1.f / sqrtf(dot(v, v))); }
__device__ __forceinline__ float max3(float3 v) { return fmaxf(v.x, fmaxf(v.y, v.z)); }
__device__ __forceinline__ float3 lerp3(float3 a, float3 b, float t) { return a + (b - a) * t; }
__device__ __forceinline__ float lerpf(float a, float b, float t) { return a + (b - a) * t; }
__device__ __forceinline__ float3 reflect3(float3 i, float3 n) { return i - n * (2.f * dot(n, i)); }

// ---- environment ------------------------------------------------------------------------------
__device__ __forceinline__ float3 environment_white(float3 d)
{
    const float sky = 1.3f, horizon = 0.6f, ground = 0.1f;
    float v = d.y > 0.f ? lerpf(horizon, sky, d.y) : lerpf(horizon, ground, -d.y);
    return f3(v, v, v);
}

// direction through the centre of texel (i, j) of a w x h equirect map
__device__ __forceinline__ float3 env_texel_dir(uint32_t i, uint32_t j, uint32_t w, uint32_t h)
{
    float u = ((float)i + 0.5f) / (float)w, v = ((float)j + 0.5f) / (float)h;
    float phi = (u - 0.5f) * 2.f * PT_PI, theta = v * PT_PI;
    float st = sinf(theta);
    return f3(st * sinf(phi), cosf(theta), -st * cosf(phi));
}

__device__ __forceinline__ uint32_t env_texel(float3 d, uint32_t w, uint32_t h)
{
    float u = 0.5f + 0.5f * atan2f(d.x, -d.z) * PT_ONE_OVER_PI;
    float v = acosf(fminf(fmaxf(d.y, -1.f), 1.f)) * PT_ONE_OVER_PI;
    uint32_t i = min((uint32_t)fmaxf(u * (float)w, 0.f), w - 1u);
    uint32_t j = min((uint32_t)fmaxf(v * (float)h, 0.f), h - 1u);
    return j * w + i;
}

struct env_view
{
    const float *rgb;
    const float *pdf_w;
    const env_alias *alias;
    uint32_t w, h;
    float factor;
};

__device__ __forceinline__ float3 env_radiance(const env_view &e, uint32_t t)
{
    const float *c = e.rgb + 3 * (size_t)t;
    return f3(__ldg(c), __ldg(c + 1), __ldg(c + 2)) * e.factor;
}

// solid-angle pdf of direction d (texel weight / (2 pi^2 sin theta))
__device__ __forceinline__ float env_pdf(const env_view &e, float3 d, uint32_t t)
{
    float st = sqrtf(fmaxf(0.f, 1.f - d.y * d.y));
    if(st <= 0.f) return 0.f;
    return __ldg(&e.pdf_w[t]) / (2.f * PT_PI * PT_PI * st);
}

// alias-table sample: u0 picks the bucket, u1 the bucket's item, (u2, u3) a point in the texel
__device__ __forceinline__ float3 env_sample(const env_view &e, float u0, float u1, float u2, float u3, float &pdf,
                                             uint32_t &texel)
{
    const uint32_t n = e.w * e.h;
    uint32_t b = min((uint32_t)(u0 * (float)n), n - 1u);
    env_alias a = e.alias[b];
    uint32_t t = u1 < a.prob ? b : a.alias;
    uint32_t i = t % e.w, j = t / e.w;
    float u = ((float)i + u2) / (float)e.w, v = ((float)j + u3) / (float)e.h;
    float phi = (u - 0.5f) * 2.f * PT_PI, theta = v * PT_PI;
    float st = sinf(theta);
    float3 d = f3(st * sinf(phi), cosf(theta), -st * cosf(phi));
    pdf = st > 0.f ? __ldg(&e.pdf_w[t]) / (2.f * PT_PI * PT_PI * st) : 0.f;
    texel = t;
    return d;
}

// ---- BSDF (metal-roughness subset of bsdf_disney.slang) ------------------------------------
struct material_view
{
    float3 base;
    float roughness; // perceptual roughness (squared into alpha by the BSDF)
    float metalness;
};

__device__ __forceinline__ float schlick_fresnel(float u)
{
    float m = fminf(fmaxf(1.f - u, 0.f), 1.f);
    return m * m * m * m * m;
}
__device__ __forceinline__ float gtr2(float ndoth, float a)
{
    float a2 = a * a;
    float t = 1.f + (a2 - 1.f) * ndoth * ndoth;
    return a2 / (PT_PI * t * t);
}
__device__ __forceinline__ float smith_ggx(float ndotv, float alpha)
{
    float a = alpha * alpha, b = ndotv * ndotv;
    return 1.f / (ndotv + sqrtf(a + b - a * b));
}

// local_frame(N): rows (tangent_x, tangent_y, N)
struct frame3
{
    float3 tx, ty, n;
};
__device__ __forceinline__ frame3 local_frame(float3 n)
{
    float len2 = n.x * n.x + n.y * n.y;
    float3 tx = len2 > 0.f ? f3(-n.y, n.x, 0.f) * (1.f / sqrtf(len2)) : f3(1.f, 0.f, 0.f);
    return frame3{tx, cross(n, tx), n};
}
__device__ __forceinline__ float3 to_local(const frame3 &f, float3 v) { return f3(dot(f.tx, v), dot(f.ty, v), dot(f.n, v)); }
__device__ __forceinline__ float3 to_world(const frame3 &f, float3 v) { return f.tx * v.x + f.ty * v.y + f.n * v.z; }

__device__ __forceinline__ float3 sample_hemisphere_cosine(float x, float y)
{
    float phi = 2.f * PT_PI * y;
    float ct = sqrtf(fmaxf(1.f - x, 0.f));
    float st = sqrtf(fmaxf(1.f - ct * ct, 0.f));
    return f3(st * cosf(phi), st * sinf(phi), ct);
}

// Heitz 2018 visible-normal sampling in the spherical-cap form of sampling.slang:98-118
__device__ __forceinline__ float3 sample_ggx_vndf(float x, float y, float3 wi, float alpha)
{
    float3 wstd = normalize(f3(wi.x * alpha, wi.y * alpha, wi.z));
    float phi = (2.f * x - 1.f) * PT_PI;
    float z = fmaf(1.f - y, 1.f + wstd.z, -wstd.z);
    float st = sqrtf(fminf(fmaxf(1.f - z * z, 0.f), 1.f));
    float3 c = f3(st * cosf(phi), st * sinf(phi), z);
    float3 m = c + wstd;
    return normalize(f3(m.x * alpha, m.y * alpha, m.z));
}

__device__ __forceinline__ float3 eval_diffuse(float alpha, float3 color, float metal, float3 V, float3 N, float3 L,
                                               float3 H, float &pdf)
{
    pdf = 0.f;
    float nol = dot(N, L);
    if(nol <= 0.f) return f3(0.f, 0.f, 0.f);
    pdf = nol * PT_ONE_OVER_PI;
    float loh = dot(L, H);
    float fl = schlick_fresnel(nol), fv = schlick_fresnel(dot(N, V));
    float fd90 = 0.5f + 2.f * loh * loh * alpha;
    float fd = lerpf(1.f, fd90, fl) * lerpf(1.f, fd90, fv);
    return color * (PT_ONE_OVER_PI * fd * (1.f - metal));
}

__device__ __forceinline__ float3 eval_specular(float alpha, float3 cspec0, float3 V, float3 N, float3 L, float3 H,
                                                float &pdf)
{
    pdf = 0.f;
    if(dot(N, L) <= 0.f) return f3(0.f, 0.f, 0.f);
    float d = gtr2(dot(N, H), alpha);
    float sv = smith_ggx(fabsf(dot(N, V)), alpha);
    pdf = 0.5f * d * sv;
    float fh = schlick_fresnel(dot(L, H));
    float3 f = lerp3(cspec0, f3(1.f, 1.f, 1.f), fh);
    float g = smith_ggx(fabsf(dot(N, L)), alpha) * sv;
    return f * (d * g);
}

struct bsdf_sample
{
    float3 dir;
    float pdf; // pdf of the sampled lobe times its selection probability (sample_disney's pdf)
    float3 f;  // the sampled lobe's value
};

// sample_disney restricted to the metal-roughness lobes; u_lobe selects diffuse vs specular,
// (x, y) drive the VNDF half vector or the cosine lobe
__device__ __forceinline__ bsdf_sample sample_bsdf(const material_view &m, float3 N, float3 V, float u_lobe, float x,
                                                   float y)
{
    bsdf_sample r;
    float diffuse_ratio = 0.5f * (1.f - m.metalness);
    float alpha = fmaxf(0.001f, m.roughness * m.roughness);
    float3 spec = lerp3(f3(0.08f, 0.08f, 0.08f), m.base, m.metalness);
    frame3 fr = local_frame(N);
    if(u_lobe < diffuse_ratio)
    {
        r.dir = to_world(fr, sample_hemisphere_cosine(x, y));
        float3 H = normalize(r.dir + V);
        r.f = eval_diffuse(alpha, m.base, m.metalness, V, N, r.dir, H, r.pdf);
        r.pdf *= diffuse_ratio;
    }
    else
    {
        float3 H = to_world(fr, sample_ggx_vndf(x, y, to_local(fr, V), alpha));
        if(dot(V, H) < 0.f) H = -H;
        r.dir = normalize(reflect3(-V, H));
        r.f = eval_specular(alpha, spec, V, N, r.dir, H, r.pdf);
        r.pdf *= 1.f - diffuse_ratio;
    }
    if(isnan(r.pdf)) r.pdf = 0.f;
    return r;
}

// eval_disney for the same subset: value and mixture pdf (the sum over lobes)
__device__ __forceinline__ float3 eval_bsdf(const material_view &m, float3 L, float3 N, float3 V, float &pdf)
{
    pdf = 0.f;
    float3 lpv = L + V;
    float len = sqrtf(dot(lpv, lpv));
    if(len < 1e-7f) return f3(0.f, 0.f, 0.f);
    float3 H = lpv * (1.f / len);
    if(dot(V, H) < 0.f) H = -H;
    if(dot(N, L) > 0.f && dot(N, H) <= 0.f) return f3(0.f, 0.f, 0.f);
    float diffuse_ratio = 0.5f * (1.f - m.metalness);
    float alpha = fmaxf(0.001f, m.roughness * m.roughness);
    float3 spec = lerp3(f3(0.08f, 0.08f, 0.08f), m.base, m.metalness);
    float pd, ps;
    float3 f = eval_diffuse(alpha, m.base, m.metalness, V, N, L, H, pd);
    f = f + eval_specular(alpha, spec, V, N, L, H, ps);
    float p = pd * diffuse_ratio + ps * (1.f - diffuse_ratio);
    if(!(p > 0.f)) return f3(0.f, 0.f, 0.f);
    pdf = p;
    return f;
}

// direct_lighting.slang:140-144
__device__ __forceinline__ float power_heuristic(float pa, float pb)
{
    float r = pb / pa;
    return 1.f / (1.f + r * r);
}

#endif // __CUDACC__

}// namespace vkg
