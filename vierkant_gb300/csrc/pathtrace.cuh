// Device math of the path tracer: environment lookup / importance sampling, vierkant's Disney BSDF
// (all lobes, iridescence included), sampling helpers and MIS weights.
//
// Restated from the reference shaders:
//   sample_disney / eval_disney   shaders/slang/ray/bsdf_disney.slang:162-296, :298-381
//   EvalDiffuse / EvalSpecular / EvalClearcoat  bsdf_disney.slang:142-160, :97-110, :129-140
//   EvalDielectricReflection / Refraction       bsdf_disney.slang:44-58, :79-95
//   GTR2, SmithGGX, SchlickFresnel, DielectricFresnel  shaders/slang/utils/bsdf.slang:9-13, :160-172, :24-33
//   sample_GTR1                   shaders/slang/utils/sampling.slang:120-129
//   local_frame, sample_GGX_VNDF, sample_hemisphere_cosine  shaders/slang/utils/sampling.slang:16-22, :79-118
//   power_heuristic               shaders/slang/ray/direct_lighting.slang:140-144
//   environment_white             shaders/slang/utils/procedural_environment.slang:7-11
//   panorama mapping              shaders/slang/unlit/panorama.slang:12-15
#pragma once

#include "internal.hpp"

#include <cuda_fp16.h>

namespace vkg
{

constexpr float PT_PI = 3.14159265358979323846f;
constexpr float PT_ONE_OVER_PI = 0.31830988618379067154f;
constexpr float PT_EPS = 1e-4f;     // ray::EPS (ray_common.slang:12)
constexpr float PT_PDF_EPS = 1e-3f; // ray::PDF_EPS (ray_common.slang:13)
constexpr float PT_TMAX = 1e4f;     // ray::DEFAULT_TMAX (ray_common.slang:15)
constexpr float PT_REGULARIZE_PDF_THRESHOLD = 1e3f; // raypipeline.slang:24
constexpr float PT_REGULARIZE_MIN_ROUGHNESS = 0.25f; // raypipeline.slang:25
// path flag bits (stored in the .w word of the path's radiance record)
constexpr uint32_t PATH_REGULARIZE = 1u; // a bounce with pdf < PT_REGULARIZE_PDF_THRESHOLD happened
constexpr uint32_t PATH_CAUSTIC = 2u;    // the reference's caustic_path marker
constexpr uint32_t PATH_NO_ENV_NEE = 4u; // the last vertex was a scattering event (no environment NEE there)

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

// back faces of a material's triangles are traced, not culled: two-sided surfaces, and objects that
// rays enter and leave (dielectric or diffuse transmission)
__host__ __device__ inline bool material_unculled(const vkg_material &m)
{
    return m.twosided != 0u || m.transmission > 0.f || m.diffuse_transmission > 0.f || m.null_surface != 0u ||
           (m.attenuation_distance > 0.f && m.attenuation_distance < 3.0e38f);
}

// a material whose candidate hits are tested for coverage (alpha mask or blend; null surfaces are
// not, raypipeline.slang:694-695)
__host__ __device__ inline bool material_alpha_tested(const vkg_material &m)
{
    return (m.blend_mode == VKG_BLEND_MASK || m.blend_mode == VKG_BLEND_BLEND) && m.null_surface == 0u;
}

// a material that uses a lobe beyond metal-roughness (the shade kernels' FULL variant)
__host__ __device__ inline bool material_full(const vkg_material &m)
{
    return m.transmission > 0.f || m.clearcoat > 0.f || m.diffuse_transmission > 0.f || m.sheen_color[0] > 0.f ||
           m.sheen_color[1] > 0.f || m.sheen_color[2] > 0.f || m.iridescence > 0.f || m.null_surface != 0u ||
           (m.attenuation_distance > 0.f && m.attenuation_distance < 3.0e38f);
}

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

// ---- chromatic dispersion (utils/bsdf.slang:46-91) -------------------------------------------------
__host__ __device__ inline bool material_dispersive(const vkg_material &m) { return m.dispersion > 0.f && m.transmission > 0.f; }

// Cauchy n(lambda) = A + B / lambda^2 (lambda in nm): B from the KHR_materials_dispersion spread
// n_F - n_C = (ior - 1) dispersion / 20 between the F (486.1 nm) and C (656.3 nm) lines, A so that
// n(587.6 nm, the d-line) = ior
__device__ __forceinline__ float cauchy_ior(float ior, float dispersion, float lambda)
{
    const float lambda_d = 587.6f;
    const float half_spread = fmul(fmul(fsub(ior, 1.f), 0.025f), dispersion);
    const float B = fmul(1046907.5f, half_spread); // 2 half_spread / (1/486.1^2 - 1/656.3^2)
    const float A = fsub(ior, fdiv(B, fmul(lambda_d, lambda_d)));
    return fadd(A, fdiv(B, fmul(lambda, lambda)));
}

// piecewise Gaussian of the CIE 1931 colour-matching fit (Wyman, Sloan & Shirley, JCGT 2013)
__device__ __forceinline__ float gaussian_lobe(float x, float mu, float sigma1, float sigma2)
{
    const float t = fmul(fsub(x, mu), x < mu ? fdiv(1.f, sigma1) : fdiv(1.f, sigma2));
    return expf(fmul(fmul(-0.5f, t), t));
}

// one wavelength (nm) -> linear Rec.709 RGB, negatives clamped (the fit's out-of-gamut colours)
__device__ __forceinline__ float3 lambda_to_rgb(float lambda)
{
    const float x = fsub(fadd(fmul(1.056f, gaussian_lobe(lambda, 599.8f, 37.9f, 31.0f)),
                              fmul(0.362f, gaussian_lobe(lambda, 442.0f, 16.0f, 26.7f))),
                         fmul(0.065f, gaussian_lobe(lambda, 501.1f, 20.4f, 26.2f)));
    const float y = fadd(fmul(0.821f, gaussian_lobe(lambda, 568.8f, 46.9f, 40.5f)),
                         fmul(0.286f, gaussian_lobe(lambda, 530.9f, 16.3f, 31.1f)));
    const float z = fadd(fmul(1.217f, gaussian_lobe(lambda, 437.0f, 11.8f, 36.0f)),
                         fmul(0.681f, gaussian_lobe(lambda, 459.0f, 26.0f, 13.8f)));
    // XYZ -> Rec.709 (row vector times the matrix, as the shader's mul(xyz, XYZ_TO_REC709))
    const float r = fadd(fadd(fmul(x, 3.2404542f), fmul(y, -1.5371385f)), fmul(z, -0.4985314f));
    const float g = fadd(fadd(fmul(x, -0.9692660f), fmul(y, 1.8760108f)), fmul(z, 0.0415560f));
    const float b = fadd(fadd(fmul(x, 0.0556434f), fmul(y, -0.2040259f)), fmul(z, 1.0572252f));
    return make_float3(fmaxf(r, 0.f), fmaxf(g, 0.f), fmaxf(b, 0.f));
}

// white balance of a uniform wavelength in [400, 700] nm (utils/bsdf.slang:79-80)
constexpr float LAMBDA_RGB_NORM_R = 1.703734f, LAMBDA_RGB_NORM_G = 2.601105f, LAMBDA_RGB_NORM_B = 2.757475f;

// ---- BSDF (bsdf_disney.slang) --------------------------------------------------------------------
struct material_view
{
    float3 base;
    float roughness; // perceptual roughness (squared into alpha by the BSDF)
    float metalness;
    float transmission, clearcoat, clearcoat_roughness;
    float3 sheen_color;
    float sheen_roughness;
    float diffuse_transmission;
    float3 dt_color;
    float iridescence, iri_ior, iri_thickness;
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
// unpolarised Fresnel reflectance of a dielectric interface, eta = n_incident / n_transmitted
// (utils/bsdf.slang:24-33)
__device__ __forceinline__ float dielectric_fresnel(float cos_i, float eta)
{
    float s2 = eta * eta * (1.f - cos_i * cos_i);
    if(s2 >= 1.f) return 1.f;
    float cos_t = sqrtf(fmaxf(1.f - s2, 0.f));
    float rs = (eta * cos_t - cos_i) / (eta * cos_t + cos_i);
    float rp = (eta * cos_i - cos_t) / (eta * cos_i + cos_t);
    return 0.5f * (rs * rs + rp * rp);
}
// refract(i, n, eta) of the shading languages: the zero vector on total internal reflection
__device__ __forceinline__ float3 refract3(float3 i, float3 n, float eta)
{
    float ni = dot(n, i);
    float k = 1.f - eta * eta * (1.f - ni * ni);
    if(k < 0.f) return f3(0.f, 0.f, 0.f);
    return i * eta - n * (eta * ni + sqrtf(k));
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

// GTR1 half vector (sampling.slang:120-129)
__device__ __forceinline__ float3 sample_gtr1(float x, float y, float roughness)
{
    float a = fmaxf(0.001f, roughness);
    float a2 = a * a;
    float phi = y * 2.f * PT_PI;
    float ct = sqrtf((1.f - powf(a2, 1.f - x)) / (1.f - a2));
    float st = fminf(fmaxf(sqrtf(1.f - ct * ct), 0.f), 1.f);
    return f3(st * cosf(phi), st * sinf(phi), ct);
}

// ---- thin-film iridescence (utils/bsdf.slang:15-17, :34-48, :83-150) ------------------------------
__device__ __forceinline__ float f_schlick(float c, float f0) { return f0 + (1.f - f0) * powf(1.f - c, 5.f); }
__device__ __forceinline__ float ior_to_f0(float t, float i)
{
    float v = (t - i) / (t + i);
    return v * v;
}
// XYZ -> linear Rec.709 (row vector times the reference's XYZ_TO_REC709 rows)
__device__ __forceinline__ float3 xyz_to_rec709(float x, float y, float z)
{
    return f3(x * 3.2404542f + y * -1.5371385f + z * -0.4985314f, x * -0.9692660f + y * 1.8760108f + z * 0.0415560f,
              x * 0.0556434f + y * -0.2040259f + z * 1.0572252f);
}
// evalSensitivity (utils/bsdf.slang:83-100): the Fourier transform of the CIE colour matching
// functions as Gaussians, val * sqrt(2 pi var) * cos(pos * phase + shift) * exp(-phase^2 var) per
// component (two Gaussians for X). Kept as its cosines c and Gaussians e so that the term of twice the
// optical path difference and phase shift follows without further transcendentals.
struct sensitivity_terms
{
    float c[4], e[4]; // X, Y, Z, second X Gaussian
};
__device__ __forceinline__ sensitivity_terms sensitivity_cos_exp(float opd, float3 shift)
{
    const float phase = 2.f * PT_PI * opd * 1.0e-9f, phase2 = phase * phase;
    sensitivity_terms t;
    t.c[0] = cosf(1.6810e+06f * phase + shift.x);
    t.c[1] = cosf(1.7953e+06f * phase + shift.y);
    t.c[2] = cosf(2.2084e+06f * phase + shift.z);
    t.c[3] = cosf(2.2399e+06f * phase + shift.x);
    t.e[0] = expf(-phase2 * 4.3278e+09f);
    t.e[1] = expf(-phase2 * 9.3046e+09f);
    t.e[2] = expf(-phase2 * 6.6121e+09f);
    t.e[3] = expf(-phase2 * 4.5282e+09f);
    return t;
}
// the terms at twice the path difference and phase shift
__device__ __forceinline__ sensitivity_terms sensitivity_double(const sensitivity_terms &t)
{
    sensitivity_terms d;
    for(int k = 0; k < 4; ++k)
    {
        d.c[k] = 2.f * t.c[k] * t.c[k] - 1.f;
        const float e2 = t.e[k] * t.e[k];
        d.e[k] = e2 * e2;
    }
    return d;
}
__device__ __forceinline__ float3 sensitivity_rgb(const sensitivity_terms &t)
{
    const float vx = 5.4856e-13f, vy = 4.4201e-13f, vz = 5.2481e-13f;
    const float sx = 4.3278e+09f, sy = 9.3046e+09f, sz = 6.6121e+09f;
    float x = vx * sqrtf(2.f * PT_PI * sx) * t.c[0] * t.e[0];
    float y = vy * sqrtf(2.f * PT_PI * sy) * t.c[1] * t.e[1];
    float z = vz * sqrtf(2.f * PT_PI * sz) * t.c[2] * t.e[2];
    x += 9.7470e-14f * sqrtf(2.f * PT_PI * 4.5282e+09f) * t.c[3] * t.e[3];
    const float inv = 1.f / 1.0685e-7f;
    return xyz_to_rec709(x * inv, y * inv, z * inv);
}
// Fresnel of a thin film of ior `film` over a base of reflectance f0, seen from outside ior `outside`.
// Not inlined: its eight cosines and exponentials would otherwise be copied into every lobe evaluation
// of every caller, and the shade kernel's code then outgrows the instruction cache
static __device__ __noinline__ float3 iridescent_fresnel(float outside, float film, float3 f0, float thickness, float cos1)
{
    const float R0 = ior_to_f0(film, outside);
    const float R12 = f_schlick(cos1, R0);
    const float T121 = 1.f - R12;
    const float r = outside / film;
    const float sin2sq = r * r * (1.f - cos1 * cos1);
    const float cos2sq = 1.f - sin2sq;
    if(cos2sq < 0.f) return f3(1.f, 1.f, 1.f);
    const float cos2 = sqrtf(cos2sq);
    auto base_ior = [](float f) {
        const float q = sqrtf(fminf(fmaxf(f, 0.f), 0.9999f) + 0.0001f);
        return (1.f + q) / (1.f - q);
    };
    const float3 bi = f3(base_ior(f0.x), base_ior(f0.y), base_ior(f0.z));
    const float3 R23 = f3(f_schlick(cos2, ior_to_f0(bi.x, film)), f_schlick(cos2, ior_to_f0(bi.y, film)),
                          f_schlick(cos2, ior_to_f0(bi.z, film)));
    const float phi12 = film < outside ? PT_PI : 0.f, phi21 = PT_PI - phi12;
    const float3 phi = f3(phi21 + (bi.x < film ? PT_PI : 0.f), phi21 + (bi.y < film ? PT_PI : 0.f),
                          phi21 + (bi.z < film ? PT_PI : 0.f));
    const float opd = 2.f * film * thickness * cos2;
    auto cl = [](float v) { return fminf(fmaxf(v, 1e-5f), 0.9999f); };
    const float3 R123 = f3(cl(R12 * R23.x), cl(R12 * R23.y), cl(R12 * R23.z));
    const float3 r123 = f3(sqrtf(R123.x), sqrtf(R123.y), sqrtf(R123.z));
    const float3 Rs = f3(T121 * T121 * R23.x / (1.f - R123.x), T121 * T121 * R23.y / (1.f - R123.y),
                         T121 * T121 * R23.z / (1.f - R123.z));
    float3 I = f3(R12, R12, R12) + Rs;
    float3 Cm = Rs - f3(T121, T121, T121);
    // the two terms m = 1, 2 of the reference's loop: the m = 2 term's cosines and Gaussians follow from
    // the m = 1 term's (cos 2a = 2 cos^2 a - 1, exp(-4 p^2 s) = exp(-p^2 s)^4), halving the
    // transcendental calls
    const sensitivity_terms t1 = sensitivity_cos_exp(opd, phi);
    Cm = Cm * r123;
    I = I + Cm * (sensitivity_rgb(t1) * 2.f);
    Cm = Cm * r123;
    I = I + Cm * (sensitivity_rgb(sensitivity_double(t1)) * 2.f);
    return f3(fmaxf(I.x, 0.f), fmaxf(I.y, 0.f), fmaxf(I.z, 0.f));
}

// EvalDiffuse with the sheen term (bsdf_disney.slang:142-160)
__device__ __forceinline__ float3 eval_diffuse(const material_view &m, float alpha, float sheen_r, float3 V, float3 N,
                                               float3 L, float3 H, float &pdf)
{
    pdf = 0.f;
    float nol = dot(N, L);
    if(nol <= 0.f) return f3(0.f, 0.f, 0.f);
    pdf = nol * PT_ONE_OVER_PI;
    float loh = dot(L, H);
    float fl = schlick_fresnel(nol), fv = schlick_fresnel(dot(N, V)), fh = schlick_fresnel(loh);
    float fd90 = 0.5f + 2.f * loh * loh * alpha;
    float fd = lerpf(1.f, fd90, fl) * lerpf(1.f, fd90, fv);
    float k = PT_ONE_OVER_PI * (1.f - m.metalness);
    return m.base * (k * fd) + m.sheen_color * (k * fh * sheen_r);
}

// EvalSpecular (bsdf_disney.slang:97-110)
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

// EvalClearcoat (bsdf_disney.slang:129-140): GTR2 with clearcoat_roughness, Smith with alpha 0.25
__device__ __forceinline__ float eval_clearcoat(float cc_rough, float cc, float3 V, float3 N, float3 L, float3 H,
                                                float &pdf)
{
    pdf = 0.f;
    if(dot(N, L) <= 0.f) return 0.f;
    float noh = dot(N, H);
    float d = gtr2(noh, cc_rough);
    pdf = d * noh / (4.f * dot(V, H));
    float f = lerpf(0.04f, 1.f, schlick_fresnel(dot(L, H)));
    float g = smith_ggx(dot(N, L), 0.25f) * smith_ggx(fabsf(dot(N, V)), 0.25f);
    return 0.25f * cc * f * d * g;
}

// EvalDielectricReflection (bsdf_disney.slang:44-58)
__device__ __forceinline__ float3 eval_dielectric_reflection(float alpha, float3 color, float eta, float3 V, float3 N,
                                                             float3 L, float3 H, float &pdf)
{
    pdf = 0.f;
    if(dot(N, L) <= 0.f) return f3(0.f, 0.f, 0.f);
    float F = dielectric_fresnel(dot(V, H), eta);
    float d = gtr2(dot(N, H), alpha);
    float sv = smith_ggx(fabsf(dot(N, V)), alpha);
    pdf = 0.5f * d * sv * F;
    float g = smith_ggx(fabsf(dot(N, L)), alpha) * sv;
    return color * (F * d * g);
}

// EvalDielectricRefraction (bsdf_disney.slang:79-95)
__device__ __forceinline__ float3 eval_dielectric_refraction(float alpha, float3 color, float eta, float3 V, float3 N,
                                                             float3 L, float3 H, float &pdf)
{
    pdf = 0.f;
    if(dot(N, L) >= 0.f) return f3(0.f, 0.f, 0.f);
    float loh = dot(L, H), voh = dot(V, H);
    float denom = loh + voh * eta;
    if(fabsf(denom) < 1e-7f) return f3(0.f, 0.f, 0.f);
    float F = dielectric_fresnel(fabsf(voh), eta);
    float d = gtr2(dot(N, H), alpha);
    float sv = smith_ggx(fabsf(dot(N, V)), alpha);
    float jac = fabsf(loh) * eta * eta / (denom * denom);
    pdf = 2.f * sv * d * fabsf(voh) * (1.f - F) * jac;
    float g = smith_ggx(fabsf(dot(N, L)), alpha) * sv;
    return color * ((1.f - F) * d * g * fabsf(voh) * 4.f * jac);
}

// EvalSpecularIridescence (bsdf_disney.slang:112-127)
__device__ __forceinline__ float3 eval_specular_iridescence(float alpha, float film_ior, float thickness, float3 cspec0,
                                                            float3 V, float3 N, float3 L, float3 H, float &pdf,
                                                            bool with_value = true)
{
    pdf = 0.f;
    if(dot(N, L) <= 0.f) return f3(0.f, 0.f, 0.f);
    float d = gtr2(dot(N, H), alpha);
    float sv = smith_ggx(fabsf(dot(N, V)), alpha);
    pdf = 0.5f * d * sv;
    if(!with_value) return f3(0.f, 0.f, 0.f);
    const float3 F = iridescent_fresnel(1.f, film_ior, cspec0, thickness, dot(V, H));
    float g = smith_ggx(fabsf(dot(N, L)), alpha) * sv;
    return F * (d * g);
}

// EvalDielectricReflectionIridescence (bsdf_disney.slang:60-77)
__device__ __forceinline__ float3 eval_dielectric_reflection_iridescence(float alpha, float3 color, float film_ior,
                                                                         float thickness, float3 cspec0, float eta,
                                                                         float3 V, float3 N, float3 L, float3 H,
                                                                         float &pdf, bool with_value = true)
{
    pdf = 0.f;
    if(dot(N, L) <= 0.f) return f3(0.f, 0.f, 0.f);
    const float voh = dot(V, H);
    float F = dielectric_fresnel(voh, eta);
    float d = gtr2(dot(N, H), alpha);
    float sv = smith_ggx(fabsf(dot(N, V)), alpha);
    pdf = 0.5f * d * sv * F;
    if(!with_value) return f3(0.f, 0.f, 0.f);
    float g = smith_ggx(fabsf(dot(N, L)), alpha) * sv;
    const float3 irF = iridescent_fresnel(1.f, film_ior, cspec0, thickness, voh);
    return color * irF * (d * g);
}

struct bsdf_sample
{
    float3 dir;
    float pdf; // pdf of the sampled lobe times its selection probability (sample_disney's pdf)
    float3 f;  // the sampled lobe's value
    bool transmission;
};

// sample_disney (bsdf_disney.slang:162-296). The reference draws a fresh random number for each lobe
// decision; here u_lobe alone makes them all, rescaled to [0, 1) inside the chosen branch, so every
// path segment uses a fixed count of draws. (x, y) drive the half vector or the cosine lobe, and y
// also makes the Fresnel reflect / refract choice of the dielectric lobe (as the reference's Xi.y does).
// eta = n_incident / n_transmitted of the hit face.
__device__ __forceinline__ bsdf_sample sample_bsdf(const material_view &m, float3 N, float3 V, float eta,
                                                   float u_lobe, float x, float y)
{
    bsdf_sample r;
    r.transmission = false;
    float diffuse_ratio = 0.5f * (1.f - m.metalness);
    float trans_weight = (1.f - m.metalness) * m.transmission;
    float alpha = fmaxf(0.001f, m.roughness * m.roughness);
    float3 spec = lerp3(f3(0.08f, 0.08f, 0.08f), m.base, m.metalness);
    frame3 fr = local_frame(N);
    if(trans_weight > 0.f && u_lobe < trans_weight)
    {
        float3 H = to_world(fr, sample_ggx_vndf(x, y, to_local(fr, V), alpha));
        if(dot(V, H) < 0.f) H = -H;
        const float3 R = reflect3(-V, H);
        const float F = dielectric_fresnel(fabsf(dot(R, H)), eta);
        float3 refr = f3(0.f, 0.f, 0.f);
        if(!(y < F)) refr = refract3(-V, H, eta);
        if(y < F)
        {
            // reflection: plain or thin-film, by the rescaled lobe uniform
            r.dir = normalize(R);
            const float ut = u_lobe / trans_weight;
            if(m.iridescence > 0.f && ut < m.iridescence)
            {
                r.f = eval_dielectric_reflection_iridescence(alpha, m.base, m.iri_ior, m.iri_thickness, spec, eta, V, N,
                                                             r.dir, H, r.pdf);
                r.pdf *= m.iridescence;
            }
            else
            {
                r.f = eval_dielectric_reflection(alpha, m.base, eta, V, N, r.dir, H, r.pdf);
                if(m.iridescence > 0.f) r.pdf *= 1.f - m.iridescence;
            }
        }
        else if(dot(refr, refr) < 1e-7f)
        {
            // total internal reflection
            r.dir = normalize(R);
            r.f = eval_dielectric_reflection(alpha, m.base, eta, V, N, r.dir, H, r.pdf);
        }
        else
        {
            r.dir = normalize(refr);
            r.f = eval_dielectric_refraction(alpha, m.base, eta, V, N, r.dir, H, r.pdf);
            r.transmission = true;
        }
        r.f = r.f * trans_weight;
        r.pdf *= trans_weight;
    }
    else
    {
        const float u = trans_weight > 0.f ? (u_lobe - trans_weight) / (1.f - trans_weight) : u_lobe;
        if(u < diffuse_ratio)
        {
            const float dt = m.diffuse_transmission;
            const float ud = u / diffuse_ratio;
            const float3 c = sample_hemisphere_cosine(x, y);
            if(dt > 0.f && ud < dt)
            {
                // Lambertian transmission: the cosine lobe of the opposite hemisphere
                r.dir = to_world(fr, f3(c.x, c.y, -c.z));
                r.f = m.dt_color * (dt * PT_ONE_OVER_PI);
                r.pdf = c.z * PT_ONE_OVER_PI * diffuse_ratio * dt;
                r.transmission = true;
            }
            else
            {
                r.dir = to_world(fr, c);
                float3 H = normalize(r.dir + V);
                r.f = eval_diffuse(m, alpha, fmaxf(0.001f, m.sheen_roughness), V, N, r.dir, H, r.pdf) * (1.f - dt);
                r.pdf *= diffuse_ratio * (1.f - dt);
            }
        }
        else
        {
            const float primary = 1.f / (1.f + m.clearcoat);
            const float us = (u - diffuse_ratio) / (1.f - diffuse_ratio);
            if(!(m.clearcoat > 0.f) || us < primary)
            {
                float3 H = to_world(fr, sample_ggx_vndf(x, y, to_local(fr, V), alpha));
                if(dot(V, H) < 0.f) H = -H;
                r.dir = normalize(reflect3(-V, H));
                const float ui = us / primary;
                if(m.iridescence > 0.f && ui < m.iridescence)
                {
                    r.f = eval_specular_iridescence(alpha, m.iri_ior, m.iri_thickness, spec, V, N, r.dir, H, r.pdf);
                    r.pdf *= primary * (1.f - diffuse_ratio) * m.iridescence;
                }
                else
                {
                    r.f = eval_specular(alpha, spec, V, N, r.dir, H, r.pdf);
                    r.pdf *= m.iridescence > 0.f ? primary * (1.f - diffuse_ratio) * (1.f - m.iridescence)
                                                 : primary * (1.f - diffuse_ratio);
                }
            }
            else
            {
                float3 H = to_world(fr, sample_gtr1(x, y, lerpf(0.1f, 0.001f, m.clearcoat)));
                if(dot(V, H) < 0.f) H = -H;
                r.dir = normalize(reflect3(-V, H));
                const float c = eval_clearcoat(m.clearcoat_roughness, m.clearcoat, V, N, r.dir, H, r.pdf);
                r.f = f3(c, c, c);
                r.pdf *= (1.f - primary) * (1.f - diffuse_ratio);
            }
        }
        r.f = r.f * (1.f - trans_weight);
        r.pdf *= 1.f - trans_weight;
    }
    if(isnan(r.pdf)) r.pdf = 0.f;
    return r;
}

// eval_disney (bsdf_disney.slang:298-381): value and mixture pdf (the sum over lobes). The clearcoat
// lobe is skipped when clearcoat == 0, where its value and pdf weight are 0.
// VALUE = false: the mixture pdf only (the thin-film Fresnel is skipped; every other value term is
// dead code the compiler removes)
template<bool VALUE = true>
__device__ __forceinline__ float3 eval_bsdf(const material_view &m, float3 L, float3 N, float3 V, float eta, float &pdf)
{
    pdf = 0.f;
    const bool refl = dot(N, L) > 0.f;
    float3 lpv = refl ? L + V : L + V * eta;
    float len = sqrtf(dot(lpv, lpv));
    if(len < 1e-7f) return f3(0.f, 0.f, 0.f);
    float3 H = lpv * (1.f / len);
    if(dot(V, H) < 0.f) H = -H;
    if(refl && dot(N, H) <= 0.f) return f3(0.f, 0.f, 0.f);
    float diffuse_ratio = 0.5f * (1.f - m.metalness);
    float primary = 1.f / (1.f + m.clearcoat);
    float trans_weight = (1.f - m.metalness) * m.transmission;
    float alpha = fmaxf(0.001f, m.roughness * m.roughness);
    float3 spec = lerp3(f3(0.08f, 0.08f, 0.08f), m.base, m.metalness);
    float3 brdf = f3(0.f, 0.f, 0.f), bsdf = brdf;
    float brdf_pdf = 0.f, bsdf_pdf = 0.f, mp;
    const float s_ir = m.iridescence;
    if(trans_weight > 0.f)
    {
        if(refl)
        {
            bsdf = eval_dielectric_reflection(alpha, m.base, eta, V, N, L, H, bsdf_pdf);
            if(s_ir > 0.f)
            {
                bsdf = bsdf * (1.f - s_ir);
                bsdf_pdf *= 1.f - s_ir;
                const float3 b2 = eval_dielectric_reflection_iridescence(alpha, m.base, m.iri_ior, m.iri_thickness,
                                                                         spec, eta, V, N, L, H, mp, VALUE);
                bsdf = bsdf + b2 * s_ir;
                bsdf_pdf += mp * s_ir;
            }
        }
        else bsdf = eval_dielectric_refraction(alpha, m.base, eta, V, N, L, H, bsdf_pdf);
    }
    if(trans_weight < 1.f)
    {
        const float dt = m.diffuse_transmission;
        brdf = eval_diffuse(m, alpha, fmaxf(0.001f, m.sheen_roughness), V, N, L, H, mp) * (1.f - dt);
        brdf_pdf = mp * diffuse_ratio * (1.f - dt);
        if(dt > 0.f && !refl)
        {
            brdf = brdf + m.dt_color * (dt * PT_ONE_OVER_PI);
            brdf_pdf += -dot(N, L) * PT_ONE_OVER_PI * diffuse_ratio * dt;
        }
        if(s_ir > 0.f)
        {
            brdf = brdf + eval_specular(alpha, spec, V, N, L, H, mp) * (1.f - s_ir);
            brdf_pdf += mp * primary * (1.f - diffuse_ratio) * (1.f - s_ir);
            brdf = brdf + eval_specular_iridescence(alpha, m.iri_ior, m.iri_thickness, spec, V, N, L, H, mp, VALUE) * s_ir;
            brdf_pdf += mp * primary * (1.f - diffuse_ratio) * s_ir;
        }
        else
        {
            brdf = brdf + eval_specular(alpha, spec, V, N, L, H, mp);
            brdf_pdf += mp * primary * (1.f - diffuse_ratio);
        }
        if(m.clearcoat > 0.f)
        {
            const float c = eval_clearcoat(m.clearcoat_roughness, m.clearcoat, V, N, L, H, mp);
            brdf = brdf + f3(c, c, c);
            brdf_pdf += mp * (1.f - primary) * (1.f - diffuse_ratio);
        }
    }
    float p = lerpf(brdf_pdf, bsdf_pdf, trans_weight);
    if(!(p > 0.f)) return f3(0.f, 0.f, 0.f);
    pdf = p;
    return lerp3(brdf, bsdf, trans_weight);
}

// eval_bsdf as one out-of-line copy: the full-material shade kernel evaluates the BSDF at three places
// (environment NEE, light NEE, the MIS pdf of the bounce), and three inlined copies of every lobe
// overflow the instruction cache
static __device__ __noinline__ float3 eval_bsdf_ool(material_view m, float3 L, float3 N, float3 V, float eta,
                                                    float &pdf)
{
    return eval_bsdf(m, L, N, V, eta, pdf);
}
// the mixture pdf alone (the MIS pdf of a bounce), out of line for the same reason
static __device__ __noinline__ float pdf_bsdf_ool(material_view m, float3 L, float3 N, float3 V, float eta)
{
    float pdf;
    eval_bsdf<false>(m, L, N, V, eta, pdf);
    return pdf;
}

// the material record as the BSDF reads it; FULL = false reads only the metal-roughness fields and
// makes the other lobes compile-time zero (for scenes whose materials have none of them)
template<bool FULL = true>
__device__ __forceinline__ material_view load_material(const vkg_material *mats, uint32_t id, bool disable_material)
{
    const vkg_material &q = mats[id];
    material_view m;
    m.base = disable_material ? f3(0.8f, 0.8f, 0.8f) : f3(q.base_color[0], q.base_color[1], q.base_color[2]);
    m.roughness = q.roughness;
    m.metalness = q.metalness;
    if constexpr(!FULL)
    {
        m.transmission = m.clearcoat = m.clearcoat_roughness = m.sheen_roughness = m.diffuse_transmission = 0.f;
        m.sheen_color = m.dt_color = f3(0.f, 0.f, 0.f);
        m.iridescence = m.iri_ior = m.iri_thickness = 0.f;
        return m;
    }
    m.iridescence = q.iridescence;
    m.iri_ior = q.iridescence_ior;
    m.iri_thickness = q.iridescence_thickness;
    m.transmission = q.transmission;
    m.clearcoat = q.clearcoat;
    m.clearcoat_roughness = q.clearcoat_roughness;
    m.sheen_color = f3(q.sheen_color[0], q.sheen_color[1], q.sheen_color[2]);
    m.sheen_roughness = q.sheen_roughness;
    m.diffuse_transmission = q.diffuse_transmission;
    m.dt_color = f3(q.diffuse_transmission_color[0], q.diffuse_transmission_color[1], q.diffuse_transmission_color[2]);
    return m;
}

// eta of a hit (raypipeline.slang:489-491) for an object in vacuum: entering through a front face
// 1 / ior, leaving through a back face ior, plus the reference's EPS; 1 for opaque materials
__device__ __forceinline__ float hit_eta(const vkg_material *mats, uint32_t id, bool back_face)
{
    const float t = mats[id].transmission;
    if(!(t > 0.f)) return 1.f;
    const float ior = mats[id].ior;
    return (back_face ? ior : 1.f / ior) + PT_EPS;
}

// the same for a surface whose ior is given (a dispersive surface's Cauchy ior)
__device__ __forceinline__ float hit_eta_ior(float ior, bool back_face) { return (back_face ? ior : 1.f / ior) + PT_EPS; }

// direct_lighting.slang:140-144
__device__ __forceinline__ float power_heuristic(float pa, float pb)
{
    float r = pb / pa;
    return 1.f / (1.f + r * r);
}

#endif // __CUDACC__

}// namespace vkg
