// Edge-avoiding a-trous denoiser over the path tracer's pixel records: the reference's denoise pass
// (src/PBRPathTracer.cpp:346-403, shaders/slang/denoise.slang) as CUDA kernels.
//
// Per pass (steps 1, 2, 4, 8, 16; PBRPathTracer.cpp:26) every pixel takes the 5x5 B3-spline kernel
// at offsets k * step (border-clamped) over albedo-demodulated radiance, each tap weighted by
//   exp(-(lum_c - lum_t)^2 / 0.9) * exp(-|n_c - n_t|^2 / 0.3) * exp(-|depth_c - depth_t|)
// (luminance of the demodulated colour with the NTSC weights, octahedral-decoded normals), and
// re-modulates with the centre's albedo clamped to >= 0.01. The three factors are evaluated as one
// exponential of the summed exponents (each factor is <= 1, so the reference's min(., 1) clamps are
// identities); pass k + 1 reads pass k's output.
//
// GB300 mapping: an HBM/L2 stencil. Per frame one kernel decodes the normals and depth into a float4
// and the clamped albedo into another; per pass one kernel turns the input colour into (demodulated
// rgb, luminance) and one filters: 25 taps x 32 B from L1/L2 (a 1280x720 frame's 15 MB of tap data
// stays in the 126 MB L2), one exp per tap.
#include "internal.hpp"
#include "pixel.cuh"

#include <cuda_runtime.h>

namespace vkg
{
namespace
{

constexpr int DN_BLOCK = 16;
constexpr uint32_t ATROUS_STEPS[5] = {1u, 2u, 4u, 8u, 16u};

__constant__ float c_kernel[25] = {
        1.f / 256.f, 1.f / 64.f, 3.f / 128.f, 1.f / 64.f, 1.f / 256.f, //
        1.f / 64.f,  1.f / 16.f, 3.f / 32.f,  1.f / 16.f, 1.f / 64.f,  //
        3.f / 128.f, 3.f / 32.f, 9.f / 64.f,  3.f / 32.f, 3.f / 128.f, //
        1.f / 64.f,  1.f / 16.f, 3.f / 32.f,  1.f / 16.f, 1.f / 64.f,  //
        1.f / 256.f, 1.f / 64.f, 3.f / 128.f, 1.f / 64.f, 1.f / 256.f};

// NTSC luminance weights (utils/color.slang:43)
constexpr float LUM_R = 0.298999994993f, LUM_G = 0.587000012398f, LUM_B = 0.114000000060f;

// per frame: (decoded normal, depth) and (albedo clamped to >= 0.01, 0)
__global__ void k_dn_geometry(const vkg_pixel_data *__restrict__ px, uint32_t n, float4 *__restrict__ geo,
                              float4 *__restrict__ alb, float *__restrict__ out_depth)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= n) return;
    const vkg_pixel_data p = px[i];
    const float2 q = unpack_snorm_2x16(p.normal);
    const float3 nv = oct_decode(q.x, q.y);
    geo[i] = make_float4(nv.x, nv.y, nv.z, p.depth);
    const float3 a = unpack_rgb8(p.albedo);
    alb[i] = make_float4(fmaxf(a.x, 0.01f), fmaxf(a.y, 0.01f), fmaxf(a.z, 0.01f), 0.f);
    if(out_depth) out_depth[i] = p.depth;
}

// per pass: the input colour (pass 0: the pixel radiance, else the previous pass) demodulated, and
// its luminance
__global__ void k_dn_demod(const vkg_pixel_data *__restrict__ px, const float4 *__restrict__ prev,
                           const float4 *__restrict__ alb, uint32_t n, float4 *__restrict__ dm)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= n) return;
    float r, g, b;
    if(prev)
    {
        const float4 c = prev[i];
        r = c.x, g = c.y, b = c.z;
    }
    else
    {
        r = px[i].radiance[0], g = px[i].radiance[1], b = px[i].radiance[2];
    }
    const float4 a = alb[i];
    r = r / a.x;
    g = g / a.y;
    b = b / a.z;
    dm[i] = make_float4(r, g, b, r * LUM_R + g * LUM_G + b * LUM_B);
}

// one a-trous pass: out = (sum_k w_k c_k / sum_k w_k) * albedo_centre
__global__ void __launch_bounds__(DN_BLOCK *DN_BLOCK)
        k_dn_filter(const float4 *__restrict__ dm, const float4 *__restrict__ geo, const float4 *__restrict__ alb,
                    uint32_t w, uint32_t h, int step, float4 *__restrict__ out)
{
    const int x = blockIdx.x * DN_BLOCK + threadIdx.x, y = blockIdx.y * DN_BLOCK + threadIdx.y;
    if(x >= (int)w || y >= (int)h) return;
    const float color_phi = 1.f / .9f, normal_phi = 1.f / .3f, position_phi = 1.f;
    const uint32_t c = (uint32_t)y * w + (uint32_t)x;
    const float4 dc = __ldg(&dm[c]), gc = __ldg(&geo[c]);
    float sr = 0.f, sg = 0.f, sb = 0.f, cw = 0.f;
#pragma unroll
    for(int k = 0; k < 25; ++k)
    {
        const int ux = min(max(x + (k % 5 - 2) * step, 0), (int)w - 1);
        const int uy = min(max(y + (k / 5 - 2) * step, 0), (int)h - 1);
        const uint32_t t = (uint32_t)uy * w + (uint32_t)ux;
        const float4 dt = __ldg(&dm[t]), gt = __ldg(&geo[t]);
        const float ld = dc.w - dt.w;
        const float ex = gc.x - gt.x, ey = gc.y - gt.y, ez = gc.z - gt.z;
        const float e = ld * ld * color_phi + (ex * ex + ey * ey + ez * ez) * normal_phi +
                        fabsf(gc.w - gt.w) * position_phi;
        const float wk = expf(-e) * c_kernel[k];
        sr += dt.x * wk;
        sg += dt.y * wk;
        sb += dt.z * wk;
        cw += wk;
    }
    const float4 a = __ldg(&alb[c]);
    out[c] = make_float4(sr / cw * a.x, sg / cw * a.y, sb / cw * a.z, 0.f);
}

__global__ void k_dn_to_rgb(const float4 *__restrict__ in, uint32_t n, float *__restrict__ rgb)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= n) return;
    const float4 v = in[i];
    rgb[3 * (size_t)i] = v.x;
    rgb[3 * (size_t)i + 1] = v.y;
    rgb[3 * (size_t)i + 2] = v.z;
}

}// namespace

// the five passes; the result in rgba (stride 4) and / or rgb (stride 3)
vkg_status denoise_run(vkg_ctx *ctx, const vkg_pixel_data *px, uint32_t w, uint32_t h, float *out_rgba,
                       float *out_rgb, float *out_depth, cudaStream_t st)
{
    const size_t n = (size_t)w * h;
    if(n == 0) return VKG_OK;
    float4 *buf = nullptr;
    cudaError_t e = cudaMallocAsync(&buf, 5 * n * sizeof(float4), st);
    if(e != cudaSuccess) return cuda_check(ctx, e, "vkg_denoise scratch");
    float4 *geo = buf, *alb = buf + n, *dm = buf + 2 * n, *ping = buf + 3 * n, *pong = buf + 4 * n;
    const uint32_t g1 = (uint32_t)((n + 255) / 256);
    k_dn_geometry<<<g1, 256, 0, st>>>(px, (uint32_t)n, geo, alb, out_depth);
    const dim3 blk(DN_BLOCK, DN_BLOCK), grid((w + DN_BLOCK - 1) / DN_BLOCK, (h + DN_BLOCK - 1) / DN_BLOCK);
    const float4 *prev = nullptr;
    for(int pass = 0; pass < 5; ++pass)
    {
        float4 *dst = (pass + 1 == 5 && out_rgba) ? reinterpret_cast<float4 *>(out_rgba) : (pass % 2 ? pong : ping);
        k_dn_demod<<<g1, 256, 0, st>>>(px, prev, alb, (uint32_t)n, dm);
        k_dn_filter<<<grid, blk, 0, st>>>(dm, geo, alb, w, h, (int)ATROUS_STEPS[pass], dst);
        prev = dst;
    }
    if(out_rgb) k_dn_to_rgb<<<g1, 256, 0, st>>>(prev, (uint32_t)n, out_rgb);
    e = cudaGetLastError();
    const cudaError_t ef = cudaFreeAsync(buf, st);
    if(e == cudaSuccess) e = ef;
    return e == cudaSuccess ? VKG_OK : cuda_check(ctx, e, "vkg_denoise");
}

}// namespace vkg

using namespace vkg;

extern "C" vkg_status vkg_denoise(vkg_ctx *ctx, const vkg_pixel_data *d_pixels, uint32_t width, uint32_t height,
                                  float *d_out_rgba, float *d_out_depth, void *stream)
{
    if(!ctx) return VKG_ERR_INVALID_ARGUMENT;
    if((width && height) && (!d_pixels || !d_out_rgba))
        return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_denoise: NULL buffer");
    if(vkg_status s = bind_device(ctx); s != VKG_OK) return s;
    return denoise_run(ctx, d_pixels, width, height, d_out_rgba, nullptr, d_out_depth,
                       static_cast<cudaStream_t>(stream));
}
