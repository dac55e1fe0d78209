// Bloom + tonemap composition of the path tracer's output: the reference's post-FX pass
// (src/PBRPathTracer.cpp:405-465) as headless CUDA kernels, display only.
//
//   bloom threshold   shaders/slang/fullscreen/bloom_thresh.slang: half-resolution image (Bloom's
//                     framebuffer, PBRPathTracer.cpp:797-799) of the bilinearly sampled HDR colour,
//                     max(c, 0) faded in by smoothstep(0.95, 1.1, NTSC luma) (Bloom.hpp brightness_thresh)
//   gaussian blur     src/GaussianBlur.cpp, shaders/slang/fullscreen/gaussian_blur.slang: 3 iterations
//                     (PBRPathTracer.cpp:799) of a horizontal and a vertical 9-tap Gaussian
//                     (GaussianBlur_<9>), clamp-to-edge
//   composition       shaders/slang/fullscreen/bloom_composition.slang + utils/tonemap.slang:
//                     1 - exp(-(hdr + bloom) * exposure), then pow(., 1 / gamma); alpha of the HDR image
//                     (the path tracer binds an empty motion image, so the motion blur takes one tap)
//
// The bloom images are RGBA16F as in the reference (Bloom::create_info_t::color_format), so every
// threshold / blur output is rounded to half precision. The reference's blur merges tap pairs into
// bilinear fetches; here the 9 taps are summed directly (the same convolution, without the texture
// unit's fixed-point filter weights). Texture sampling is restated as bilinear filtering with
// clamp-to-edge addressing at texel centres. The 9-tap kernel is crocore::createGaussianKernel_1D
// (crocore, a submodule absent from the reference checkout; pinned commit unknown) with sigma
// deduced from the size: restated as the normalised Gaussian exp(-x^2 / (2 sigma^2)), x = -4..4,
// sigma = 0.3 ((9 - 1) / 2 - 1) + 0.8 = 1.7.
#include "internal.hpp"

#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cmath>

namespace vkg
{
namespace
{

__constant__ float c_blur[9];

__device__ __forceinline__ float4 ld_half4(const __half *p)
{
    const __half2 a = reinterpret_cast<const __half2 *>(p)[0], b = reinterpret_cast<const __half2 *>(p)[1];
    const float2 fa = __half22float2(a), fb = __half22float2(b);
    return make_float4(fa.x, fa.y, fb.x, fb.y);
}
__device__ __forceinline__ void st_half4(__half *p, float4 v)
{
    reinterpret_cast<__half2 *>(p)[0] = __floats2half2_rn(v.x, v.y);
    reinterpret_cast<__half2 *>(p)[1] = __floats2half2_rn(v.z, v.w);
}

// bilinear sample at texture coordinate (u, v) in [0, 1] of a w x h image, clamp-to-edge
template<class Load>
__device__ __forceinline__ float4 bilinear(Load load, uint32_t w, uint32_t h, float u, float v)
{
    const float x = u * (float)w - 0.5f, y = v * (float)h - 0.5f;
    const float x0f = floorf(x), y0f = floorf(y);
    const float fx = x - x0f, fy = y - y0f;
    const int x0 = min(max((int)x0f, 0), (int)w - 1), x1 = min(max((int)x0f + 1, 0), (int)w - 1);
    const int y0 = min(max((int)y0f, 0), (int)h - 1), y1 = min(max((int)y0f + 1, 0), (int)h - 1);
    const float4 a = load(x0, y0), b = load(x1, y0), c = load(x0, y1), d = load(x1, y1);
    auto lerp4 = [](float4 p, float4 q, float t) {
        return make_float4(p.x + (q.x - p.x) * t, p.y + (q.y - p.y) * t, p.z + (q.z - p.z) * t, p.w + (q.w - p.w) * t);
    };
    return lerp4(lerp4(a, b, fx), lerp4(c, d, fx), fy);
}

__global__ void k_bloom_thresh(const float4 *__restrict__ hdr, uint32_t w, uint32_t h, uint32_t bw, uint32_t bh,
                               __half *__restrict__ out, float lo, float hi)
{
    const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if(x >= bw || y >= bh) return;
    const float u = ((float)x + 0.5f) / (float)bw, v = ((float)y + 0.5f) / (float)bh;
    float4 c = bilinear([&](int i, int j) { return __ldg(&hdr[(size_t)j * w + i]); }, w, h, u, v);
    c = make_float4(fmaxf(c.x, 0.f), fmaxf(c.y, 0.f), fmaxf(c.z, 0.f), fmaxf(c.w, 0.f));
    const float br = c.x * 0.299f + c.y * 0.587f + c.z * 0.114f;
    const float t = fminf(fmaxf((br - lo) / (hi - lo), 0.f), 1.f);
    const float s = t * t * (3.f - 2.f * t);
    // lerp((0, 0, 0, 1), c, s)
    st_half4(out + 4 * ((size_t)y * bw + x), make_float4(c.x * s, c.y * s, c.z * s, 1.f + (c.w - 1.f) * s));
}

// one separable blur pass (dx, dy) = (1, 0) or (0, 1)
__global__ void k_blur(const __half *__restrict__ in, uint32_t w, uint32_t h, int dx, int dy, __half *__restrict__ out)
{
    const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if(x >= w || y >= h) return;
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for(int k = -4; k <= 4; ++k)
    {
        const int i = min(max((int)x + k * dx, 0), (int)w - 1), j = min(max((int)y + k * dy, 0), (int)h - 1);
        const float4 v = ld_half4(in + 4 * ((size_t)j * w + i));
        const float wk = c_blur[k + 4];
        acc.x += v.x * wk;
        acc.y += v.y * wk;
        acc.z += v.z * wk;
        acc.w += v.w * wk;
    }
    st_half4(out + 4 * ((size_t)y * w + x), acc);
}

__global__ void k_composite(const float4 *__restrict__ hdr, const __half *__restrict__ bloom, uint32_t w, uint32_t h,
                            uint32_t bw, uint32_t bh, float exposure, float inv_gamma, float4 *__restrict__ out)
{
    const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if(x >= w || y >= h) return;
    const float4 c = hdr[(size_t)y * w + x];
    float3 b = make_float3(0.f, 0.f, 0.f);
    if(bloom)
    {
        const float u = ((float)x + 0.5f) / (float)w, v = ((float)y + 0.5f) / (float)h;
        const float4 s = bilinear([&](int i, int j) { return ld_half4(bloom + 4 * ((size_t)j * bw + i)); }, bw, bh, u, v);
        b = make_float3(s.x, s.y, s.z);
    }
    float r = 1.f - expf(-(c.x + b.x) * exposure), g = 1.f - expf(-(c.y + b.y) * exposure),
          bl = 1.f - expf(-(c.z + b.z) * exposure);
    r = powf(r, inv_gamma);
    g = powf(g, inv_gamma);
    bl = powf(bl, inv_gamma);
    out[(size_t)y * w + x] = make_float4(r, g, bl, c.w);
}

}// namespace
}// namespace vkg

using namespace vkg;

extern "C" vkg_status vkg_post_fx_default(vkg_post_fx_settings *s)
{
    if(!s) return VKG_ERR_INVALID_ARGUMENT;
    // PBRPathTracer::settings_t (PBRPathTracer.hpp:74-86), Bloom::create_info_t, PBRPathTracer.cpp:797-799
    *s = vkg_post_fx_settings{};
    s->tonemap = 1;
    s->bloom = 1;
    s->exposure = 2.f;
    s->gamma = 1.f;
    s->brightness_thresh[0] = 0.95f;
    s->brightness_thresh[1] = 1.1f;
    s->blur_iterations = 3;
    return VKG_OK;
}

extern "C" vkg_status vkg_post_fx(vkg_ctx *ctx, const float *d_hdr_rgba, uint32_t width, uint32_t height,
                                  const vkg_post_fx_settings *s, float *d_out_rgba, void *stream)
{
    if(!ctx) return VKG_ERR_INVALID_ARGUMENT;
    if(!s || ((width && height) && (!d_hdr_rgba || !d_out_rgba)))
        return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_post_fx: NULL argument");
    if(!(s->gamma > 0.f) || !std::isfinite(s->exposure) || !(s->brightness_thresh[1] > s->brightness_thresh[0]) ||
       s->blur_iterations > 64)
        return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_post_fx: invalid settings");
    if(width == 0 || height == 0) return VKG_OK;
    if(vkg_status st = bind_device(ctx); st != VKG_OK) return st;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const size_t n = (size_t)width * height;
    if(!s->tonemap)
    {
        // no post-FX: the HDR image itself (PBRPathTracer.cpp:411)
        VKG_TRY_CUDA(ctx, cudaMemcpyAsync(d_out_rgba, d_hdr_rgba, n * 4 * sizeof(float), cudaMemcpyDeviceToDevice, st));
        return VKG_OK;
    }
    // the 9-tap kernel, normalised in double (sigma from the size, see the file comment)
    float wts[9];
    {
        const double sigma = 0.3 * ((9 - 1) * 0.5 - 1) + 0.8;
        double sum = 0, k[9];
        for(int i = 0; i < 9; ++i)
        {
            const double x = i - 4;
            k[i] = std::exp(-x * x / (2 * sigma * sigma));
            sum += k[i];
        }
        for(int i = 0; i < 9; ++i) wts[i] = (float)(k[i] / sum);
    }
    VKG_TRY_CUDA(ctx, cudaMemcpyToSymbolAsync(c_blur, wts, sizeof(wts), 0, cudaMemcpyHostToDevice, st));
    const uint32_t bw = std::max<uint32_t>(width / 2, 1), bh = std::max<uint32_t>(height / 2, 1);
    __half *bl = nullptr;
    if(s->bloom)
    {
        VKG_TRY_CUDA(ctx, cudaMallocAsync(&bl, 2 * (size_t)bw * bh * 4 * sizeof(__half), st));
        __half *ping = bl, *pong = bl + (size_t)bw * bh * 4;
        const dim3 blk(16, 16), g((bw + 15) / 16, (bh + 15) / 16);
        k_bloom_thresh<<<g, blk, 0, st>>>(reinterpret_cast<const float4 *>(d_hdr_rgba), width, height, bw, bh, ping,
                                          s->brightness_thresh[0], s->brightness_thresh[1]);
        for(uint32_t it = 0; it < s->blur_iterations; ++it)
        {
            k_blur<<<g, blk, 0, st>>>(ping, bw, bh, 1, 0, pong);
            k_blur<<<g, blk, 0, st>>>(pong, bw, bh, 0, 1, ping);
        }
    }
    const dim3 blk(16, 16), g((width + 15) / 16, (height + 15) / 16);
    k_composite<<<g, blk, 0, st>>>(reinterpret_cast<const float4 *>(d_hdr_rgba), bl, width, height, bw, bh,
                                   s->exposure, 1.f / s->gamma, reinterpret_cast<float4 *>(d_out_rgba));
    cudaError_t e = cudaGetLastError();
    if(bl)
    {
        const cudaError_t ef = cudaFreeAsync(bl, st);
        if(e == cudaSuccess) e = ef;
    }
    return e == cudaSuccess ? VKG_OK : cuda_check(ctx, e, "vkg_post_fx");
}
