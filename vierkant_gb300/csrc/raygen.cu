// Camera-ray generation on the GPU (the wavefront "generate" stage for ray batches).
//
// Pinhole convention of shaders/slang/raypipeline.slang:58-89 with the projection of
// include/vierkant/projection.hpp:48-57 (aperture 0): ndc = 2 * (pixel + jitter) / size - 1,
// camera-space direction (ndc.x * tan(fovy/2) * aspect, -ndc.y * tan(fovy/2), -1), rotated by the
// camera basis and normalised as v * (1 / sqrt(dot(v, v))). Every operation is separately rounded,
// so the rays are bit-identical to the host statement of the same formula.
// Jitter: ray r = s*W*H + y*W + x takes PCG32(seed, stream) draws 2r and 2r+1 (O(log r) jump-ahead).
#include "internal.hpp"

namespace vkg
{
namespace
{

__global__ void k_camera_rays(vkg_camera cam, uint64_t seed, uint64_t stream, uint64_t total, vkg_ray *__restrict__ out)
{
    uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if(r >= total) return;
    const uint64_t per = (uint64_t)cam.width * cam.height;
    const uint64_t p = r % per;
    const uint32_t x = (uint32_t)(p % cam.width), y = (uint32_t)(p / cam.width);
    pcg32 g = pcg32_seed(seed, stream);
    pcg32_advance(g, 2u * r);
    const float jx = u01(pcg32_next(g));
    const float jy = u01(pcg32_next(g));
    const float sx = fdiv(fadd((float)x, jx), (float)cam.width);
    const float sy = fdiv(fadd((float)y, jy), (float)cam.height);
    const float nx = fsub(fmul(2.0f, sx), 1.0f), ny = fsub(fmul(2.0f, sy), 1.0f);
    const float cx = fmul(nx, fmul(cam.tan_half_fovy, cam.aspect));
    const float cy = -fmul(ny, cam.tan_half_fovy);
    const float cz = -1.0f;
    float d[3];
    for(int a = 0; a < 3; ++a) d[a] = fadd(fadd(fmul(cam.right[a], cx), fmul(cam.up[a], cy)), fmul(cam.back[a], cz));
    const float inv = frcp(fsqrt(dot3(d[0], d[1], d[2], d[0], d[1], d[2])));
    float4 w0 = make_float4(cam.eye[0], cam.eye[1], cam.eye[2], 1e-4f);
    float4 w1 = make_float4(fmul(d[0], inv), fmul(d[1], inv), fmul(d[2], inv), 1e4f);
    float4 *o = reinterpret_cast<float4 *>(out + r);
    o[0] = w0;
    o[1] = w1;
}

}// namespace
}// namespace vkg

using namespace vkg;

extern "C" vkg_status vkg_camera_rays(vkg_ctx *ctx, const vkg_camera *cam, uint64_t seed, uint64_t stream,
                                      uint32_t spp, vkg_ray *d_rays, void *stream_)
{
    if(!ctx) return VKG_ERR_INVALID_ARGUMENT;
    if(!cam || !d_rays) return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_camera_rays: NULL argument");
    if(cam->width == 0 || cam->height == 0 || spp == 0) return VKG_OK;
    if(reinterpret_cast<uintptr_t>(d_rays) & 15u)
        return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_camera_rays: ray buffer must be 16-byte aligned");
    if(vkg_status s = bind_device(ctx); s != VKG_OK) return s;
    const uint64_t total = (uint64_t)cam->width * cam->height * spp;
    const int T = 256;
    const uint64_t grid = (total + T - 1) / T;
    if(grid > 0x7FFFFFFFull) return set_error(ctx, VKG_ERR_CAPACITY, "vkg_camera_rays: too many rays");
    k_camera_rays<<<(unsigned)grid, T, 0, static_cast<cudaStream_t>(stream_)>>>(*cam, seed, stream, total, d_rays);
    return cuda_check(ctx, cudaGetLastError(), "k_camera_rays");
}
