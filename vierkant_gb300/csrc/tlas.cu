// Two-level ray queries (vkg_tlas_closest_hit / vkg_tlas_any_hit): one thread per ray through
// trace_tlas (tlas.cuh). The top-level build lives with the other builds in bvh_build.cu.
#include "tlas.cuh"

namespace vkg
{
namespace
{

constexpr int TLAS_THREADS = 128;

template<bool ANY>
__global__ void __launch_bounds__(TLAS_THREADS)
        k_tlas_trace(const node8 *__restrict__ tnodes, const inst_rec *__restrict__ inst,
                     const blas_ref *__restrict__ blas, const vkg_ray *__restrict__ rays, uint32_t n,
                     vkg_inst_hit *__restrict__ hits, uint32_t *__restrict__ occluded, int cull)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= n) return;
    const float4 *rp = reinterpret_cast<const float4 *>(rays + i);
    const float4 r0 = __ldg(rp), r1 = __ldg(rp + 1);
    const tlas_result r = trace_tlas<ANY>(tnodes, inst, blas, r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, r1.z, r1.w, cull);
    if(ANY)
        occluded[i] = r.occluded ? 1u : 0u;
    else
    {
        uint4 *o = reinterpret_cast<uint4 *>(hits + i);
        o[0] = make_uint4(r.prim, r.inst, __float_as_uint(r.t), __float_as_uint(r.u));
        o[1] = make_uint4(__float_as_uint(r.v), 0u, 0u, 0u);
    }
}

__global__ void k_tlas_miss(uint32_t n, vkg_inst_hit *__restrict__ hits, uint32_t *__restrict__ occluded)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= n) return;
    if(hits) hits[i] = vkg_inst_hit{VKG_MISS, VKG_MISS, 0.f, 0.f, 0.f, {0u, 0u, 0u}};
    if(occluded) occluded[i] = 0u;
}

template<bool ANY>
vkg_status launch(vkg_ctx *ctx, const vkg_tlas *t, const vkg_ray *rays, uint32_t n, vkg_inst_hit *hits,
                  uint32_t *occ, uint32_t flags, void *stream)
{
    if(!ctx) return VKG_ERR_INVALID_ARGUMENT;
    if(!t) return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "two-level query: NULL TLAS");
    if(n == 0) return VKG_OK;
    if(!rays || (ANY ? !occ : !hits)) return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "two-level query: NULL buffer");
    if(reinterpret_cast<uintptr_t>(rays) % 16 || reinterpret_cast<uintptr_t>(ANY ? (void *)occ : (void *)hits) % 16)
        return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "two-level query: buffers must be 16-byte aligned");
    if(vkg_status s = bind_device(ctx); s != VKG_OK) return s;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const uint32_t grid = (n + TLAS_THREADS - 1) / TLAS_THREADS;
    if(t->num_instances == 0)
        k_tlas_miss<<<grid, TLAS_THREADS, 0, st>>>(n, ANY ? nullptr : hits, ANY ? occ : nullptr);
    else
        k_tlas_trace<ANY><<<grid, TLAS_THREADS, 0, st>>>(t->top.d_nodes, t->d_inst, t->d_blas, rays, n, hits, occ,
                                                         (flags & VKG_RAY_CULL_BACK_FACES) ? CULL_BACK : CULL_NONE);
    return cuda_check(ctx, cudaGetLastError(), "k_tlas_trace");
}

}// namespace
}// namespace vkg

using namespace vkg;

extern "C" {

vkg_status vkg_tlas_closest_hit(vkg_ctx *ctx, const vkg_tlas *tlas, const vkg_ray *d_rays, uint32_t n,
                                vkg_inst_hit *d_hits, uint32_t flags, void *stream)
{
    return launch<false>(ctx, tlas, d_rays, n, d_hits, nullptr, flags, stream);
}

vkg_status vkg_tlas_any_hit(vkg_ctx *ctx, const vkg_tlas *tlas, const vkg_ray *d_rays, uint32_t n, uint32_t *d_occluded,
                            uint32_t flags, void *stream)
{
    return launch<true>(ctx, tlas, d_rays, n, nullptr, d_occluded, flags, stream);
}

}// extern "C"
