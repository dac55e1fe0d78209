// Closest-hit / any-hit traversal of the 8-wide quantised BVH (software traversal: GB300 has no
// RT cores). Replaces the RT-core TraceRay of shaders/slang/raypipeline.slang:182 and the
// RayQuery visibility test of shaders/slang/ray/visibility_test.slang:45-87.
//
// One thread per ray; the traversal itself is trace_ray() in traverse.cuh.
//
// Work per ray (the roofline's algorithmic unit): 32 B ray in + 16 B hit out from HBM, plus
// 96 B per node visit and 48 B per triangle test from L2/L1.
#include "traverse.cuh"

#include <algorithm>
#include <cstdlib>
#include <string>

namespace vkg
{
namespace
{

constexpr int TRACE_THREADS = 128;

// STACK: traversal stack entries; 64 serve BVHs up to 10 levels deep (7 (depth - 1) + 1 entries)
template<bool ANY, bool STATS, int STACK>
__global__ void __launch_bounds__(TRACE_THREADS)
        k_trace(const node8 *__restrict__ nodes, const tri_rec *__restrict__ tris, const vkg_ray *__restrict__ rays,
                uint32_t n, vkg_hit *__restrict__ hits, uint32_t *__restrict__ occluded, int cull,
                unsigned long long *__restrict__ counters)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long visits = 0, tests = 0;
    if(i < n)
    {
        const float4 *rp = reinterpret_cast<const float4 *>(rays + i);
        const float4 r0 = __ldg(rp), r1 = __ldg(rp + 1);
        trace_result r = trace_ray<ANY, STATS, STACK>(nodes, tris, r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, r1.z, r1.w,
                                                      cull, visits, tests, counters);
        if(ANY) { occluded[i] = r.occluded ? 1u : 0u; }
        else
        {
            reinterpret_cast<uint4 *>(hits)[i] =
                    make_uint4(r.prim, __float_as_uint(r.t), __float_as_uint(r.u), __float_as_uint(r.v));
        }
    }
    if(STATS)
    {
        for(int o = 16; o > 0; o >>= 1)
        {
            visits += __shfl_down_sync(0xffffffffu, visits, o);
            tests += __shfl_down_sync(0xffffffffu, tests, o);
        }
        if((threadIdx.x & 31u) == 0 && counters)
        {
            atomicAdd(&counters[0], visits);
            atomicAdd(&counters[1], tests);
        }
    }
}

// Persistent variant: a fixed grid of warps; every lane whose ray has finished takes the next ray
// index from a global counter (one atomic per warp and refill), so warps stay full until the batch
// is exhausted instead of idling behind their slowest ray.
template<bool ANY, bool STATS>
__global__ void __launch_bounds__(TRACE_THREADS)
        k_trace_persistent(const node8 *__restrict__ nodes, const tri_rec *__restrict__ tris,
                           const vkg_ray *__restrict__ rays, uint32_t n, vkg_hit *__restrict__ hits,
                           uint32_t *__restrict__ occluded, int cull, unsigned long long *__restrict__ counters,
                           uint32_t *__restrict__ next_ray)
{
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t lt = (1u << lane) - 1u;
    unsigned long long visits = 0, tests = 0;
    ray_state s;
    uint2 stack[TRAVERSAL_STACK];
    s.st = stack;
    uint32_t cur = 0xFFFFFFFFu;
    bool exhausted = false;
    for(;;)
    {
        const bool need = cur == 0xFFFFFFFFu && !exhausted;
        const unsigned m = __ballot_sync(0xffffffffu, need);
        if(m)
        {
            const uint32_t leader = __ffs(m) - 1;
            uint32_t base = 0;
            if(lane == leader) base = atomicAdd(next_ray, (uint32_t)__popc(m));
            base = __shfl_sync(0xffffffffu, base, leader);
            if(need)
            {
                const uint32_t idx = base + __popc(m & lt);
                if(idx < n)
                {
                    const float4 *rp = reinterpret_cast<const float4 *>(rays + idx);
                    const float4 r0 = __ldg(rp), r1 = __ldg(rp + 1);
                    ray_init(s, r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, r1.z, r1.w);
                    cur = idx;
                }
                else exhausted = true;
            }
        }
        const bool active = cur != 0xFFFFFFFFu;
        if(!__any_sync(0xffffffffu, active)) break;
        if(active && !ray_step<ANY, STATS>(s, nodes, tris, cull, visits, tests, counters))
        {
            const trace_result r = ray_result(s);
            if(ANY) occluded[cur] = r.occluded ? 1u : 0u;
            else
                reinterpret_cast<uint4 *>(hits)[cur] =
                        make_uint4(r.prim, __float_as_uint(r.t), __float_as_uint(r.u), __float_as_uint(r.v));
            cur = 0xFFFFFFFFu;
        }
    }
    if(STATS)
    {
        for(int o = 16; o > 0; o >>= 1)
        {
            visits += __shfl_down_sync(0xffffffffu, visits, o);
            tests += __shfl_down_sync(0xffffffffu, tests, o);
        }
        if(lane == 0 && counters)
        {
            atomicAdd(&counters[0], visits);
            atomicAdd(&counters[1], tests);
        }
    }
}

template<bool ANY, bool STATS>
void launch_persistent(vkg_ctx *ctx, const vkg_bvh *bvh, const vkg_ray *d_rays, uint32_t n, vkg_hit *d_hits,
                       uint32_t *d_occ, int cull, cudaStream_t st)
{
    static int blocks_per_sm = 0;
    if(blocks_per_sm == 0)
    {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, k_trace_persistent<ANY, STATS>, TRACE_THREADS,
                                                      0);
        if(blocks_per_sm < 1) blocks_per_sm = 1;
    }
    uint32_t grid = (uint32_t)ctx->num_sms * (uint32_t)blocks_per_sm;
    const uint32_t need = (n + TRACE_THREADS - 1) / TRACE_THREADS;
    if(grid > need) grid = need;
    cudaMemsetAsync(ctx->d_work, 0, sizeof(uint32_t), st);
    k_trace_persistent<ANY, STATS><<<grid, TRACE_THREADS, 0, st>>>(bvh->d_nodes, bvh->d_tris, d_rays, n, d_hits, d_occ,
                                                                   cull, ctx->d_counters, ctx->d_work);
}

// kernel choice: the one-thread-per-ray kernel by default (faster on mixed primary/bounce batches);
// VKG_TRACE_KERNEL=persistent selects the refilling persistent kernel
bool use_persistent()
{
    static int v = -1;
    if(v < 0)
    {
        const char *e = getenv("VKG_TRACE_KERNEL");
        v = (e && std::string(e) == "persistent") ? 1 : 0;
    }
    return v == 1;
}

template<bool ANY, bool STATS>
void launch_simple(bool small_stack, uint32_t grid, cudaStream_t st, const vkg_bvh *bvh, const vkg_ray *rays,
                   uint32_t n, vkg_hit *hits, uint32_t *occ, int cull, unsigned long long *counters)
{
    if(small_stack)
        k_trace<ANY, STATS, 64><<<grid, TRACE_THREADS, 0, st>>>(bvh->d_nodes, bvh->d_tris, rays, n, hits, occ, cull,
                                                                counters);
    else
        k_trace<ANY, STATS, (int)TRAVERSAL_STACK><<<grid, TRACE_THREADS, 0, st>>>(bvh->d_nodes, bvh->d_tris, rays, n,
                                                                                   hits, occ, cull, counters);
}

__global__ void k_fill_miss(vkg_hit *hits, uint32_t *occluded, uint32_t n)
{
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= n) return;
    if(hits) reinterpret_cast<uint4 *>(hits)[i] = make_uint4(VKG_MISS, 0u, 0u, 0u);
    if(occluded) occluded[i] = 0u;
}

vkg_status launch_trace(vkg_ctx *ctx, const vkg_bvh *bvh, const vkg_ray *d_rays, uint32_t n, vkg_hit *d_hits,
                        uint32_t *d_occ, uint32_t flags, cudaStream_t st)
{
    const uint32_t grid = (n + TRACE_THREADS - 1) / TRACE_THREADS;
    if(bvh->num_tris == 0 || bvh->num_nodes == 0)
    {
        k_fill_miss<<<grid, TRACE_THREADS, 0, st>>>(d_hits, d_occ, n);
        return cuda_check(ctx, cudaGetLastError(), "k_fill_miss");
    }
    const int cull = (flags & VKG_RAY_CULL_BACK_FACES) ? 1 : 0;
    const bool stats = (flags & VKG_RAY_COUNT_STATS) != 0;
    if(use_persistent())
    {
        if(d_occ)
        {
            if(stats) launch_persistent<true, true>(ctx, bvh, d_rays, n, nullptr, d_occ, cull, st);
            else launch_persistent<true, false>(ctx, bvh, d_rays, n, nullptr, d_occ, cull, st);
        }
        else
        {
            if(stats) launch_persistent<false, true>(ctx, bvh, d_rays, n, d_hits, nullptr, cull, st);
            else launch_persistent<false, false>(ctx, bvh, d_rays, n, d_hits, nullptr, cull, st);
        }
        return cuda_check(ctx, cudaGetLastError(), "k_trace_persistent");
    }
    const bool small = bvh->depth <= 10;
    if(d_occ)
    {
        if(stats) launch_simple<true, true>(small, grid, st, bvh, d_rays, n, nullptr, d_occ, cull, ctx->d_counters);
        else launch_simple<true, false>(small, grid, st, bvh, d_rays, n, nullptr, d_occ, cull, ctx->d_counters);
    }
    else
    {
        if(stats) launch_simple<false, true>(small, grid, st, bvh, d_rays, n, d_hits, nullptr, cull, ctx->d_counters);
        else launch_simple<false, false>(small, grid, st, bvh, d_rays, n, d_hits, nullptr, cull, ctx->d_counters);
    }
    return cuda_check(ctx, cudaGetLastError(), "k_trace");
}

vkg_status check_common(vkg_ctx *ctx, const vkg_bvh *bvh, const void *rays, const void *out, const char *fn)
{
    if(!ctx) return VKG_ERR_INVALID_ARGUMENT;
    if(!bvh) return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "%s: bvh is NULL", fn);
    if(!rays || !out) return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "%s: NULL ray or output buffer", fn);
    if((reinterpret_cast<uintptr_t>(rays) & 15u) || (reinterpret_cast<uintptr_t>(out) & 3u))
        return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "%s: ray buffer must be 16-byte aligned", fn);
    return bind_device(ctx);
}

}// namespace
}// namespace vkg

using namespace vkg;

extern "C" vkg_status vkg_closest_hit(vkg_ctx *ctx, const vkg_bvh *bvh, const vkg_ray *d_rays, uint32_t num_rays,
                                      vkg_hit *d_hits, uint32_t flags, void *stream)
{
    if(num_rays == 0) return VKG_OK;
    if(vkg_status s = check_common(ctx, bvh, d_rays, d_hits, "vkg_closest_hit"); s != VKG_OK) return s;
    if(reinterpret_cast<uintptr_t>(d_hits) & 15u)
        return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_closest_hit: hit buffer must be 16-byte aligned");
    return launch_trace(ctx, bvh, d_rays, num_rays, d_hits, nullptr, flags, static_cast<cudaStream_t>(stream));
}

extern "C" vkg_status vkg_any_hit(vkg_ctx *ctx, const vkg_bvh *bvh, const vkg_ray *d_rays, uint32_t num_rays,
                                  uint32_t *d_occluded, uint32_t flags, void *stream)
{
    if(num_rays == 0) return VKG_OK;
    if(vkg_status s = check_common(ctx, bvh, d_rays, d_occluded, "vkg_any_hit"); s != VKG_OK) return s;
    return launch_trace(ctx, bvh, d_rays, num_rays, nullptr, d_occluded, flags, static_cast<cudaStream_t>(stream));
}

extern "C" vkg_status vkg_closest_hit_host(vkg_ctx *ctx, const vkg_bvh *bvh, const vkg_ray *h_rays,
                                           uint32_t num_rays, vkg_hit *h_hits, uint32_t flags, void *stream)
{
    if(!ctx) return VKG_ERR_INVALID_ARGUMENT;
    if(num_rays == 0) return VKG_OK;
    if(!bvh || !h_rays || !h_hits)
        return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_closest_hit_host: NULL argument");
    if(vkg_status s = bind_device(ctx); s != VKG_OK) return s;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const size_t rb = sizeof(vkg_ray) * (size_t)num_rays, hb = sizeof(vkg_hit) * (size_t)num_rays;
    if(ctx->stage_rays_bytes < rb)
    {
        cudaFree(ctx->d_stage_rays);
        ctx->d_stage_rays = nullptr;
        ctx->stage_rays_bytes = 0;
        VKG_TRY_CUDA(ctx, cudaMalloc(&ctx->d_stage_rays, rb));
        ctx->stage_rays_bytes = rb;
    }
    if(ctx->stage_hits_bytes < hb)
    {
        cudaFree(ctx->d_stage_hits);
        ctx->d_stage_hits = nullptr;
        ctx->stage_hits_bytes = 0;
        VKG_TRY_CUDA(ctx, cudaMalloc(&ctx->d_stage_hits, hb));
        ctx->stage_hits_bytes = hb;
    }
    // Chunks of HOST_CHUNK rays alternate between two streams: chunk c's upload, trace and download
    // are ordered on its stream, so the upload of c + 1 and the download of c - 1 (two copy engines)
    // run under the trace of c. Each chunk has its own region of the staging buffers.
    constexpr uint32_t HOST_CHUNK = 1u << 20;
    const uint32_t chunks = (num_rays + HOST_CHUNK - 1) / HOST_CHUNK;
    auto *d_rays = static_cast<vkg_ray *>(ctx->d_stage_rays);
    auto *d_hits = static_cast<vkg_hit *>(ctx->d_stage_hits);
    // (the persistent kernels share one work counter, so they are not run on two streams at once)
    if(chunks == 1 || use_persistent())
    {
        VKG_TRY_CUDA(ctx, cudaMemcpyAsync(d_rays, h_rays, rb, cudaMemcpyHostToDevice, st));
        vkg_status s = launch_trace(ctx, bvh, d_rays, num_rays, d_hits, nullptr, flags, st);
        if(s != VKG_OK) return s;
        VKG_TRY_CUDA(ctx, cudaMemcpyAsync(h_hits, d_hits, hb, cudaMemcpyDeviceToHost, st));
        VKG_TRY_CUDA(ctx, cudaStreamSynchronize(st));
        return VKG_OK;
    }
    for(int k = 0; k < 2; ++k)
        if(!ctx->pipe[k]) VKG_TRY_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->pipe[k], cudaStreamNonBlocking));
    for(int k = 0; k < 3; ++k)
        if(!ctx->pipe_ev[k]) VKG_TRY_CUDA(ctx, cudaEventCreateWithFlags(&ctx->pipe_ev[k], cudaEventDisableTiming));
    // fork: both streams start after the work already queued on the caller's stream
    VKG_TRY_CUDA(ctx, cudaEventRecord(ctx->pipe_ev[0], st));
    for(int k = 0; k < 2; ++k) VKG_TRY_CUDA(ctx, cudaStreamWaitEvent(ctx->pipe[k], ctx->pipe_ev[0], 0));
    vkg_status status = VKG_OK;
    for(uint32_t c = 0; c < chunks && status == VKG_OK; ++c)
    {
        cudaStream_t ps = ctx->pipe[c & 1u];
        const size_t first = (size_t)c * HOST_CHUNK;
        const uint32_t n = (uint32_t)std::min<size_t>(HOST_CHUNK, num_rays - first);
        cudaError_t e = cudaMemcpyAsync(d_rays + first, h_rays + first, n * sizeof(vkg_ray), cudaMemcpyHostToDevice, ps);
        if(e != cudaSuccess)
        {
            status = cuda_check(ctx, e, "vkg_closest_hit_host");
            break;
        }
        status = launch_trace(ctx, bvh, d_rays + first, n, d_hits + first, nullptr, flags, ps);
        if(status != VKG_OK) break;
        e = cudaMemcpyAsync(h_hits + first, d_hits + first, n * sizeof(vkg_hit), cudaMemcpyDeviceToHost, ps);
        if(e != cudaSuccess) status = cuda_check(ctx, e, "vkg_closest_hit_host");
    }
    // join: the caller's stream waits for both (also after an error, so nothing is left in flight)
    for(int k = 0; k < 2; ++k)
    {
        cudaEventRecord(ctx->pipe_ev[1 + k], ctx->pipe[k]);
        cudaStreamWaitEvent(st, ctx->pipe_ev[1 + k], 0);
    }
    const cudaError_t e = cudaStreamSynchronize(st);
    if(status != VKG_OK) return status;
    if(e != cudaSuccess) return cuda_check(ctx, e, "vkg_closest_hit_host");
    return VKG_OK;
}

extern "C" vkg_status vkg_ray_stats_get(vkg_ctx *ctx, uint64_t *node_visits, uint64_t *tri_tests, int reset)
{
    if(!ctx) return VKG_ERR_INVALID_ARGUMENT;
    if(vkg_status s = bind_device(ctx); s != VKG_OK) return s;
    unsigned long long h[4] = {0, 0, 0, 0};
    VKG_TRY_CUDA(ctx, cudaDeviceSynchronize());
    VKG_TRY_CUDA(ctx, cudaMemcpy(h, ctx->d_counters, sizeof(h), cudaMemcpyDeviceToHost));
    if(node_visits) *node_visits = h[0];
    if(tri_tests) *tri_tests = h[1];
    if(reset) VKG_TRY_CUDA(ctx, cudaMemset(ctx->d_counters, 0, sizeof(h)));
    if(h[2] & 1ull)
        return set_error(ctx, VKG_ERR_STACK_OVERFLOW, "a traversal exceeded its %u-entry stack", TRAVERSAL_STACK);
    return VKG_OK;
}
