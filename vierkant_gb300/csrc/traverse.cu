// Closest-hit / any-hit traversal of the 8-wide quantised BVH (software traversal: GB300 has no
// RT cores). Replaces the RT-core TraceRay of shaders/slang/raypipeline.slang:182 and the
// RayQuery visibility test of shaders/slang/ray/visibility_test.slang:45-87.
//
// One thread per ray. Per node: six 16-byte loads (96 B node), slab tests of all children as
// fmaf(q, 2^e * inv_d, (origin - o) * inv_d) (two per axis per child), children sorted by entry
// distance with an 8-key sorting network, leaf children intersected first (closest leaves shrink
// best_t before any subtree is visited), internal children pushed far-to-near with their entry
// distance so a pop can be skipped once best_t has passed it. Triangle test: the reference's
// Moeller-Trumbore (src/intersection.cpp:114-129) op for op on 48-byte records.
//
// Work per ray (the roofline's algorithmic unit): 32 B ray in + 16 B hit out from HBM, plus
// 96 B per node visit and 48 B per triangle test from L2/L1.
#include "internal.hpp"

namespace vkg
{
namespace
{

constexpr int TRACE_THREADS = 128;

__device__ __forceinline__ uint32_t tenc(float f)
{
    uint32_t b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float tdec(uint32_t u)
{
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u);
}

__device__ __forceinline__ void cswap(unsigned long long &a, unsigned long long &b)
{
    unsigned long long lo = a < b ? a : b, hi = a < b ? b : a;
    a = lo;
    b = hi;
}

// Batcher odd-even merge network, 19 comparators
__device__ __forceinline__ void sort8(unsigned long long k[8])
{
    cswap(k[0], k[1]); cswap(k[2], k[3]); cswap(k[4], k[5]); cswap(k[6], k[7]);
    cswap(k[0], k[2]); cswap(k[1], k[3]); cswap(k[4], k[6]); cswap(k[5], k[7]);
    cswap(k[1], k[2]); cswap(k[5], k[6]);
    cswap(k[0], k[4]); cswap(k[1], k[5]); cswap(k[2], k[6]); cswap(k[3], k[7]);
    cswap(k[2], k[4]); cswap(k[3], k[5]);
    cswap(k[1], k[2]); cswap(k[3], k[4]); cswap(k[5], k[6]);
}

__device__ __forceinline__ uint32_t sel4(const uint4 &w, uint32_t j)
{
    uint32_t a = (j & 1u) ? w.y : w.x;
    uint32_t b = (j & 1u) ? w.w : w.z;
    return (j & 2u) ? b : a;
}

__device__ __forceinline__ float safe_rcp(float d)
{
    float dd = fabsf(d) < 1e-20f ? copysignf(1e-20f, d) : d;
    return __frcp_rn(dd);
}

__device__ __forceinline__ float qbyte(uint32_t w, int k) { return (float)((w >> (8 * (k & 3))) & 0xFFu); }

template<bool ANY, bool STATS>
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
        const float ox = r0.x, oy = r0.y, oz = r0.z, tmin = r0.w;
        const float dx = r1.x, dy = r1.y, dz = r1.z, tmax = r1.w;
        const float ix = safe_rcp(dx), iy = safe_rcp(dy), iz = safe_rcp(dz);
        const bool negx = ix < 0.f, negy = iy < 0.f, negz = iz < 0.f;

        float best_t = tmax, bu = 0.f, bv = 0.f;
        uint32_t best = VKG_MISS;
        bool done = false;
        uint32_t st_node[TRAVERSAL_STACK];
        float st_t[TRAVERSAL_STACK];
        int sp = 0;
        st_node[0] = 0;
        st_t[0] = tmin;
        sp = 1;

        while(sp > 0 && !done)
        {
            --sp;
            const uint32_t ni = st_node[sp];
            if(st_t[sp] > best_t) continue;
            if(STATS) ++visits;
            const uint4 *np = reinterpret_cast<const uint4 *>(nodes + ni);
            const uint4 w0 = __ldg(np), w1 = __ldg(np + 1), w2 = __ldg(np + 2);
            const uint4 w3 = __ldg(np + 3), w4 = __ldg(np + 4), w5 = __ldg(np + 5);
            const uint32_t meta = w0.w;
            const uint32_t nch = meta >> 24;
            const float tox = __fmul_rn(__fsub_rn(__uint_as_float(w0.x), ox), ix);
            const float toy = __fmul_rn(__fsub_rn(__uint_as_float(w0.y), oy), iy);
            const float toz = __fmul_rn(__fsub_rn(__uint_as_float(w0.z), oz), iz);
            const float sx = __fmul_rn(exp_scale(meta & 0xFFu), ix);
            const float sy = __fmul_rn(exp_scale((meta >> 8) & 0xFFu), iy);
            const float sz = __fmul_rn(exp_scale((meta >> 16) & 0xFFu), iz);
            // near / far quantised planes per axis (swap lo/hi for negative directions)
            const uint32_t nx0 = negx ? w2.z : w1.x, nx1 = negx ? w2.w : w1.y;
            const uint32_t fx0 = negx ? w1.x : w2.z, fx1 = negx ? w1.y : w2.w;
            const uint32_t ny0 = negy ? w3.x : w1.z, ny1 = negy ? w3.y : w1.w;
            const uint32_t fy0 = negy ? w1.z : w3.x, fy1 = negy ? w1.w : w3.y;
            const uint32_t nz0 = negz ? w3.z : w2.x, nz1 = negz ? w3.w : w2.y;
            const uint32_t fz0 = negz ? w2.x : w3.z, fz1 = negz ? w2.y : w3.w;

            unsigned long long key[8];
#pragma unroll
            for(int k = 0; k < 8; ++k)
            {
                key[k] = ~0ull;
                if((uint32_t)k < nch)
                {
                    const uint32_t wnx = k < 4 ? nx0 : nx1, wfx = k < 4 ? fx0 : fx1;
                    const uint32_t wny = k < 4 ? ny0 : ny1, wfy = k < 4 ? fy0 : fy1;
                    const uint32_t wnz = k < 4 ? nz0 : nz1, wfz = k < 4 ? fz0 : fz1;
                    const float tnx = fmaf(qbyte(wnx, k), sx, tox), tfx = fmaf(qbyte(wfx, k), sx, tox);
                    const float tny = fmaf(qbyte(wny, k), sy, toy), tfy = fmaf(qbyte(wfy, k), sy, toy);
                    const float tnz = fmaf(qbyte(wnz, k), sz, toz), tfz = fmaf(qbyte(wfz, k), sz, toz);
                    const float tn = fmaxf(fmaxf(tnx, tny), fmaxf(tnz, tmin));
                    const float tf = fminf(fminf(tfx, tfy), fminf(tfz, best_t));
                    if(tn <= tf) key[k] = ((unsigned long long)tenc(tn) << 32) | (unsigned long long)k;
                }
            }
            sort8(key);

            // leaf children, nearest first
#pragma unroll
            for(int h = 0; h < 8; ++h)
            {
                if(key[h] == ~0ull || done) break;
                const uint32_t k = (uint32_t)(key[h] & 7ull);
                const uint32_t c = (k & 4u) ? sel4(w5, k & 3u) : sel4(w4, k & 3u);
                if(!(c & LEAF_BIT)) continue;
                if(tdec((uint32_t)(key[h] >> 32)) > best_t) continue;
                const uint32_t start = c & 0x07FFFFFFu, cnt = ((c >> 27) & 0xFu) + 1u;
                for(uint32_t ti = start; ti < start + cnt; ++ti)
                {
                    const float4 *tp = reinterpret_cast<const float4 *>(tris + ti);
                    const float4 a = __ldg(tp), b = __ldg(tp + 1), cc = __ldg(tp + 2);
                    if(STATS) ++tests;
                    float t, u, v;
                    if(!tri_test(a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w, cc.x, ox, oy, oz, dx, dy, dz, cull, t, u, v))
                        continue;
                    if(!(t > tmin && t < tmax)) continue;
                    if(ANY)
                    {
                        done = true;
                        break;
                    }
                    const uint32_t prim = __float_as_uint(cc.y);
                    if(t < best_t || (t == best_t && prim < best))
                    {
                        best_t = t;
                        best = prim;
                        bu = u;
                        bv = v;
                    }
                }
            }
            if(done) break;
            // internal children, farthest pushed first
#pragma unroll
            for(int h = 7; h >= 0; --h)
            {
                if(key[h] == ~0ull) continue;
                const uint32_t k = (uint32_t)(key[h] & 7ull);
                const uint32_t c = (k & 4u) ? sel4(w5, k & 3u) : sel4(w4, k & 3u);
                if(c & LEAF_BIT) continue;
                if(sp < (int)TRAVERSAL_STACK)
                {
                    st_node[sp] = c;
                    st_t[sp] = tdec((uint32_t)(key[h] >> 32));
                    ++sp;
                }
                else if(counters) { atomicOr(&counters[2], 1ull); }
            }
        }
        if(ANY) { occluded[i] = done ? 1u : 0u; }
        else
        {
            uint4 out;
            if(best == VKG_MISS) out = make_uint4(VKG_MISS, 0u, 0u, 0u);
            else out = make_uint4(best, __float_as_uint(best_t), __float_as_uint(bu), __float_as_uint(bv));
            reinterpret_cast<uint4 *>(hits)[i] = out;
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
    if(d_occ)
    {
        if(stats)
            k_trace<true, true><<<grid, TRACE_THREADS, 0, st>>>(bvh->d_nodes, bvh->d_tris, d_rays, n, nullptr, d_occ,
                                                                cull, ctx->d_counters);
        else
            k_trace<true, false><<<grid, TRACE_THREADS, 0, st>>>(bvh->d_nodes, bvh->d_tris, d_rays, n, nullptr, d_occ,
                                                                 cull, ctx->d_counters);
    }
    else
    {
        if(stats)
            k_trace<false, true><<<grid, TRACE_THREADS, 0, st>>>(bvh->d_nodes, bvh->d_tris, d_rays, n, d_hits,
                                                                 nullptr, cull, ctx->d_counters);
        else
            k_trace<false, false><<<grid, TRACE_THREADS, 0, st>>>(bvh->d_nodes, bvh->d_tris, d_rays, n, d_hits,
                                                                  nullptr, cull, ctx->d_counters);
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
    VKG_TRY_CUDA(ctx, cudaMemcpyAsync(ctx->d_stage_rays, h_rays, rb, cudaMemcpyHostToDevice, st));
    vkg_status s = launch_trace(ctx, bvh, static_cast<const vkg_ray *>(ctx->d_stage_rays), num_rays,
                                static_cast<vkg_hit *>(ctx->d_stage_hits), nullptr, flags, st);
    if(s != VKG_OK) return s;
    VKG_TRY_CUDA(ctx, cudaMemcpyAsync(h_hits, ctx->d_stage_hits, hb, cudaMemcpyDeviceToHost, st));
    VKG_TRY_CUDA(ctx, cudaStreamSynchronize(st));
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
