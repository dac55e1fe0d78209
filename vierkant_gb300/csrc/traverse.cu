// Closest-hit / any-hit traversal of the 8-wide quantised BVH (software traversal: GB300 has no
// RT cores). Replaces the RT-core TraceRay of shaders/slang/raypipeline.slang:182 and the
// RayQuery visibility test of shaders/slang/ray/visibility_test.slang:45-87.
//
// One thread per ray; the traversal itself is trace_ray() in traverse.cuh. Large batches are traced
// in bins (origin cell x direction): neighbouring threads then follow similar paths through the tree,
// so a warp's lanes stay busy together and share node loads in L1.
//
// Work per ray (the roofline's algorithmic unit): 32 B ray in + 16 B hit out from HBM, plus
// 96 B per node visit and 48 B per triangle test from L2/L1.
#include "traverse.cuh"

#include <algorithm>
#include <cstdlib>
#include <string>
#include <vector>

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
                unsigned long long *__restrict__ counters, const uint32_t *__restrict__ perm,
                const uint32_t *__restrict__ reordered)
{
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long visits = 0, tests = 0;
    if(j < n)
    {
        // thread j traces ray perm[j] when the batch was binned (and some tile did not keep its order)
        const uint32_t i = (perm && __ldg(reordered)) ? __ldg(perm + j) : j;
        const float4 *rp = reinterpret_cast<const float4 *>(rays + i);
        const float4 r0 = __ldg(rp), r1 = __ldg(rp + 1);
        const trace_result r = trace_ray<ANY, STATS, STACK>(nodes, tris, r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, r1.z,
                                                            r1.w, cull, visits, tests, counters);
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
                           uint32_t *__restrict__ next_ray, const uint32_t *__restrict__ perm,
                           const uint32_t *__restrict__ reordered)
{
    if(perm && __ldg(reordered) == 0u) perm = nullptr;
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
                const uint32_t pos = base + __popc(m & lt);
                if(pos < n)
                {
                    const uint32_t idx = perm ? __ldg(perm + pos) : pos; // the ray at traced position pos
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
        if(active && !ray_step_auto<ANY, STATS>(s, nodes, tris, cull, visits, tests, counters))
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
                       uint32_t *d_occ, int cull, cudaStream_t st, const uint32_t *perm, const uint32_t *reordered)
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
                                                                   cull, ctx->d_counters, ctx->d_work, perm, reordered);
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
                   uint32_t n, vkg_hit *hits, uint32_t *occ, int cull, unsigned long long *counters,
                   const uint32_t *perm, const uint32_t *reordered)
{
    if(small_stack)
        k_trace<ANY, STATS, 64><<<grid, TRACE_THREADS, 0, st>>>(bvh->d_nodes, bvh->d_tris, rays, n, hits, occ, cull,
                                                                counters, perm, reordered);
    else
        k_trace<ANY, STATS, (int)TRAVERSAL_STACK><<<grid, TRACE_THREADS, 0, st>>>(
                bvh->d_nodes, bvh->d_tris, rays, n, hits, occ, cull, counters, perm, reordered);
}

// ---- ray binning -------------------------------------------------------------------------------
// bin = (Morton index of the origin's cell in an 8 x 8 x 8 grid over the scene box) * 64 + direction
// bin (8 x 8 cells of the octahedral map of the direction). Cell-major order keeps the rays of one
// region of the scene together; within a cell, rays of similar direction. Within a bin the rays
// keep roughly the order they came in (for a camera or bounce batch: pixel order, itself spatially
// coherent): tiles keep their order, and within a tile the ranks follow the order in which its warps
// reach the bin's counter, each warp walking a contiguous part of the tile. An order shuffled within
// the bins traces slower than the given order.
// Counting sort over T tiles of consecutive rays:
//   k_bin_keys     every ray's bin (16 bits)
//   k_bin_tiles    one CTA per tile: each ray's rank among the tile's rays of its bin (shared-memory
//                  counters) and the tile's bin histogram -> M[t][bin]; a tile whose rays are
//                  coherent already (most 32-ray steps in one bin: camera rays) keeps its order as
//                  one run in an extra bin placed after all others
//   k_bin_columns  per bin, M[.][bin] scanned over the tiles in place (exclusive); S[bin] = total
//   k_bin_offsets  F = exclusive scan of S: the bins' first positions
//   k_bin_place    perm[F[bin] + M[t][bin] + rank] = ray
constexpr int BIN_CELL_BITS = 3;                                            // per axis
constexpr int BIN_DIR_BITS = 3;                                             // per octahedral axis
constexpr uint32_t NUM_BINS = 1u << (3 * BIN_CELL_BITS + 2 * BIN_DIR_BITS); // 32,768
constexpr uint32_t BIN_MIN_RAYS = 1u << 19;
constexpr int BIN_THREADS = 1024;                                           // per tile CTA
constexpr uint32_t BIN_MAX_TILE = 40u * BIN_THREADS;                        // ranks fit 16 bits
// slot NUM_BINS (KEEP_BIN): the rays of tiles that keep their order; the count rows are padded to
// whole groups of 32 slots
constexpr uint32_t KEEP_BIN = NUM_BINS;
constexpr uint32_t BIN_SLOTS = NUM_BINS + 32;
constexpr size_t BIN_SMEM = sizeof(uint32_t) * BIN_SLOTS;                    // 128 KB + 128 B
static_assert(NUM_BINS == BIN_THREADS * 32, "32 bins per thread");
static_assert(BIN_SLOTS <= 65536 && BIN_MAX_TILE <= 65536, "bin and rank are packed in 16 bits each");

__device__ __forceinline__ uint32_t spread3(uint32_t v) { return (v & 1u) | ((v & 2u) << 2) | ((v & 4u) << 4); }

__device__ __forceinline__ uint32_t cell_coord(float p, float lo, float scale)
{
    // NaN converts to 0; out-of-box origins clamp to the border cells
    const int c = __float2int_rz((p - lo) * scale);
    return (uint32_t)min(max(c, 0), (1 << BIN_CELL_BITS) - 1);
}

__device__ __forceinline__ uint32_t dir_bin(float dx, float dy, float dz)
{
    constexpr float R = (float)(1 << BIN_DIR_BITS);
    const float a = fabsf(dx) + fabsf(dy) + fabsf(dz);
    float u = 0.f, v = 0.f;
    if(a > 0.f)
    {
        const float ia = 1.f / a;
        u = dx * ia;
        v = dy * ia;
        if(dz < 0.f)
        {
            const float fu = (1.f - fabsf(v)) * copysignf(1.f, u), fv = (1.f - fabsf(u)) * copysignf(1.f, v);
            u = fu;
            v = fv;
        }
    }
    const int qu = min(max(__float2int_rz((u + 1.f) * (0.5f * R)), 0), (1 << BIN_DIR_BITS) - 1);
    const int qv = min(max(__float2int_rz((v + 1.f) * (0.5f * R)), 0), (1 << BIN_DIR_BITS) - 1);
    return (uint32_t)qu | ((uint32_t)qv << BIN_DIR_BITS);
}

__device__ __forceinline__ uint32_t ray_bin(float4 r0, float4 r1, float3 lo, float3 scale)
{
    const uint32_t cell = spread3(cell_coord(r0.x, lo.x, scale.x)) | (spread3(cell_coord(r0.y, lo.y, scale.y)) << 1) |
                          (spread3(cell_coord(r0.z, lo.z, scale.z)) << 2);
    return (cell << (2 * BIN_DIR_BITS)) | dir_bin(r1.x, r1.y, r1.z);
}

__global__ void __launch_bounds__(256)
        k_bin_keys(const vkg_ray *__restrict__ rays, uint32_t n_cap, const uint32_t *__restrict__ d_n, float3 lo,
                   float3 scale, uint16_t *__restrict__ bins, uint32_t *__restrict__ reordered)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i == 0) *reordered = 0u; // k_bin_tiles counts the tiles that do not keep their order
    const uint32_t n = d_n ? min(*d_n, n_cap) : n_cap;
    if(i >= n) return;
    const float4 *rp = reinterpret_cast<const float4 *>(rays + i);
    bins[i] = (uint16_t)ray_bin(__ldg(rp), __ldg(rp + 1), lo, scale);
}

// Each warp walks its own contiguous 1/32 of the tile, 32 rays a step. Steps whose rays all share
// one bin extend a run of that bin; a run takes its ranks with one atomic when it ends (its keys are
// written then), so a stretch of coherent rays costs one atomic instead of one per step and warp
// (all warps of a camera tile would otherwise queue on the same few counters). In other steps each
// ray takes its rank with its own atomic.
__global__ void __launch_bounds__(BIN_THREADS)
        k_bin_tiles(const uint16_t *__restrict__ bins, uint32_t n_cap, const uint32_t *__restrict__ d_n, uint32_t tile,
                    uint32_t *__restrict__ keys, uint32_t *__restrict__ M, uint32_t *__restrict__ reordered)
{
    const uint32_t n = d_n ? min(*d_n, n_cap) : n_cap;
    extern __shared__ uint32_t h[];
    __shared__ uint32_t uniform_steps;
    for(uint32_t b = threadIdx.x; b < BIN_SLOTS; b += BIN_THREADS) h[b] = 0u;
    if(threadIdx.x == 0) uniform_steps = 0u;
    __syncthreads();
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    // (tiles past a device-side count are empty: they keep their order and write a zero row)
    const uint32_t start = blockIdx.x * tile, end = start < n ? min(start + tile, n) : start;
    const uint32_t per_warp = tile / 32u; // a multiple of 32
    const uint32_t w0 = start + warp * per_warp, w1 = min(w0 + per_warp, end);
    // a tile most of whose 32-ray steps fall into one bin each is coherent already (camera rays):
    // it keeps its order, as one run in KEEP_BIN
    constexpr int U = 8; // steps whose bins are loaded together
    {
        uint32_t u_steps = 0;
        for(uint32_t r0 = w0; r0 < w1; r0 += 32u * U)
        {
            uint32_t bu[U];
#pragma unroll
            for(int u = 0; u < U; ++u)
            {
                const uint32_t i = r0 + 32u * u + lane;
                bu[u] = i < w1 ? (uint32_t)__ldg(bins + i) : 0xFFFFFFFFu;
            }
#pragma unroll
            for(int u = 0; u < U; ++u)
            {
                const uint32_t r = r0 + 32u * u;
                if(r >= w1) break; // warp-uniform
                const bool valid = r + lane < w1;
                const uint32_t b0 = __shfl_sync(0xffffffffu, bu[u], 0);
                u_steps += __all_sync(0xffffffffu, !valid || bu[u] == b0) ? 1u : 0u;
            }
        }
        if(lane == 0 && u_steps) atomicAdd(&uniform_steps, u_steps);
    }
    __syncthreads();
    const uint32_t steps = (end - start + 31u) / 32u;
    if(2u * uniform_steps >= steps)
    {
        for(uint32_t i = start + threadIdx.x; i < end; i += BIN_THREADS) keys[i] = KEEP_BIN | ((i - start) << 16);
        if(threadIdx.x == 0) h[KEEP_BIN] = end - start;
        __syncthreads();
        uint32_t *row = M + (size_t)blockIdx.x * BIN_SLOTS;
        for(uint32_t b = threadIdx.x; b < BIN_SLOTS; b += BIN_THREADS) row[b] = h[b];
        return;
    }
    if(threadIdx.x == 0) atomicAdd(reordered, 1u);
    uint32_t run_bin = 0xFFFFFFFFu, run_start = 0, run_len = 0;
    // a run's ranks: one atomic, then its keys
    auto flush = [&]() {
        if(run_len == 0) return;
        uint32_t base = 0;
        if(lane == 0) base = atomicAdd(&h[run_bin], run_len);
        base = __shfl_sync(0xffffffffu, base, 0);
        for(uint32_t j = lane; j < run_len; j += 32u) keys[run_start + j] = run_bin | ((base + j) << 16);
        run_len = 0;
        run_bin = 0xFFFFFFFFu;
    };
    for(uint32_t r0 = w0; r0 < w1; r0 += 32u * U)
    {
        uint32_t bu[U];
#pragma unroll
        for(int u = 0; u < U; ++u)
        {
            const uint32_t i = r0 + 32u * u + lane;
            bu[u] = i < w1 ? (uint32_t)__ldg(bins + i) : 0xFFFFFFFFu;
        }
#pragma unroll
        for(int u = 0; u < U; ++u)
        {
            const uint32_t r = r0 + 32u * u;
            if(r >= w1) break; // warp-uniform
            const uint32_t i = r + lane;
            const bool valid = i < w1;
            const uint32_t bin = bu[u];
            const uint32_t b0 = __shfl_sync(0xffffffffu, bin, 0); // lane 0 is always valid
            if(__all_sync(0xffffffffu, !valid || bin == b0))
            {
                const uint32_t cnt = min(32u, w1 - r);
                if(b0 != run_bin)
                {
                    flush();
                    run_bin = b0;
                    run_start = r;
                }
                run_len += cnt;
                continue;
            }
            flush();
            if(valid) keys[i] = bin | (atomicAdd(&h[bin], 1u) << 16);
        }
    }
    flush();
    __syncthreads();
    uint32_t *row = M + (size_t)blockIdx.x * BIN_SLOTS;
    for(uint32_t b = threadIdx.x; b < BIN_SLOTS; b += BIN_THREADS) row[b] = h[b];
}

// CTA = 32 bins (lanes) x 32 chunks of consecutive tiles (warps): chunk sums, their scan per bin in
// shared memory, then the chunk's entries rewritten as the bin's running count before the tile
__global__ void __launch_bounds__(1024)
        k_bin_columns(uint32_t *__restrict__ M, uint32_t tiles, uint32_t *__restrict__ S,
                      const uint32_t *__restrict__ reordered)
{
    if(*reordered == 0u) return; // every tile keeps its order: the batch is traced as given
    __shared__ uint32_t part[32][33];
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t b = blockIdx.x * 32u + lane;
    const uint32_t per = (tiles + 31u) / 32u;
    const uint32_t t0 = min(warp * per, tiles), t1 = min(t0 + per, tiles);
    uint32_t sum = 0;
    for(uint32_t t = t0; t < t1; ++t) sum += M[(size_t)t * BIN_SLOTS + b];
    part[warp][lane] = sum;
    __syncthreads();
    if(warp == 0)
    {
        uint32_t run = 0;
        for(int w = 0; w < 32; ++w)
        {
            const uint32_t c = part[w][lane];
            part[w][lane] = run;
            run += c;
        }
        S[b] = run;
    }
    __syncthreads();
    uint32_t run = part[warp][lane];
    for(uint32_t t = t0; t < t1; ++t)
    {
        uint32_t *p = M + (size_t)t * BIN_SLOTS + b;
        const uint32_t c = *p;
        *p = run;
        run += c;
    }
}

// F = exclusive scan of S, one CTA: S staged in shared memory (a pad word after every 32 keeps the
// per-thread runs of 32 consecutive bins free of bank conflicts), 32 bins per thread
constexpr size_t BIN_SCAN_SMEM = sizeof(uint32_t) * (NUM_BINS + NUM_BINS / 32);
__global__ void __launch_bounds__(BIN_THREADS)
        k_bin_offsets(const uint32_t *__restrict__ S, uint32_t *__restrict__ F, const uint32_t *__restrict__ reordered)
{
    if(*reordered == 0u) return;
    extern __shared__ uint32_t sm[];
    __shared__ uint32_t warp_sum[32];
    const uint32_t t = threadIdx.x, lane = t & 31u, warp = t >> 5;
    for(uint32_t b = t; b < NUM_BINS; b += BIN_THREADS) sm[b + (b >> 5)] = __ldg(S + b);
    __syncthreads();
    uint32_t *mine = sm + t * 33u; // bins t*32 .. t*32+31
    uint32_t total = 0;
    for(int k = 0; k < 32; ++k) total += mine[k];
    uint32_t x = total;
    for(int o = 1; o < 32; o <<= 1)
    {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if(lane >= (uint32_t)o) x += y;
    }
    if(lane == 31) warp_sum[warp] = x;
    __syncthreads();
    if(warp == 0)
    {
        uint32_t w = warp_sum[lane];
        for(int o = 1; o < 32; o <<= 1)
        {
            const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if(lane >= (uint32_t)o) w += y;
        }
        warp_sum[lane] = w;
    }
    __syncthreads();
    uint32_t acc = (warp ? warp_sum[warp - 1] : 0u) + x - total;
    for(int k = 0; k < 32; ++k)
    {
        const uint32_t c = mine[k];
        mine[k] = acc;
        acc += c;
    }
    __syncthreads();
    for(uint32_t b = t; b < NUM_BINS; b += BIN_THREADS) F[b] = sm[b + (b >> 5)];
    if(t == BIN_THREADS - 1) F[KEEP_BIN] = acc; // the kept rays follow all bins
}

__global__ void __launch_bounds__(256)
        k_bin_place(const uint32_t *__restrict__ keys, uint32_t n_cap, const uint32_t *__restrict__ d_n, uint32_t tile,
                    const uint32_t *__restrict__ M, const uint32_t *__restrict__ F, uint32_t *__restrict__ perm,
                    const uint32_t *__restrict__ reordered)
{
    if(*reordered == 0u) return;
    const uint32_t n = d_n ? min(*d_n, n_cap) : n_cap;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= n) return;
    const uint32_t k = keys[i], bin = k & 0xFFFFu, t = i / tile;
    perm[__ldg(F + bin) + M[(size_t)t * BIN_SLOTS + bin] + (k >> 16)] = i;
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
    // reordered: device word, the number of tiles the binning reordered (0: trace in the given order)
    const uint32_t *reordered = nullptr;
    const uint32_t *perm = bin_rays(ctx, bvh, d_rays, n, nullptr, flags, st, &reordered);
    if(use_persistent())
    {
        if(d_occ)
        {
            if(stats) launch_persistent<true, true>(ctx, bvh, d_rays, n, nullptr, d_occ, cull, st, perm, reordered);
            else launch_persistent<true, false>(ctx, bvh, d_rays, n, nullptr, d_occ, cull, st, perm, reordered);
        }
        else
        {
            if(stats) launch_persistent<false, true>(ctx, bvh, d_rays, n, d_hits, nullptr, cull, st, perm, reordered);
            else launch_persistent<false, false>(ctx, bvh, d_rays, n, d_hits, nullptr, cull, st, perm, reordered);
        }
        if(perm) bin_rays_done(ctx, st);
        return cuda_check(ctx, cudaGetLastError(), "k_trace_persistent");
    }
    const bool small = bvh->depth <= 10;
    if(d_occ)
    {
        if(stats) launch_simple<true, true>(small, grid, st, bvh, d_rays, n, nullptr, d_occ, cull, ctx->d_counters, perm, reordered);
        else launch_simple<true, false>(small, grid, st, bvh, d_rays, n, nullptr, d_occ, cull, ctx->d_counters, perm, reordered);
    }
    else
    {
        if(stats) launch_simple<false, true>(small, grid, st, bvh, d_rays, n, d_hits, nullptr, cull, ctx->d_counters, perm, reordered);
        else launch_simple<false, false>(small, grid, st, bvh, d_rays, n, d_hits, nullptr, cull, ctx->d_counters, perm, reordered);
    }
    if(perm) bin_rays_done(ctx, st);
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

const uint32_t *bin_rays(vkg_ctx *ctx, const vkg_bvh *bvh, const vkg_ray *d_rays, uint32_t n, const uint32_t *d_n,
                         uint32_t flags, cudaStream_t st, const uint32_t **reordered_out)
{
    *reordered_out = nullptr;
    if((flags & VKG_RAY_KEEP_ORDER) || n < BIN_MIN_RAYS || !bvh) return nullptr;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if(cudaStreamIsCapturing(st, &cap) != cudaSuccess || cap != cudaStreamCaptureStatusNone)
    {
        cudaGetLastError();
        return nullptr;
    }
    // the shared-memory opt-in is a per-device attribute
    static uint64_t smem_set = 0;
    const uint64_t dev_bit = 1ull << (ctx->device & 63);
    if(!(smem_set & dev_bit))
    {
        if(cudaFuncSetAttribute(k_bin_tiles, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)BIN_SMEM) != cudaSuccess ||
           cudaFuncSetAttribute(k_bin_offsets, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)BIN_SCAN_SMEM) !=
                   cudaSuccess)
        {
            cudaGetLastError();
            return nullptr;
        }
        smem_set |= dev_bit;
    }
    // tiles of whole 1024-ray rounds: one per SM, or more of BIN_MAX_TILE rays each for larger batches
    const size_t per_sm = ((size_t)n + (size_t)ctx->num_sms - 1) / (size_t)ctx->num_sms;
    const uint32_t tile =
            (uint32_t)std::min<size_t>(BIN_MAX_TILE, (per_sm + BIN_THREADS - 1) / BIN_THREADS * BIN_THREADS);
    const uint32_t tiles = (uint32_t)(((size_t)n + tile - 1) / tile);
    auto &b = ctx->bins;
    if(!b.done && cudaEventCreateWithFlags(&b.done, cudaEventDisableTiming) != cudaSuccess)
    {
        b.done = nullptr;
        cudaGetLastError();
        return nullptr;
    }
    // the previous call's kernels may still use the scratch (another stream)
    if(cudaStreamWaitEvent(st, b.done, 0) != cudaSuccess)
    {
        cudaGetLastError();
        return nullptr;
    }
    if(b.cap < n || b.tiles_cap < tiles)
    {
        // cudaFree waits for the device, so nothing in flight still uses the old buffers
        cudaFree(b.keys);
        cudaFree(b.perm);
        cudaFree(b.tile_counts);
        cudaFree(b.bin_totals);
        b = vkg_ctx::ray_bins{nullptr, nullptr, nullptr, nullptr, 0, 0, b.done};
        // bin_totals: S, F, the count of reordered tiles
        if(cudaMalloc(&b.keys, sizeof(uint32_t) * (size_t)n) != cudaSuccess ||
           cudaMalloc(&b.perm, sizeof(uint32_t) * (size_t)n) != cudaSuccess ||
           cudaMalloc(&b.tile_counts, sizeof(uint32_t) * (size_t)BIN_SLOTS * tiles) != cudaSuccess ||
           cudaMalloc(&b.bin_totals, sizeof(uint32_t) * (2 * (size_t)BIN_SLOTS + 1)) != cudaSuccess)
        {
            cudaFree(b.keys);
            cudaFree(b.perm);
            cudaFree(b.tile_counts);
            cudaFree(b.bin_totals);
            b = vkg_ctx::ray_bins{nullptr, nullptr, nullptr, nullptr, 0, 0, b.done};
            cudaGetLastError();
            return nullptr;
        }
        b.cap = n;
        b.tiles_cap = tiles;
    }
    float3 lo, scale;
    float *plo = &lo.x, *ps = &scale.x;
    for(int a = 0; a < 3; ++a)
    {
        plo[a] = bvh->scene_min[a];
        const float ext = bvh->scene_max[a] - bvh->scene_min[a];
        ps[a] = ext > 0.f ? (float)(1 << BIN_CELL_BITS) / ext : 0.f;
    }
    uint32_t *S = b.bin_totals, *F = b.bin_totals + BIN_SLOTS;
    // the 16-bit bins live in the first half of perm's storage until k_bin_place overwrites it
    // (k_bin_tiles reads them before; k_bin_place reads only keys)
    uint16_t *bins16 = reinterpret_cast<uint16_t *>(b.perm);
    uint32_t *reordered = b.bin_totals + 2 * BIN_SLOTS;
    k_bin_keys<<<(n + 255) / 256, 256, 0, st>>>(d_rays, n, d_n, lo, scale, bins16, reordered);
    k_bin_tiles<<<tiles, BIN_THREADS, BIN_SMEM, st>>>(bins16, n, d_n, tile, b.keys, b.tile_counts, reordered);
    k_bin_columns<<<BIN_SLOTS / 32, 1024, 0, st>>>(b.tile_counts, tiles, S, reordered);
    k_bin_offsets<<<1, BIN_THREADS, BIN_SCAN_SMEM, st>>>(S, F, reordered);
    k_bin_place<<<(n + 255) / 256, 256, 0, st>>>(b.keys, n, d_n, tile, b.tile_counts, F, b.perm, reordered);
    *reordered_out = reordered;
    return b.perm;
}

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

namespace vkg
{
namespace
{
// Chunk sizes of the host variant's pipeline: 2^20 rays, with a ramp of 2^18 and 2^19 at the start
// (the first trace waits only for a short upload; each upload still ends before the trace before it,
// as uploads run about twice as fast as traces) and a 2^18 chunk at the end (a short last download).
// One chunk up to 2^20 rays.
std::vector<uint32_t> host_chunks(uint32_t n)
{
    constexpr uint32_t FULL = 1u << 20, SMALL = 1u << 18;
    std::vector<uint32_t> out;
    if(n <= FULL)
    {
        out.push_back(n);
        return out;
    }
    uint32_t left = n;
    for(uint32_t s: {SMALL, 2 * SMALL})
    {
        out.push_back(s);
        left -= s;
    }
    while(left > FULL + SMALL)
    {
        out.push_back(FULL);
        left -= FULL;
    }
    if(left > 2 * SMALL)
    {
        out.push_back(left - SMALL);
        left = SMALL;
    }
    out.push_back(left);
    return out;
}
}// namespace
}// namespace vkg

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
    // Chunks flow through three engines at once: one stream uploads the chunks back to back, two
    // streams trace alternate chunks (each chunk after its upload), one stream downloads each chunk's
    // hits after its trace. Each chunk has its own region of the staging buffers, so nothing waits
    // for a buffer to be free. The chunks are traced in their given order: binning a chunk costs more
    // than it saves at this size (the one-call variant bins large batches).
    const std::vector<uint32_t> sizes = host_chunks(num_rays);
    const uint32_t chunks = (uint32_t)sizes.size();
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
    for(cudaStream_t &p: ctx->pipe)
        if(!p) VKG_TRY_CUDA(ctx, cudaStreamCreateWithFlags(&p, cudaStreamNonBlocking));
    for(cudaEvent_t &e: ctx->pipe_ev)
        if(!e) VKG_TRY_CUDA(ctx, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    cudaStream_t up = ctx->pipe[2], down = ctx->pipe[3];
    cudaEvent_t up_done = ctx->pipe_ev[5], trace_done = ctx->pipe_ev[6];
    // fork: every stream starts after the work already queued on the caller's stream
    VKG_TRY_CUDA(ctx, cudaEventRecord(ctx->pipe_ev[0], st));
    for(cudaStream_t p: ctx->pipe) VKG_TRY_CUDA(ctx, cudaStreamWaitEvent(p, ctx->pipe_ev[0], 0));
    // (an event is re-recorded for the next chunk only after the wait on its last record is queued)
    vkg_status status = VKG_OK;
    size_t first = 0;
    for(uint32_t c = 0; c < chunks && status == VKG_OK; first += sizes[c], ++c)
    {
        cudaStream_t ts = ctx->pipe[c & 1u];
        const uint32_t n = sizes[c];
        cudaError_t e = cudaMemcpyAsync(d_rays + first, h_rays + first, n * sizeof(vkg_ray), cudaMemcpyHostToDevice, up);
        if(e == cudaSuccess) e = cudaEventRecord(up_done, up);
        if(e == cudaSuccess) e = cudaStreamWaitEvent(ts, up_done, 0);
        if(e != cudaSuccess)
        {
            status = cuda_check(ctx, e, "vkg_closest_hit_host");
            break;
        }
        status = launch_trace(ctx, bvh, d_rays + first, n, d_hits + first, nullptr, flags | VKG_RAY_KEEP_ORDER, ts);
        if(status != VKG_OK) break;
        e = cudaEventRecord(trace_done, ts);
        if(e == cudaSuccess) e = cudaStreamWaitEvent(down, trace_done, 0);
        if(e == cudaSuccess)
            e = cudaMemcpyAsync(h_hits + first, d_hits + first, n * sizeof(vkg_hit), cudaMemcpyDeviceToHost, down);
        if(e != cudaSuccess) status = cuda_check(ctx, e, "vkg_closest_hit_host");
    }
    // join: the caller's stream waits for every stream (also after an error, so nothing is left in flight)
    for(int k = 0; k < 4; ++k)
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
