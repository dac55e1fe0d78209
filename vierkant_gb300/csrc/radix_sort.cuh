// Stable LSD radix sort of (key, value) pairs, 8 bits per pass: per-tile digit histograms, one
// exclusive scan over all (digit, tile) counts, and a scatter whose ranks within a warp come from
// __match_any_sync. Used by the BVH builds (Morton codes). The optional d_n points to a device-side
// element count (<= the capacity the grid was sized for).
#pragma once

#include "internal.hpp"

namespace vkg
{
namespace
{

constexpr int SORT_THREADS = 256;
constexpr int SORT_ITEMS = 16;
constexpr int SORT_TILE = SORT_THREADS * SORT_ITEMS; // keys per block

__global__ void k_radix_hist(const uint32_t *__restrict__ keys, uint32_t n_cap, int shift, uint32_t *__restrict__ counts,
                             uint32_t nblocks, const uint32_t *__restrict__ d_n = nullptr)
{
    const uint32_t n = d_n ? min(*d_n, n_cap) : n_cap;
    __shared__ uint32_t hist[256];
    hist[threadIdx.x] = 0;
    __syncthreads();
    size_t base = (size_t)blockIdx.x * SORT_TILE;
    for(int it = 0; it < SORT_ITEMS; ++it)
    {
        size_t i = base + (size_t)it * SORT_THREADS + threadIdx.x;
        if(i < n) atomicAdd(&hist[(keys[i] >> shift) & 0xFFu], 1u);
    }
    __syncthreads();
    counts[(size_t)threadIdx.x * nblocks + blockIdx.x] = hist[threadIdx.x];
}

// exclusive scan of `count` words in place (single CTA of 1024 threads)
__global__ void k_scan_exclusive(uint32_t *__restrict__ data, uint32_t count, uint32_t *__restrict__ total)
{
    __shared__ uint32_t warp_sums[32];
    __shared__ uint32_t carry;
    if(threadIdx.x == 0) carry = 0;
    __syncthreads();
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    for(uint32_t base = 0; base < count; base += 1024u)
    {
        uint32_t i = base + threadIdx.x;
        uint32_t v = i < count ? data[i] : 0u;
        uint32_t x = v;
        for(int o = 1; o < 32; o <<= 1)
        {
            uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if(lane >= (uint32_t)o) x += y;
        }
        if(lane == 31) warp_sums[warp] = x;
        __syncthreads();
        if(warp == 0)
        {
            uint32_t w = warp_sums[lane];
            for(int o = 1; o < 32; o <<= 1)
            {
                uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
                if(lane >= (uint32_t)o) w += y;
            }
            warp_sums[lane] = w; // inclusive over warps
        }
        __syncthreads();
        uint32_t warp_prefix = warp ? warp_sums[warp - 1] : 0u;
        uint32_t c = carry;
        if(i < count) data[i] = c + warp_prefix + x - v;
        __syncthreads();
        if(threadIdx.x == 1023) carry = c + warp_sums[31];
        __syncthreads();
    }
    if(threadIdx.x == 0 && total) *total = carry;
}

__global__ void k_radix_scatter(const uint32_t *__restrict__ keys_in, const uint32_t *__restrict__ vals_in, uint32_t n_cap,
                                int shift, const uint32_t *__restrict__ offsets, uint32_t nblocks,
                                uint32_t *__restrict__ keys_out, uint32_t *__restrict__ vals_out,
                                const uint32_t *__restrict__ d_n = nullptr)
{
    const uint32_t n = d_n ? min(*d_n, n_cap) : n_cap;
    __shared__ uint32_t s_off[256];
    __shared__ uint32_t s_warp[8][257];
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    s_off[tid] = offsets[(size_t)tid * nblocks + blockIdx.x];
    const uint32_t lt_mask = (1u << lane) - 1u;
    size_t base = (size_t)blockIdx.x * SORT_TILE;
    for(int it = 0; it < SORT_ITEMS; ++it)
    {
        for(uint32_t j = tid; j < 8u * 257u; j += SORT_THREADS) (&s_warp[0][0])[j] = 0u;
        __syncthreads();
        size_t i = base + (size_t)it * SORT_THREADS + tid;
        bool valid = i < n;
        uint32_t key = valid ? keys_in[i] : 0u;
        uint32_t val = valid ? vals_in[i] : 0u;
        uint32_t digit = valid ? ((key >> shift) & 0xFFu) : 256u;
        uint32_t peers = __match_any_sync(0xffffffffu, digit);
        uint32_t rank = __popc(peers & lt_mask);
        if(rank == 0) s_warp[warp][digit] = __popc(peers);
        __syncthreads();
        // exclusive prefix over the 8 warps for digit `tid`
        uint32_t run = 0;
        for(int w = 0; w < 8; ++w)
        {
            uint32_t c = s_warp[w][tid];
            s_warp[w][tid] = run;
            run += c;
        }
        __syncthreads();
        if(valid)
        {
            uint32_t pos = s_off[digit] + s_warp[warp][digit] + rank;
            keys_out[pos] = key;
            vals_out[pos] = val;
        }
        __syncthreads();
        s_off[tid] += run;
        __syncthreads();
    }
}

// ---- Karras radix tree ------------------------------------------------------------------------
__device__ __forceinline__ int kdelta(const uint32_t *codes, int64_t n, int64_t i, int64_t j)
{
    if(j < 0 || j >= n) return -1;
    uint32_t a = codes[i], b = codes[j];
    if(a == b) return 32 + __clz((uint32_t)i ^ (uint32_t)j);
    return __clz(a ^ b);
}


}// namespace
}// namespace vkg
