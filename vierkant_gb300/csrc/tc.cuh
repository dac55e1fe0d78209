// Blackwell (sm_103a) tensor-core building blocks in inline PTX: mbarriers with bounded waits,
// TMEM allocation, tcgen05.mma (kind::f16, BF16 x BF16 -> FP32, operands in shared memory) with
// its commit, tcgen05.ld, and the shared-memory matrix descriptor for the canonical no-swizzle
// K-major layout.
//
// Canonical K-major layout without swizzle (PTX ISA, tcgen05 shared memory matrix layouts): the
// operand is cut into core matrices of 8 rows x 16 bytes (8 BF16), each stored as 128 contiguous
// bytes (row r at r * 16). Core matrix (row group i, K group j) starts at i * SBO + j * LBO. This
// file uses LBO = 128 (K groups adjacent) and SBO = K * 16 (one row group after another), so an
// R x K operand occupies exactly R * K * 2 bytes and one MMA step of K = 16 advances the start
// address by 256 bytes.
#pragma once

#include <cstdint>

namespace vkg
{
namespace tc
{

// a wait gives up after this many mbarrier.try_wait attempts or this much wall time, whichever first
constexpr uint32_t WAIT_LIMIT = 1u << 24;
constexpr uint64_t WAIT_NS = 1000000000ull; // 1 s

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(count));
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n}\n"
                 : "=r"(ok)
                 : "r"(smem_addr(bar)), "r"(parity)
                 : "memory");
    return ok != 0;
}

__device__ __forceinline__ uint64_t global_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// true once the phase with the given parity completed; false after max_tries attempts or max_ns
__device__ __forceinline__ bool mbar_wait_for(uint64_t *bar, uint32_t parity, uint32_t max_tries, uint64_t max_ns)
{
    if(mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = global_ns();
    for(uint32_t i = 0; i < max_tries; ++i)
    {
        if(mbar_try_wait(bar, parity)) return true;
        if((i & 255u) == 255u && global_ns() - t0 > max_ns) return false;
    }
    return false;
}

// the kernels' wait: at most WAIT_LIMIT attempts or WAIT_NS
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity)
{
    return mbar_wait_for(bar, parity, WAIT_LIMIT, WAIT_NS);
}

// ---- named barriers over one warpgroup (128 threads); id 0 is __syncthreads' ----------------------
__device__ __forceinline__ void wg_sync(uint32_t id) { asm volatile("barrier.sync %0, 128;\n" ::"r"(id) : "memory"); }

// barrier over the warpgroup that also ORs a predicate across its threads
__device__ __forceinline__ bool wg_sync_or(uint32_t id, bool pred)
{
    uint32_t out;
    asm volatile("{\n\t.reg .pred p, q;\n\tsetp.ne.u32 q, %1, 0;\n\tbarrier.red.or.pred p, %2, 128, q;\n\t"
                 "selp.u32 %0, 1, 0, p;\n}\n"
                 : "=r"(out)
                 : "r"((uint32_t)pred), "r"(id)
                 : "memory");
    return out != 0;
}

// ---- TMEM ----------------------------------------------------------------------------------------
// one full warp; the base address is written to *slot (shared memory)
__device__ __forceinline__ void tmem_alloc(uint32_t *slot, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_addr(slot)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }
// generic-proxy shared-memory writes -> visible to the tensor core (async proxy)
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

// ---- descriptors -----------------------------------------------------------------------------------
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1u << 46; // descriptor version (tcgen05)
    // base offset 0, absolute LBO mode 0, layout type 0 = no swizzle
    return d;
}

// kind::f16 instruction descriptor: D FP32, A and B BF16, both K-major, shape M x N
__host__ __device__ constexpr uint32_t idesc_bf16(uint32_t M, uint32_t N)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((N >> 3) << 17) | ((M >> 4) << 24);
}

// D[tmem] (+)= A * B^T for one K = 16 step; issued by a single thread
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, bool accumulate)
{
    asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
                 "l"(adesc), "l"(bdesc), "r"(idesc), "r"((uint32_t)accumulate)
                 : "memory");
}

// the mbarrier receives one arrival once every MMA issued so far by this thread has completed
__device__ __forceinline__ void mma_commit(uint64_t *bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(smem_addr(bar))
                 : "memory");
}

// 16 consecutive FP32 columns of this thread's TMEM lane (32x32b shape: warp w reads lanes 32w..32w+31)
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16])
{
    uint32_t r[16];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                 : "r"(taddr)
                 : "memory");
#pragma unroll
    for(int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmem_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory"); }

// byte offset of element (row, k) of an R x K BF16 operand in the canonical layout above
__host__ __device__ constexpr uint32_t canon_offset(uint32_t row, uint32_t k, uint32_t K)
{
    return (row >> 3) * (K * 16u) + (k >> 3) * 128u + (row & 7u) * 16u + (k & 7u) * 2u;
}

}// namespace tc
}// namespace vkg
