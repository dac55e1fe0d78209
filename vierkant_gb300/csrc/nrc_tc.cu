// Neural radiance cache inference on the 5th-generation tensor cores (tcgen05, sm_103a).
//
// One CTA of 256 threads owns a tile of 128 queries at a time (persistent over tiles):
//   1. two threads per query encode it (hash-grid levels 0..7 / levels 8..15 + SH + material,
//      nrc_encode.cuh) straight into shared memory as the BF16 A operand of layer 0 (128 x 80,
//      canonical K-major layout, tc.cuh);
//   2. thread 0 issues the layer's tcgen05.mma steps (M = 128, N = 64 or 16, K = 16 each) against
//      the weights, which stay in shared memory for the kernel's lifetime, and commits them to an
//      mbarrier; the FP32 accumulator lives in TMEM (64 columns);
//   3. after the mbarrier (bounded wait), the two threads of a query read its TMEM lane (32 columns
//      each), apply ReLU, pack BF16 and write the next layer's A operand back to shared memory; the
//      last layer's first three columns are the prediction.
// The numerics equal the mma.sync twin (nrc.cu): BF16 inputs / weights / activations, FP32
// accumulation; only the summation order inside an MMA differs.
//
// A wait that runs out (it never should) sets bit 0 of the error word, lets any MMA still in flight
// finish (bounded), frees the TMEM and returns.
#include "nrc_encode.cuh"
#include "tc.cuh"

#include <algorithm>

namespace vkg
{
namespace nrc
{

constexpr uint32_t TC_THREADS = 128, TC_INFER_THREADS = 256, TC_TILE = 128, TC_TMEM_COLS = 64;
constexpr uint32_t TC_W_BYTES = NPARAM * 2;      // all six layers, BF16 B operands (45,056 B)
constexpr uint32_t TC_A_BYTES = TC_TILE * IN * 2; // one A operand (20,480 B)
constexpr uint32_t TC_SMEM = TC_W_BYTES + TC_A_BYTES;
constexpr uint32_t TC_TIMEOUT = 1u;

namespace
{

__device__ __forceinline__ uint32_t eff_n(uint32_t n, const uint32_t *d_n) { return d_n ? min(*d_n, n) : n; }

// FP32 master weights ([in][out] row-major per layer) -> BF16 B operands: layer l as N x K, K-major
__global__ void k_pack_tc(const float *__restrict__ W, uint16_t *__restrict__ wtc)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if(e >= NPARAM) return;
    int l = 0;
    while(l + 1 < NLAYER && e >= layer_off(l + 1)) ++l;
    const int K = layer_in(l), N = layer_out(l), local = e - layer_off(l);
    const int k = local / N, n = local - k * N;
    const __nv_bfloat16 b = __float2bfloat16_rn(W[e]);
    wtc[(layer_off(l) * 2 + tc::canon_offset(n, k, K)) / 2] = *reinterpret_cast<const uint16_t *>(&b);
}

// FP32 master weights -> BF16 operands of the backward: layer l as K_l x N_l (rows = the layer's
// inputs, K = its outputs), K-major, so that D (128 x K_l) = G_l (128 x N_l) W_l^T is one UMMA chain
__global__ void k_pack_tc_t(const float *__restrict__ W, uint16_t *__restrict__ wtc_t)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if(e >= NPARAM) return;
    int l = 0;
    while(l + 1 < NLAYER && e >= layer_off(l + 1)) ++l;
    const int N = layer_out(l), local = e - layer_off(l);
    const int k = local / N, n = local - k * N;
    const __nv_bfloat16 b = __float2bfloat16_rn(W[e]);
    wtc_t[(layer_off(l) * 2 + tc::canon_offset(k, n, N)) / 2] = *reinterpret_cast<const uint16_t *>(&b);
}

// FUSED: encode the feature records here; else read the encoded inputs X (n x 40 u32) written by k_encode
template<bool FUSED>
__global__ void __launch_bounds__(TC_INFER_THREADS)
        k_infer_tc(const float *__restrict__ feats, const uint32_t *__restrict__ X, uint32_t n_cap,
                   const uint32_t *__restrict__ d_n, grid_config gc, const __half2 *__restrict__ grid,
                   const uint16_t *__restrict__ wtc, float *__restrict__ Y, uint32_t *__restrict__ err)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ uint64_t mbar;
    __shared__ uint32_t tslot;
    uint8_t *sw = smem, *sa = smem + TC_W_BYTES;
    const uint32_t tid = threadIdx.x, warp = tid >> 5;
    // thread t works on row r = t mod 128 of the tile; its half h = t / 128 picks the hash-grid levels
    // it encodes (0..7 or 8..15 + the SH / material inputs) and the TMEM columns it drains (warp w reads
    // TMEM lanes 32 (w mod 4) .. + 31)
    const uint32_t r = tid & (TC_TILE - 1), h = tid >> 7;

    for(uint32_t i = tid; i < TC_W_BYTES / 16; i += TC_INFER_THREADS)
        reinterpret_cast<uint4 *>(sw)[i] = reinterpret_cast<const uint4 *>(wtc)[i];
    if(warp == 0) tc::tmem_alloc(&tslot, TC_TMEM_COLS);
    if(tid == 0) tc::mbar_init(&mbar, 1);
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tslot, lane_base = ((warp & 3u) * 32u) << 16;
    const uint32_t sw_addr = tc::smem_addr(sw), sa_addr = tc::smem_addr(sa);
    const uint32_t n = eff_n(n_cap, d_n), tiles = (n + TC_TILE - 1) / TC_TILE;
    uint32_t phase = 0;
    bool failed = false;

    for(uint32_t tile = blockIdx.x; tile < tiles && !failed; tile += gridDim.x)
    {
        const uint32_t q = tile * TC_TILE + r;
        if constexpr(!FUSED)
        {
            // half h copies 16-byte groups h, h + 2, ... of row r
            const uint4 *src = reinterpret_cast<const uint4 *>(X + (size_t)(IN / 2) * q);
#pragma unroll
            for(int j = h; j < IN / 8; j += 2)
                *reinterpret_cast<uint4 *>(sa + tc::canon_offset(r, 8 * j, IN)) =
                        q < n ? src[j] : make_uint4(0u, 0u, 0u, 0u);
        }
        else if(h == 0)
        {
            uint32_t x[8];
            if(q < n)
            {
                const float *f = feats + (size_t)FEAT * q;
                float px, py, pz;
                normalised_pos(gc, f, px, py, pz);
                encode_levels<0, 8>(gc, grid, px, py, pz, x);
            }
            else
                for(int j = 0; j < 8; ++j) x[j] = 0u;
#pragma unroll
            for(int j = 0; j < 2; ++j)
                *reinterpret_cast<uint4 *>(sa + tc::canon_offset(r, 8 * j, IN)) =
                        make_uint4(x[4 * j], x[4 * j + 1], x[4 * j + 2], x[4 * j + 3]);
        }
        else
        {
            uint32_t x[32];
            if(q < n)
            {
                const float *f = feats + (size_t)FEAT * q;
                float px, py, pz;
                normalised_pos(gc, f, px, py, pz);
                encode_levels<8, 16>(gc, grid, px, py, pz, x);
                encode_rest(f, x + 8);
            }
            else
                for(int j = 0; j < 32; ++j) x[j] = 0u;
#pragma unroll
            for(int j = 0; j < 8; ++j)
                *reinterpret_cast<uint4 *>(sa + tc::canon_offset(r, 16 + 8 * j, IN)) =
                        make_uint4(x[4 * j], x[4 * j + 1], x[4 * j + 2], x[4 * j + 3]);
        }
        tc::fence_async_smem();
        tc::fence_before_sync();
        __syncthreads();
#pragma unroll 1
        for(int l = 0; l < NLAYER; ++l)
        {
            const uint32_t K = layer_in(l), N = layer_out(l);
            if(tid == 0)
            {
                tc::fence_after_sync();
                const uint32_t idesc = tc::idesc_bf16(TC_TILE, N);
                const uint32_t wb = sw_addr + (uint32_t)layer_off(l) * 2u;
                for(uint32_t s = 0; s < K / 16; ++s)
                    tc::mma_bf16(tmem, tc::smem_desc(sa_addr + 256u * s, 128u, K * 16u),
                                 tc::smem_desc(wb + 256u * s, 128u, K * 16u), idesc, s > 0);
                tc::mma_commit(&mbar);
            }
            const bool ok = tc::mbar_wait(&mbar, phase);
            if(__syncthreads_or(!ok))
            {
                failed = true;
                break;
            }
            phase ^= 1u;
            tc::fence_after_sync();
            if(l + 1 < NLAYER)
            {
                // this thread's 32 of the 64 columns of row r
                uint32_t hv[16];
#pragma unroll
                for(int c = 0; c < 2; ++c)
                {
                    float v[16];
                    tc::tmem_ld16(tmem + lane_base + 32u * h + 16u * c, v);
                    tc::tmem_ld_wait();
#pragma unroll
                    for(int j = 0; j < 8; ++j) hv[8 * c + j] = pack_bf16(fmaxf(v[2 * j], 0.f), fmaxf(v[2 * j + 1], 0.f));
                }
#pragma unroll
                for(int j = 0; j < 4; ++j)
                    *reinterpret_cast<uint4 *>(sa + tc::canon_offset(r, 32 * h + 8 * j, HID)) =
                            make_uint4(hv[4 * j], hv[4 * j + 1], hv[4 * j + 2], hv[4 * j + 3]);
                tc::fence_async_smem();
            }
            else if(h == 0)
            {
                float v[16];
                tc::tmem_ld16(tmem + lane_base, v);
                tc::tmem_ld_wait();
                if(q < n)
                {
                    Y[3 * (size_t)q] = v[0];
                    Y[3 * (size_t)q + 1] = v[1];
                    Y[3 * (size_t)q + 2] = v[2];
                }
            }
            tc::fence_before_sync();
            __syncthreads();
        }
    }
    if(failed)
    {
        if(tid == 0) atomicOr(err, TC_TIMEOUT);
        tc::mbar_wait(&mbar, phase); // the MMAs in flight, if any
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if(warp == 0) tc::tmem_dealloc(tmem, TC_TMEM_COLS);
}

// diagnostic: D (128 x N, FP32) = A (128 x K BF16, row-major) * B^T (N x K BF16, row-major) through the
// same descriptors, one CTA
__global__ void __launch_bounds__(TC_THREADS)
        k_tc_gemm(const uint16_t *__restrict__ A, const uint16_t *__restrict__ B, uint32_t K, uint32_t N,
                  float *__restrict__ D, uint32_t *__restrict__ err)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ uint64_t mbar;
    __shared__ uint32_t tslot;
    const uint32_t tid = threadIdx.x, warp = tid >> 5;
    uint8_t *sa = smem, *sb = smem + TC_TILE * K * 2;
    for(uint32_t k = 0; k < K; ++k)
        *reinterpret_cast<uint16_t *>(sa + tc::canon_offset(tid, k, K)) = A[(size_t)tid * K + k];
    for(uint32_t e = tid; e < N * K; e += TC_THREADS)
        *reinterpret_cast<uint16_t *>(sb + tc::canon_offset(e / K, e % K, K)) = B[e];
    if(warp == 0) tc::tmem_alloc(&tslot, TC_TMEM_COLS);
    if(tid == 0) tc::mbar_init(&mbar, 1);
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tslot;
    if(tid == 0)
    {
        const uint32_t idesc = tc::idesc_bf16(TC_TILE, N);
        for(uint32_t s = 0; s < K / 16; ++s)
            tc::mma_bf16(tmem, tc::smem_desc(tc::smem_addr(sa) + 256u * s, 128u, K * 16u),
                         tc::smem_desc(tc::smem_addr(sb) + 256u * s, 128u, K * 16u), idesc, s > 0);
        tc::mma_commit(&mbar);
    }
    const bool ok = tc::mbar_wait(&mbar, 0);
    if(__syncthreads_or(!ok))
    {
        if(tid == 0) atomicOr(err, TC_TIMEOUT);
        tc::mbar_wait(&mbar, 0);
    }
    else
    {
        tc::fence_after_sync();
        for(uint32_t c = 0; c < N / 16; ++c)
        {
            float v[16];
            tc::tmem_ld16(tmem + ((warp * 32u) << 16) + 16u * c, v);
            tc::tmem_ld_wait();
            for(int j = 0; j < 16; ++j) D[(size_t)tid * N + 16 * c + j] = v[j];
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if(warp == 0) tc::tmem_dealloc(tmem, TC_TMEM_COLS);
}

// ---- pipelined inference: independent warpgroups ------------------------------------------------
// The single-tile kernel above leaves the tensor core idle while a layer's epilogue (TMEM -> registers
// -> ReLU / BF16 -> shared memory) runs, and the epilogue, not the MMA, sets its time. Here a CTA of
// NWG warpgroups (128 threads each) runs NWG tiles at once: warpgroup g owns 64 TMEM columns
// [64 g, 64 g + 64), one A operand in shared memory, one mbarrier and named barrier g + 1, and its
// thread 0 issues its own MMAs; so while one warpgroup drains its accumulator the tensor core works
// on another's layer. The weights (all six layers, 45 KB) are shared. Thread r of a warpgroup owns
// row r of its tile (TMEM lane r: warp w reads lanes 32 (w mod 4) .. + 31). Inputs are the encoded
// BF16 records of k_encode.
// TRAIN: also store the hidden activations H1..H5 (BF16, 5 x 64 per record in natural column order,
// the layout the backward reads) as the training forward.
template<int NWG, bool TRAIN>
__global__ void __launch_bounds__(NWG * 128)
        k_infer_tc_wg(const uint32_t *__restrict__ X, uint32_t n_cap, const uint32_t *__restrict__ d_n,
                      const uint16_t *__restrict__ wtc, float *__restrict__ Y, uint32_t *__restrict__ err,
                      uint32_t *__restrict__ H)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ uint64_t mbar[NWG];
    __shared__ uint32_t tslot;
    const uint32_t tid = threadIdx.x, warp = tid >> 5, g = tid >> 7, r = tid & 127u;
    uint8_t *sw = smem, *sa = smem + TC_W_BYTES + g * TC_A_BYTES;
    for(uint32_t i = tid; i < TC_W_BYTES / 16; i += NWG * 128)
        reinterpret_cast<uint4 *>(sw)[i] = reinterpret_cast<const uint4 *>(wtc)[i];
    // TMEM columns: 64 per warpgroup, allocated as a power of two of at least 32
    static_assert(NWG >= 1 && NWG <= 8, "at most 512 TMEM columns");
    constexpr uint32_t COLS = NWG * 64 <= 64 ? 64 : (NWG * 64 <= 128 ? 128 : (NWG * 64 <= 256 ? 256 : 512));
    if(warp == 0) tc::tmem_alloc(&tslot, COLS);
    if(tid < NWG) tc::mbar_init(&mbar[tid], 1);
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tslot + 64u * g, lane_base = ((warp & 3u) * 32u) << 16;
    const uint32_t sw_addr = tc::smem_addr(sw), sa_addr = tc::smem_addr(sa);
    const uint32_t n = eff_n(n_cap, d_n), tiles = (n + TC_TILE - 1) / TC_TILE;
    const uint32_t bar_id = g + 1;
    uint32_t phase = 0;
    bool failed = false;

    for(uint32_t tile = blockIdx.x * NWG + g; tile < tiles && !failed; tile += gridDim.x * NWG)
    {
        const uint32_t q = tile * TC_TILE + r;
        const uint4 *src = reinterpret_cast<const uint4 *>(X + (size_t)(IN / 2) * q);
#pragma unroll
        for(int j = 0; j < IN / 8; ++j)
            *reinterpret_cast<uint4 *>(sa + tc::canon_offset(r, 8 * j, IN)) = q < n ? src[j] : make_uint4(0u, 0u, 0u, 0u);
        tc::fence_async_smem();
        tc::fence_before_sync();
        tc::wg_sync(bar_id);
#pragma unroll 1
        for(int l = 0; l < NLAYER; ++l)
        {
            const uint32_t K = layer_in(l), N = layer_out(l);
            if(r == 0)
            {
                tc::fence_after_sync();
                const uint32_t idesc = tc::idesc_bf16(TC_TILE, N);
                const uint32_t wb = sw_addr + (uint32_t)layer_off(l) * 2u;
                for(uint32_t s = 0; s < K / 16; ++s)
                    tc::mma_bf16(tmem, tc::smem_desc(sa_addr + 256u * s, 128u, K * 16u),
                                 tc::smem_desc(wb + 256u * s, 128u, K * 16u), idesc, s > 0);
                tc::mma_commit(&mbar[g]);
            }
            const bool ok = tc::mbar_wait(&mbar[g], phase);
            if(tc::wg_sync_or(bar_id, !ok))
            {
                failed = true;
                break;
            }
            phase ^= 1u;
            tc::fence_after_sync();
            if(l + 1 < NLAYER)
            {
                // two TMEM loads in flight per wait
#pragma unroll
                for(int c2 = 0; c2 < 2; ++c2)
                {
                    float v[2][16];
                    tc::tmem_ld16(tmem + lane_base + 32u * c2, v[0]);
                    tc::tmem_ld16(tmem + lane_base + 32u * c2 + 16u, v[1]);
                    tc::tmem_ld_wait();
#pragma unroll
                    for(int cc = 0; cc < 2; ++cc)
                    {
                        const int c = 2 * c2 + cc;
                        uint32_t hv[8];
#pragma unroll
                        for(int j = 0; j < 8; ++j)
                            hv[j] = pack_bf16(fmaxf(v[cc][2 * j], 0.f), fmaxf(v[cc][2 * j + 1], 0.f));
                        *reinterpret_cast<uint4 *>(sa + tc::canon_offset(r, 16 * c, HID)) =
                                make_uint4(hv[0], hv[1], hv[2], hv[3]);
                        *reinterpret_cast<uint4 *>(sa + tc::canon_offset(r, 16 * c + 8, HID)) =
                                make_uint4(hv[4], hv[5], hv[6], hv[7]);
                        if(TRAIN && q < n)
                        {
                            uint4 *hp = reinterpret_cast<uint4 *>(H + (size_t)q * (5 * HID / 2) + l * (HID / 2) + 8 * c);
                            hp[0] = make_uint4(hv[0], hv[1], hv[2], hv[3]);
                            hp[1] = make_uint4(hv[4], hv[5], hv[6], hv[7]);
                        }
                    }
                }
                tc::fence_async_smem();
            }
            else
            {
                float v[16];
                tc::tmem_ld16(tmem + lane_base, v);
                tc::tmem_ld_wait();
                if(q < n)
                {
                    Y[3 * (size_t)q] = v[0];
                    Y[3 * (size_t)q + 1] = v[1];
                    Y[3 * (size_t)q + 2] = v[2];
                }
            }
            tc::fence_before_sync();
            tc::wg_sync(bar_id);
        }
    }
    if(failed)
    {
        if(r == 0) atomicOr(err, TC_TIMEOUT);
        tc::mbar_wait(&mbar[g], phase); // this warpgroup's MMAs in flight, if any
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if(warp == 0) tc::tmem_dealloc(tslot, COLS);
}

// ---- backward through the layers on tcgen05 ------------------------------------------------------
// The mma.sync k_backward restated on the tensor cores with the warpgroup pipeline of k_infer_tc_wg:
// per tile of 128 records, thread r owns record q = 128 tile + r:
//   dy = dL/dy of the relative L2 loss (|y - t|^2 / (y^2 + 0.01), mean over 3n) -> G block 5 and the
//   BF16 A operand (128 x 16);
//   for l = 5 .. 1: D = G_l W_l^T (UMMA, TMEM), G_{l-1} = D * [H_l > 0] rounded to BF16 -> G block
//   l - 1 and the next A operand (128 x 64);
//   dX (the 32 hash-grid features) = G_0 W_0^T (N = 32) -> dXg in FP32.
// Quantisation points equal k_backward's (FP32 sums, mask in FP32, BF16 rounding of each G); only
// the summation order inside an MMA differs. Weights: wtc_t (k_pack_tc_t), resident in shared memory.
constexpr uint32_t TC_G_BYTES = TC_TILE * HID * 2; // one A operand of the backward (16,384 B)
template<int NWG>
__global__ void __launch_bounds__(NWG * 128)
        k_backward_tc_wg(const uint32_t *__restrict__ H, const float *__restrict__ Y, const float *__restrict__ T,
                         uint32_t n_cap, const uint32_t *__restrict__ d_n, const uint16_t *__restrict__ wtc_t,
                         uint32_t *__restrict__ G, float *__restrict__ dXg, float *__restrict__ loss_sum,
                         uint32_t *__restrict__ err)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ uint64_t mbar[NWG];
    __shared__ uint32_t tslot;
    const uint32_t tid = threadIdx.x, warp = tid >> 5, g = tid >> 7, r = tid & 127u;
    uint8_t *sw = smem, *sa = smem + TC_W_BYTES + g * TC_G_BYTES;
    for(uint32_t i = tid; i < TC_W_BYTES / 16; i += NWG * 128)
        reinterpret_cast<uint4 *>(sw)[i] = reinterpret_cast<const uint4 *>(wtc_t)[i];
    static_assert(NWG >= 1 && NWG <= 8, "at most 512 TMEM columns");
    constexpr uint32_t COLS = NWG * 64 <= 64 ? 64 : (NWG * 64 <= 128 ? 128 : (NWG * 64 <= 256 ? 256 : 512));
    if(warp == 0) tc::tmem_alloc(&tslot, COLS);
    if(tid < NWG) tc::mbar_init(&mbar[tid], 1);
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tslot + 64u * g, lane_base = ((warp & 3u) * 32u) << 16;
    const uint32_t sw_addr = tc::smem_addr(sw), sa_addr = tc::smem_addr(sa);
    const uint32_t n = eff_n(n_cap, d_n), tiles = (n + TC_TILE - 1) / TC_TILE;
    const float inv_count = n ? 1.f / (3.f * (float)n) : 0.f;
    const uint32_t bar_id = g + 1;
    uint32_t phase = 0;
    bool failed = false;
    float loss = 0.f;

    for(uint32_t tile = blockIdx.x * NWG + g; tile < tiles && !failed; tile += gridDim.x * NWG)
    {
        const uint32_t q = tile * TC_TILE + r;
        const bool valid = q < n;
        // dL/dy (raw columns 0..2 of 16)
        float dy[3] = {0.f, 0.f, 0.f};
        if(valid)
            for(int c = 0; c < 3; ++c)
            {
                const float y = Y[(size_t)q * 3 + c], t = T[(size_t)q * 3 + c];
                const float den = y * y + 0.01f;
                const float e = y - t;
                loss += e * e / den;
                dy[c] = 2.f * e / den * inv_count;
            }
        const uint32_t gy0 = pack_bf16(dy[0], dy[1]), gy1 = pack_bf16(dy[2], 0.f);
        if(valid)
        {
            uint4 *gp = reinterpret_cast<uint4 *>(G + (size_t)q * 168 + 160);
            gp[0] = make_uint4(gy0, gy1, 0u, 0u);
            gp[1] = make_uint4(0u, 0u, 0u, 0u);
        }
        // A operand 128 x 16 (K = 16): columns 0..7 and 8..15
        *reinterpret_cast<uint4 *>(sa + tc::canon_offset(r, 0, 16)) = make_uint4(gy0, gy1, 0u, 0u);
        *reinterpret_cast<uint4 *>(sa + tc::canon_offset(r, 8, 16)) = make_uint4(0u, 0u, 0u, 0u);
        tc::fence_async_smem();
        tc::fence_before_sync();
        tc::wg_sync(bar_id);
#pragma unroll 1
        for(int l = NLAYER - 1; l >= 0; --l)
        {
            // D (128 x rows) = A (128 x K') * B^T with B = W_l as rows = inputs, K' = outputs
            const uint32_t Kp = layer_out(l), rows = l == 0 ? 32u : (uint32_t)layer_in(l);
            if(r == 0)
            {
                tc::fence_after_sync();
                const uint32_t idesc = tc::idesc_bf16(TC_TILE, rows);
                const uint32_t wb = sw_addr + (uint32_t)layer_off(l) * 2u;
                for(uint32_t s = 0; s < Kp / 16; ++s)
                    tc::mma_bf16(tmem, tc::smem_desc(sa_addr + 256u * s, 128u, Kp * 16u),
                                 tc::smem_desc(wb + 256u * s, 128u, Kp * 16u), idesc, s > 0);
                tc::mma_commit(&mbar[g]);
            }
            const bool ok = tc::mbar_wait(&mbar[g], phase);
            if(tc::wg_sync_or(bar_id, !ok))
            {
                failed = true;
                break;
            }
            phase ^= 1u;
            tc::fence_after_sync();
            if(l > 0)
            {
                // G_{l-1} = dH_l * [H_l > 0]; H_l is block l - 1 of H
                const uint4 *hp = reinterpret_cast<const uint4 *>(H + (size_t)q * 160 + (l - 1) * 32);
#pragma unroll
                for(int c = 0; c < 4; ++c)
                {
                    float v[16];
                    tc::tmem_ld16(tmem + lane_base + 16u * c, v);
                    tc::tmem_ld_wait();
                    const uint4 h0 = valid ? hp[2 * c] : make_uint4(0u, 0u, 0u, 0u);
                    const uint4 h1 = valid ? hp[2 * c + 1] : make_uint4(0u, 0u, 0u, 0u);
                    const uint32_t hw[8] = {h0.x, h0.y, h0.z, h0.w, h1.x, h1.y, h1.z, h1.w};
                    uint32_t gv[8];
#pragma unroll
                    for(int j = 0; j < 8; ++j)
                    {
                        const float m0 = (hw[j] & 0x7FFFu) ? 1.f : 0.f, m1 = ((hw[j] >> 16) & 0x7FFFu) ? 1.f : 0.f;
                        gv[j] = pack_bf16(v[2 * j] * m0, v[2 * j + 1] * m1);
                    }
                    *reinterpret_cast<uint4 *>(sa + tc::canon_offset(r, 16 * c, HID)) = make_uint4(gv[0], gv[1], gv[2], gv[3]);
                    *reinterpret_cast<uint4 *>(sa + tc::canon_offset(r, 16 * c + 8, HID)) =
                            make_uint4(gv[4], gv[5], gv[6], gv[7]);
                    if(valid)
                    {
                        uint4 *gp = reinterpret_cast<uint4 *>(G + (size_t)q * 168 + (l - 1) * 32 + 8 * c);
                        gp[0] = make_uint4(gv[0], gv[1], gv[2], gv[3]);
                        gp[1] = make_uint4(gv[4], gv[5], gv[6], gv[7]);
                    }
                }
                tc::fence_async_smem();
            }
            else
            {
                // dX of the 32 hash-grid features, FP32
#pragma unroll
                for(int c = 0; c < 2; ++c)
                {
                    float v[16];
                    tc::tmem_ld16(tmem + lane_base + 16u * c, v);
                    tc::tmem_ld_wait();
                    if(valid)
                    {
                        float4 *dp = reinterpret_cast<float4 *>(dXg + (size_t)q * 32 + 16 * c);
#pragma unroll
                        for(int j = 0; j < 4; ++j) dp[j] = make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
                    }
                }
            }
            tc::fence_before_sync();
            tc::wg_sync(bar_id);
        }
    }
    for(int o = 16; o > 0; o >>= 1) loss += __shfl_down_sync(0xffffffffu, loss, o);
    if((tid & 31u) == 0 && loss_sum) atomicAdd(loss_sum, loss * inv_count);
    if(failed)
    {
        if(r == 0) atomicOr(err, TC_TIMEOUT);
        tc::mbar_wait(&mbar[g], phase);
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if(warp == 0) tc::tmem_dealloc(tslot, COLS);
}

// diagnostic: the error path every tcgen05 kernel here takes when a wait runs out, run to its end on
// purpose. Each CTA allocates TMEM and waits on an mbarrier that nothing arrives on, with a limit of
// limit_ns instead of the kernels' 1 s; the wait gives up, the CTA sets TC_TIMEOUT, waits a second
// time (bounded, as the kernels do for MMAs in flight), frees its TMEM and returns. elapsed_ns: the
// longest time one CTA spent in the two waits.
constexpr uint32_t PROBE_TMEM_COLS = 32;
__global__ void __launch_bounds__(TC_THREADS)
        k_wait_probe(uint64_t limit_ns, uint32_t *__restrict__ err, unsigned long long *__restrict__ elapsed_ns)
{
    __shared__ uint64_t mbar;
    __shared__ uint32_t tslot;
    const uint32_t tid = threadIdx.x, warp = tid >> 5;
    if(warp == 0) tc::tmem_alloc(&tslot, PROBE_TMEM_COLS);
    if(tid == 0) tc::mbar_init(&mbar, 1);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tslot;
    const uint64_t t0 = tc::global_ns();
    const bool ok = tc::mbar_wait_for(&mbar, 0, tc::WAIT_LIMIT, limit_ns);
    if(__syncthreads_or(!ok))
    {
        if(tid == 0) atomicOr(err, TC_TIMEOUT);
        tc::mbar_wait_for(&mbar, 0, tc::WAIT_LIMIT, limit_ns);
    }
    if(tid == 0) atomicMax(elapsed_ns, (unsigned long long)(tc::global_ns() - t0));
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if(warp == 0) tc::tmem_dealloc(tmem, PROBE_TMEM_COLS);
}

// ---- weight gradients on tcgen05 --------------------------------------------------------------
// dW_l[k][o] = sum over records s of H_l[s][k] * G_l[s][o] (H_0 = the encoded inputs X, G_l the
// gradient of layer l's pre-activation, both BF16 as the backward stored them). As one UMMA chain per
// layer and chunk of 128 records: D (128 x N_l, FP32 in TMEM) += A (128 x 128) * B (N_l x 128)^T with
// A = H_l^T zero-padded to 128 rows and B = G_l^T, both K-major over the records. The six
// accumulators (336 TMEM columns) stay resident while the CTA walks its chunks; two shared-memory
// buffer pairs let the staging of one layer overlap the MMAs of the previous one.
constexpr uint32_t WG_TC_THREADS = 256, WG_TC_CHUNK = 128, WG_TC_TMEM = 512;
constexpr uint32_t WG_A_BYTES = 128 * WG_TC_CHUNK * 2, WG_B_BYTES = 64 * WG_TC_CHUNK * 2;
// two buffer pairs (96 KB) padded so that a single CTA fits per SM (its TMEM allocation takes all 512
// columns)
constexpr uint32_t WG_TC_SMEM = 120u * 1024u;

__device__ __forceinline__ uint32_t tmem_col(int l) { return l < NLAYER - 1 ? 64u * (uint32_t)l : 320u; }

// 16 BF16 values (8 u32) of record s into rows [r0, r0 + 16) of a K-major operand (K = 128 records)
__device__ __forceinline__ void scatter16(uint8_t *buf, uint32_t r0, uint32_t s, const uint4 (&v)[2])
{
    const uint32_t w[8] = {v[0].x, v[0].y, v[0].z, v[0].w, v[1].x, v[1].y, v[1].z, v[1].w};
#pragma unroll
    for(int j = 0; j < 8; ++j)
    {
        *reinterpret_cast<uint16_t *>(buf + tc::canon_offset(r0 + 2 * j, s, WG_TC_CHUNK)) = (uint16_t)(w[j] & 0xFFFFu);
        *reinterpret_cast<uint16_t *>(buf + tc::canon_offset(r0 + 2 * j + 1, s, WG_TC_CHUNK)) = (uint16_t)(w[j] >> 16);
    }
}

__global__ void __launch_bounds__(WG_TC_THREADS)
        k_wgrad_tc(const uint32_t *__restrict__ X, const uint32_t *__restrict__ H, const uint32_t *__restrict__ G,
                   uint32_t n_cap, const uint32_t *__restrict__ d_n, float *__restrict__ dW, uint32_t *__restrict__ err)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ uint64_t mbar[2];
    __shared__ uint32_t tslot;
    uint8_t *sA[2] = {smem, smem + WG_A_BYTES}, *sB[2] = {smem + 2 * WG_A_BYTES, smem + 2 * WG_A_BYTES + WG_B_BYTES};
    const uint32_t tid = threadIdx.x, warp = tid >> 5, s = tid & (WG_TC_CHUNK - 1), h = tid >> 7;
    // A rows past a layer's inputs stay zero: clear both A buffers once
    for(uint32_t i = tid; i < 2 * WG_A_BYTES / 16; i += WG_TC_THREADS)
        reinterpret_cast<uint4 *>(smem)[i] = make_uint4(0u, 0u, 0u, 0u);
    if(warp == 0) tc::tmem_alloc(&tslot, WG_TC_TMEM);
    if(tid == 0)
    {
        tc::mbar_init(&mbar[0], 1);
        tc::mbar_init(&mbar[1], 1);
    }
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tslot;
    const uint32_t n = d_n ? min(*d_n, n_cap) : n_cap;
    const uint32_t chunks = (n + WG_TC_CHUNK - 1) / WG_TC_CHUNK;
    uint32_t phase[2] = {0u, 0u};
    bool used[2] = {false, false}, failed = false, any = false;
    for(uint32_t c = blockIdx.x; c < chunks && !failed; c += gridDim.x)
    {
        const uint32_t r = c * WG_TC_CHUNK + s;
        const bool valid = r < n;
#pragma unroll 1
        for(int l = 0; l < NLAYER; ++l)
        {
            const uint32_t b = (uint32_t)l & 1u, K = layer_in(l), N = layer_out(l);
            if(used[b])
            {
                // the MMAs that read this buffer pair last must be done before it is overwritten
                const bool ok = tc::mbar_wait(&mbar[b], phase[b]);
                if(__syncthreads_or(!ok))
                {
                    failed = true;
                    break;
                }
                phase[b] ^= 1u;
                used[b] = false;
            }
            // A: this record's layer inputs in blocks of 16 rows, the two halves of the CTA alternating
            const uint32_t *arow = l == 0 ? X + (size_t)r * 40 : H + (size_t)r * 160 + 32 * (l - 1);
            for(uint32_t k0 = 16 * h; k0 < K; k0 += 32)
            {
                uint4 v[2] = {make_uint4(0u, 0u, 0u, 0u), make_uint4(0u, 0u, 0u, 0u)};
                if(valid)
                {
                    v[0] = *reinterpret_cast<const uint4 *>(arow + k0 / 2);
                    v[1] = *reinterpret_cast<const uint4 *>(arow + k0 / 2 + 4);
                }
                scatter16(sA[b], k0, s, v);
            }
            if(b == 0 && l > 0 && h == 1)
                // rows 64..79 of buffer 0 still hold layer 0's last inputs
                for(uint32_t k = 64; k < 80; ++k)
                    *reinterpret_cast<uint16_t *>(sA[b] + tc::canon_offset(k, s, WG_TC_CHUNK)) = 0;
            // B: this record's output gradients in blocks of 16 rows
            const uint32_t *grow = G + (size_t)r * 168 + (l == NLAYER - 1 ? 160 : 32 * l);
            for(uint32_t o0 = 16 * h; o0 < N; o0 += 32)
            {
                uint4 v[2] = {make_uint4(0u, 0u, 0u, 0u), make_uint4(0u, 0u, 0u, 0u)};
                if(valid)
                {
                    v[0] = *reinterpret_cast<const uint4 *>(grow + o0 / 2);
                    v[1] = *reinterpret_cast<const uint4 *>(grow + o0 / 2 + 4);
                }
                scatter16(sB[b], o0, s, v);
            }
            tc::fence_async_smem();
            tc::fence_before_sync();
            __syncthreads();
            if(tid == 0)
            {
                tc::fence_after_sync();
                const uint32_t idesc = tc::idesc_bf16(128, N);
                const uint32_t a0 = tc::smem_addr(sA[b]), b0 = tc::smem_addr(sB[b]);
                for(uint32_t k = 0; k < WG_TC_CHUNK / 16; ++k)
                    tc::mma_bf16(tmem + tmem_col(l), tc::smem_desc(a0 + 256u * k, 128u, WG_TC_CHUNK * 16u),
                                 tc::smem_desc(b0 + 256u * k, 128u, WG_TC_CHUNK * 16u), idesc, any || k > 0);
                tc::mma_commit(&mbar[b]);
            }
            used[b] = true;
        }
        any = true;
    }
    // the last MMAs of both buffers
    for(int b = 0; b < 2 && !failed; ++b)
        if(used[b])
        {
            const bool ok = tc::mbar_wait(&mbar[b], phase[b]);
            if(__syncthreads_or(!ok)) failed = true;
            else
            {
                phase[b] ^= 1u;
                used[b] = false;
            }
        }
    if(failed)
    {
        if(tid == 0) atomicOr(err, TC_TIMEOUT);
        for(int b = 0; b < 2; ++b)
            if(used[b]) tc::mbar_wait(&mbar[b], phase[b]);
    }
    else if(any)
    {
        tc::fence_after_sync();
        // lane k = 32 (warp mod 4) + lane of TMEM holds row k of every layer's accumulator
        const uint32_t k = 32u * (warp & 3u) + (tid & 31u), lane_base = (32u * (warp & 3u)) << 16;
#pragma unroll 1
        for(int l = 0; l < NLAYER; ++l)
        {
            const uint32_t K = layer_in(l), N = layer_out(l);
            for(uint32_t c0 = 16u * h; c0 < N; c0 += 32u)
            {
                float v[16];
                tc::tmem_ld16(tmem + lane_base + tmem_col(l) + c0, v);
                tc::tmem_ld_wait();
                if(k < K)
                    for(int j = 0; j < 16; ++j)
                        if(c0 + j < N) atomicAdd(&dW[layer_off(l) + k * N + c0 + j], v[j]);
            }
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if(warp == 0) tc::tmem_dealloc(tmem, WG_TC_TMEM);
}

}// namespace

vkg_status nrc_wgrad_tc(vkg_ctx *ctx, const uint32_t *X, const uint32_t *H, const uint32_t *G, uint32_t n,
                        const uint32_t *d_n, float *dW, uint32_t *err, cudaStream_t st)
{
    if(n == 0) return VKG_OK;
    VKG_TRY_CUDA(ctx, cudaFuncSetAttribute(k_wgrad_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)WG_TC_SMEM));
    const uint32_t chunks = (n + WG_TC_CHUNK - 1) / WG_TC_CHUNK;
    const uint32_t grid = std::min<uint32_t>(chunks, (uint32_t)ctx->num_sms);
    k_wgrad_tc<<<grid, WG_TC_THREADS, WG_TC_SMEM, st>>>(X, H, G, n, d_n, dW, err);
    return cuda_check(ctx, cudaGetLastError(), "k_wgrad_tc");
}

vkg_status nrc_pack_tc(vkg_ctx *ctx, const float *W, uint16_t *wtc, cudaStream_t st, uint16_t *wtc_t)
{
    k_pack_tc<<<(NPARAM + 255) / 256, 256, 0, st>>>(W, wtc);
    if(wtc_t) k_pack_tc_t<<<(NPARAM + 255) / 256, 256, 0, st>>>(W, wtc_t);
    return cuda_check(ctx, cudaGetLastError(), "k_pack_tc");
}

// the pipelined MLP over encoded inputs X: inference (H null) or the training forward (H receives the
// activations)
template<int NWG>
vkg_status launch_forward_tc(vkg_ctx *ctx, const uint16_t *wtc, const uint32_t *X, uint32_t n, const uint32_t *d_n,
                             float *Y, uint32_t *H, uint32_t *err, cudaStream_t st)
{
    const uint32_t smem = TC_W_BYTES + NWG * TC_A_BYTES;
    auto kern = H ? k_infer_tc_wg<NWG, true> : k_infer_tc_wg<NWG, false>;
    VKG_TRY_CUDA(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    VKG_TRY_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, NWG * 128, smem));
    // TMEM: a resident CTA holds NWG x 64 of the SM's 512 columns
    per_sm = std::max(1, std::min(per_sm, 512 / (NWG * 64)));
    const uint32_t tiles = (n + TC_TILE - 1) / TC_TILE;
    const uint32_t grid_n = std::min<uint32_t>((tiles + NWG - 1) / NWG, (uint32_t)(ctx->num_sms * per_sm));
    kern<<<grid_n, NWG * 128, smem, st>>>(X, n, d_n, wtc, Y, err, H);
    return cuda_check(ctx, cudaGetLastError(), "k_infer_tc_wg");
}

vkg_status nrc_forward_tc(vkg_ctx *ctx, const uint16_t *wtc, const uint32_t *X, uint32_t n, const uint32_t *d_n,
                          float *Y, uint32_t *H, uint32_t *err, cudaStream_t st)
{
    if(n == 0) return VKG_OK;
    // as many tiles in flight per SM as the batch fills: eight warpgroups once every SM gets eight tiles
    const uint32_t tiles = (n + TC_TILE - 1) / TC_TILE, sms = (uint32_t)ctx->num_sms;
    if(tiles >= 8 * sms) return launch_forward_tc<8>(ctx, wtc, X, n, d_n, Y, H, err, st);
    if(tiles >= 4 * sms) return launch_forward_tc<4>(ctx, wtc, X, n, d_n, Y, H, err, st);
    return launch_forward_tc<2>(ctx, wtc, X, n, d_n, Y, H, err, st);
}

template<int NWG>
vkg_status launch_backward_tc(vkg_ctx *ctx, const uint16_t *wtc_t, const uint32_t *H, const float *Y, const float *T,
                              uint32_t n, const uint32_t *d_n, uint32_t *G, float *dXg, float *loss, uint32_t *err,
                              cudaStream_t st)
{
    const uint32_t smem = TC_W_BYTES + NWG * TC_G_BYTES;
    VKG_TRY_CUDA(ctx, cudaFuncSetAttribute(k_backward_tc_wg<NWG>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    VKG_TRY_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_backward_tc_wg<NWG>, NWG * 128, smem));
    per_sm = std::max(1, std::min(per_sm, 512 / (NWG * 64)));
    const uint32_t tiles = (n + TC_TILE - 1) / TC_TILE;
    const uint32_t grid_n = std::min<uint32_t>((tiles + NWG - 1) / NWG, (uint32_t)(ctx->num_sms * per_sm));
    k_backward_tc_wg<NWG><<<grid_n, NWG * 128, smem, st>>>(H, Y, T, n, d_n, wtc_t, G, dXg, loss, err);
    return cuda_check(ctx, cudaGetLastError(), "k_backward_tc_wg");
}

vkg_status nrc_backward_tc(vkg_ctx *ctx, const uint16_t *wtc_t, const uint32_t *H, const float *Y, const float *T,
                           uint32_t n, const uint32_t *d_n, uint32_t *G, float *dXg, float *loss, uint32_t *err,
                           cudaStream_t st)
{
    if(n == 0) return VKG_OK;
    const uint32_t tiles = (n + TC_TILE - 1) / TC_TILE, sms = (uint32_t)ctx->num_sms;
    if(tiles >= 8 * sms) return launch_backward_tc<8>(ctx, wtc_t, H, Y, T, n, d_n, G, dXg, loss, err, st);
    if(tiles >= 4 * sms) return launch_backward_tc<4>(ctx, wtc_t, H, Y, T, n, d_n, G, dXg, loss, err, st);
    return launch_backward_tc<2>(ctx, wtc_t, H, Y, T, n, d_n, G, dXg, loss, err, st);
}

vkg_status nrc_infer_tc(vkg_ctx *ctx, const grid_config &gc, const __half2 *grid, const uint16_t *wtc,
                        const float *feats, const uint32_t *X, uint32_t n, const uint32_t *d_n, float *Y, uint32_t *err,
                        cudaStream_t st)
{
    if(n == 0) return VKG_OK;
    if(X) return nrc_forward_tc(ctx, wtc, X, n, d_n, Y, nullptr, err, st);
    auto kern = X ? k_infer_tc<false> : k_infer_tc<true>;
    VKG_TRY_CUDA(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TC_SMEM));
    int per_sm = 0;
    VKG_TRY_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, TC_INFER_THREADS, TC_SMEM));
    // TMEM: every resident CTA holds 64 of the SM's 512 columns
    per_sm = std::max(1, std::min(per_sm, (int)(512 / TC_TMEM_COLS)));
    const uint32_t tiles = (n + TC_TILE - 1) / TC_TILE;
    const uint32_t grid_n = std::min<uint32_t>(tiles, (uint32_t)(ctx->num_sms * per_sm));
    kern<<<grid_n, TC_INFER_THREADS, TC_SMEM, st>>>(feats, X, n, d_n, gc, grid, wtc, Y, err);
    return cuda_check(ctx, cudaGetLastError(), "k_infer_tc");
}

}// namespace nrc
}// namespace vkg

using namespace vkg;

extern "C" vkg_status vkg_diag_wait_timeout(vkg_ctx *ctx, uint32_t num_ctas, uint64_t limit_ns, uint32_t *d_err,
                                            uint64_t *d_elapsed_ns, void *stream)
{
    if(!ctx) return VKG_ERR_INVALID_ARGUMENT;
    if(!d_err || !d_elapsed_ns || num_ctas == 0 || num_ctas > 4096 || limit_ns == 0 || limit_ns > 100000000ull)
        return set_error(ctx, VKG_ERR_INVALID_ARGUMENT,
                         "vkg_diag_wait_timeout: need 1 <= num_ctas <= 4096 and 0 < limit_ns <= 1e8");
    if(vkg_status s = bind_device(ctx); s != VKG_OK) return s;
    nrc::k_wait_probe<<<num_ctas, nrc::TC_THREADS, 0, static_cast<cudaStream_t>(stream)>>>(
            limit_ns, d_err, reinterpret_cast<unsigned long long *>(d_elapsed_ns));
    return cuda_check(ctx, cudaGetLastError(), "k_wait_probe");
}

extern "C" vkg_status vkg_diag_tc_gemm(vkg_ctx *ctx, const uint16_t *d_a, const uint16_t *d_b, uint32_t k,
                                       uint32_t n, float *d_d, uint32_t *d_err, void *stream)
{
    if(!ctx) return VKG_ERR_INVALID_ARGUMENT;
    if(!d_a || !d_b || !d_d || !d_err || k == 0 || k % 16 || k > 256 || n < 16 || n > nrc::TC_TMEM_COLS || n % 16)
        return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_diag_tc_gemm: need 16 <= n <= 64, k <= 256, multiples of 16");
    if(vkg_status s = bind_device(ctx); s != VKG_OK) return s;
    const uint32_t smem = nrc::TC_TILE * k * 2 + n * k * 2;
    VKG_TRY_CUDA(ctx, cudaFuncSetAttribute(nrc::k_tc_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    nrc::k_tc_gemm<<<1, nrc::TC_THREADS, smem, static_cast<cudaStream_t>(stream)>>>(d_a, d_b, k, n, d_d, d_err);
    return cuda_check(ctx, cudaGetLastError(), "k_tc_gemm");
}
