// Neural radiance cache: encodings, fully-fused tensor-core MLP (forward / backward), weight
// gradients, hash-grid gradients and Adam. Shape and encodings: see nrc.cuh.
//
// MLP kernels keep a warp's 16 samples in registers from layer to layer: the FP32 accumulator
// fragment of an m16n8k16 MMA for output columns (16j .. 16j+15) is exactly the A fragment of the
// next layer's k-tile j, so ReLU + BF16 packing is the only work between layers. B fragments
// (weights, and transposed weights for the backward) are pre-packed per lane and staged in shared
// memory. This mma.sync path is the correctness twin of the tcgen05 inference kernel
// (nrc_tc.cu) and the training path.
#include "nrc_encode.cuh"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

struct vkg_nrc
{
    vkg_ctx *ctx = nullptr;
    vkg_nrc_config cfg{};
    vkg::nrc::grid_config gc{};
    uint32_t table = 0;          // entries per level
    size_t ngrid = 0;            // grid parameters (levels * table * 2)
    float lr = 1e-2f, b1 = 0.9f, b2 = 0.99f, eps = 1e-15f;
    uint32_t *d_state = nullptr; // [0] Adam steps taken, [1] 1 if the current step has records
    float *grid = nullptr, *grid_g = nullptr, *grid_m = nullptr, *grid_v = nullptr;
    __half2 *grid_h = nullptr;
    float *w = nullptr, *w_g = nullptr, *w_m = nullptr, *w_v = nullptr;
    uint2 *frag = nullptr, *fragT = nullptr;
    uint16_t *wtc = nullptr;     // BF16 weights in the tcgen05 operand layout
    uint16_t *wtc_t = nullptr;   // the same, transposed per layer (the backward's operands)
    uint32_t *d_err = nullptr;   // tensor-core kernel error word
    uint32_t tc_infer = 1;       // 1: mma.sync MLP, 2: tcgen05 MLP, 3: tcgen05 MLP with the encoding fused
    bool tc_train = false;       // weight gradients on tcgen05 (else FP32 CUDA cores)
    bool tc_forward = false;     // the training forward on tcgen05 (else the mma.sync twin)
    // training / inference scratch, sized for `cap` samples
    uint32_t cap = 0;
    uint32_t *X = nullptr, *H = nullptr, *G = nullptr;
    float *Y = nullptr, *dXg = nullptr, *loss = nullptr;
};

namespace vkg
{
namespace nrc
{
namespace
{

constexpr int MLP_THREADS = 128;

__device__ __forceinline__ float bf_lo(uint32_t v) { return __uint_as_float(v << 16); }
__device__ __forceinline__ float bf_hi(uint32_t v) { return __uint_as_float(v & 0xFFFF0000u); }

__device__ __forceinline__ void mma16816(float (&d)[4], const uint32_t (&a)[4], uint2 b)
{
    asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                 "{%0,%1,%2,%3};\n"
                 : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
                 : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b.x), "r"(b.y));
}

// accumulator fragments of 2*KT n-tiles -> A fragments of KT k-tiles (optionally ReLU)
template<int KT, bool RELU>
__device__ __forceinline__ void acc_to_a(const float (&acc)[2 * KT][4], uint32_t (&a)[KT][4])
{
#pragma unroll
    for(int k = 0; k < KT; ++k)
    {
        float v[8];
#pragma unroll
        for(int q = 0; q < 4; ++q)
        {
            v[q] = acc[2 * k][q];
            v[4 + q] = acc[2 * k + 1][q];
        }
        if(RELU)
#pragma unroll
            for(int q = 0; q < 8; ++q) v[q] = fmaxf(v[q], 0.f);
        a[k][0] = pack_bf16(v[0], v[1]);
        a[k][1] = pack_bf16(v[2], v[3]);
        a[k][2] = pack_bf16(v[4], v[5]);
        a[k][3] = pack_bf16(v[6], v[7]);
    }
}

// one dense layer for a 16-row tile: acc[N/8] = a[K/16] x W
template<int KT, int NT>
__device__ __forceinline__ void layer(const uint32_t (&a)[KT][4], const uint2 *__restrict__ sw, int lane,
                                      float (&acc)[NT][4])
{
#pragma unroll
    for(int j = 0; j < NT; ++j)
    {
        acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
#pragma unroll
        for(int k = 0; k < KT; ++k) mma16816(acc[j], a[k], sw[(k * NT + j) * 32 + lane]);
    }
}

__device__ __forceinline__ uint32_t eff_count(uint32_t n, const uint32_t *d_n) { return d_n ? min(*d_n, n) : n; }

__global__ void k_encode(const float *__restrict__ feats, uint32_t n, const uint32_t *__restrict__ d_n, grid_config gc,
                         const __half2 *__restrict__ grid, uint32_t *__restrict__ X)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= eff_count(n, d_n)) return;
    encode_record(gc, grid, feats + (size_t)FEAT * i, X + (size_t)(IN / 2) * i);
}

// ---- fused forward -------------------------------------------------------------------------------
// TRAIN: also saves H1..H5 (BF16) for the backward
template<bool TRAIN>
__global__ void __launch_bounds__(MLP_THREADS)
        k_forward(const uint32_t *__restrict__ X, uint32_t n_cap, const uint32_t *__restrict__ d_n,
                  const uint2 *__restrict__ wfrag, float *__restrict__ Y, uint32_t *__restrict__ H)
{
    __shared__ uint2 sw[NFRAG];
    for(int i = threadIdx.x; i < NFRAG; i += blockDim.x) sw[i] = wfrag[i];
    __syncthreads();
    const uint32_t n = eff_count(n_cap, d_n);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int g = lane >> 2, tig = lane & 3;
    const uint32_t ntiles = (n + 15) / 16;
    for(uint32_t tile = blockIdx.x * nw + warp; tile < ntiles; tile += gridDim.x * nw)
    {
        const uint32_t ra = tile * 16 + g, rb = ra + 8;
        const bool va = ra < n, vb = rb < n;
        uint32_t a0[5][4];
#pragma unroll
        for(int k = 0; k < 5; ++k)
        {
            a0[k][0] = va ? X[(size_t)ra * 40 + 8 * k + tig] : 0u;
            a0[k][1] = vb ? X[(size_t)rb * 40 + 8 * k + tig] : 0u;
            a0[k][2] = va ? X[(size_t)ra * 40 + 8 * k + tig + 4] : 0u;
            a0[k][3] = vb ? X[(size_t)rb * 40 + 8 * k + tig + 4] : 0u;
        }
        float acc[8][4];
        uint32_t h[4][4];
        layer<5, 8>(a0, sw + frag_off(0), lane, acc);
        acc_to_a<4, true>(acc, h);
#pragma unroll
        for(int l = 1; l <= 5; ++l)
        {
            if(TRAIN)
            {
                const int blk = (l - 1) * 32;
#pragma unroll
                for(int k = 0; k < 4; ++k)
                {
                    if(va)
                    {
                        H[(size_t)ra * 160 + blk + 8 * k + tig] = h[k][0];
                        H[(size_t)ra * 160 + blk + 8 * k + tig + 4] = h[k][2];
                    }
                    if(vb)
                    {
                        H[(size_t)rb * 160 + blk + 8 * k + tig] = h[k][1];
                        H[(size_t)rb * 160 + blk + 8 * k + tig + 4] = h[k][3];
                    }
                }
            }
            if(l == 5) break;
            layer<4, 8>(h, sw + frag_off(l), lane, acc);
            acc_to_a<4, true>(acc, h);
        }
        float o[2][4];
        layer<4, 2>(h, sw + frag_off(5), lane, o);
        if(tig == 0)
        {
            if(va)
            {
                Y[(size_t)ra * 3] = o[0][0];
                Y[(size_t)ra * 3 + 1] = o[0][1];
            }
            if(vb)
            {
                Y[(size_t)rb * 3] = o[0][2];
                Y[(size_t)rb * 3 + 1] = o[0][3];
            }
        }
        else if(tig == 1)
        {
            if(va) Y[(size_t)ra * 3 + 2] = o[0][0];
            if(vb) Y[(size_t)rb * 3 + 2] = o[0][2];
        }
    }
}

// ---- fused backward (activation gradients) -------------------------------------------------------
__device__ __forceinline__ float relu_mask(uint32_t hpair, bool hi)
{
    const uint32_t bits = hi ? (hpair >> 16) : (hpair & 0xFFFFu);
    return (bits & 0x7FFFu) ? 1.f : 0.f;
}

__global__ void __launch_bounds__(MLP_THREADS)
        k_backward(const uint32_t *__restrict__ H, const float *__restrict__ Y, const float *__restrict__ T,
                   uint32_t n_cap, const uint32_t *__restrict__ d_n, const uint2 *__restrict__ wfragT,
                   uint32_t *__restrict__ G, float *__restrict__ dXg, float *__restrict__ loss_sum)
{
    __shared__ uint2 sw[NFRAG];
    for(int i = threadIdx.x; i < NFRAG; i += blockDim.x) sw[i] = wfragT[i];
    __syncthreads();
    const uint32_t n = eff_count(n_cap, d_n);
    const float inv_count = n ? 1.f / (3.f * (float)n) : 0.f;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int g = lane >> 2, tig = lane & 3;
    const uint32_t ntiles = (n + 15) / 16;
    float loss = 0.f;
    for(uint32_t tile = blockIdx.x * nw + warp; tile < ntiles; tile += gridDim.x * nw)
    {
        const uint32_t ra = tile * 16 + g, rb = ra + 8;
        const bool va = ra < n, vb = rb < n;
        // dL/dy of the relative L2 loss for columns 2tig, 2tig+1 (only 0..2 exist)
        float dy[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for(int q = 0; q < 4; ++q)
        {
            const uint32_t r = q < 2 ? ra : rb;
            const int c = 2 * tig + (q & 1);
            if((q < 2 ? va : vb) && c < 3)
            {
                const float y = Y[(size_t)r * 3 + c], t = T[(size_t)r * 3 + c];
                const float den = y * y + 0.01f;
                const float e = y - t;
                loss += e * e / den;
                dy[q] = 2.f * e / den * inv_count;
            }
        }
        uint32_t gy[1][4] = {{pack_bf16(dy[0], dy[1]), pack_bf16(dy[2], dy[3]), 0u, 0u}};
        if(va)
        {
            G[(size_t)ra * 168 + 160 + tig] = gy[0][0];
            G[(size_t)ra * 168 + 160 + tig + 4] = 0u;
        }
        if(vb)
        {
            G[(size_t)rb * 168 + 160 + tig] = gy[0][1];
            G[(size_t)rb * 168 + 160 + tig + 4] = 0u;
        }
        float acc[8][4];
        uint32_t gz[4][4];
        // layer 5: dH5 = G5 * W5^T (K' = 16)
        layer<1, 8>(gy, sw + fragT_off(5), lane, acc);
#pragma unroll
        for(int l = 5; l >= 1; --l)
        {
            // G_{l-1} = dH_l * [H_l > 0]; H_l is block l-1 of H
            const int blk = (l - 1) * 32;
#pragma unroll
            for(int j = 0; j < 8; ++j)
            {
                const int u = blk + 4 * j + tig;
                const uint32_t ha = va ? H[(size_t)ra * 160 + u] : 0u, hb = vb ? H[(size_t)rb * 160 + u] : 0u;
                acc[j][0] *= relu_mask(ha, false);
                acc[j][1] *= relu_mask(ha, true);
                acc[j][2] *= relu_mask(hb, false);
                acc[j][3] *= relu_mask(hb, true);
            }
            acc_to_a<4, false>(acc, gz);
            const int gb = (l - 1) * 32;
#pragma unroll
            for(int k = 0; k < 4; ++k)
            {
                if(va)
                {
                    G[(size_t)ra * 168 + gb + 8 * k + tig] = gz[k][0];
                    G[(size_t)ra * 168 + gb + 8 * k + tig + 4] = gz[k][2];
                }
                if(vb)
                {
                    G[(size_t)rb * 168 + gb + 8 * k + tig] = gz[k][1];
                    G[(size_t)rb * 168 + gb + 8 * k + tig + 4] = gz[k][3];
                }
            }
            if(l > 1) layer<4, 8>(gz, sw + fragT_off(l - 1), lane, acc);
        }
        // dX (first 32 columns: the hash-grid features) = G0 * W0^T
        float dx[4][4];
        {
            const uint2 *s0 = sw + fragT_off(0);
#pragma unroll
            for(int j = 0; j < 4; ++j)
            {
                dx[j][0] = dx[j][1] = dx[j][2] = dx[j][3] = 0.f;
#pragma unroll
                for(int k = 0; k < 4; ++k) mma16816(dx[j], gz[k], s0[(k * 10 + j) * 32 + lane]);
            }
        }
#pragma unroll
        for(int j = 0; j < 4; ++j)
        {
            if(va)
            {
                dXg[(size_t)ra * 32 + 8 * j + 2 * tig] = dx[j][0];
                dXg[(size_t)ra * 32 + 8 * j + 2 * tig + 1] = dx[j][1];
            }
            if(vb)
            {
                dXg[(size_t)rb * 32 + 8 * j + 2 * tig] = dx[j][2];
                dXg[(size_t)rb * 32 + 8 * j + 2 * tig + 1] = dx[j][3];
            }
        }
    }
    for(int o = 16; o > 0; o >>= 1) loss += __shfl_down_sync(0xffffffffu, loss, o);
    if(lane == 0 && loss_sum) atomicAdd(loss_sum, loss * inv_count);
}

// ---- weight gradients: dW_l = H_l^T G_l (FP32, 4x4 register blocks, 128-sample chunks) ----------
constexpr int WG_THREADS = 256;
constexpr int WG_CHUNK = 64;

__device__ __forceinline__ void bf16_row_to_smem(const uint32_t *src, int words, float *dst)
{
    for(int w = 0; w < words; ++w)
    {
        const uint32_t v = src[w];
        dst[2 * w] = bf_lo(v);
        dst[2 * w + 1] = bf_hi(v);
    }
}

__global__ void __launch_bounds__(WG_THREADS)
        k_wgrad(const uint32_t *__restrict__ X, const uint32_t *__restrict__ H, const uint32_t *__restrict__ G,
                uint32_t n_cap, const uint32_t *__restrict__ d_n, float *__restrict__ dW)
{
    const uint32_t n = eff_count(n_cap, d_n);
    __shared__ __align__(16) float sA[WG_CHUNK][IN];
    __shared__ __align__(16) float sB[WG_CHUNK][HID];
    for(int l = 0; l < NLAYER; ++l)
    {
        const int K = layer_in(l), N = layer_out(l);
        const int nb = (K / 4) * (N / 4);
        float acc[2][16];
#pragma unroll
        for(int q = 0; q < 2; ++q)
#pragma unroll
            for(int e = 0; e < 16; ++e) acc[q][e] = 0.f;
        for(uint32_t c0 = blockIdx.x * WG_CHUNK; c0 < n; c0 += gridDim.x * WG_CHUNK)
        {
            __syncthreads();
            for(int s = threadIdx.x; s < WG_CHUNK; s += blockDim.x)
            {
                const uint32_t r = c0 + s;
                if(r < n)
                {
                    if(l == 0) bf16_row_to_smem(X + (size_t)r * 40, 40, sA[s]);
                    else bf16_row_to_smem(H + (size_t)r * 160 + (l - 1) * 32, 32, sA[s]);
                    const int gb = l == NLAYER - 1 ? 160 : l * 32;
                    bf16_row_to_smem(G + (size_t)r * 168 + gb, N / 2, sB[s]);
                }
                else
                {
                    for(int k = 0; k < K; ++k) sA[s][k] = 0.f;
                    for(int o = 0; o < N; ++o) sB[s][o] = 0.f;
                }
            }
            __syncthreads();
#pragma unroll
            for(int q = 0; q < 2; ++q)
            {
                const int b = threadIdx.x + q * WG_THREADS;
                if(b >= nb) continue;
                const int k0 = (b / (N / 4)) * 4, o0 = (b % (N / 4)) * 4;
                for(int s = 0; s < WG_CHUNK; ++s)
                {
                    const float4 a = *reinterpret_cast<const float4 *>(&sA[s][k0]);
                    const float4 bb = *reinterpret_cast<const float4 *>(&sB[s][o0]);
                    const float av[4] = {a.x, a.y, a.z, a.w}, bv[4] = {bb.x, bb.y, bb.z, bb.w};
#pragma unroll
                    for(int i = 0; i < 4; ++i)
#pragma unroll
                        for(int j = 0; j < 4; ++j) acc[q][i * 4 + j] += av[i] * bv[j];
                }
            }
        }
#pragma unroll
        for(int q = 0; q < 2; ++q)
        {
            const int b = threadIdx.x + q * WG_THREADS;
            if(b >= nb) continue;
            const int k0 = (b / (N / 4)) * 4, o0 = (b % (N / 4)) * 4;
#pragma unroll
            for(int i = 0; i < 4; ++i)
#pragma unroll
                for(int j = 0; j < 4; ++j) atomicAdd(&dW[layer_off(l) + (k0 + i) * N + o0 + j], acc[q][i * 4 + j]);
        }
    }
}

__global__ void k_grid_backward(const float *__restrict__ feats, uint32_t n, const uint32_t *__restrict__ d_n,
                                grid_config gc, const float *__restrict__ dXg, float *__restrict__ grid_g)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= eff_count(n, d_n)) return;
    float px, py, pz;
    normalised_pos(gc, feats + (size_t)FEAT * i, px, py, pz);
    const uint32_t T = 1u << gc.log2_t;
    for(uint32_t l = 0; l < gc.levels; ++l)
    {
        const float g0 = dXg[(size_t)i * 32 + 2 * l], g1 = dXg[(size_t)i * 32 + 2 * l + 1];
        if(g0 == 0.f && g1 == 0.f) continue;
        corner_iter c = level_setup(gc, l, px, py, pz);
#pragma unroll
        for(int k = 0; k < 8; ++k)
        {
            float w;
            const uint32_t idx = corner_index(c, k, w);
            float *p = grid_g + 2 * ((size_t)l * T + idx);
            atomicAdd(p, w * g0);
            atomicAdd(p + 1, w * g1);
        }
    }
}

// An optimiser step starts on the device: it counts (and runs) only if its batch has records, so a
// frame whose training paths all escaped leaves the parameters and the moments untouched.
__global__ void k_adam_begin(const uint32_t *__restrict__ d_n, uint32_t *__restrict__ state)
{
    const bool active = d_n == nullptr || *d_n > 0;
    state[1] = active ? 1u : 0u;
    if(active) state[0] += 1u;
}

// Adam (Kingma & Ba 2015) with bias correction 1 - beta^t, t the device step count; gradients are
// consumed (zeroed). Each thread updates one pair of parameters so the FP16 copy (feature pairs) is
// written from values it owns.
__global__ void k_adam(float *__restrict__ p, float *__restrict__ g, float *__restrict__ m, float *__restrict__ v,
                       size_t n, float lr, float b1, float b2, float eps, const uint32_t *__restrict__ state,
                       __half2 *__restrict__ half_copy)
{
    if(state[1] == 0) return;
    const float t = (float)state[0];
    const float c1 = 1.f - powf(b1, t), c2 = 1.f - powf(b2, t);
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for(size_t i2 = (size_t)blockIdx.x * blockDim.x + threadIdx.x; 2 * i2 < n; i2 += stride)
    {
        const float2 gi = reinterpret_cast<const float2 *>(g)[i2];
        float2 mi = reinterpret_cast<const float2 *>(m)[i2], vi = reinterpret_cast<const float2 *>(v)[i2];
        float2 pi = reinterpret_cast<const float2 *>(p)[i2];
        mi.x = b1 * mi.x + (1.f - b1) * gi.x;
        mi.y = b1 * mi.y + (1.f - b1) * gi.y;
        vi.x = b2 * vi.x + (1.f - b2) * gi.x * gi.x;
        vi.y = b2 * vi.y + (1.f - b2) * gi.y * gi.y;
        pi.x = pi.x - lr * (mi.x / c1) / (sqrtf(vi.x / c2) + eps);
        pi.y = pi.y - lr * (mi.y / c1) / (sqrtf(vi.y / c2) + eps);
        reinterpret_cast<float2 *>(m)[i2] = mi;
        reinterpret_cast<float2 *>(v)[i2] = vi;
        reinterpret_cast<float2 *>(p)[i2] = pi;
        reinterpret_cast<float2 *>(g)[i2] = make_float2(0.f, 0.f);
        if(half_copy) half_copy[i2] = __floats2half2_rn(pi.x, pi.y);
    }
}

// FP16 copy of the FP32 master grid
__global__ void k_to_half(const float *__restrict__ p, size_t n, __half2 *__restrict__ half_copy)
{
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for(size_t i2 = (size_t)blockIdx.x * blockDim.x + threadIdx.x; 2 * i2 < n; i2 += stride)
    {
        const float2 v = reinterpret_cast<const float2 *>(p)[i2];
        half_copy[i2] = __floats2half2_rn(v.x, v.y);
    }
}

// pack the FP32 master weights into per-lane B fragments (forward) and transposed fragments (backward)
__global__ void k_pack(const float *__restrict__ W, uint2 *__restrict__ frag, uint2 *__restrict__ fragT)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if(e >= NFRAG) return;
    int l = 0;
    while(l + 1 < NLAYER && e >= frag_off(l + 1)) ++l;
    const int K = layer_in(l), N = layer_out(l), lane = e & 31, g = lane >> 2, tig = lane & 3;
    const float *w = W + layer_off(l);
    {
        const int idx = (e - frag_off(l)) >> 5;
        const int kt = idx / (N / 8), j = idx % (N / 8);
        const int n = 8 * j + g, k = 16 * kt + 2 * tig;
        frag[e] = make_uint2(pack_bf16(w[k * N + n], w[(k + 1) * N + n]), pack_bf16(w[(k + 8) * N + n], w[(k + 9) * N + n]));
    }
    {
        // transposed: B' = W^T (K' = N, N' = K)
        const int idx = (e - fragT_off(l)) >> 5;
        const int kt = idx / (K / 8), j = idx % (K / 8);
        const int n = 8 * j + g, k = 16 * kt + 2 * tig; // n indexes W rows (inputs), k W columns (outputs)
        fragT[e] = make_uint2(pack_bf16(w[n * N + k], w[n * N + k + 1]), pack_bf16(w[n * N + k + 8], w[n * N + k + 9]));
    }
}

__global__ void k_init(float *__restrict__ grid, __half2 *__restrict__ grid_h, size_t ngrid, float *__restrict__ W,
                       uint64_t seed)
{
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for(size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < ngrid / 2; i += stride)
    {
        pcg32 r = pcg32_seed(seed, i);
        const float a = (u01(pcg32_next(r)) * 2.f - 1.f) * 1e-4f, b = (u01(pcg32_next(r)) * 2.f - 1.f) * 1e-4f;
        grid[2 * i] = a;
        grid[2 * i + 1] = b;
        grid_h[i] = __floats2half2_rn(a, b);
    }
    for(size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < NPARAM; i += stride)
    {
        int l = 0;
        while(l + 1 < NLAYER && (int)i >= layer_off(l + 1)) ++l;
        const int K = layer_in(l), N = layer_out(l);
        const int o = ((int)i - layer_off(l)) % N;
        pcg32 r = pcg32_seed(seed ^ 0x9E3779B97F4A7C15ull, i);
        const float bound = sqrtf(6.f / (float)(K + (l == NLAYER - 1 ? 3 : N)));
        W[i] = (l == NLAYER - 1 && o >= 3) ? 0.f : (u01(pcg32_next(r)) * 2.f - 1.f) * bound;
    }
}

}// namespace

vkg_status nrc_ensure(vkg_nrc *c, uint32_t n)
{
    if(n <= c->cap) return VKG_OK;
    cudaFree(c->X);
    cudaFree(c->H);
    cudaFree(c->G);
    cudaFree(c->Y);
    cudaFree(c->dXg);
    c->X = c->H = c->G = nullptr;
    c->Y = c->dXg = nullptr;
    c->cap = 0;
    cudaError_t e = cudaSuccess;
    auto al = [&](void **p, size_t b) {
        if(e == cudaSuccess) e = cudaMalloc(p, b);
    };
    al((void **)&c->X, (size_t)n * 40 * 4);
    al((void **)&c->H, (size_t)n * 160 * 4);
    al((void **)&c->G, (size_t)n * 168 * 4);
    al((void **)&c->Y, (size_t)n * 3 * 4);
    al((void **)&c->dXg, (size_t)n * 32 * 4);
    if(e != cudaSuccess) return cuda_check(c->ctx, e, "nrc buffers");
    c->cap = n;
    return VKG_OK;
}

// n: capacity (host); d_n: optional device-side count (<= n) of the valid records
vkg_status nrc_encode(vkg_nrc *c, const float *feats, uint32_t n, const uint32_t *d_n, uint32_t *X, cudaStream_t st)
{
    if(n == 0) return VKG_OK;
    k_encode<<<(n + 127) / 128, 128, 0, st>>>(feats, n, d_n, c->gc, c->grid_h, X);
    return cuda_check(c->ctx, cudaGetLastError(), "k_encode");
}

vkg_status nrc_forward(vkg_nrc *c, const uint32_t *X, uint32_t n, const uint32_t *d_n, float *Y, cudaStream_t st)
{
    if(n == 0) return VKG_OK;
    const uint32_t tiles = (n + 15) / 16, per_cta = MLP_THREADS / 32;
    const uint32_t grid = std::min<uint32_t>((tiles + per_cta - 1) / per_cta, (uint32_t)c->ctx->num_sms * 8);
    k_forward<false><<<grid, MLP_THREADS, 0, st>>>(X, n, d_n, c->frag, Y, nullptr);
    return cuda_check(c->ctx, cudaGetLastError(), "k_forward");
}

vkg_status nrc_backward(vkg_nrc *c, const float *feats, const float *targets, uint32_t n, const uint32_t *d_n,
                        cudaStream_t st)
{
    if(n == 0) return VKG_OK;
    if(vkg_status s = nrc_ensure(c, n); s != VKG_OK) return s;
    if(vkg_status s = nrc_encode(c, feats, n, d_n, c->X, st); s != VKG_OK) return s;
    const uint32_t tiles = (n + 15) / 16, per_cta = MLP_THREADS / 32;
    const uint32_t grid = std::min<uint32_t>((tiles + per_cta - 1) / per_cta, (uint32_t)c->ctx->num_sms * 8);
    // the training forward and backward: on tcgen05 (train_kernel 3), else the mma.sync twins
    if(c->tc_forward)
    {
        if(vkg_status s = nrc_forward_tc(c->ctx, c->wtc, c->X, n, d_n, c->Y, c->H, c->d_err, st); s != VKG_OK) return s;
    }
    else
        k_forward<true><<<grid, MLP_THREADS, 0, st>>>(c->X, n, d_n, c->frag, c->Y, c->H);
    if(c->tc_forward)
    {
        if(vkg_status s = nrc_backward_tc(c->ctx, c->wtc_t, c->H, c->Y, targets, n, d_n, c->G, c->dXg, c->loss,
                                          c->d_err, st);
           s != VKG_OK)
            return s;
    }
    else
        k_backward<<<grid, MLP_THREADS, 0, st>>>(c->H, c->Y, targets, n, d_n, c->fragT, c->G, c->dXg, c->loss);
    if(c->tc_train)
    {
        if(vkg_status s = nrc_wgrad_tc(c->ctx, c->X, c->H, c->G, n, d_n, c->w_g, c->d_err, st); s != VKG_OK) return s;
    }
    else
    {
        const uint32_t wg = std::min<uint32_t>((n + WG_CHUNK - 1) / WG_CHUNK, (uint32_t)c->ctx->num_sms * 2);
        k_wgrad<<<wg, WG_THREADS, 0, st>>>(c->X, c->H, c->G, n, d_n, c->w_g);
    }
    k_grid_backward<<<(n + 127) / 128, 128, 0, st>>>(feats, n, d_n, c->gc, c->dXg, c->grid_g);
    return cuda_check(c->ctx, cudaGetLastError(), "nrc backward");
}

// d_n: optional device-side record count of the batch; an empty batch takes no step
vkg_status nrc_adam(vkg_nrc *c, const uint32_t *d_n, cudaStream_t st)
{
    const uint32_t blocks = (uint32_t)c->ctx->num_sms * 8;
    k_adam_begin<<<1, 1, 0, st>>>(d_n, c->d_state);
    k_adam<<<blocks, 256, 0, st>>>(c->grid, c->grid_g, c->grid_m, c->grid_v, c->ngrid, c->lr, c->b1, c->b2, c->eps,
                                   c->d_state, c->grid_h);
    k_adam<<<64, 256, 0, st>>>(c->w, c->w_g, c->w_m, c->w_v, NPARAM, c->lr, c->b1, c->b2, c->eps, c->d_state, nullptr);
    k_pack<<<(NFRAG + 255) / 256, 256, 0, st>>>(c->w, c->frag, c->fragT);
    if(vkg_status s = nrc_pack_tc(c->ctx, c->w, c->wtc, st, c->wtc_t); s != VKG_OK) return s;
    return cuda_check(c->ctx, cudaGetLastError(), "nrc adam");
}

const vkg_nrc_config &nrc_config(const vkg_nrc *c) { return c->cfg; }

vkg_status nrc_predict(vkg_nrc *c, const float *feats, uint32_t n, const uint32_t *d_n, uint32_t *X, float *Y,
                       cudaStream_t st)
{
    if(c->tc_infer == 3) return nrc_infer_tc(c->ctx, c->gc, c->grid_h, c->wtc, feats, nullptr, n, d_n, Y, c->d_err, st);
    if(c->tc_infer == 2)
    {
        if(vkg_status s = nrc_encode(c, feats, n, d_n, X, st); s != VKG_OK) return s;
        return nrc_infer_tc(c->ctx, c->gc, c->grid_h, c->wtc, feats, X, n, d_n, Y, c->d_err, st);
    }
    if(vkg_status s = nrc_encode(c, feats, n, d_n, X, st); s != VKG_OK) return s;
    return nrc_forward(c, X, n, d_n, Y, st);
}

vkg_status nrc_train(vkg_nrc *c, const float *feats, const float *targets, uint32_t n, const uint32_t *d_n,
                     cudaStream_t st)
{
    if(vkg_status s = nrc_backward(c, feats, targets, n, d_n, st); s != VKG_OK) return s;
    return nrc_adam(c, d_n, st);
}

}// namespace nrc
}// namespace vkg

using namespace vkg;
using namespace vkg::nrc;

extern "C" {

vkg_status vkg_nrc_config_default(vkg_nrc_config *c)
{
    if(!c) return VKG_ERR_INVALID_ARGUMENT;
    *c = vkg_nrc_config{};
    c->levels = 16;
    c->log2_table_size = 19;
    c->base_resolution = 16;
    c->max_resolution = 2048;
    c->learning_rate = 1e-2f;
    c->beta1 = 0.9f;
    c->beta2 = 0.99f;
    c->epsilon = 1e-15f;
    c->seed = 1337;
    c->scene_min[0] = c->scene_min[1] = c->scene_min[2] = -1.f;
    c->scene_max[0] = c->scene_max[1] = c->scene_max[2] = 1.f;
    c->batch_size = 65536;
    c->train_paths = 65536;
    c->terminate_depth = 2;
    c->train_depth = 4;
    c->train_steps = 0;
    return VKG_OK;
}

vkg_status vkg_nrc_create(vkg_ctx *ctx, const vkg_nrc_config *cfg, vkg_nrc **out)
{
    if(!ctx) return VKG_ERR_INVALID_ARGUMENT;
    if(!cfg || !out) return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_nrc_create: NULL argument");
    *out = nullptr;
    if(cfg->levels == 0 || cfg->levels > 16 || cfg->log2_table_size < 10 || cfg->log2_table_size > 24 ||
       cfg->base_resolution < 2 || cfg->max_resolution < cfg->base_resolution)
        return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_nrc_create: invalid hash-grid configuration");
    if(vkg_status s = bind_device(ctx); s != VKG_OK) return s;
    if(cfg->batch_size == 0 || cfg->batch_size > (1u << 24) || cfg->train_paths > (1u << 24) || cfg->train_depth > 16)
        return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_nrc_create: invalid training configuration");
    if(cfg->infer_kernel > 3)
        return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_nrc_create: infer_kernel must be 0..3");
    if(cfg->train_kernel > 3)
        return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_nrc_create: train_kernel must be 0..3");
    auto *c = new vkg_nrc();
    c->ctx = ctx;
    c->cfg = *cfg;
    // default inference: the pipelined tcgen05 MLP after the shared encoding (2,073,600 queries: 1.152 ms,
    // the mma.sync twin 1.138 ms; the encoding is ~85 % of either)
    c->tc_infer = cfg->infer_kernel ? cfg->infer_kernel : 2u;
    // default: everything on tcgen05 (per 65,536-record step 0.479 ms, against 0.482 ms with the mma.sync
    // forward / backward and 0.574 ms with the FP32 weight gradients)
    c->tc_train = cfg->train_kernel != 1;
    c->tc_forward = cfg->train_kernel == 3 || cfg->train_kernel == 0;
    c->gc.levels = cfg->levels;
    c->gc.log2_t = cfg->log2_table_size;
    c->gc.base_res = cfg->base_resolution;
    c->gc.growth = cfg->levels > 1 ? expf((logf((float)cfg->max_resolution) - logf((float)cfg->base_resolution)) /
                                          (float)(cfg->levels - 1))
                                   : 1.f;
    for(int a = 0; a < 3; ++a)
    {
        c->gc.smin[a] = cfg->scene_min[a];
        const float ext = cfg->scene_max[a] - cfg->scene_min[a];
        c->gc.sinv[a] = ext > 0.f ? 1.f / ext : 0.f;
    }
    c->lr = cfg->learning_rate;
    c->b1 = cfg->beta1;
    c->b2 = cfg->beta2;
    c->eps = cfg->epsilon;
    c->table = 1u << cfg->log2_table_size;
    c->ngrid = (size_t)cfg->levels * c->table * 2;
    cudaError_t e = cudaSuccess;
    auto al = [&](void **p, size_t b) {
        if(e == cudaSuccess) e = cudaMalloc(p, b);
    };
    al((void **)&c->grid, c->ngrid * 4);
    al((void **)&c->grid_g, c->ngrid * 4);
    al((void **)&c->grid_m, c->ngrid * 4);
    al((void **)&c->grid_v, c->ngrid * 4);
    al((void **)&c->grid_h, c->ngrid * 2);
    al((void **)&c->w, NPARAM * 4);
    al((void **)&c->w_g, NPARAM * 4);
    al((void **)&c->w_m, NPARAM * 4);
    al((void **)&c->w_v, NPARAM * 4);
    al((void **)&c->frag, NFRAG * 8);
    al((void **)&c->fragT, NFRAG * 8);
    al((void **)&c->loss, 4 * 4);
    al((void **)&c->d_state, 2 * sizeof(uint32_t));
    al((void **)&c->wtc, NPARAM * 2);
    al((void **)&c->wtc_t, NPARAM * 2);
    al((void **)&c->d_err, sizeof(uint32_t));
    if(e == cudaSuccess)
    {
        for(void *p: {(void *)c->grid_g, (void *)c->grid_m, (void *)c->grid_v})
            if(e == cudaSuccess) e = cudaMemset(p, 0, c->ngrid * 4);
        for(void *p: {(void *)c->w_g, (void *)c->w_m, (void *)c->w_v})
            if(e == cudaSuccess) e = cudaMemset(p, 0, NPARAM * 4);
        if(e == cudaSuccess) e = cudaMemset(c->loss, 0, 16);
        if(e == cudaSuccess) e = cudaMemset(c->d_state, 0, 2 * sizeof(uint32_t));
        if(e == cudaSuccess) e = cudaMemset(c->d_err, 0, sizeof(uint32_t));
    }
    if(e != cudaSuccess)
    {
        vkg_nrc_destroy(c);
        return cuda_check(ctx, e, "vkg_nrc_create");
    }
    k_init<<<ctx->num_sms * 8, 256>>>(c->grid, c->grid_h, c->ngrid, c->w, cfg->seed);
    k_pack<<<(NFRAG + 255) / 256, 256>>>(c->w, c->frag, c->fragT);
    if(vkg_status s = nrc_pack_tc(ctx, c->w, c->wtc, nullptr, c->wtc_t); s != VKG_OK)
    {
        vkg_nrc_destroy(c);
        return s;
    }
    e = cudaDeviceSynchronize();
    if(e != cudaSuccess)
    {
        vkg_nrc_destroy(c);
        return cuda_check(ctx, e, "vkg_nrc_create init");
    }
    *out = c;
    return VKG_OK;
}

vkg_status vkg_nrc_destroy(vkg_nrc *c)
{
    if(!c) return VKG_OK;
    if(c->ctx) bind_device(c->ctx);
    for(void *p: {(void *)c->grid, (void *)c->grid_g, (void *)c->grid_m, (void *)c->grid_v, (void *)c->grid_h,
                  (void *)c->w, (void *)c->w_g, (void *)c->w_m, (void *)c->w_v, (void *)c->frag, (void *)c->fragT,
                  (void *)c->loss, (void *)c->d_state, (void *)c->wtc, (void *)c->wtc_t, (void *)c->d_err, (void *)c->X, (void *)c->H, (void *)c->G, (void *)c->Y,
                  (void *)c->dXg})
        cudaFree(p);
    delete c;
    return VKG_OK;
}

vkg_status vkg_nrc_info(const vkg_nrc *c, vkg_nrc_info_t *out)
{
    if(!c || !out) return VKG_ERR_INVALID_ARGUMENT;
    *out = vkg_nrc_info_t{};
    out->levels = c->gc.levels;
    out->table_size = c->table;
    out->growth = c->gc.growth;
    for(uint32_t l = 0; l < c->gc.levels && l < 16; ++l) out->level_resolution[l] = level_res(c->gc, l);
    out->num_mlp_params = NPARAM;
    out->num_grid_params = (uint64_t)c->ngrid;
    out->d_mlp_params = c->w;
    out->d_grid_params = c->grid;
    out->d_mlp_grads = c->w_g;
    out->d_grid_grads = c->grid_g;
    if(vkg_status s = bind_device(c->ctx); s != VKG_OK) return s;
    VKG_TRY_CUDA(c->ctx, cudaMemcpy(&out->step, c->d_state, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    VKG_TRY_CUDA(c->ctx, cudaMemcpy(&out->kernel_error, c->d_err, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    out->infer_kernel = c->tc_infer;
    out->train_kernel = c->tc_forward ? 3u : (c->tc_train ? 2u : 1u);
    return VKG_OK;
}

vkg_status vkg_nrc_infer(vkg_nrc *c, const float *d_feats, uint32_t n, float *d_rgb, void *stream)
{
    if(!c) return VKG_ERR_INVALID_ARGUMENT;
    if(n == 0) return VKG_OK;
    if(!d_feats || !d_rgb) return set_error(c->ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_nrc_infer: NULL buffer");
    if(vkg_status s = bind_device(c->ctx); s != VKG_OK) return s;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if(c->tc_infer == 3)
        return nrc_infer_tc(c->ctx, c->gc, c->grid_h, c->wtc, d_feats, nullptr, n, nullptr, d_rgb, c->d_err, st);
    if(vkg_status s = nrc_ensure(c, n); s != VKG_OK) return s;
    if(vkg_status s = nrc_encode(c, d_feats, n, nullptr, c->X, st); s != VKG_OK) return s;
    if(c->tc_infer == 2) return nrc_infer_tc(c->ctx, c->gc, c->grid_h, c->wtc, d_feats, c->X, n, nullptr, d_rgb, c->d_err, st);
    return nrc_forward(c, c->X, n, nullptr, d_rgb, st);
}

vkg_status vkg_nrc_backward(vkg_nrc *c, const float *d_feats, const float *d_targets, uint32_t n, void *stream)
{
    if(!c) return VKG_ERR_INVALID_ARGUMENT;
    if(!d_feats || !d_targets) return set_error(c->ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_nrc_backward: NULL buffer");
    if(vkg_status s = bind_device(c->ctx); s != VKG_OK) return s;
    return nrc_backward(c, d_feats, d_targets, n, nullptr, static_cast<cudaStream_t>(stream));
}

vkg_status vkg_nrc_adam_step(vkg_nrc *c, void *stream)
{
    if(!c) return VKG_ERR_INVALID_ARGUMENT;
    if(vkg_status s = bind_device(c->ctx); s != VKG_OK) return s;
    return nrc_adam(c, nullptr, static_cast<cudaStream_t>(stream));
}

vkg_status vkg_nrc_train_step(vkg_nrc *c, const float *d_feats, const float *d_targets, uint32_t n, float *h_loss,
                              void *stream)
{
    if(!c) return VKG_ERR_INVALID_ARGUMENT;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if(vkg_status s = bind_device(c->ctx); s != VKG_OK) return s;
    if(h_loss) VKG_TRY_CUDA(c->ctx, cudaMemsetAsync(c->loss, 0, 4, st));
    if(vkg_status s = nrc_backward(c, d_feats, d_targets, n, nullptr, st); s != VKG_OK) return s;
    if(vkg_status s = nrc_adam(c, nullptr, st); s != VKG_OK) return s;
    if(h_loss)
    {
        VKG_TRY_CUDA(c->ctx, cudaMemcpyAsync(h_loss, c->loss, 4, cudaMemcpyDeviceToHost, st));
        VKG_TRY_CUDA(c->ctx, cudaStreamSynchronize(st));
    }
    return VKG_OK;
}

vkg_status vkg_nrc_load_params(vkg_nrc *c, const float *d_mlp, const float *d_grid, void *stream)
{
    if(!c) return VKG_ERR_INVALID_ARGUMENT;
    if(vkg_status s = bind_device(c->ctx); s != VKG_OK) return s;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if(d_mlp) VKG_TRY_CUDA(c->ctx, cudaMemcpyAsync(c->w, d_mlp, NPARAM * 4, cudaMemcpyDeviceToDevice, st));
    if(d_grid)
    {
        VKG_TRY_CUDA(c->ctx, cudaMemcpyAsync(c->grid, d_grid, c->ngrid * 4, cudaMemcpyDeviceToDevice, st));
        // refresh the FP16 copy the encoder reads
        k_to_half<<<c->ctx->num_sms * 8, 256, 0, st>>>(c->grid, c->ngrid, c->grid_h);
    }
    k_pack<<<(NFRAG + 255) / 256, 256, 0, st>>>(c->w, c->frag, c->fragT);
    if(vkg_status s = nrc_pack_tc(c->ctx, c->w, c->wtc, st, c->wtc_t); s != VKG_OK) return s;
    return cuda_check(c->ctx, cudaGetLastError(), "vkg_nrc_load_params");
}

}// extern "C"

namespace
{
// checkpoint file header, 128 bytes little-endian
struct nrc_ckpt_header
{
    char magic[8];            // "VKGNRC01"
    uint32_t version;         // 1
    uint32_t header_bytes;    // 128
    uint32_t levels, log2_table_size, base_resolution, max_resolution;
    uint32_t num_mlp_params, step;
    uint64_t num_grid_params;
    float learning_rate, beta1, beta2, epsilon;
    float scene_min[3], scene_max[3];
    uint64_t payload_bytes;
    uint64_t checksum;        // FNV-1a 64 of the payload
    uint8_t reserved[24];
};
static_assert(sizeof(nrc_ckpt_header) == 128, "checkpoint header layout");

uint64_t fnv1a64(const void *data, size_t n, uint64_t h = 1469598103934665603ull)
{
    const auto *p = static_cast<const uint8_t *>(data);
    for(size_t i = 0; i < n; ++i)
    {
        h ^= p[i];
        h *= 1099511628211ull;
    }
    return h;
}

nrc_ckpt_header ckpt_header(const vkg_nrc *c, uint32_t step)
{
    nrc_ckpt_header h{};
    std::memcpy(h.magic, "VKGNRC01", 8);
    h.version = 1;
    h.header_bytes = sizeof(nrc_ckpt_header);
    h.levels = c->cfg.levels;
    h.log2_table_size = c->cfg.log2_table_size;
    h.base_resolution = c->cfg.base_resolution;
    h.max_resolution = c->cfg.max_resolution;
    h.num_mlp_params = NPARAM;
    h.step = step;
    h.num_grid_params = c->ngrid;
    h.learning_rate = c->lr;
    h.beta1 = c->b1;
    h.beta2 = c->b2;
    h.epsilon = c->eps;
    for(int a = 0; a < 3; ++a)
    {
        h.scene_min[a] = c->cfg.scene_min[a];
        h.scene_max[a] = c->cfg.scene_max[a];
    }
    h.payload_bytes = (3ull * NPARAM + 3ull * c->ngrid) * sizeof(float);
    return h;
}
}// namespace

extern "C" {

vkg_status vkg_nrc_save(vkg_nrc *c, const char *path, void *stream)
{
    if(!c) return VKG_ERR_INVALID_ARGUMENT;
    if(!path) return set_error(c->ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_nrc_save: NULL path");
    if(vkg_status s = bind_device(c->ctx); s != VKG_OK) return s;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    uint32_t step = 0;
    std::vector<float> buf(3ull * NPARAM + 3ull * c->ngrid);
    float *dst = buf.data();
    for(const float *src: {c->w, c->w_m, c->w_v})
    {
        VKG_TRY_CUDA(c->ctx, cudaMemcpyAsync(dst, src, NPARAM * sizeof(float), cudaMemcpyDeviceToHost, st));
        dst += NPARAM;
    }
    for(const float *src: {c->grid, c->grid_m, c->grid_v})
    {
        VKG_TRY_CUDA(c->ctx, cudaMemcpyAsync(dst, src, c->ngrid * sizeof(float), cudaMemcpyDeviceToHost, st));
        dst += c->ngrid;
    }
    VKG_TRY_CUDA(c->ctx, cudaMemcpyAsync(&step, c->d_state, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    VKG_TRY_CUDA(c->ctx, cudaStreamSynchronize(st));
    nrc_ckpt_header h = ckpt_header(c, step);
    h.checksum = fnv1a64(buf.data(), buf.size() * sizeof(float));
    std::FILE *f = std::fopen(path, "wb");
    if(!f) return set_error(c->ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_nrc_save: cannot open %s", path);
    const bool ok = std::fwrite(&h, sizeof(h), 1, f) == 1 &&
                    std::fwrite(buf.data(), sizeof(float), buf.size(), f) == buf.size();
    const bool closed = std::fclose(f) == 0;
    if(!ok || !closed) return set_error(c->ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_nrc_save: write to %s failed", path);
    return VKG_OK;
}

vkg_status vkg_nrc_load(vkg_nrc *c, const char *path, void *stream)
{
    if(!c) return VKG_ERR_INVALID_ARGUMENT;
    if(!path) return set_error(c->ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_nrc_load: NULL path");
    if(vkg_status s = bind_device(c->ctx); s != VKG_OK) return s;
    std::FILE *f = std::fopen(path, "rb");
    if(!f) return set_error(c->ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_nrc_load: cannot open %s", path);
    nrc_ckpt_header h{};
    std::vector<float> buf;
    const char *why = nullptr;
    if(std::fread(&h, sizeof(h), 1, f) != 1) why = "short header";
    else if(std::memcmp(h.magic, "VKGNRC01", 8) != 0 || h.version != 1 || h.header_bytes != sizeof(h))
        why = "not a version-1 cache checkpoint";
    else
    {
        const nrc_ckpt_header want = ckpt_header(c, 0);
        bool same = h.levels == want.levels && h.log2_table_size == want.log2_table_size &&
                    h.base_resolution == want.base_resolution && h.max_resolution == want.max_resolution &&
                    h.num_mlp_params == want.num_mlp_params && h.num_grid_params == want.num_grid_params &&
                    h.payload_bytes == want.payload_bytes;
        for(int a = 0; a < 3; ++a)
            same = same && h.scene_min[a] == want.scene_min[a] && h.scene_max[a] == want.scene_max[a];
        if(!same) why = "grid layout or scene box differs from this cache's configuration";
        else
        {
            buf.resize(h.payload_bytes / sizeof(float));
            if(std::fread(buf.data(), sizeof(float), buf.size(), f) != buf.size()) why = "short payload";
            else if(std::fgetc(f) != EOF) why = "trailing bytes after the payload";
            else if(fnv1a64(buf.data(), buf.size() * sizeof(float)) != h.checksum) why = "checksum mismatch";
        }
    }
    std::fclose(f);
    if(why) return set_error(c->ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_nrc_load: %s: %s", path, why);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const float *src = buf.data();
    for(float *dst: {c->w, c->w_m, c->w_v})
    {
        VKG_TRY_CUDA(c->ctx, cudaMemcpyAsync(dst, src, NPARAM * sizeof(float), cudaMemcpyHostToDevice, st));
        src += NPARAM;
    }
    for(float *dst: {c->grid, c->grid_m, c->grid_v})
    {
        VKG_TRY_CUDA(c->ctx, cudaMemcpyAsync(dst, src, c->ngrid * sizeof(float), cudaMemcpyHostToDevice, st));
        src += c->ngrid;
    }
    VKG_TRY_CUDA(c->ctx, cudaMemcpyAsync(c->d_state, &h.step, sizeof(uint32_t), cudaMemcpyHostToDevice, st));
    // the operand copies the kernels read
    k_to_half<<<c->ctx->num_sms * 8, 256, 0, st>>>(c->grid, c->ngrid, c->grid_h);
    k_pack<<<(NFRAG + 255) / 256, 256, 0, st>>>(c->w, c->frag, c->fragT);
    if(vkg_status s = nrc_pack_tc(c->ctx, c->w, c->wtc, st, c->wtc_t); s != VKG_OK) return s;
    VKG_TRY_CUDA(c->ctx, cudaStreamSynchronize(st));
    return cuda_check(c->ctx, cudaGetLastError(), "vkg_nrc_load");
}

}// extern "C"
