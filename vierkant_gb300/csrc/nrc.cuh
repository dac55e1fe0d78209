// Neural radiance cache: shared definitions (network shape, feature record, encodings).
//
// Not in the reference (vierkant has no learned component). Network: 80 inputs -> 5 hidden layers
// of width 64 (ReLU, no biases) -> RGB, BF16 weights and activations, FP32 accumulation.
// Inputs: position through a multiresolution hash grid (Mueller et al. 2022: 16 levels x 2
// features, 2^19 FP16 entries per level, trilinear), outgoing direction and normal through real
// spherical harmonics of degree 4 (bands 0..3, 16 coefficients each), roughness and albedo;
// 68 values padded to 80. Loss: relative L2 (y - t)^2 / (sg(y)^2 + 0.01). Optimiser: Adam.
#pragma once

#include "internal.hpp"

#include <cuda_bf16.h>
#include <cuda_fp16.h>

namespace vkg
{
namespace nrc
{

constexpr int IN = 80;     // padded input width
constexpr int HID = 64;    // hidden width
constexpr int OUTP = 16;   // padded output width (3 used)
constexpr int NLAYER = 6;  // weight matrices: 80x64, 4 x 64x64, 64x16
constexpr int FEAT = 13;   // feature record: pos3, dir3, normal3, roughness, albedo3
constexpr int GRID_FEATS = 32;

// per-layer input / output widths and offsets into the FP32 master weight array ([in][out] row-major)
__host__ __device__ constexpr int layer_in(int l) { return l == 0 ? IN : HID; }
__host__ __device__ constexpr int layer_out(int l) { return l == NLAYER - 1 ? OUTP : HID; }
__host__ __device__ constexpr int layer_off(int l)
{
    int o = 0;
    for(int i = 0; i < l; ++i) o += layer_in(i) * layer_out(i);
    return o;
}
constexpr int NPARAM = layer_off(NLAYER); // 22,528

// fragment-packed BF16 weights for m16n8k16 B operands: per layer (K/16) x (N/8) x 32 lanes x uint2
__host__ __device__ constexpr int frag_count(int l) { return (layer_in(l) / 16) * (layer_out(l) / 8) * 32; }
__host__ __device__ constexpr int frag_off(int l)
{
    int o = 0;
    for(int i = 0; i < l; ++i) o += frag_count(i);
    return o;
}
constexpr int NFRAG = frag_off(NLAYER); // 5,632 uint2 = 45,056 B
// transposed weights (backward): layer l as (N/16) x (K/8) x 32 lanes -- same total per layer
__host__ __device__ constexpr int fragT_count(int l) { return (layer_out(l) / 16) * (layer_in(l) / 8) * 32; }
__host__ __device__ constexpr int fragT_off(int l)
{
    int o = 0;
    for(int i = 0; i < l; ++i) o += fragT_count(i);
    return o;
}

// activations saved by the training forward: H1..H5 (64 each) per sample, BF16
constexpr int ACT = 5 * HID;
// gradients w.r.t. pre-activations saved by the backward: G5 (16) + G0..G4 (64 each)
constexpr int GRAD = OUTP + 5 * HID;

struct grid_config
{
    uint32_t levels, log2_t, base_res;
    float growth;
    float smin[3], sinv[3]; // position normalisation: p = (x - smin) * sinv
};

__host__ __device__ inline uint32_t level_res(const grid_config &g, uint32_t l)
{
    float r = (float)g.base_res;
    for(uint32_t i = 0; i < l; ++i) r *= g.growth;
    return (uint32_t)r;
}

// entry points for the path tracer. n is the capacity of the arrays; d_n (optional) points to the
// device-side count (<= n) of valid records, so queue lengths never travel to the host.
const vkg_nrc_config &nrc_config(const vkg_nrc *c);
// encoded inputs of n records: n x 40 u32 (80 BF16 values per record)
constexpr size_t ENCODED_BYTES = IN * 2;
// predictions (n x 3 fp32) for n feature records (n x FEAT fp32); X is caller-owned scratch of n x ENCODED_BYTES
vkg_status nrc_predict(vkg_nrc *c, const float *feats, uint32_t n, const uint32_t *d_n, uint32_t *X, float *Y,
                       cudaStream_t st);
// tcgen05 inference (nrc_tc.cu): BF16 B operands of all layers (NPARAM x 2 bytes, canonical K-major)
vkg_status nrc_pack_tc(vkg_ctx *ctx, const float *W, uint16_t *wtc, cudaStream_t st, uint16_t *wtc_t = nullptr);
vkg_status nrc_backward_tc(vkg_ctx *ctx, const uint16_t *wtc_t, const uint32_t *H, const float *Y, const float *T,
                           uint32_t n, const uint32_t *d_n, uint32_t *G, float *dXg, float *loss, uint32_t *err,
                           cudaStream_t st);
// MLP on tcgen05 over the encoded inputs X (n x 40 u32), or, with X == nullptr, encoding + MLP fused;
// err receives 1 if a tensor-core wait ran out
vkg_status nrc_infer_tc(vkg_ctx *ctx, const grid_config &gc, const __half2 *grid, const uint16_t *wtc,
                        const float *feats, const uint32_t *X, uint32_t n, const uint32_t *d_n, float *Y, uint32_t *err,
                        cudaStream_t st);
// weight gradients of n records on tcgen05 (accumulated into dW); err receives 1 if a wait ran out
vkg_status nrc_forward_tc(vkg_ctx *ctx, const uint16_t *wtc, const uint32_t *X, uint32_t n, const uint32_t *d_n,
                          float *Y, uint32_t *H, uint32_t *err, cudaStream_t st);
vkg_status nrc_wgrad_tc(vkg_ctx *ctx, const uint32_t *X, const uint32_t *H, const uint32_t *G, uint32_t n,
                        const uint32_t *d_n, float *dW, uint32_t *err, cudaStream_t st);
// one optimiser step (backward + Adam) on n records; records past *d_n contribute nothing
vkg_status nrc_train(vkg_nrc *c, const float *feats, const float *targets, uint32_t n, const uint32_t *d_n,
                     cudaStream_t st);

}// namespace nrc
}// namespace vkg
