// Neural radiance cache: the input encoding shared by the mma.sync and tcgen05 kernels.
#pragma once

#include "nrc.cuh"

namespace vkg
{
namespace nrc
{

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi)
{
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t *>(&v);
}

// ---- encodings ---------------------------------------------------------------------------------
__device__ __forceinline__ void sh4(float x, float y, float z, float *o)
{
    // real spherical harmonics, bands 0..3
    const float xx = x * x, yy = y * y, zz = z * z;
    o[0] = 0.28209479177387814f;
    o[1] = -0.48860251190291987f * y;
    o[2] = 0.48860251190291987f * z;
    o[3] = -0.48860251190291987f * x;
    o[4] = 1.0925484305920792f * x * y;
    o[5] = -1.0925484305920792f * y * z;
    o[6] = 0.31539156525252005f * (3.f * zz - 1.f);
    o[7] = -1.0925484305920792f * x * z;
    o[8] = 0.5462742152960396f * (xx - yy);
    o[9] = -0.5900435899266435f * y * (3.f * xx - yy);
    o[10] = 2.890611442640554f * x * y * z;
    o[11] = -0.4570457994644658f * y * (5.f * zz - 1.f);
    o[12] = 0.3731763325901154f * z * (5.f * zz - 3.f);
    o[13] = -0.4570457994644658f * x * (5.f * zz - 1.f);
    o[14] = 1.445305721320277f * z * (xx - yy);
    o[15] = -0.5900435899266435f * x * (xx - 3.f * yy);
}

struct corner_iter
{
    uint32_t res, table;
    bool dense;
    int cx, cy, cz;
    float fx, fy, fz;
};

__device__ __forceinline__ corner_iter level_setup(const grid_config &gc, uint32_t l, float px, float py, float pz)
{
    corner_iter c;
    c.res = level_res(gc, l);
    c.table = 1u << gc.log2_t;
    const uint64_t r1 = (uint64_t)c.res + 1;
    c.dense = r1 * r1 * r1 <= (uint64_t)c.table;
    const float x = px * (float)c.res, y = py * (float)c.res, z = pz * (float)c.res;
    // the cell is clamped so p = 1 interpolates inside the last cell (every corner stays in range)
    const float top = (float)(c.res - 1);
    const float flx = fminf(floorf(x), top), fly = fminf(floorf(y), top), flz = fminf(floorf(z), top);
    c.cx = (int)flx;
    c.cy = (int)fly;
    c.cz = (int)flz;
    c.fx = x - flx;
    c.fy = y - fly;
    c.fz = z - flz;
    return c;
}

__device__ __forceinline__ uint32_t corner_index(const corner_iter &c, int k, float &w)
{
    const uint32_t x = (uint32_t)(c.cx + (k & 1)), y = (uint32_t)(c.cy + ((k >> 1) & 1)),
                   z = (uint32_t)(c.cz + ((k >> 2) & 1));
    w = ((k & 1) ? c.fx : 1.f - c.fx) * ((k & 2) ? c.fy : 1.f - c.fy) * ((k & 4) ? c.fz : 1.f - c.fz);
    if(c.dense) return x + y * (c.res + 1) + z * (c.res + 1) * (c.res + 1);
    return (x * 1u ^ y * 2654435761u ^ z * 805459861u) & (c.table - 1u);
}

__device__ __forceinline__ void normalised_pos(const grid_config &gc, const float *f, float &px, float &py, float &pz)
{
    px = fminf(fmaxf((f[0] - gc.smin[0]) * gc.sinv[0], 0.f), 1.f);
    py = fminf(fmaxf((f[1] - gc.smin[1]) * gc.sinv[1], 0.f), 1.f);
    pz = fminf(fmaxf((f[2] - gc.smin[2]) * gc.sinv[2], 0.f), 1.f);
}

// hash-grid features of levels [l0, l1) of one record: out[l - l0] = BF16 pair of level l
// (levels at or past gc.levels give zeros)
template<int L0, int L1>
__device__ __forceinline__ void encode_levels(const grid_config &gc, const __half2 *__restrict__ grid, float px,
                                              float py, float pz, uint32_t *out)
{
    const uint32_t T = 1u << gc.log2_t;
#pragma unroll
    for(int l = L0; l < L1; ++l)
    {
        uint32_t word = 0u;
        if((uint32_t)l < gc.levels)
        {
            corner_iter c = level_setup(gc, l, px, py, pz);
            float f0 = 0.f, f1 = 0.f;
#pragma unroll
            for(int k = 0; k < 8; ++k)
            {
                float w;
                const uint32_t idx = corner_index(c, k, w);
                const float2 v = __half22float2(grid[(size_t)l * T + idx]);
                f0 += w * v.x;
                f1 += w * v.y;
            }
            word = pack_bf16(f0, f1);
        }
        out[l - L0] = word;
    }
}

// the non-grid inputs (words 16..39): SH of the direction and of the normal, roughness, albedo, padding
__device__ __forceinline__ void encode_rest(const float *f, uint32_t *out)
{
    float s[16];
    sh4(f[3], f[4], f[5], s);
#pragma unroll
    for(int k = 0; k < 8; ++k) out[k] = pack_bf16(s[2 * k], s[2 * k + 1]);
    sh4(f[6], f[7], f[8], s);
#pragma unroll
    for(int k = 0; k < 8; ++k) out[8 + k] = pack_bf16(s[2 * k], s[2 * k + 1]);
    out[16] = pack_bf16(f[9], f[10]);
    out[17] = pack_bf16(f[11], f[12]);
#pragma unroll
    for(int k = 18; k < 24; ++k) out[k] = 0u;
}

// the 80 BF16 inputs of one feature record as 40 u32 (BF16 pairs): 16 levels x 2 hash-grid features,
// 16 SH coefficients of the direction, 16 of the normal, roughness, albedo, zero padding
__device__ __forceinline__ void encode_record(const grid_config &gc, const __half2 *__restrict__ grid, const float *f,
                                              uint32_t *out)
{
    float px, py, pz;
    normalised_pos(gc, f, px, py, pz);
    encode_levels<0, 16>(gc, grid, px, py, pz, out);
    encode_rest(f, out + 16);
}

}// namespace nrc
}// namespace vkg
