/*
 * CPU restatement of the reference's denoise pass: five edge-avoiding a-trous passes
 * (src/PBRPathTracer.cpp:26, :346-403; shaders/slang/denoise.slang:33-102) and the pixel-record
 * packing it reads (octahedral_map.slang:9-55, color.slang:6-18). TEST INFRASTRUCTURE ONLY
 * (CPU oracle): tests compare the GPU's vkg_denoise and the tracer's pixel records against it.
 * The weights are evaluated literally as the shader writes them: three exponentials per tap, each
 * clamped by min(., 1), the tap colour divided by its own clamped albedo.
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

void orc_oct_encode(const float n[3], float p[2])
{
    float s = 1.f / (fabsf(n[0]) + fabsf(n[1]) + fabsf(n[2]));
    float px = n[0] * s, py = n[1] * s;
    if(n[2] < 0.f)
    {
        float qx = (1.f - fabsf(py)) * (px >= 0.f ? 1.f : -1.f);
        float qy = (1.f - fabsf(px)) * (py >= 0.f ? 1.f : -1.f);
        px = qx;
        py = qy;
    }
    p[0] = px;
    p[1] = py;
}

void orc_oct_decode(const float p[2], float n[3])
{
    float nx = p[0], ny = p[1], nz = 1.f - fabsf(p[0]) - fabsf(p[1]);
    if(nz < 0.f)
    {
        nx = (1.f - fabsf(p[1])) * (p[0] >= 0.f ? 1.f : -1.f);
        ny = (1.f - fabsf(p[0])) * (p[1] >= 0.f ? 1.f : -1.f);
    }
    float inv = 1.f / sqrtf(nx * nx + ny * ny + nz * nz);
    n[0] = nx * inv;
    n[1] = ny * inv;
    n[2] = nz * inv;
}

uint32_t orc_pack_snorm_2x16(float x, float y)
{
    if(x != x || y != y) return 0u;
    x = fminf(fmaxf(x, -1.f), 1.f);
    y = fminf(fmaxf(y, -1.f), 1.f);
    int ix = (int)rintf(x * 32767.f), iy = (int)rintf(y * 32767.f);
    return ((uint32_t)ix & 0xFFFFu) | ((uint32_t)iy << 16);
}

void orc_unpack_snorm_2x16(uint32_t p, float out[2])
{
    int ix = (int)(int16_t)(p & 0xFFFFu), iy = (int)(int16_t)(p >> 16);
    out[0] = fmaxf((float)ix / 32767.f, -1.f);
    out[1] = fmaxf((float)iy / 32767.f, -1.f);
}

static uint32_t q8(float v) { return (uint32_t)(fminf(fmaxf(v, 0.f), 1.f) * 255.f); }

uint32_t orc_pack_rgba8(float r, float g, float b, float a) { return q8(r) | (q8(g) << 8) | (q8(b) << 16) | (q8(a) << 24); }

void orc_unpack_rgb8(uint32_t c, float out[3])
{
    out[0] = (float)(c & 0xFFu) / 255.f;
    out[1] = (float)((c >> 8) & 0xFFu) / 255.f;
    out[2] = (float)((c >> 16) & 0xFFu) / 255.f;
}

static const float KERNEL[25] = {
        1.f / 256.f, 1.f / 64.f, 3.f / 128.f, 1.f / 64.f, 1.f / 256.f, 1.f / 64.f, 1.f / 16.f, 3.f / 32.f, 1.f / 16.f,
        1.f / 64.f,  3.f / 128.f, 3.f / 32.f, 9.f / 64.f, 3.f / 32.f, 3.f / 128.f, 1.f / 64.f, 1.f / 16.f, 3.f / 32.f,
        1.f / 16.f,  1.f / 64.f,  1.f / 256.f, 1.f / 64.f, 3.f / 128.f, 1.f / 64.f, 1.f / 256.f};

static const float LUM[3] = {0.298999994993f, 0.587000012398f, 0.114000000060f};

/* one pass; prev = NULL reads the pixel radiance */
static void pass(const orc_pixel *px, const float *prev, uint32_t w, uint32_t h, int step, float *out)
{
    const float color_phi = 1.f / .9f, normal_phi = 1.f / .3f, position_phi = 1.f;
    for(uint32_t y = 0; y < h; ++y)
        for(uint32_t x = 0; x < w; ++x)
        {
            const uint32_t c = y * w + x;
            float cval[3], nval[3], q[2], alb[3], eff[3], dmc[3];
            for(int k = 0; k < 3; ++k) cval[k] = prev ? prev[4 * (size_t)c + k] : px[c].radiance[k];
            orc_unpack_snorm_2x16(px[c].normal, q);
            orc_oct_decode(q, nval);
            float depth_c = px[c].depth;
            orc_unpack_rgb8(px[c].albedo, alb);
            for(int k = 0; k < 3; ++k)
            {
                eff[k] = fmaxf(alb[k], 0.01f);
                dmc[k] = cval[k] / eff[k];
            }
            float lum_c = dmc[0] * LUM[0] + dmc[1] * LUM[1] + dmc[2] * LUM[2];
            float sum[3] = {0, 0, 0}, cum = 0.f;
            for(int i = 0; i < 25; ++i)
            {
                int ux = (int)x + (i % 5 - 2) * step, uy = (int)y + (i / 5 - 2) * step;
                ux = ux < 0 ? 0 : (ux > (int)w - 1 ? (int)w - 1 : ux);
                uy = uy < 0 ? 0 : (uy > (int)h - 1 ? (int)h - 1 : uy);
                const uint32_t t = (uint32_t)uy * w + (uint32_t)ux;
                float ct[3], at[3], dt[3], nt[3];
                for(int k = 0; k < 3; ++k) ct[k] = prev ? prev[4 * (size_t)t + k] : px[t].radiance[k];
                orc_unpack_rgb8(px[t].albedo, at);
                for(int k = 0; k < 3; ++k) dt[k] = ct[k] / fmaxf(at[k], 0.01f);
                float lum_t = dt[0] * LUM[0] + dt[1] * LUM[1] + dt[2] * LUM[2];
                float ld = lum_c - lum_t;
                float c_w = fminf(expf(-(ld * ld) * color_phi), 1.f);
                orc_unpack_snorm_2x16(px[t].normal, q);
                orc_oct_decode(q, nt);
                float ex = nval[0] - nt[0], ey = nval[1] - nt[1], ez = nval[2] - nt[2];
                float n_w = fminf(expf(-(ex * ex + ey * ey + ez * ez) * normal_phi), 1.f);
                float p_w = expf(-fabsf(depth_c - px[t].depth) * position_phi);
                float wgt = c_w * n_w * p_w * KERNEL[i];
                for(int k = 0; k < 3; ++k) sum[k] += dt[k] * wgt;
                cum += wgt;
            }
            for(int k = 0; k < 3; ++k) out[4 * (size_t)c + k] = sum[k] / cum * eff[k];
            out[4 * (size_t)c + 3] = 0.f;
        }
}

void orc_denoise(const orc_pixel *px, uint32_t w, uint32_t h, float *out_rgba)
{
    static const int steps[5] = {1, 2, 4, 8, 16};
    const size_t n = (size_t)w * h;
    float *a = (float *)malloc(4 * n * sizeof(float)), *b = (float *)malloc(4 * n * sizeof(float));
    const float *prev = NULL;
    for(int p = 0; p < 5; ++p)
    {
        float *dst = p == 4 ? out_rgba : (p % 2 ? b : a);
        pass(px, prev, w, h, steps[p], dst);
        prev = dst;
    }
    free(a);
    free(b);
}
