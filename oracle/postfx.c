/*
 * CPU restatement of the reference's bloom + tonemap composition (src/PBRPathTracer.cpp:405-465,
 * src/Bloom.cpp, src/GaussianBlur.cpp, shaders/slang/fullscreen/bloom_thresh.slang,
 * gaussian_blur.slang, bloom_composition.slang, utils/tonemap.slang:21-24). TEST INFRASTRUCTURE ONLY
 * (CPU oracle): the GPU's vkg_post_fx is compared against it.
 *
 * Texture sampling is bilinear with clamp-to-edge at texel centres; the bloom images are RGBA16F
 * (every threshold / blur result rounded to half precision, _Float16 round-to-nearest-even); the
 * blur is the 9-tap convolution the reference's paired bilinear taps add up to. The 9 weights are
 * crocore::createGaussianKernel_1D<9> with sigma deduced from the size (crocore is an absent
 * submodule; restated as the normalised Gaussian with sigma = 0.3 ((9 - 1) / 2 - 1) + 0.8 = 1.7:
 * that kernel's parity is unpinned).
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>

static float h16(float v) { return (float)(_Float16)v; }

static void sample(const float *img, uint32_t w, uint32_t h, float u, float v, float out[4])
{
    float x = u * (float)w - 0.5f, y = v * (float)h - 0.5f;
    float x0f = floorf(x), y0f = floorf(y);
    float fx = x - x0f, fy = y - y0f;
    int xi = (int)x0f, yi = (int)y0f;
    int x0 = xi < 0 ? 0 : (xi > (int)w - 1 ? (int)w - 1 : xi), x1 = xi + 1 < 0 ? 0 : (xi + 1 > (int)w - 1 ? (int)w - 1 : xi + 1);
    int y0 = yi < 0 ? 0 : (yi > (int)h - 1 ? (int)h - 1 : yi), y1 = yi + 1 < 0 ? 0 : (yi + 1 > (int)h - 1 ? (int)h - 1 : yi + 1);
    for(int c = 0; c < 4; ++c)
    {
        float a = img[4 * ((size_t)y0 * w + x0) + c], b = img[4 * ((size_t)y0 * w + x1) + c];
        float d = img[4 * ((size_t)y1 * w + x0) + c], e = img[4 * ((size_t)y1 * w + x1) + c];
        float top = a + (b - a) * fx, bot = d + (e - d) * fx;
        out[c] = top + (bot - top) * fy;
    }
}

void orc_post_fx(const float *hdr, uint32_t w, uint32_t h, int tonemap, int bloom, float exposure, float gamma,
                 float lo, float hi, uint32_t iterations, float *out)
{
    const size_t n = (size_t)w * h;
    if(!tonemap)
    {
        for(size_t i = 0; i < 4 * n; ++i) out[i] = hdr[i];
        return;
    }
    float wts[9];
    {
        double sigma = 0.3 * ((9 - 1) * 0.5 - 1) + 0.8, sum = 0, k[9];
        for(int i = 0; i < 9; ++i)
        {
            double x = i - 4;
            k[i] = exp(-x * x / (2 * sigma * sigma));
            sum += k[i];
        }
        for(int i = 0; i < 9; ++i) wts[i] = (float)(k[i] / sum);
    }
    uint32_t bw = w / 2 ? w / 2 : 1, bh = h / 2 ? h / 2 : 1;
    float *a = NULL, *b = NULL;
    if(bloom)
    {
        a = (float *)malloc(4 * (size_t)bw * bh * sizeof(float));
        b = (float *)malloc(4 * (size_t)bw * bh * sizeof(float));
        /* threshold (bloom_thresh.slang): max(c, 0), lerp((0,0,0,1), c, smoothstep(lo, hi, luma)) */
        for(uint32_t y = 0; y < bh; ++y)
            for(uint32_t x = 0; x < bw; ++x)
            {
                float c[4];
                sample(hdr, w, h, ((float)x + 0.5f) / (float)bw, ((float)y + 0.5f) / (float)bh, c);
                for(int k = 0; k < 4; ++k) c[k] = fmaxf(c[k], 0.f);
                float br = c[0] * 0.299f + c[1] * 0.587f + c[2] * 0.114f;
                float t = fminf(fmaxf((br - lo) / (hi - lo), 0.f), 1.f);
                float s = t * t * (3.f - 2.f * t);
                float *o = a + 4 * ((size_t)y * bw + x);
                o[0] = h16(c[0] * s);
                o[1] = h16(c[1] * s);
                o[2] = h16(c[2] * s);
                o[3] = h16(1.f + (c[3] - 1.f) * s);
            }
        for(uint32_t it = 0; it < iterations; ++it)
            for(int pass = 0; pass < 2; ++pass)
            {
                const float *src = pass ? b : a;
                float *dst = pass ? a : b;
                for(uint32_t y = 0; y < bh; ++y)
                    for(uint32_t x = 0; x < bw; ++x)
                    {
                        float acc[4] = {0, 0, 0, 0};
                        for(int k = -4; k <= 4; ++k)
                        {
                            int i = (int)x + (pass ? 0 : k), j = (int)y + (pass ? k : 0);
                            i = i < 0 ? 0 : (i > (int)bw - 1 ? (int)bw - 1 : i);
                            j = j < 0 ? 0 : (j > (int)bh - 1 ? (int)bh - 1 : j);
                            for(int c = 0; c < 4; ++c) acc[c] += src[4 * ((size_t)j * bw + i) + c] * wts[k + 4];
                        }
                        for(int c = 0; c < 4; ++c) dst[4 * ((size_t)y * bw + x) + c] = h16(acc[c]);
                    }
            }
    }
    /* composition (bloom_composition.slang, tonemap_exposure) */
    for(uint32_t y = 0; y < h; ++y)
        for(uint32_t x = 0; x < w; ++x)
        {
            const float *c = hdr + 4 * ((size_t)y * w + x);
            float bl[4] = {0, 0, 0, 0};
            if(bloom) sample(a, bw, bh, ((float)x + 0.5f) / (float)w, ((float)y + 0.5f) / (float)h, bl);
            float *o = out + 4 * ((size_t)y * w + x);
            for(int k = 0; k < 3; ++k) o[k] = powf(1.f - expf(-(c[k] + bl[k]) * exposure), 1.f / gamma);
            o[3] = c[3];
        }
    free(a);
    free(b);
}
