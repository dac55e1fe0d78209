// DCT JPEG decoder with Huffman coding (ITU-T T.81): sequential (Annex F) and progressive (Annex G:
// spectral selection and successive approximation, end-of-band runs) frames. Marker segments,
// canonical Huffman tables (F.2.2.3's code-length decoding), DC prediction per component, run-length
// AC coefficients in zig-zag order collected per block over all scans, then dequantisation, a
// separable floating-point inverse DCT, level shift, chroma replication and the JFIF YCbCr -> RGB
// conversion.
#include "jpeg.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace vkg
{
namespace
{

// natural (row-major) index of the k-th coefficient in zig-zag order
constexpr uint8_t ZIGZAG[64] = {0,  1,  8,  16, 9,  2,  3,  10, 17, 24, 32, 25, 18, 11, 4,  5,
                                12, 19, 26, 33, 40, 48, 41, 34, 27, 20, 13, 6,  7,  14, 21, 28,
                                35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23, 30, 37, 44, 51,
                                58, 59, 52, 45, 38, 31, 39, 46, 53, 60, 61, 54, 47, 55, 62, 63};

struct huffman
{
    bool defined = false;
    int32_t mincode[17], maxcode[18], valptr[17];
    uint8_t vals[256];
    uint32_t nvals = 0;
};

struct component
{
    uint32_t id, h, v, tq;
    uint32_t td = 0, ta = 0;
    uint32_t bw = 0, bh = 0; // blocks per row / column in the plane (whole MCUs)
    std::vector<int16_t> coef; // per block 64 coefficients in zig-zag order, over all scans
    std::vector<uint8_t> plane;
    int32_t pred = 0;
};

struct decoder
{
    const uint8_t *p, *end;
    std::string &err;
    uint16_t q[4][64];
    bool q_defined[4] = {false, false, false, false};
    huffman dc[4], ac[4];
    std::vector<component> comps;
    uint32_t width = 0, height = 0, hmax = 1, vmax = 1, mcux = 0, mcuy = 0, restart = 0;
    bool frame = false, adobe = false, progressive = false;
    uint32_t ss = 0, se = 63, ah = 0, al = 0; // the current scan's band and successive approximation
    uint32_t eobrun = 0;                     // blocks left in the current end-of-band run
    uint8_t adobe_transform = 1;
    // entropy-coded bit reader
    const uint8_t *s = nullptr;
    uint32_t acc = 0;
    int nbits = 0;
    bool hit_marker = false;

    bool fail(const char *m)
    {
        err = m;
        return false;
    }

    uint32_t u16(const uint8_t *x) { return (uint32_t)x[0] << 8 | x[1]; }

    bool build_huffman(huffman &t, const uint8_t *counts, const uint8_t *vals, uint32_t nvals)
    {
        // canonical codes (Annex C): lengths in order, codes consecutive within a length
        t.nvals = nvals;
        std::memcpy(t.vals, vals, nvals);
        int32_t code = 0;
        uint32_t k = 0;
        for(int l = 1; l <= 16; ++l)
        {
            const uint32_t n = counts[l - 1];
            t.valptr[l] = (int32_t)k;
            t.mincode[l] = code;
            code += (int32_t)n;
            k += n;
            t.maxcode[l] = n ? code - 1 : -1;
            if(code > (1 << l)) return fail("JPEG: over-subscribed Huffman table");
            code <<= 1;
        }
        t.maxcode[17] = 0x7FFFFFFF;
        t.defined = true;
        return true;
    }

    // ---- bit reader over the entropy-coded segment (0xFF 0x00 is a data byte 0xFF; any other
    // marker ends the data: zeros are fed after it)
    void fill()
    {
        while(nbits <= 24)
        {
            uint32_t b = 0;
            if(!hit_marker && s < end)
            {
                b = *s;
                if(b == 0xFF)
                {
                    const uint32_t n = s + 1 < end ? s[1] : 0xD9u;
                    if(n == 0x00) s += 2;
                    else
                    {
                        hit_marker = true;
                        b = 0;
                    }
                }
                else
                    ++s;
            }
            acc |= b << (24 - nbits);
            nbits += 8;
        }
    }
    uint32_t bits(int n)
    {
        if(n == 0) return 0;
        fill();
        const uint32_t r = acc >> (32 - n);
        acc <<= n;
        nbits -= n;
        return r;
    }
    int decode(const huffman &t, bool &ok)
    {
        fill();
        int32_t code = 0;
        for(int l = 1; l <= 16; ++l)
        {
            code = (code << 1) | (int32_t)(acc >> 31);
            acc <<= 1;
            --nbits;
            if(code <= t.maxcode[l] && t.maxcode[l] >= 0)
            {
                const int32_t j = t.valptr[l] + code - t.mincode[l];
                if(j < 0 || (uint32_t)j >= t.nvals) break;
                return t.vals[j];
            }
        }
        ok = false;
        return 0;
    }
    static int32_t extend(uint32_t v, int t) { return t && v < (1u << (t - 1)) ? (int32_t)v - (1 << t) + 1 : (int32_t)v; }

    // ---- one block of a scan into the component's coefficients at block (bx, by)
    bool block(component &c, uint32_t bx, uint32_t by)
    {
        int16_t *z = c.coef.data() + ((size_t)by * c.bw + bx) * 64;
        bool ok = true;
        if(ss == 0)
        {
            // DC: the whole coefficient (sequential), its high bits (first scan) or one more bit
            if(ah == 0)
            {
                if(!dc[c.td].defined) return fail("JPEG: scan uses an undefined Huffman table");
                const int t = decode(dc[c.td], ok);
                if(!ok || t > 11) return fail("JPEG: bad DC code");
                c.pred += extend(bits(t), t);
                z[0] = (int16_t)(c.pred * (1 << al));
            }
            else if(bits(1))
                z[0] = (int16_t)(z[0] | (1 << al));
            if(!progressive) return ac_first(c, z, 1);
            return true;
        }
        return ah == 0 ? ac_first(c, z, ss) : ac_refine(c, z);
    }

    // AC coefficients k0..se of a sequential block or a progressive first scan (values << al); an
    // end-of-band symbol ends this block and, in progressive scans, starts a run over the next ones
    bool ac_first(component &c, int16_t *z, uint32_t k0)
    {
        if(eobrun > 0)
        {
            --eobrun;
            return true;
        }
        const huffman &ha = ac[c.ta];
        if(!ha.defined) return fail("JPEG: scan uses an undefined Huffman table");
        bool ok = true;
        for(uint32_t k = k0; k <= se;)
        {
            const int rs = decode(ha, ok);
            if(!ok) return fail("JPEG: bad AC code");
            const int r = rs >> 4, sz = rs & 15;
            if(sz == 0)
            {
                if(r == 15)
                {
                    k += 16;
                    continue;
                }
                if(progressive) eobrun = (1u << r) - 1u + (r ? bits(r) : 0u);
                break;
            }
            k += (uint32_t)r;
            if(k > se) return fail("JPEG: AC run past the band");
            z[k] = (int16_t)(extend(bits(sz), sz) * (1 << al));
            ++k;
        }
        return true;
    }

    // the refinement bit of an already non-zero coefficient
    void refine(int16_t &v)
    {
        if(bits(1) && (v & (1 << al)) == 0) v = (int16_t)(v + (v >= 0 ? (1 << al) : -(1 << al)));
    }

    // a progressive AC refinement scan (G.1.2.3): newly non-zero coefficients (+-1 << al) placed after
    // r zero-history coefficients, a correction bit for every non-zero one passed on the way, and for
    // every non-zero coefficient after the end of band
    bool ac_refine(component &c, int16_t *z)
    {
        const huffman &ha = ac[c.ta];
        if(!ha.defined) return fail("JPEG: scan uses an undefined Huffman table");
        bool ok = true;
        uint32_t k = ss;
        if(eobrun == 0)
        {
            for(; k <= se; ++k)
            {
                const int rs = decode(ha, ok);
                if(!ok) return fail("JPEG: bad AC code");
                int r = rs >> 4;
                const int sz = rs & 15;
                int v = 0;
                if(sz)
                {
                    if(sz != 1) return fail("JPEG: bad refinement code");
                    v = bits(1) ? (1 << al) : -(1 << al);
                }
                else if(r != 15)
                {
                    eobrun = (1u << r) + (r ? bits(r) : 0u);
                    break;
                }
                while(k <= se)
                {
                    int16_t &w = z[k];
                    if(w != 0)
                        refine(w);
                    else if(--r < 0)
                        break;
                    ++k;
                }
                if(v)
                {
                    if(k > se) return fail("JPEG: refinement past the band");
                    z[k] = (int16_t)v;
                }
            }
        }
        if(eobrun > 0)
        {
            for(; k <= se; ++k)
                if(z[k] != 0) refine(z[k]);
            --eobrun;
        }
        return true;
    }

    // dequantise every block and transform it into the component's plane
    void reconstruct()
    {
        for(component &c: comps)
        {
            const uint16_t *qt = q[c.tq];
            for(uint32_t by = 0; by < c.bh; ++by)
                for(uint32_t bx = 0; bx < c.bw; ++bx)
                {
                    const int16_t *z = c.coef.data() + ((size_t)by * c.bw + bx) * 64;
                    float F[64];
                    for(int k = 0; k < 64; ++k) F[ZIGZAG[k]] = (float)z[k] * (float)qt[k];
                    idct(F, c.plane.data() + (size_t)by * 8 * c.bw * 8 + (size_t)bx * 8, c.bw * 8);
                }
        }
    }

    // f(x, y) = 1/4 sum_u sum_v C(u) C(v) F(v, u) cos((2x + 1) u pi / 16) cos((2y + 1) v pi / 16),
    // C(0) = 1 / sqrt 2, else 1; then + 128, rounded and clamped to [0, 255]
    static void idct(const float *F, uint8_t *out, size_t stride)
    {
        static float T[8][8]; // T[x][u] = C(u) / 2 cos((2x + 1) u pi / 16)
        static bool init = false;
        if(!init)
        {
            for(int x = 0; x < 8; ++x)
                for(int u = 0; u < 8; ++u)
                    T[x][u] = (float)((u == 0 ? std::sqrt(0.5) : 1.0) * 0.5 *
                                      std::cos((2 * x + 1) * u * 3.14159265358979323846 / 16.0));
            init = true;
        }
        float tmp[64];
        for(int v = 0; v < 8; ++v) // rows of coefficients -> rows of x
            for(int x = 0; x < 8; ++x)
            {
                float acc = 0.f;
                for(int u = 0; u < 8; ++u) acc += T[x][u] * F[v * 8 + u];
                tmp[v * 8 + x] = acc;
            }
        for(int y = 0; y < 8; ++y)
            for(int x = 0; x < 8; ++x)
            {
                float acc = 0.f;
                for(int v = 0; v < 8; ++v) acc += T[y][v] * tmp[v * 8 + x];
                const float val = std::floor(acc + 128.5f);
                out[(size_t)y * stride + x] = (uint8_t)std::min(255.f, std::max(0.f, val));
            }
    }

    // the restart marker after each interval: re-align, expect RSTn, reset the predictions
    bool restart_marker()
    {
        acc = 0;
        nbits = 0;
        if(!(s + 1 < end && s[0] == 0xFF && s[1] >= 0xD0 && s[1] <= 0xD7)) return fail("JPEG: missing restart marker");
        s += 2;
        hit_marker = false;
        for(component &c: comps) c.pred = 0;
        eobrun = 0;
        return true;
    }

    bool scan(const uint8_t *seg, uint32_t len)
    {
        if(!frame) return fail("JPEG: scan before the frame header");
        const uint32_t ns = seg[0];
        if(ns < 1 || ns > 4 || len < 4 + 2 * ns) return fail("JPEG: bad scan header");
        std::vector<component *> sc;
        for(uint32_t i = 0; i < ns; ++i)
        {
            const uint32_t id = seg[1 + 2 * i], t = seg[2 + 2 * i];
            component *c = nullptr;
            for(component &k: comps)
                if(k.id == id) c = &k;
            if(!c || (t >> 4) > 3 || (t & 15) > 3) return fail("JPEG: scan names an unknown component or table");
            c->td = t >> 4;
            c->ta = t & 15;
            sc.push_back(c);
        }
        const uint8_t *tail = seg + 1 + 2 * ns;
        ss = tail[0];
        se = tail[1];
        ah = tail[2] >> 4;
        al = tail[2] & 15;
        if(!progressive && (ss != 0 || se != 63 || tail[2] != 0)) return fail("JPEG: bad sequential scan");
        // progressive: a DC band alone, AC bands of one component; each refinement adds one bit
        if(progressive && (se > 63 || ss > se || (ss == 0 && se != 0) || (ss > 0 && ns != 1) || al > 13 ||
                           (ah != 0 && ah != al + 1)))
            return fail("JPEG: bad progressive scan");
        for(component *c: sc)
            if(!q_defined[c->tq]) return fail("JPEG: undefined quantisation table");
        for(component &c: comps) c.pred = 0;
        eobrun = 0;
        s = seg + len;
        acc = 0;
        nbits = 0;
        hit_marker = false;
        uint32_t done = 0;
        if(ns == 1)
        {
            // one component, its blocks in raster order over the component's own extent
            component &c = *sc[0];
            const uint32_t cw = (width * c.h + hmax - 1) / hmax, ch = (height * c.v + vmax - 1) / vmax;
            const uint32_t nbx = (cw + 7) / 8, nby = (ch + 7) / 8;
            for(uint32_t by = 0; by < nby; ++by)
                for(uint32_t bx = 0; bx < nbx; ++bx)
                {
                    if(restart && done && done % restart == 0 && !restart_marker()) return false;
                    if(!block(c, bx, by)) return false;
                    ++done;
                }
        }
        else
        {
            for(uint32_t my = 0; my < mcuy; ++my)
                for(uint32_t mx = 0; mx < mcux; ++mx)
                {
                    if(restart && done && done % restart == 0 && !restart_marker()) return false;
                    for(component *c: sc)
                        for(uint32_t v = 0; v < c->v; ++v)
                            for(uint32_t h = 0; h < c->h; ++h)
                                if(!block(*c, mx * c->h + h, my * c->v + v)) return false;
                    ++done;
                }
        }
        // continue after the entropy-coded data: at the next marker that is not a restart marker
        const uint8_t *m = s;
        while(m + 1 < end && !(m[0] == 0xFF && m[1] != 0x00 && !(m[1] >= 0xD0 && m[1] <= 0xD7))) ++m;
        p = m;
        return true;
    }

    bool run(std::vector<uint8_t> &rgba, uint32_t &w_out, uint32_t &h_out)
    {
        if(end - p < 4 || p[0] != 0xFF || p[1] != 0xD8) return fail("JPEG: no SOI marker");
        p += 2;
        bool scanned = false;
        while(true)
        {
            while(p < end && *p != 0xFF) ++p; // tolerate fill bytes before a marker
            while(p < end && *p == 0xFF) ++p;
            if(p >= end) break;
            const uint8_t mk = *p++;
            if(mk == 0xD9) break; // EOI
            if(mk == 0x01 || (mk >= 0xD0 && mk <= 0xD7)) continue;
            if(end - p < 2) return fail("JPEG: truncated segment");
            const uint32_t len = u16(p);
            if(len < 2 || (size_t)(end - p) < len) return fail("JPEG: truncated segment");
            const uint8_t *seg = p + 2;
            const uint32_t n = len - 2;
            p += len;
            if(mk == 0xC0 || mk == 0xC1 || mk == 0xC2)
            {
                progressive = mk == 0xC2;
                if(frame) return fail("JPEG: second frame header");
                if(n < 6 || seg[0] != 8) return fail("JPEG: only 8-bit samples are supported");
                height = u16(seg + 1);
                width = u16(seg + 3);
                const uint32_t nf = seg[5];
                if(width == 0 || height == 0 || width > 16384 || height > 16384) return fail("JPEG: bad image size");
                if((nf != 1 && nf != 3) || n < 6 + 3 * nf) return fail("JPEG: only grey or three-component images");
                for(uint32_t i = 0; i < nf; ++i)
                {
                    component c;
                    c.id = seg[6 + 3 * i];
                    c.h = seg[7 + 3 * i] >> 4;
                    c.v = seg[7 + 3 * i] & 15;
                    c.tq = seg[8 + 3 * i];
                    if(c.h < 1 || c.h > 4 || c.v < 1 || c.v > 4 || c.tq > 3) return fail("JPEG: bad component");
                    hmax = std::max(hmax, c.h);
                    vmax = std::max(vmax, c.v);
                    comps.push_back(c);
                }
                if(nf == 1) comps[0].h = comps[0].v = hmax = vmax = 1; // a lone component is not subsampled
                mcux = (width + 8 * hmax - 1) / (8 * hmax);
                mcuy = (height + 8 * vmax - 1) / (8 * vmax);
                for(component &c: comps)
                {
                    c.bw = mcux * c.h;
                    c.bh = mcuy * c.v;
                    c.coef.assign((size_t)c.bw * c.bh * 64, 0);
                    c.plane.assign((size_t)c.bw * 8 * c.bh * 8, 0);
                }
                frame = true;
            }
            else if(mk == 0xC3 || (mk >= 0xC5 && mk <= 0xCF && mk != 0xC8 && mk != 0xCC))
                return fail("JPEG: lossless, hierarchical or arithmetic-coded images are not supported");
            else if(mk == 0xDB)
            {
                for(uint32_t k = 0; k < n;)
                {
                    const uint32_t pq = seg[k] >> 4, tq = seg[k] & 15;
                    if(tq > 3 || pq > 1 || k + 1 + 64 * (pq + 1) > n) return fail("JPEG: bad quantisation table");
                    for(int i = 0; i < 64; ++i)
                        q[tq][i] = pq ? (uint16_t)u16(seg + k + 1 + 2 * i) : seg[k + 1 + i];
                    q_defined[tq] = true;
                    k += 1 + 64 * (pq + 1);
                }
            }
            else if(mk == 0xC4)
            {
                for(uint32_t k = 0; k < n;)
                {
                    if(k + 17 > n) return fail("JPEG: bad Huffman table");
                    const uint32_t tc = seg[k] >> 4, th = seg[k] & 15;
                    uint32_t total = 0;
                    for(int i = 0; i < 16; ++i) total += seg[k + 1 + i];
                    if(tc > 1 || th > 3 || total > 256 || k + 17 + total > n) return fail("JPEG: bad Huffman table");
                    if(!build_huffman(tc ? ac[th] : dc[th], seg + k + 1, seg + k + 17, total)) return false;
                    k += 17 + total;
                }
            }
            else if(mk == 0xDD)
            {
                if(n < 2) return fail("JPEG: bad restart interval");
                restart = u16(seg);
            }
            else if(mk == 0xEE)
            {
                // Adobe: a transform flag of 0 marks three components as RGB, not YCbCr
                if(n >= 12 && std::memcmp(seg, "Adobe", 5) == 0)
                {
                    adobe = true;
                    adobe_transform = seg[11];
                }
            }
            else if(mk == 0xDA)
            {
                if(n < 1 || !scan(seg, n)) return err.empty() ? fail("JPEG: bad scan") : false;
                scanned = true;
            }
        }
        if(!frame || !scanned) return fail("JPEG: no image data");
        reconstruct();
        // colour: planes upsampled by replication, then YCbCr -> RGB (JFIF) unless Adobe says RGB
        rgba.assign((size_t)width * height * 4, 255);
        const bool ycc = comps.size() == 3 && !(adobe && adobe_transform == 0);
        for(uint32_t y = 0; y < height; ++y)
            for(uint32_t x = 0; x < width; ++x)
            {
                float v[3];
                for(size_t k = 0; k < comps.size(); ++k)
                {
                    const component &c = comps[k];
                    const uint32_t sx = x * c.h / hmax, sy = y * c.v / vmax;
                    v[k] = c.plane[(size_t)sy * c.bw * 8 + sx];
                }
                uint8_t *o = rgba.data() + ((size_t)y * width + x) * 4;
                if(comps.size() == 1)
                    o[0] = o[1] = o[2] = (uint8_t)v[0];
                else if(!ycc)
                    for(int k = 0; k < 3; ++k) o[k] = (uint8_t)v[k];
                else
                {
                    const float Y = v[0], cb = v[1] - 128.f, cr = v[2] - 128.f;
                    const float rgb[3] = {Y + 1.402f * cr, Y - 0.344136f * cb - 0.714136f * cr, Y + 1.772f * cb};
                    for(int k = 0; k < 3; ++k)
                        o[k] = (uint8_t)std::min(255.f, std::max(0.f, std::floor(rgb[k] + 0.5f)));
                }
            }
        w_out = width;
        h_out = height;
        return true;
    }
};

}// namespace

bool jpeg_decode(const uint8_t *data, size_t size, std::vector<uint8_t> &rgba, uint32_t &width, uint32_t &height,
                 std::string &err)
{
    err.clear();
    if(!data) return false;
    decoder d{data, data + size, err};
    return d.run(rgba, width, height);
}

}// namespace vkg
