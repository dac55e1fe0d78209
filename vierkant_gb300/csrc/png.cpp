// PNG decoding for the glTF loader: see png.hpp.
#include "png.hpp"

#include <algorithm>
#include <cstring>

namespace vkg
{
namespace
{

// LSB-first bit reader over a byte range (DEFLATE packs bits from the low end of each byte)
struct bit_reader
{
    const uint8_t *p;
    size_t n, pos = 0;
    uint32_t buf = 0;
    int cnt = 0;

    bool need(int k)
    {
        while(cnt < k)
        {
            if(pos >= n) return false;
            buf |= (uint32_t)p[pos++] << cnt;
            cnt += 8;
        }
        return true;
    }
    bool bits(int k, uint32_t &v)
    {
        if(k == 0)
        {
            v = 0;
            return true;
        }
        if(!need(k)) return false;
        v = buf & ((1u << k) - 1u);
        buf >>= k;
        cnt -= k;
        return true;
    }
    void align()
    {
        buf = 0;
        cnt = 0;
    }
};

// canonical Huffman code: counts per length and the symbols in code order
struct huffman
{
    uint16_t count[16] = {};
    std::vector<uint16_t> symbol;

    // false for an over-subscribed set of lengths (an incomplete one is allowed, as zlib does for
    // single-code distance trees)
    bool build(const uint8_t *lengths, int n)
    {
        std::fill(count, count + 16, (uint16_t)0);
        for(int i = 0; i < n; ++i) ++count[lengths[i]];
        count[0] = 0;
        int left = 1;
        for(int len = 1; len < 16; ++len)
        {
            left <<= 1;
            left -= count[len];
            if(left < 0) return false;
        }
        uint16_t offs[16];
        offs[1] = 0;
        for(int len = 1; len < 15; ++len) offs[len + 1] = (uint16_t)(offs[len] + count[len]);
        symbol.assign((size_t)n, 0);
        for(int i = 0; i < n; ++i)
            if(lengths[i]) symbol[offs[lengths[i]]++] = (uint16_t)i;
        return true;
    }

    // one symbol, code bits read most significant first; -1 on a bad code or the end of input
    int decode(bit_reader &br) const
    {
        int code = 0, first = 0, index = 0;
        for(int len = 1; len < 16; ++len)
        {
            uint32_t b;
            if(!br.bits(1, b)) return -1;
            code |= (int)b;
            const int c = count[len];
            if(code - c < first) return symbol[(size_t)(index + (code - first))];
            index += c;
            first += c;
            first <<= 1;
            code <<= 1;
        }
        return -1;
    }
};

constexpr uint16_t LEN_BASE[29] = {3,  4,  5,  6,  7,  8,  9,  10, 11,  13,  15,  17,  19,  23, 27,
                                   31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
constexpr uint8_t LEN_EXTRA[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
constexpr uint16_t DIST_BASE[30] = {1,   2,   3,   4,   5,   7,    9,    13,   17,   25,   33,   49,   65,    97,    129,
                                    193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
constexpr uint8_t DIST_EXTRA[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};

bool inflate_block(bit_reader &br, const huffman &lit, const huffman &dist, std::vector<uint8_t> &out, size_t max_out,
                   std::string &err)
{
    for(;;)
    {
        const int sym = lit.decode(br);
        if(sym < 0) return err = "deflate: bad literal / length code", false;
        if(sym < 256)
        {
            if(out.size() >= max_out) return err = "deflate: output larger than expected", false;
            out.push_back((uint8_t)sym);
            continue;
        }
        if(sym == 256) return true;
        const int li = sym - 257;
        if(li >= 29) return err = "deflate: bad length symbol", false;
        uint32_t extra;
        if(!br.bits(LEN_EXTRA[li], extra)) return err = "deflate: truncated", false;
        const size_t len = LEN_BASE[li] + extra;
        const int ds = dist.decode(br);
        if(ds < 0 || ds >= 30) return err = "deflate: bad distance code", false;
        if(!br.bits(DIST_EXTRA[ds], extra)) return err = "deflate: truncated", false;
        const size_t d = DIST_BASE[ds] + extra;
        if(d > out.size()) return err = "deflate: distance past the start", false;
        if(out.size() + len > max_out) return err = "deflate: output larger than expected", false;
        const size_t from = out.size() - d;
        for(size_t k = 0; k < len; ++k) out.push_back(out[from + k]);
    }
}

}// namespace

bool inflate_raw(const uint8_t *data, size_t size, std::vector<uint8_t> &out, size_t max_out, std::string &err)
{
    bit_reader br{data, size};
    out.clear();
    uint32_t last = 0;
    while(!last)
    {
        uint32_t type;
        if(!br.bits(1, last) || !br.bits(2, type)) return err = "deflate: truncated", false;
        if(type == 0)
        {
            // stored: LEN and NLEN on a byte boundary
            br.align();
            if(br.pos + 4 > size) return err = "deflate: truncated stored block", false;
            const uint32_t len = (uint32_t)data[br.pos] | ((uint32_t)data[br.pos + 1] << 8);
            const uint32_t nlen = (uint32_t)data[br.pos + 2] | ((uint32_t)data[br.pos + 3] << 8);
            br.pos += 4;
            if((len ^ 0xFFFFu) != nlen) return err = "deflate: stored block length mismatch", false;
            if(br.pos + len > size) return err = "deflate: truncated stored block", false;
            if(out.size() + len > max_out) return err = "deflate: output larger than expected", false;
            out.insert(out.end(), data + br.pos, data + br.pos + len);
            br.pos += len;
            continue;
        }
        huffman lit, dist;
        if(type == 1)
        {
            uint8_t l[288], dl[30];
            for(int i = 0; i < 144; ++i) l[i] = 8;
            for(int i = 144; i < 256; ++i) l[i] = 9;
            for(int i = 256; i < 280; ++i) l[i] = 7;
            for(int i = 280; i < 288; ++i) l[i] = 8;
            for(int i = 0; i < 30; ++i) dl[i] = 5;
            lit.build(l, 288);
            dist.build(dl, 30);
        }
        else if(type == 2)
        {
            uint32_t hlit, hdist, hclen;
            if(!br.bits(5, hlit) || !br.bits(5, hdist) || !br.bits(4, hclen)) return err = "deflate: truncated", false;
            hlit += 257;
            hdist += 1;
            hclen += 4;
            if(hlit > 286 || hdist > 30) return err = "deflate: bad code counts", false;
            static const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
            uint8_t cl[19] = {};
            for(uint32_t i = 0; i < hclen; ++i)
            {
                uint32_t v;
                if(!br.bits(3, v)) return err = "deflate: truncated", false;
                cl[order[i]] = (uint8_t)v;
            }
            huffman clh;
            if(!clh.build(cl, 19)) return err = "deflate: bad code-length code", false;
            uint8_t lens[316] = {};
            uint32_t k = 0;
            while(k < hlit + hdist)
            {
                const int sym = clh.decode(br);
                if(sym < 0) return err = "deflate: bad code-length symbol", false;
                if(sym < 16)
                {
                    lens[k++] = (uint8_t)sym;
                    continue;
                }
                uint32_t rep, val = 0, extra;
                if(sym == 16)
                {
                    if(k == 0) return err = "deflate: repeat with no previous length", false;
                    val = lens[k - 1];
                    if(!br.bits(2, extra)) return err = "deflate: truncated", false;
                    rep = 3 + extra;
                }
                else if(sym == 17)
                {
                    if(!br.bits(3, extra)) return err = "deflate: truncated", false;
                    rep = 3 + extra;
                }
                else
                {
                    if(!br.bits(7, extra)) return err = "deflate: truncated", false;
                    rep = 11 + extra;
                }
                if(k + rep > hlit + hdist) return err = "deflate: code lengths overrun", false;
                while(rep--) lens[k++] = (uint8_t)val;
            }
            if(lens[256] == 0) return err = "deflate: no end-of-block code", false;
            if(!lit.build(lens, (int)hlit) || !dist.build(lens + hlit, (int)hdist))
                return err = "deflate: bad Huffman lengths", false;
        }
        else
            return err = "deflate: reserved block type", false;
        if(!inflate_block(br, lit, dist, out, max_out, err)) return false;
    }
    return true;
}

namespace
{
uint32_t be32(const uint8_t *p) { return ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | p[3]; }

int paeth(int a, int b, int c)
{
    const int p = a + b - c, pa = std::abs(p - a), pb = std::abs(p - b), pc = std::abs(p - c);
    return pa <= pb && pa <= pc ? a : (pb <= pc ? b : c);
}
}// namespace

bool png_decode(const uint8_t *data, size_t size, std::vector<uint8_t> &rgba, uint32_t &width, uint32_t &height,
                std::string &err)
{
    static const uint8_t sig[8] = {137, 80, 78, 71, 13, 10, 26, 10};
    if(size < 8 || std::memcmp(data, sig, 8) != 0) return err = "not a PNG file", false;
    size_t pos = 8;
    uint32_t w = 0, h = 0, depth = 0, ctype = 0, interlace = 0;
    bool have_ihdr = false;
    std::vector<uint8_t> idat, palette, trns;
    for(;;)
    {
        if(pos + 8 > size) return err = "PNG: truncated chunk", false;
        const uint32_t len = be32(data + pos);
        const uint8_t *type = data + pos + 4;
        if(len > size || pos + 12 + (size_t)len > size) return err = "PNG: truncated chunk", false;
        const uint8_t *body = data + pos + 8;
        if(std::memcmp(type, "IHDR", 4) == 0)
        {
            if(len != 13) return err = "PNG: bad IHDR", false;
            w = be32(body);
            h = be32(body + 4);
            depth = body[8];
            ctype = body[9];
            interlace = body[12];
            if(body[10] != 0 || body[11] != 0) return err = "PNG: unknown compression or filter method", false;
            have_ihdr = true;
        }
        else if(std::memcmp(type, "PLTE", 4) == 0)
            palette.assign(body, body + len);
        else if(std::memcmp(type, "tRNS", 4) == 0)
            trns.assign(body, body + len);
        else if(std::memcmp(type, "IDAT", 4) == 0)
            idat.insert(idat.end(), body, body + len);
        else if(std::memcmp(type, "IEND", 4) == 0)
            break;
        pos += 12 + (size_t)len;
    }
    if(!have_ihdr) return err = "PNG: no IHDR", false;
    if(w == 0 || h == 0 || w > 32768 || h > 32768) return err = "PNG: size out of range", false;
    if(interlace) return err = "PNG: interlaced images are not supported", false;
    int channels;
    switch(ctype)
    {
        case 0: channels = 1; break;
        case 2: channels = 3; break;
        case 3: channels = 1; break;
        case 4: channels = 2; break;
        case 6: channels = 4; break;
        default: return err = "PNG: unknown colour type", false;
    }
    const bool depth_ok = depth == 8 || depth == 16 || ((ctype == 0 || ctype == 3) && (depth == 1 || depth == 2 || depth == 4));
    if(!depth_ok || (ctype == 3 && depth == 16)) return err = "PNG: unsupported bit depth", false;
    if(ctype == 3 && (palette.empty() || palette.size() % 3)) return err = "PNG: missing palette", false;
    const size_t bits_pp = (size_t)channels * depth;
    const size_t stride = (w * bits_pp + 7) / 8;
    const size_t bpp = std::max<size_t>(1, bits_pp / 8);
    if(idat.size() < 2 || (idat[0] & 0x0Fu) != 8 || (idat[1] & 0x20u) || ((idat[0] << 8) | idat[1]) % 31)
        return err = "PNG: bad zlib header", false;
    std::vector<uint8_t> raw;
    const size_t expect = (stride + 1) * (size_t)h;
    if(!inflate_raw(idat.data() + 2, idat.size() - 2, raw, expect, err)) return false;
    if(raw.size() != expect) return err = "PNG: image data size mismatch", false;
    // unfilter in place
    std::vector<uint8_t> prev(stride, 0);
    std::vector<uint8_t> img(stride * (size_t)h);
    for(uint32_t y = 0; y < h; ++y)
    {
        const uint8_t f = raw[y * (stride + 1)];
        const uint8_t *in = raw.data() + y * (stride + 1) + 1;
        uint8_t *cur = img.data() + y * stride;
        for(size_t x = 0; x < stride; ++x)
        {
            const int a = x >= bpp ? cur[x - bpp] : 0, b = prev[x], c = x >= bpp ? prev[x - bpp] : 0;
            int v = in[x];
            switch(f)
            {
                case 0: break;
                case 1: v += a; break;
                case 2: v += b; break;
                case 3: v += (a + b) >> 1; break;
                case 4: v += paeth(a, b, c); break;
                default: return err = "PNG: unknown filter type", false;
            }
            cur[x] = (uint8_t)v;
        }
        std::memcpy(prev.data(), cur, stride);
    }
    // expand to RGBA8
    rgba.assign((size_t)w * h * 4, 255);
    auto sample = [&](const uint8_t *row, uint32_t x, int ch) -> uint32_t {
        if(depth == 8) return row[(size_t)x * channels + ch];
        if(depth == 16) return row[((size_t)x * channels + ch) * 2]; // the high byte
        const uint32_t per = 8 / depth, byte = row[x / per], shift = 8 - depth * (x % per + 1);
        return (byte >> shift) & ((1u << depth) - 1u);
    };
    const uint32_t scale = depth < 8 ? 255u / ((1u << depth) - 1u) : 1u;
    for(uint32_t y = 0; y < h; ++y)
    {
        const uint8_t *row = img.data() + y * stride;
        for(uint32_t x = 0; x < w; ++x)
        {
            uint8_t *o = rgba.data() + ((size_t)y * w + x) * 4;
            if(ctype == 3)
            {
                const uint32_t i = sample(row, x, 0);
                if((size_t)i * 3 + 2 >= palette.size()) return err = "PNG: palette index out of range", false;
                o[0] = palette[i * 3];
                o[1] = palette[i * 3 + 1];
                o[2] = palette[i * 3 + 2];
                o[3] = i < trns.size() ? trns[i] : 255;
            }
            else if(ctype == 0 || ctype == 4)
            {
                const uint8_t g = (uint8_t)(sample(row, x, 0) * scale);
                o[0] = o[1] = o[2] = g;
                if(ctype == 4) o[3] = (uint8_t)sample(row, x, 1);
            }
            else
            {
                for(int c = 0; c < 3; ++c) o[c] = (uint8_t)sample(row, x, c);
                if(ctype == 6) o[3] = (uint8_t)sample(row, x, 3);
            }
        }
    }
    width = w;
    height = h;
    return true;
}

}// namespace vkg
