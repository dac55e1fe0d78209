// glTF 2.0 scene ingestion for the path tracer (host only): the reference's model/gltf.cpp path
// (src/model/gltf.cpp, tinygltf underneath) restated without third-party code.
//
// Reads .gltf (JSON; buffers as base64 data URIs or files next to it) and .glb (binary container).
// Produces, for the default scene (`scene`, else scene 0, else every node that is nobody's child):
//   * one mesh per (mesh, triangle primitive) with float positions and uint32 indices (sequential
//     when a primitive has none); other primitive modes are skipped, as the reference does
//     (gltf.cpp:1126-1130);
//   * one instance per node placement of each primitive, nodes visited breadth first from the scene's
//     roots as the reference does (gltf.cpp:1063-1218), the world transform composed parent x local
//     with 4x4 matrices in double (local = the node's `matrix`, else T * R * S; gltf.cpp:136-159);
//     the primitive's material, 0 when it has none (the reference's default index);
//   * the materials (gltf.cpp:316-560): base colour, metallic (default 1), roughness (default 1),
//     emissive x KHR_materials_emissive_strength, doubleSided, KHR_materials_transmission,
//     KHR_materials_ior, KHR_materials_dispersion, KHR_materials_clearcoat, KHR_materials_sheen, KHR_materials_iridescence (the
//     film thickness is the range's maximum, as the shader reads it), KHR_materials_diffuse_transmission,
//     KHR_materials_volume (attenuation colour / distance) and KHR_materials_scatter /
//     KHR_materials_volume_scatter (gltf.cpp:476-500, :634-657); a default material when the asset
//     has none;
//   * KHR_lights_punctual lights placed by their nodes (gltf.cpp:1043-1061, :1182-1190), converted as
//     convert_light does (punctual_light.hpp:92-111): position = translation, direction = R (0,0,-1),
//     tangent = R (1,0,0), R the node's rotation (its world matrix's columns normalised).
//   * per primitive NORMAL, TEXCOORD_0 (float, or normalised unsigned integers) and TANGENT (xyz; when
//     absent but NORMAL and TEXCOORD_0 are there, computed as Geometry::compute_tangents does,
//     Geometry.cpp:196-252); the textures the materials use (baseColor, metallicRoughness, normal,
//     emissive -- which zeroes the emissive factor, as gltf.cpp:377 does -- transmission, diffuse
//     transmission factor / colour), one per glTF texture: its image decoded from PNG or JPEG
//     (sequential or progressive; data URI, file or buffer view) with its sampler's wrap modes (REPEAT
//     by default); a texture whose image cannot be decoded (another format, a lossless or arithmetic-
//     coded JPEG) is counted in skipped_textures and its material slots left empty. The colour texture's KHR_texture_transform
//     becomes the material's uv_transform.
// Not read: occlusion, skins, morph targets, animations, cameras, volume
// thickness, specular, sparse accessors, quantised positions. The reference composes transforms as
// translation / quaternion / scale triples and projects shear away (transform.hpp:106-128); the
// matrix composition here is the same for every chain without shear.
#include "internal.hpp"
#include "jpeg.hpp"
#include "png.hpp"

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <deque>
#include <fstream>
#include <limits>
#include <string>
#include <vector>

namespace
{

// ---- a small JSON reader -------------------------------------------------------------------
struct jv
{
    enum kind_t { NUL, BOOL, NUM, STR, ARR, OBJ } kind = NUL;
    bool b = false;
    double n = 0;
    std::string s;
    std::vector<jv> a;
    std::vector<std::pair<std::string, jv>> o;

    const jv *get(const char *k) const
    {
        if(kind != OBJ) return nullptr;
        for(const auto &kv: o)
            if(kv.first == k) return &kv.second;
        return nullptr;
    }
    double num(const char *k, double def) const
    {
        const jv *v = get(k);
        return v && v->kind == NUM ? v->n : def;
    }
    long idx(const char *k) const
    {
        const jv *v = get(k);
        return v && v->kind == NUM && v->n >= 0 && v->n == std::floor(v->n) ? (long)v->n : -1;
    }
    const std::string *str(const char *k) const
    {
        const jv *v = get(k);
        return v && v->kind == STR ? &v->s : nullptr;
    }
    const std::vector<jv> *arr(const char *k) const
    {
        const jv *v = get(k);
        return v && v->kind == ARR ? &v->a : nullptr;
    }
};

struct json_parser
{
    const char *p, *end;
    std::string err;
    int depth = 0;

    void ws()
    {
        while(p < end && (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r')) ++p;
    }
    bool fail(const char *m)
    {
        if(err.empty()) err = m;
        return false;
    }
    bool lit(const char *w)
    {
        const size_t n = std::strlen(w);
        if((size_t)(end - p) < n || std::strncmp(p, w, n) != 0) return false;
        p += n;
        return true;
    }
    static void utf8(std::string &out, uint32_t c)
    {
        if(c < 0x80) out += (char)c;
        else if(c < 0x800)
        {
            out += (char)(0xC0 | (c >> 6));
            out += (char)(0x80 | (c & 0x3F));
        }
        else if(c < 0x10000)
        {
            out += (char)(0xE0 | (c >> 12));
            out += (char)(0x80 | ((c >> 6) & 0x3F));
            out += (char)(0x80 | (c & 0x3F));
        }
        else
        {
            out += (char)(0xF0 | (c >> 18));
            out += (char)(0x80 | ((c >> 12) & 0x3F));
            out += (char)(0x80 | ((c >> 6) & 0x3F));
            out += (char)(0x80 | (c & 0x3F));
        }
    }
    bool hex4(uint32_t &v)
    {
        if(end - p < 4) return false;
        v = 0;
        for(int i = 0; i < 4; ++i)
        {
            const char c = *p++;
            v <<= 4;
            if(c >= '0' && c <= '9') v |= (uint32_t)(c - '0');
            else if(c >= 'a' && c <= 'f') v |= (uint32_t)(c - 'a' + 10);
            else if(c >= 'A' && c <= 'F') v |= (uint32_t)(c - 'A' + 10);
            else return false;
        }
        return true;
    }
    bool string(std::string &out)
    {
        if(p >= end || *p != '"') return fail("expected a string");
        ++p;
        while(p < end && *p != '"')
        {
            char c = *p++;
            if(c != '\\')
            {
                out += c;
                continue;
            }
            if(p >= end) return fail("unterminated escape");
            c = *p++;
            switch(c)
            {
                case '"': out += '"'; break;
                case '\\': out += '\\'; break;
                case '/': out += '/'; break;
                case 'b': out += '\b'; break;
                case 'f': out += '\f'; break;
                case 'n': out += '\n'; break;
                case 'r': out += '\r'; break;
                case 't': out += '\t'; break;
                case 'u':
                {
                    uint32_t u;
                    if(!hex4(u)) return fail("bad \\u escape");
                    if(u >= 0xD800 && u < 0xDC00 && end - p >= 6 && p[0] == '\\' && p[1] == 'u')
                    {
                        p += 2;
                        uint32_t lo;
                        if(!hex4(lo) || lo < 0xDC00 || lo >= 0xE000) return fail("bad surrogate pair");
                        u = 0x10000 + ((u - 0xD800) << 10) + (lo - 0xDC00);
                    }
                    utf8(out, u);
                    break;
                }
                default: return fail("bad escape");
            }
        }
        if(p >= end) return fail("unterminated string");
        ++p;
        return true;
    }
    bool value(jv &v)
    {
        if(++depth > 256) return fail("nesting too deep");
        ws();
        if(p >= end) return fail("unexpected end");
        bool ok = true;
        if(*p == '{')
        {
            v.kind = jv::OBJ;
            ++p;
            ws();
            if(p < end && *p == '}') ++p;
            else
                for(;;)
                {
                    ws();
                    std::string k;
                    if(!string(k)) return false;
                    ws();
                    if(p >= end || *p != ':') return fail("expected ':'");
                    ++p;
                    v.o.emplace_back(std::move(k), jv{});
                    if(!value(v.o.back().second)) return false;
                    ws();
                    if(p < end && *p == ',')
                    {
                        ++p;
                        continue;
                    }
                    if(p < end && *p == '}')
                    {
                        ++p;
                        break;
                    }
                    return fail("expected ',' or '}'");
                }
        }
        else if(*p == '[')
        {
            v.kind = jv::ARR;
            ++p;
            ws();
            if(p < end && *p == ']') ++p;
            else
                for(;;)
                {
                    v.a.emplace_back();
                    if(!value(v.a.back())) return false;
                    ws();
                    if(p < end && *p == ',')
                    {
                        ++p;
                        continue;
                    }
                    if(p < end && *p == ']')
                    {
                        ++p;
                        break;
                    }
                    return fail("expected ',' or ']'");
                }
        }
        else if(*p == '"')
        {
            v.kind = jv::STR;
            ok = string(v.s);
        }
        else if(lit("true"))
        {
            v.kind = jv::BOOL;
            v.b = true;
        }
        else if(lit("false")) v.kind = jv::BOOL;
        else if(lit("null")) v.kind = jv::NUL;
        else
        {
            char *e = nullptr;
            std::string tok;
            while(p < end && std::strchr("+-0123456789.eE", *p)) tok += *p++;
            if(tok.empty()) return fail("unexpected character");
            v.kind = jv::NUM;
            v.n = std::strtod(tok.c_str(), &e);
            if(!e || *e) return fail("bad number");
        }
        --depth;
        return ok;
    }
};

// ---- the asset ------------------------------------------------------------------------------
struct mesh_t
{
    std::vector<float> xyz;
    std::vector<uint32_t> idx;
    std::vector<float> nrm; // the primitive's NORMAL attribute (3 per vertex), empty when it has none
    std::vector<float> uv;  // TEXCOORD_0 (2 per vertex), empty when it has none
    std::vector<float> tng; // TANGENT xyz or computed tangents (3 per vertex), empty when neither
};

struct texture_t
{
    std::vector<uint8_t> rgba; // empty: the image could not be decoded
    uint32_t width = 0, height = 0, wrap_s = VKG_WRAP_REPEAT, wrap_t = VKG_WRAP_REPEAT;
};

}// namespace

struct vkg_gltf
{
    std::vector<mesh_t> meshes;
    std::vector<vkg_instance> instances;
    std::vector<vkg_material> materials;
    std::vector<vkg_light> lights;
    std::vector<texture_t> textures;
    uint32_t skipped_primitives = 0, skipped_textures = 0;
};

namespace
{

struct loader
{
    std::string err;
    std::string dir;
    jv doc;
    std::vector<std::vector<uint8_t>> buffers;

    bool fail(const char *fmt, ...)
    {
        if(!err.empty()) return false;
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        std::vsnprintf(buf, sizeof(buf), fmt, ap);
        va_end(ap);
        err = buf;
        return false;
    }

    static bool read_file(const std::string &path, std::vector<uint8_t> &out)
    {
        std::ifstream f(path, std::ios::binary);
        if(!f) return false;
        f.seekg(0, std::ios::end);
        const std::streamoff n = f.tellg();
        if(n < 0) return false;
        f.seekg(0);
        out.resize((size_t)n);
        return n == 0 || (bool)f.read(reinterpret_cast<char *>(out.data()), n);
    }

    static bool base64(const std::string &in, size_t from, std::vector<uint8_t> &out)
    {
        auto val = [](char c) -> int {
            if(c >= 'A' && c <= 'Z') return c - 'A';
            if(c >= 'a' && c <= 'z') return c - 'a' + 26;
            if(c >= '0' && c <= '9') return c - '0' + 52;
            if(c == '+') return 62;
            if(c == '/') return 63;
            return -1;
        };
        uint32_t acc = 0;
        int bits = 0;
        for(size_t i = from; i < in.size(); ++i)
        {
            if(in[i] == '=') break;
            const int v = val(in[i]);
            if(v < 0) return false;
            acc = (acc << 6) | (uint32_t)v;
            bits += 6;
            if(bits >= 8)
            {
                bits -= 8;
                out.push_back((uint8_t)((acc >> bits) & 0xFFu));
            }
        }
        return true;
    }

    bool parse_json(const char *b, size_t n)
    {
        json_parser jp{b, b + n, {}, 0};
        if(!jp.value(doc)) return fail("JSON: %s", jp.err.c_str());
        jp.ws();
        if(jp.p != jp.end) return fail("JSON: trailing characters");
        if(doc.kind != jv::OBJ) return fail("JSON: the document is not an object");
        return true;
    }

    bool load(const std::string &path)
    {
        const size_t slash = path.find_last_of("/\\");
        dir = slash == std::string::npos ? std::string() : path.substr(0, slash + 1);
        std::vector<uint8_t> file;
        if(!read_file(path, file)) return fail("cannot read '%s'", path.c_str());
        std::vector<uint8_t> glb_bin;
        bool have_bin = false;
        if(file.size() >= 12 && std::memcmp(file.data(), "glTF", 4) == 0)
        {
            // binary container: header, JSON chunk, optional BIN chunk
            uint32_t version, length;
            std::memcpy(&version, file.data() + 4, 4);
            std::memcpy(&length, file.data() + 8, 4);
            if(version != 2 || length > file.size()) return fail("GLB: bad header");
            size_t off = 12;
            bool have_json = false;
            while(off + 8 <= length)
            {
                uint32_t clen, ctype;
                std::memcpy(&clen, file.data() + off, 4);
                std::memcpy(&ctype, file.data() + off + 4, 4);
                off += 8;
                if(clen > length - off) return fail("GLB: chunk past the end");
                if(ctype == 0x4E4F534Au && !have_json)
                {
                    if(!parse_json(reinterpret_cast<const char *>(file.data() + off), clen)) return false;
                    have_json = true;
                }
                else if(ctype == 0x004E4942u && !have_bin)
                {
                    glb_bin.assign(file.begin() + (std::ptrdiff_t)off, file.begin() + (std::ptrdiff_t)(off + clen));
                    have_bin = true;
                }
                off += (clen + 3u) & ~3u;
            }
            if(!have_json) return fail("GLB: no JSON chunk");
        }
        else if(!parse_json(reinterpret_cast<const char *>(file.data()), file.size()))
            return false;
        const jv *asset = doc.get("asset");
        const std::string *ver = asset ? asset->str("version") : nullptr;
        if(!ver || ver->empty() || (*ver)[0] != '2') return fail("asset.version must be 2.x");
        if(const auto *bufs = doc.arr("buffers"))
            for(size_t i = 0; i < bufs->size(); ++i)
            {
                const jv &b = (*bufs)[i];
                const std::string *uri = b.str("uri");
                std::vector<uint8_t> data;
                if(!uri)
                {
                    if(!have_bin || i != 0) return fail("buffer %zu has no uri and no GLB chunk", i);
                    data = glb_bin;
                }
                else if(uri->rfind("data:", 0) == 0)
                {
                    const size_t comma = uri->find(',');
                    if(comma == std::string::npos || uri->find(";base64") == std::string::npos ||
                       !base64(*uri, comma + 1, data))
                        return fail("buffer %zu: unsupported data URI", i);
                }
                else if(!read_file(dir + *uri, data))
                    return fail("buffer %zu: cannot read '%s'", i, uri->c_str());
                const double bl = b.num("byteLength", -1);
                if(bl < 0 || (double)data.size() < bl) return fail("buffer %zu is shorter than its byteLength", i);
                buffers.push_back(std::move(data));
            }
        return true;
    }

    // the elements of an accessor as doubles (components per element in `comps`)
    // want_float: float components only (or, with unorm_ok, also normalised unsigned bytes / shorts,
    // mapped to [0, 1]); else integer components only
    bool accessor(long ai, const char *what, std::vector<double> &out, int &comps, bool want_float, bool unorm_ok = false)
    {
        const auto *accs = doc.arr("accessors");
        if(!accs || ai < 0 || (size_t)ai >= accs->size()) return fail("%s: accessor %ld missing", what, ai);
        const jv &a = (*accs)[(size_t)ai];
        if(a.get("sparse")) return fail("%s: sparse accessors are not supported", what);
        const std::string *type = a.str("type");
        comps = !type ? 0 : *type == "SCALAR" ? 1 : *type == "VEC2" ? 2 : *type == "VEC3" ? 3 : *type == "VEC4" ? 4 : 0;
        if(!comps) return fail("%s: unsupported accessor type", what);
        const long ct = (long)a.num("componentType", 0);
        const size_t csize = ct == 5120 || ct == 5121 ? 1 : ct == 5122 || ct == 5123 ? 2 : ct == 5125 || ct == 5126 ? 4 : 0;
        const jv *nz = a.get("normalized");
        const bool unorm = unorm_ok && nz && nz->kind == jv::BOOL && nz->b && (ct == 5121 || ct == 5123);
        if(!csize || (want_float && ct != 5126 && !unorm) || (!want_float && ct == 5126))
            return fail("%s: unsupported component type %ld", what, ct);
        const double count = a.num("count", -1);
        if(count < 0 || count > 1e9) return fail("%s: bad count", what);
        const size_t n = (size_t)count;
        out.assign(n * (size_t)comps, 0.0);
        const long bvi = a.idx("bufferView");
        if(bvi < 0) return true; // all zeros (glTF 3.6.2.3)
        const auto *bvs = doc.arr("bufferViews");
        if(!bvs || (size_t)bvi >= bvs->size()) return fail("%s: bufferView %ld missing", what, bvi);
        const jv &bv = (*bvs)[(size_t)bvi];
        const long bi = bv.idx("buffer");
        if(bi < 0 || (size_t)bi >= buffers.size()) return fail("%s: buffer %ld missing", what, bi);
        const std::vector<uint8_t> &buf = buffers[(size_t)bi];
        const size_t elem = csize * (size_t)comps;
        const size_t stride = bv.get("byteStride") ? (size_t)bv.num("byteStride", 0) : elem;
        const size_t view_off = (size_t)bv.num("byteOffset", 0), view_len = (size_t)bv.num("byteLength", 0);
        const size_t acc_off = (size_t)a.num("byteOffset", 0);
        if(stride < elem || view_off + view_len > buf.size() ||
           (n && acc_off + stride * (n - 1) + elem > view_len))
            return fail("%s: accessor %ld reads past its buffer view", what, ai);
        const uint8_t *base = buf.data() + view_off + acc_off;
        for(size_t i = 0; i < n; ++i)
            for(int c = 0; c < comps; ++c)
            {
                const uint8_t *q = base + i * stride + (size_t)c * csize;
                double v = 0;
                switch(ct)
                {
                    case 5120: v = (double)*reinterpret_cast<const int8_t *>(q); break;
                    case 5121: v = (double)*q; break;
                    case 5122: { int16_t t; std::memcpy(&t, q, 2); v = t; break; }
                    case 5123: { uint16_t t; std::memcpy(&t, q, 2); v = t; break; }
                    case 5125: { uint32_t t; std::memcpy(&t, q, 4); v = t; break; }
                    default: { float t; std::memcpy(&t, q, 4); v = t; break; }
                }
                out[i * (size_t)comps + (size_t)c] = unorm ? v / (ct == 5121 ? 255.0 : 65535.0) : v;
            }
        return true;
    }

    // Geometry::compute_tangents (Geometry.cpp:196-252): per-triangle UV-derivative tangents summed at
    // the vertices, Gram-Schmidt against the normal, negated unless dot(cross(n, t), b) < 0
    static void compute_tangents(mesh_t &M)
    {
        const size_t nv = M.xyz.size() / 3;
        std::vector<float> t(nv * 3, 0.f), b(nv * 3, 0.f);
        for(size_t i = 0; i + 2 < M.idx.size(); i += 3)
        {
            const uint32_t a = M.idx[i], bb = M.idx[i + 1], c = M.idx[i + 2];
            const float *v0 = &M.xyz[3 * (size_t)a], *v1 = &M.xyz[3 * (size_t)bb], *v2 = &M.xyz[3 * (size_t)c];
            const float *u0 = &M.uv[2 * (size_t)a], *u1 = &M.uv[2 * (size_t)bb], *u2 = &M.uv[2 * (size_t)c];
            const float x1 = v1[0] - v0[0], x2 = v2[0] - v0[0], y1 = v1[1] - v0[1], y2 = v2[1] - v0[1];
            const float z1 = v1[2] - v0[2], z2 = v2[2] - v0[2];
            const float s1 = u1[0] - u0[0], s2 = u2[0] - u0[0], t1 = u1[1] - u0[1], t2 = u2[1] - u0[1];
            const float r = 1.f / (s1 * t2 - s2 * t1);
            const float sd[3] = {(t2 * x1 - t1 * x2) * r, (t2 * y1 - t1 * y2) * r, (t2 * z1 - t1 * z2) * r};
            const float td[3] = {(s1 * x2 - s2 * x1) * r, (s1 * y2 - s2 * y1) * r, (s1 * z2 - s2 * z1) * r};
            for(uint32_t v: {a, bb, c})
                for(int k = 0; k < 3; ++k)
                {
                    t[3 * (size_t)v + k] += sd[k];
                    b[3 * (size_t)v + k] += td[k];
                }
        }
        M.tng.assign(nv * 3, 0.f);
        for(size_t v = 0; v < nv; ++v)
        {
            const float *n = &M.nrm[3 * v], *tv = &t[3 * v], *bv = &b[3 * v];
            const float d = n[0] * tv[0] + n[1] * tv[1] + n[2] * tv[2];
            float o[3] = {tv[0] - n[0] * d, tv[1] - n[1] * d, tv[2] - n[2] * d};
            const float len = std::sqrt(o[0] * o[0] + o[1] * o[1] + o[2] * o[2]);
            for(float &x: o) x = len > 0.f ? x / len : 0.f;
            const float cr[3] = {n[1] * tv[2] - n[2] * tv[1], n[2] * tv[0] - n[0] * tv[2], n[0] * tv[1] - n[1] * tv[0]};
            const float sign = (cr[0] * bv[0] + cr[1] * bv[1] + cr[2] * bv[2]) < 0.f ? 1.f : -1.f;
            for(int k = 0; k < 3; ++k) M.tng[3 * v + k] = o[k] * sign;
        }
    }

    // the bytes of image ii: a data URI, a file next to the asset, or a buffer view
    bool image_bytes(long ii, std::vector<uint8_t> &out)
    {
        const auto *imgs = doc.arr("images");
        if(!imgs || ii < 0 || (size_t)ii >= imgs->size()) return fail("image %ld missing", ii);
        const jv &im = (*imgs)[(size_t)ii];
        if(const std::string *uri = im.str("uri"))
        {
            if(uri->rfind("data:", 0) == 0)
            {
                const size_t comma = uri->find(',');
                if(comma == std::string::npos || uri->find(";base64") == std::string::npos || !base64(*uri, comma + 1, out))
                    return fail("image %ld: unreadable data uri", ii);
                return true;
            }
            if(!read_file(dir + *uri, out)) return fail("image %ld: cannot read '%s'", ii, uri->c_str());
            return true;
        }
        const long bvi = im.idx("bufferView");
        const auto *bvs = doc.arr("bufferViews");
        if(bvi < 0 || !bvs || (size_t)bvi >= bvs->size()) return fail("image %ld has no uri and no bufferView", ii);
        const jv &bv = (*bvs)[(size_t)bvi];
        const long bi = bv.idx("buffer");
        if(bi < 0 || (size_t)bi >= buffers.size()) return fail("image %ld: buffer %ld missing", ii, bi);
        const size_t off = (size_t)bv.num("byteOffset", 0), len = (size_t)bv.num("byteLength", 0);
        if(off + len > buffers[(size_t)bi].size()) return fail("image %ld: buffer view past its buffer", ii);
        out.assign(buffers[(size_t)bi].begin() + (long)off, buffers[(size_t)bi].begin() + (long)(off + len));
        return true;
    }

    // the asset's textures: PNG images decoded with their samplers' wrap modes; false only on a
    // malformed reference (a texture whose image is not a PNG is kept empty and counted)
    bool textures(vkg_gltf &G)
    {
        const auto *texs = doc.arr("textures");
        if(!texs) return true;
        const auto *samplers = doc.arr("samplers");
        auto wrap = [](double w) -> uint32_t {
            return w == 33071 ? VKG_WRAP_CLAMP_TO_EDGE : w == 33648 ? VKG_WRAP_MIRRORED_REPEAT : VKG_WRAP_REPEAT;
        };
        for(size_t ti = 0; ti < texs->size(); ++ti)
        {
            const jv &t = (*texs)[ti];
            texture_t T;
            const long si = t.idx("sampler");
            if(samplers && si >= 0 && (size_t)si < samplers->size())
            {
                T.wrap_s = wrap((*samplers)[(size_t)si].num("wrapS", 10497));
                T.wrap_t = wrap((*samplers)[(size_t)si].num("wrapT", 10497));
            }
            const long src = t.idx("source");
            std::vector<uint8_t> bytes;
            if(src < 0) return fail("texture %zu has no source image", ti);
            if(!image_bytes(src, bytes)) return false;
            // PNG or JPEG by their signatures (the MIME type is advisory); anything else is skipped
            std::string perr;
            const bool is_jpeg = bytes.size() >= 2 && bytes[0] == 0xFF && bytes[1] == 0xD8;
            const bool ok = is_jpeg ? vkg::jpeg_decode(bytes.data(), bytes.size(), T.rgba, T.width, T.height, perr)
                                    : vkg::png_decode(bytes.data(), bytes.size(), T.rgba, T.width, T.height, perr);
            if(!ok)
            {
                T.rgba.clear();
                ++G.skipped_textures;
            }
            G.textures.push_back(std::move(T));
        }
        return true;
    }

    static void mat_mul(const double *A, const double *B, double *C) // column-major 4x4
    {
        double r[16];
        for(int c = 0; c < 4; ++c)
            for(int rr = 0; rr < 4; ++rr)
            {
                double s = 0;
                for(int k = 0; k < 4; ++k) s += A[k * 4 + rr] * B[c * 4 + k];
                r[c * 4 + rr] = s;
            }
        std::memcpy(C, r, sizeof(r));
    }

    static void local_matrix(const jv &node, double *M)
    {
        const auto *m = node.arr("matrix");
        if(m && m->size() == 16)
        {
            for(int i = 0; i < 16; ++i) M[i] = (*m)[(size_t)i].kind == jv::NUM ? (*m)[(size_t)i].n : (i % 5 == 0);
            return;
        }
        double t[3] = {0, 0, 0}, s[3] = {1, 1, 1}, q[4] = {0, 0, 0, 1}; // q = (x, y, z, w)
        auto rd = [&](const char *k, double *dst, size_t n) {
            const auto *v = node.arr(k);
            if(v && v->size() == n)
                for(size_t i = 0; i < n; ++i)
                    if((*v)[i].kind == jv::NUM) dst[i] = (*v)[i].n;
        };
        rd("translation", t, 3);
        rd("scale", s, 3);
        rd("rotation", q, 4);
        const double x = q[0], y = q[1], z = q[2], w = q[3];
        const double R[9] = {1 - 2 * (y * y + z * z), 2 * (x * y + z * w),     2 * (x * z - y * w),
                             2 * (x * y - z * w),     1 - 2 * (x * x + z * z), 2 * (y * z + x * w),
                             2 * (x * z + y * w),     2 * (y * z - x * w),     1 - 2 * (x * x + y * y)}; // columns
        for(int c = 0; c < 3; ++c)
        {
            for(int r = 0; r < 3; ++r) M[c * 4 + r] = R[c * 3 + r] * s[c];
            M[c * 4 + 3] = 0;
        }
        M[12] = t[0], M[13] = t[1], M[14] = t[2], M[15] = 1;
    }

    static float clampf(double v, double lo, double hi) { return (float)std::min(std::max(v, lo), hi); }

    vkg_material material(const jv &m)
    {
        vkg_material r;
        vkg_material_defaults(&r);
        auto rd = [&](const jv *o, const char *k, float *dst, size_t n) {
            const auto *v = o ? o->arr(k) : nullptr;
            if(v && v->size() >= n)
                for(size_t i = 0; i < n; ++i)
                    if((*v)[i].kind == jv::NUM) dst[i] = (float)(*v)[i].n;
        };
        const jv *pbr = m.get("pbrMetallicRoughness");
        rd(pbr, "baseColorFactor", r.base_color, 3);
        float bc[4] = {r.base_color[0], r.base_color[1], r.base_color[2], 1.f};
        rd(pbr, "baseColorFactor", bc, 4);
        r.alpha = bc[3];
        // alphaMode (gltf.cpp:323-326 of the reference): OPAQUE (default), BLEND, MASK; alphaCutoff 0.5
        if(const std::string *am = m.str("alphaMode"))
            r.blend_mode = *am == "BLEND" ? VKG_BLEND_BLEND : (*am == "MASK" ? VKG_BLEND_MASK : VKG_BLEND_OPAQUE);
        r.alpha_cutoff = (float)m.num("alphaCutoff", 0.5);
        r.metalness = pbr ? clampf(pbr->num("metallicFactor", 1.0), 0, 1) : 1.f;
        r.roughness = pbr ? (float)pbr->num("roughnessFactor", 1.0) : 1.f;
        float em[3] = {0, 0, 0};
        rd(&m, "emissiveFactor", em, 3);
        float strength = 1.f;
        const jv *ext = m.get("extensions");
        if(ext && ext->kind == jv::OBJ)
        {
            if(const jv *e = ext->get("KHR_materials_emissive_strength"))
                strength = (float)e->num("emissiveStrength", 1.0);
            if(const jv *e = ext->get("KHR_materials_transmission"))
                r.transmission = clampf(e->num("transmissionFactor", 0.0), 0, 1);
            if(const jv *e = ext->get("KHR_materials_ior")) r.ior = (float)e->num("ior", 1.5);
            if(const jv *e = ext->get("KHR_materials_dispersion")) r.dispersion = (float)e->num("dispersion", 0.0);
            if(const jv *e = ext->get("KHR_materials_clearcoat"))
            {
                r.clearcoat = (float)std::max(0.0, e->num("clearcoatFactor", 0.0));
                r.clearcoat_roughness = (float)std::max(0.0, e->num("clearcoatRoughnessFactor", 0.0));
            }
            if(const jv *e = ext->get("KHR_materials_sheen"))
            {
                r.sheen_color[0] = r.sheen_color[1] = r.sheen_color[2] = 0.f;
                rd(e, "sheenColorFactor", r.sheen_color, 3);
                r.sheen_roughness = (float)std::max(0.0, e->num("sheenRoughnessFactor", 0.0));
            }
            if(const jv *e = ext->get("KHR_materials_iridescence"))
            {
                r.iridescence = clampf(e->num("iridescenceFactor", 0.0), 0, 1);
                r.iridescence_ior = (float)e->num("iridescenceIOR", 1.3);
                r.iridescence_thickness = (float)e->num("iridescenceThicknessMaximum", 400.0);
            }
            if(const jv *e = ext->get("KHR_materials_diffuse_transmission"))
            {
                r.diffuse_transmission = clampf(e->num("diffuseTransmissionFactor", 0.0), 0, 1);
                rd(e, "diffuseTransmissionColorFactor", r.diffuse_transmission_color, 3);
            }
            if(const jv *e = ext->get("KHR_materials_volume"))
            {
                // attenuation colour / distance (absent distance: infinite, no medium); the
                // thickness factor drives no part of the path tracer and is not stored
                rd(e, "attenuationColor", r.attenuation_color, 3);
                r.attenuation_distance = (float)e->num("attenuationDistance", (double)r.attenuation_distance);
            }
            // KHR_materials_scatter (scatterFactor, default 0) or the older KHR_materials_volume_scatter
            // (no factor: implicitly 1): multi-scatter colour and Henyey-Greenstein anisotropy
            const jv *sc = ext->get("KHR_materials_scatter");
            const bool unified = sc != nullptr;
            if(!sc) sc = ext->get("KHR_materials_volume_scatter");
            if(sc)
            {
                rd(sc, "multiscatterColorFactor", r.scatter_color, 3);
                r.phase_g = (float)sc->num("scatterAnisotropy", 0.0);
                r.scatter_factor = (float)sc->num("scatterFactor", unified ? 0.0 : 1.0);
            }
        }
        // texture slots: glTF texture indices, resolved to NO_TEXTURE later if the image fails
        auto tex = [](const jv *info) -> uint32_t {
            const long i = info ? info->idx("index") : -1;
            return i >= 0 ? (uint32_t)i : VKG_NO_TEXTURE;
        };
        r.tex_color = tex(pbr ? pbr->get("baseColorTexture") : nullptr);
        // KHR_texture_transform of the colour texture, the one the reference keeps per entry
        // (texture_transform, gltf.cpp:162-194; RayBuilder.cpp:596-597): T(offset) R(rotation about -z)
        // S(scale) applied to (u, v, 0, 1)
        if(const jv *bct = pbr ? pbr->get("baseColorTexture") : nullptr)
            if(const jv *bx = bct->get("extensions"))
                if(const jv *tt = bx->get("KHR_texture_transform"))
                {
                    float off[2] = {0.f, 0.f}, sc[2] = {1.f, 1.f};
                    rd(tt, "offset", off, 2);
                    rd(tt, "scale", sc, 2);
                    const double rot = tt->num("rotation", 0.0), c = std::cos(rot), sn = std::sin(rot);
                    const float t6[6] = {(float)(c * sc[0]), (float)(sn * sc[1]), off[0],
                                         (float)(-sn * sc[0]), (float)(c * sc[1]), off[1]};
                    std::memcpy(r.uv_transform, t6, sizeof(t6));
                    r.has_uv_transform = 1u;
                }
        r.tex_ao_rough_metal = tex(pbr ? pbr->get("metallicRoughnessTexture") : nullptr);
        r.tex_normal = tex(m.get("normalTexture"));
        r.tex_emission = tex(m.get("emissiveTexture"));
        if(r.tex_emission != VKG_NO_TEXTURE) em[0] = em[1] = em[2] = 0.f; // the texture alone (gltf.cpp:377)
        if(ext && ext->kind == jv::OBJ)
        {
            if(const jv *e = ext->get("KHR_materials_transmission")) r.tex_transmission = tex(e->get("transmissionTexture"));
            if(const jv *e = ext->get("KHR_materials_diffuse_transmission"))
            {
                r.tex_diffuse_transmission = tex(e->get("diffuseTransmissionTexture"));
                r.tex_diffuse_transmission_color = tex(e->get("diffuseTransmissionColorTexture"));
            }
        }
        for(int c = 0; c < 3; ++c) r.emission[c] = em[c] * strength;
        const jv *ds = m.get("doubleSided");
        r.twosided = ds && ds->kind == jv::BOOL && ds->b ? 1u : 0u;
        if(r.transmission > 0.f && !(r.ior > 0.f)) r.ior = 1.5f;
        return r;
    }

    bool run(vkg_gltf &G)
    {
        // materials
        if(const auto *ms = doc.arr("materials"))
            for(const jv &m: *ms) G.materials.push_back(material(m));
        if(G.materials.empty())
        {
            vkg_material d;
            vkg_material_defaults(&d);
            G.materials.push_back(d);
        }
        if(!textures(G)) return false;
        // material slots of missing or undecoded textures stay empty
        for(vkg_material &m: G.materials)
            for(uint32_t *slot: {&m.tex_color, &m.tex_normal, &m.tex_emission, &m.tex_ao_rough_metal, &m.tex_transmission,
                                 &m.tex_diffuse_transmission, &m.tex_diffuse_transmission_color})
                if(*slot != VKG_NO_TEXTURE && (*slot >= G.textures.size() || G.textures[*slot].rgba.empty()))
                    *slot = VKG_NO_TEXTURE;
        // meshes: one per triangle primitive
        const auto *meshes = doc.arr("meshes");
        std::vector<std::vector<std::pair<uint32_t, uint32_t>>> prim_of(meshes ? meshes->size() : 0); // (mesh, material)
        for(size_t mi = 0; meshes && mi < meshes->size(); ++mi)
        {
            const auto *prims = (*meshes)[mi].arr("primitives");
            for(size_t pi = 0; prims && pi < prims->size(); ++pi)
            {
                const jv &pr = (*prims)[pi];
                if((long)pr.num("mode", 4) != 4)
                {
                    ++G.skipped_primitives;
                    continue;
                }
                const jv *attr = pr.get("attributes");
                const long pos = attr ? attr->idx("POSITION") : -1;
                if(pos < 0) return fail("mesh %zu primitive %zu has no POSITION", mi, pi);
                std::vector<double> p, ix;
                int comps = 0;
                if(!accessor(pos, "POSITION", p, comps, true)) return false;
                if(comps != 3) return fail("mesh %zu primitive %zu: POSITION is not VEC3", mi, pi);
                mesh_t M;
                M.xyz.assign(p.begin(), p.end());
                const size_t nv = p.size() / 3;
                // vertex normals (the reference's loader reads them into its vertices, gltf.cpp:
                // NORMAL -> Vertex::normal) for smooth shading
                if(const long na = attr->idx("NORMAL"); na >= 0)
                {
                    std::vector<double> nn;
                    int nc = 0;
                    if(!accessor(na, "NORMAL", nn, nc, true)) return false;
                    if(nc != 3 || nn.size() != p.size())
                        return fail("mesh %zu primitive %zu: NORMAL is not VEC3 per vertex", mi, pi);
                    M.nrm.assign(nn.begin(), nn.end());
                }
                if(const long ta = attr->idx("TEXCOORD_0"); ta >= 0)
                {
                    std::vector<double> tt;
                    int tc = 0;
                    if(!accessor(ta, "TEXCOORD_0", tt, tc, true, true)) return false;
                    if(tc != 2 || tt.size() != nv * 2)
                        return fail("mesh %zu primitive %zu: TEXCOORD_0 is not VEC2 per vertex", mi, pi);
                    M.uv.assign(tt.begin(), tt.end());
                }
                if(const long ga = attr->idx("TANGENT"); ga >= 0)
                {
                    std::vector<double> gg;
                    int gc = 0;
                    if(!accessor(ga, "TANGENT", gg, gc, true)) return false;
                    if(gc != 4 || gg.size() != nv * 4)
                        return fail("mesh %zu primitive %zu: TANGENT is not VEC4 per vertex", mi, pi);
                    M.tng.resize(nv * 3);
                    for(size_t k = 0; k < nv; ++k)
                        for(int c = 0; c < 3; ++c) M.tng[3 * k + c] = (float)gg[4 * k + c];
                }
                const long ia = pr.idx("indices");
                if(ia >= 0)
                {
                    int ic = 0;
                    if(!accessor(ia, "indices", ix, ic, false)) return false;
                    if(ic != 1) return fail("mesh %zu primitive %zu: indices are not SCALAR", mi, pi);
                }
                else
                {
                    ix.resize(nv);
                    for(size_t k = 0; k < nv; ++k) ix[k] = (double)k;
                }
                if(ix.size() % 3) return fail("mesh %zu primitive %zu: index count not a multiple of 3", mi, pi);
                for(double v: ix)
                    if(v >= (double)nv) return fail("mesh %zu primitive %zu: index %g out of range", mi, pi, v);
                M.idx.assign(ix.begin(), ix.end());
                if(M.tng.empty() && !M.uv.empty() && !M.nrm.empty()) compute_tangents(M);
                long mat = pr.idx("material");
                if(mat < 0 || (size_t)mat >= G.materials.size()) mat = 0;
                prim_of[mi].push_back({(uint32_t)G.meshes.size(), (uint32_t)mat});
                G.meshes.push_back(std::move(M));
            }
        }
        // light assets (KHR_lights_punctual)
        struct light_asset
        {
            uint32_t type;
            float color[3], intensity, range, inner, outer;
        };
        std::vector<light_asset> lassets;
        if(const jv *ext = doc.get("extensions"))
            if(const jv *lp = ext->get("KHR_lights_punctual"))
                if(const auto *ls = lp->arr("lights"))
                    for(const jv &l: *ls)
                    {
                        light_asset a{};
                        const std::string *t = l.str("type");
                        a.type = t && *t == "spot" ? VKG_LIGHT_SPOT : t && *t == "directional" ? VKG_LIGHT_DIRECTIONAL
                                                                                                : VKG_LIGHT_OMNI;
                        a.color[0] = a.color[1] = a.color[2] = 1.f;
                        if(const auto *c = l.arr("color"); c && c->size() == 3)
                            for(int k = 0; k < 3; ++k) a.color[k] = (float)(*c)[(size_t)k].n;
                        a.intensity = (float)l.num("intensity", 1.0);
                        const double r = l.num("range", 0.0);
                        a.range = r > 0 ? (float)r : std::numeric_limits<float>::infinity();
                        const jv *spot = l.get("spot");
                        a.inner = spot ? (float)spot->num("innerConeAngle", 0.0) : 0.f;
                        a.outer = spot ? (float)spot->num("outerConeAngle", 0.7853981633974483) : 0.7853981633974483f;
                        lassets.push_back(a);
                    }
        // the scene's nodes, breadth first
        const auto *nodes = doc.arr("nodes");
        const size_t nn = nodes ? nodes->size() : 0;
        std::vector<long> roots;
        const auto *scenes = doc.arr("scenes");
        long si = doc.idx("scene");
        if(scenes && !scenes->empty())
        {
            if(si < 0 || (size_t)si >= scenes->size()) si = 0;
            if(const auto *rn = (*scenes)[(size_t)si].arr("nodes"))
                for(const jv &r: *rn) roots.push_back(r.kind == jv::NUM ? (long)r.n : -1);
        }
        else
        {
            std::vector<char> child(nn, 0);
            for(size_t i = 0; i < nn; ++i)
                if(const auto *ch = (*nodes)[i].arr("children"))
                    for(const jv &c: *ch)
                        if(c.kind == jv::NUM && c.n >= 0 && (size_t)c.n < nn) child[(size_t)c.n] = 1;
            for(size_t i = 0; i < nn; ++i)
                if(!child[i]) roots.push_back((long)i);
        }
        struct item
        {
            long node;
            double world[16];
            int depth;
        };
        std::deque<item> q;
        const double I[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
        for(long r: roots)
        {
            item it{r, {}, 0};
            std::memcpy(it.world, I, sizeof(I));
            q.push_back(it);
        }
        size_t visits = 0;
        while(!q.empty())
        {
            item it = q.front();
            q.pop_front();
            if(it.node < 0 || (size_t)it.node >= nn) continue;
            if(it.depth > 1000 || ++visits > 100000000) return fail("node hierarchy too deep or cyclic");
            const jv &node = (*nodes)[(size_t)it.node];
            double L[16], W[16];
            local_matrix(node, L);
            mat_mul(it.world, L, W);
            const long mesh = node.idx("mesh");
            if(mesh >= 0 && (size_t)mesh < prim_of.size())
                for(const auto &pm: prim_of[(size_t)mesh])
                {
                    vkg_instance inst{};
                    for(int r = 0; r < 3; ++r)
                        for(int c = 0; c < 4; ++c) inst.transform[r * 4 + c] = (float)W[c * 4 + r];
                    inst.blas = pm.first;
                    inst.material = pm.second;
                    G.instances.push_back(inst);
                }
            if(const jv *ext = node.get("extensions"))
                if(const jv *lp = ext->get("KHR_lights_punctual"))
                {
                    const long li = lp->idx("light");
                    if(li >= 0 && (size_t)li < lassets.size())
                    {
                        const light_asset &a = lassets[(size_t)li];
                        // the node's rotation: its world matrix's columns normalised
                        float rot[9];
                        for(int c = 0; c < 3; ++c)
                        {
                            const double len = std::sqrt(W[c * 4] * W[c * 4] + W[c * 4 + 1] * W[c * 4 + 1] +
                                                         W[c * 4 + 2] * W[c * 4 + 2]);
                            for(int r = 0; r < 3; ++r) rot[r * 3 + c] = (float)(len > 0 ? W[c * 4 + r] / len : (r == c));
                        }
                        const float tr[3] = {(float)W[12], (float)W[13], (float)W[14]};
                        vkg_light_source src{a.type, {a.color[0], a.color[1], a.color[2]}, a.intensity, a.range,
                                             a.inner, a.outer, {1.f, 1.f}};
                        vkg_light l;
                        vkg_light_convert(&src, rot, tr, &l);
                        G.lights.push_back(l);
                    }
                }
            if(const auto *ch = node.arr("children"))
                for(const jv &c: *ch)
                {
                    item nx{c.kind == jv::NUM ? (long)c.n : -1, {}, it.depth + 1};
                    std::memcpy(nx.world, W, sizeof(W));
                    q.push_back(nx);
                }
        }
        return true;
    }
};

}// namespace

extern "C" {

vkg_status vkg_gltf_load(const char *path, vkg_gltf **out, char *err, size_t err_len)
{
    if(err && err_len) err[0] = 0;
    if(!path || !out) return VKG_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    loader L;
    auto *G = new vkg_gltf();
    if(!L.load(path) || !L.run(*G))
    {
        if(err && err_len) std::snprintf(err, err_len, "%s", L.err.c_str());
        delete G;
        return VKG_ERR_INVALID_ARGUMENT;
    }
    *out = G;
    return VKG_OK;
}

vkg_status vkg_gltf_counts_get(const vkg_gltf *g, vkg_gltf_counts *out)
{
    if(!g || !out) return VKG_ERR_INVALID_ARGUMENT;
    *out = vkg_gltf_counts{};
    out->num_meshes = (uint32_t)g->meshes.size();
    out->num_instances = (uint32_t)g->instances.size();
    out->num_materials = (uint32_t)g->materials.size();
    out->num_lights = (uint32_t)g->lights.size();
    out->skipped_primitives = g->skipped_primitives;
    out->num_textures = (uint32_t)g->textures.size();
    out->skipped_textures = g->skipped_textures;
    return VKG_OK;
}

vkg_status vkg_gltf_mesh(const vkg_gltf *g, uint32_t i, const float **xyz, uint32_t *num_vertices,
                         const uint32_t **indices, uint32_t *num_tris)
{
    if(!g || i >= g->meshes.size() || !xyz || !num_vertices || !indices || !num_tris) return VKG_ERR_INVALID_ARGUMENT;
    const auto &M = g->meshes[i];
    *xyz = M.xyz.data();
    *num_vertices = (uint32_t)(M.xyz.size() / 3);
    *indices = M.idx.data();
    *num_tris = (uint32_t)(M.idx.size() / 3);
    return VKG_OK;
}

vkg_status vkg_gltf_mesh_texcoords(const vkg_gltf *g, uint32_t i, const float **uv)
{
    if(!g || i >= g->meshes.size() || !uv) return VKG_ERR_INVALID_ARGUMENT;
    *uv = g->meshes[i].uv.empty() ? nullptr : g->meshes[i].uv.data();
    return VKG_OK;
}

vkg_status vkg_gltf_mesh_tangents(const vkg_gltf *g, uint32_t i, const float **tangents)
{
    if(!g || i >= g->meshes.size() || !tangents) return VKG_ERR_INVALID_ARGUMENT;
    *tangents = g->meshes[i].tng.empty() ? nullptr : g->meshes[i].tng.data();
    return VKG_OK;
}

vkg_status vkg_gltf_textures(const vkg_gltf *g, vkg_texture_desc *out)
{
    if(!g || (!out && !g->textures.empty())) return VKG_ERR_INVALID_ARGUMENT;
    for(size_t i = 0; i < g->textures.size(); ++i)
    {
        const texture_t &T = g->textures[i];
        // an undecoded image: a 1 x 1 white texture keeps the indices aligned (no material uses it)
        static const uint8_t white[4] = {255, 255, 255, 255};
        out[i] = vkg_texture_desc{T.rgba.empty() ? white : T.rgba.data(), T.rgba.empty() ? 1u : T.width,
                                  T.rgba.empty() ? 1u : T.height, T.wrap_s, T.wrap_t};
    }
    return VKG_OK;
}

vkg_status vkg_gltf_mesh_normals(const vkg_gltf *g, uint32_t i, const float **normals)
{
    if(!g || i >= g->meshes.size() || !normals) return VKG_ERR_INVALID_ARGUMENT;
    const auto &M = g->meshes[i];
    *normals = M.nrm.empty() ? nullptr : M.nrm.data();
    return VKG_OK;
}

vkg_status vkg_gltf_instances(const vkg_gltf *g, vkg_instance *out)
{
    if(!g || (!out && !g->instances.empty())) return VKG_ERR_INVALID_ARGUMENT;
    if(!g->instances.empty()) std::memcpy(out, g->instances.data(), g->instances.size() * sizeof(vkg_instance));
    return VKG_OK;
}

vkg_status vkg_gltf_materials(const vkg_gltf *g, vkg_material *out)
{
    if(!g || !out) return VKG_ERR_INVALID_ARGUMENT;
    std::memcpy(out, g->materials.data(), g->materials.size() * sizeof(vkg_material));
    return VKG_OK;
}

vkg_status vkg_gltf_lights(const vkg_gltf *g, vkg_light *out)
{
    if(!g || (!out && !g->lights.empty())) return VKG_ERR_INVALID_ARGUMENT;
    if(!g->lights.empty()) std::memcpy(out, g->lights.data(), g->lights.size() * sizeof(vkg_light));
    return VKG_OK;
}

vkg_status vkg_gltf_destroy(vkg_gltf *g)
{
    delete g;
    return VKG_OK;
}

}// extern "C"
