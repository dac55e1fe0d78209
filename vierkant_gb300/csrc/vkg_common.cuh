// Shared host/device building blocks of libvkg: exactly-rounded float helpers, PCG32, the
// reference's shader RNG pair, the Moeller-Trumbore triangle test and the 8-wide node layout.
//
// Bit-exactness rule: everything that feeds a value compared bit-for-bit with the CPU reference
// (ray generation, triangle tests, Morton codes, quantised boxes) goes through the VKG_* helpers,
// which map to the round-to-nearest intrinsics on the device (never contracted into FMA) and to
// plain operators on the host (the library is compiled with -ffp-contract=off).
#pragma once

#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define VKG_HD __host__ __device__ __forceinline__
#else
#define VKG_HD inline
#endif

namespace vkg
{

#if defined(__CUDA_ARCH__)
VKG_HD float fmul(float a, float b) { return __fmul_rn(a, b); }
VKG_HD float fadd(float a, float b) { return __fadd_rn(a, b); }
VKG_HD float fsub(float a, float b) { return __fsub_rn(a, b); }
VKG_HD float fdiv(float a, float b) { return __fdiv_rn(a, b); }
VKG_HD float frcp(float a) { return __frcp_rn(a); }
VKG_HD float fsqrt(float a) { return __fsqrt_rn(a); }
VKG_HD uint32_t f2u(float f) { return __float_as_uint(f); }
VKG_HD float u2f(uint32_t u) { return __uint_as_float(u); }
#else
VKG_HD float fmul(float a, float b) { return a * b; }
VKG_HD float fadd(float a, float b) { return a + b; }
VKG_HD float fsub(float a, float b) { return a - b; }
VKG_HD float fdiv(float a, float b) { return a / b; }
VKG_HD float frcp(float a) { return 1.0f / a; }
VKG_HD float fsqrt(float a) { return __builtin_sqrtf(a); }
VKG_HD uint32_t f2u(float f)
{
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
}
VKG_HD float u2f(uint32_t u)
{
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}
#endif

// glm-order dot / cross (left-to-right sums; see intersection.cpp call sites)
VKG_HD float dot3(float ax, float ay, float az, float bx, float by, float bz)
{
    return fadd(fadd(fmul(ax, bx), fmul(ay, by)), fmul(az, bz));
}

// ---- PCG32 (O'Neill 2014: XSH-RR output, 64-bit LCG state, odd stream increment) ------------
constexpr uint64_t PCG_MULT = 6364136223846793005ull;

struct pcg32
{
    uint64_t state, inc;
};

VKG_HD uint32_t pcg32_next(pcg32 &g)
{
    uint64_t old = g.state;
    g.state = old * PCG_MULT + g.inc;
    uint32_t xs = static_cast<uint32_t>(((old >> 18u) ^ old) >> 27u);
    uint32_t rot = static_cast<uint32_t>(old >> 59u);
    return (xs >> rot) | (xs << ((0u - rot) & 31u));
}

VKG_HD pcg32 pcg32_seed(uint64_t initstate, uint64_t initseq)
{
    pcg32 g{0u, (initseq << 1u) | 1u};
    pcg32_next(g);
    g.state += initstate;
    pcg32_next(g);
    return g;
}

// jump ahead by `delta` draws in O(log delta) (Brown 1994, arbitrary-stride LCG skipping)
VKG_HD void pcg32_advance(pcg32 &g, uint64_t delta)
{
    uint64_t cur_mult = PCG_MULT, cur_plus = g.inc, acc_mult = 1u, acc_plus = 0u;
    while(delta > 0)
    {
        if(delta & 1u)
        {
            acc_mult *= cur_mult;
            acc_plus = acc_plus * cur_mult + cur_plus;
        }
        cur_plus = (cur_mult + 1u) * cur_plus;
        cur_mult *= cur_mult;
        delta >>= 1u;
    }
    g.state = acc_mult * g.state + acc_plus;
}

// uniform float in [0, 1): top 24 bits times 2^-24 (exact)
VKG_HD float u01(uint32_t x) { return static_cast<float>(x >> 8) * 5.9604644775390625e-8f; }

// ---- reference shader RNG: hash.slang:47-56, random.slang:27-36 ----------------------------
VKG_HD uint32_t xxhash32(uint32_t lhs, uint32_t rhs)
{
    const uint32_t P2 = 2246822519u, P3 = 3266489917u, P4 = 668265263u, P5 = 374761393u;
    uint32_t h = lhs + P5 + rhs * P3;
    h = P4 * ((h << 17) | (h >> (32 - 17)));
    h = P2 * (h ^ (h >> 15));
    h = P3 * (h ^ (h >> 13));
    return h ^ (h >> 16);
}

VKG_HD uint32_t lcg(uint32_t &prev)
{
    prev = 1664525u * prev + 1013904223u;
    return prev & 0x00FFFFFFu;
}

VKG_HD float rnd(uint32_t &prev) { return static_cast<float>(lcg(prev)) / static_cast<float>(0x01000000); }

// ---- Moeller-Trumbore, op for op as src/intersection.cpp:114-129 -------------------------
// (v0, e1 = v1 - v0, e2 = v2 - v0 precomputed with the same subtraction). Returns 1 on
// INTERSECT. cull != 0 additionally rejects det < 0 (clockwise seen from the ray origin).
VKG_HD int tri_test(float v0x, float v0y, float v0z, float e1x, float e1y, float e1z, float e2x, float e2y, float e2z,
                    float ox, float oy, float oz, float dx, float dy, float dz, int cull, float &t, float &u, float &v)
{
    // pvec = cross(d, e2)
    float px = fsub(fmul(dy, e2z), fmul(e2y, dz));
    float py = fsub(fmul(dz, e2x), fmul(e2z, dx));
    float pz = fsub(fmul(dx, e2y), fmul(e2x, dy));
    float det = dot3(e1x, e1y, e1z, px, py, pz);
    const float eps = 10.0e-10f;
    if(det > -eps && det < eps) return 0;
    if(cull && det < 0.f) return 0;
    float inv_det = frcp(det);
    float tx = fsub(ox, v0x), ty = fsub(oy, v0y), tz = fsub(oz, v0z);
    float uu = fmul(inv_det, dot3(tx, ty, tz, px, py, pz));
    if(uu < 0.0f || uu > 1.0f) return 0;
    // qvec = cross(tvec, e1)
    float qx = fsub(fmul(ty, e1z), fmul(e1y, tz));
    float qy = fsub(fmul(tz, e1x), fmul(e1z, tx));
    float qz = fsub(fmul(tx, e1y), fmul(e1x, ty));
    float vv = fmul(dot3(dx, dy, dz, qx, qy, qz), inv_det);
    if(vv < 0.0f || fadd(uu, vv) > 1.0f) return 0;
    t = fmul(dot3(e2x, e2y, e2z, qx, qy, qz), inv_det);
    u = uu;
    v = vv;
    return 1;
}

// ---- 8-wide node (96 B = 6 x 16 B) ------------------------------------------------------
//   [0]  origin.xyz (fp32), exps[3] (2^(e-127) scales), nchild
//   [16] qlo x[8], qlo y[8]   [32] qlo z[8], qhi x[8]   [48] qhi y[8], qhi z[8]
//   [64] child[8]: internal -> node index; leaf -> 0x80000000 | (count-1) << 27 | first triangle
struct alignas(16) node8
{
    float origin[3];
    uint8_t exps[3];
    uint8_t nchild;
    uint8_t qlo[3][8];
    uint8_t qhi[3][8];
    uint32_t child[8];
};
static_assert(sizeof(node8) == 96, "node8 must be 96 bytes");

// triangle record (48 B = 3 x 16 B): v0.xyz, e1.xyz, e2.xyz, triangle id, 2 pad words
struct alignas(16) tri_rec
{
    float v[9];
    uint32_t prim;
    uint32_t pad[2];
};
static_assert(sizeof(tri_rec) == 48, "tri_rec must be 48 bytes");

constexpr uint32_t LEAF_BIT = 0x80000000u;
constexpr uint32_t LEAF_MAX_LIMIT = 16;
constexpr uint32_t MAX_TRIS = 1u << 27;

VKG_HD float exp_scale(uint32_t e) { return u2f(e << 23); }

VKG_HD uint32_t expand10(uint32_t v)
{
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

}// namespace vkg
