// Traversal core shared by the ray-query kernels (traverse.cu) and the path tracer's queue
// kernels (pathtrace.cu): one ray, 8-wide quantised BVH, closest hit or any hit.
//
// Per node: six 16-byte loads (96 B node), slab tests of all children as
// fmaf(q, 2^e * inv_d, (origin - o) * inv_d), children ordered by entry distance with an 8-key
// sorting network on 32-bit keys, leaf children intersected first (nearest first), internal
// children pushed far-to-near with their entry distance so a pop is skipped once best_t has passed
// it. Triangle test: the reference's Moeller-Trumbore (src/intersection.cpp:114-129) op for op.
// ray_step() processes one node, so a persistent kernel can refill lanes whose ray has finished.
#pragma once

#include "internal.hpp"

namespace vkg
{

// culling modes: none, all back faces (RAY_FLAG_CULL_BACK_FACING_TRIANGLES), or back faces of
// triangles whose record is not flagged two-sided (per-instance TRIANGLE_FACING_CULL_DISABLE,
// src/RayBuilder.cpp:521-522)
enum cull_mode : int
{
    CULL_NONE = 0,
    CULL_BACK = 1,
    CULL_BACK_UNLESS_TWOSIDED = 2
};
constexpr uint32_t TRI_FLAG_TWOSIDED = 1u;
constexpr uint32_t TRI_FLAG_TRANSMISSIVE = 2u; // light shadow rays pass: transmission > 0 or a null surface
constexpr uint32_t TRI_FLAG_ALPHA = 4u;        // candidate hits are tested for coverage (alpha mask / blend)

// Candidate filter of the traversal (the any-hit stage): with `active` false the test compiles away.
// Otherwise a candidate hit that would count (the nearest so far, or any for an any-hit query) on a
// triangle flagged TRI_FLAG_ALPHA (single level), or inside an instance whose material
// tests_material() (two levels), counts only if accept(instance, triangle, u, v) says so. The
// filter's answer depends on the candidate alone, never on the order candidates are met in.
struct no_filter
{
    static constexpr bool active = false;
    __device__ __forceinline__ bool accept(uint32_t, uint32_t, float, float) const { return true; }
    __device__ __forceinline__ bool tests_material(uint32_t) const { return false; }
};

struct trace_result
{
    uint32_t prim;
    float t, u, v;
    bool occluded;
};

__device__ __forceinline__ uint32_t tenc(float f)
{
    uint32_t b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float tdec(uint32_t u)
{
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u);
}

// Child keys: an entry distance as an ordered 32-bit key with its low 3 bits replaced by the slot.
// For a ray with tmin >= +0 every entry distance is >= +0, whose float bits order like the values:
// the key is the bits with the sign cleared (so -0 and +0 agree). Other rays use tenc / tdec.
template<bool POS>
__device__ __forceinline__ uint32_t child_key(float tn, uint32_t k)
{
    return POS ? ((__float_as_uint(tn) & 0x7FFFFFF8u) | k) : ((tenc(tn) & ~7u) | k);
}
template<bool POS>
__device__ __forceinline__ float key_dist(uint32_t key)
{
    return POS ? __uint_as_float(key & 0x7FFFFFF8u) : tdec(key & ~7u);
}
// the key mode of a ray: its tmin's sign bit clear
__device__ __forceinline__ bool key_pos(float tmin) { return !(__float_as_uint(tmin) & 0x80000000u); }

__device__ __forceinline__ void cswap(uint32_t &a, uint32_t &b)
{
    const uint32_t lo = min(a, b), hi = max(a, b);
    a = lo;
    b = hi;
}

// Batcher odd-even merge network, 19 comparators
__device__ __forceinline__ void sort8(uint32_t k[8])
{
    cswap(k[0], k[1]); cswap(k[2], k[3]); cswap(k[4], k[5]); cswap(k[6], k[7]);
    cswap(k[0], k[2]); cswap(k[1], k[3]); cswap(k[4], k[6]); cswap(k[5], k[7]);
    cswap(k[1], k[2]); cswap(k[5], k[6]);
    cswap(k[0], k[4]); cswap(k[1], k[5]); cswap(k[2], k[6]); cswap(k[3], k[7]);
    cswap(k[2], k[4]); cswap(k[3], k[5]);
    cswap(k[1], k[2]); cswap(k[3], k[4]); cswap(k[5], k[6]);
}

__device__ __forceinline__ uint32_t sel4(const uint4 &w, uint32_t j)
{
    uint32_t a = (j & 1u) ? w.y : w.x;
    uint32_t b = (j & 1u) ? w.w : w.z;
    return (j & 2u) ? b : a;
}

__device__ __forceinline__ float safe_rcp(float d)
{
    float dd = fabsf(d) < 1e-20f ? copysignf(1e-20f, d) : d;
    return __frcp_rn(dd);
}

__device__ __forceinline__ float qbyte(uint32_t w, int k) { return (float)((w >> (8 * (k & 3))) & 0xFFu); }



// per-ray traversal state. The stack (STACK entries) is a separate local-memory array the state
// points to: a struct that holds the array itself is placed in local memory as a whole, fields
// included, and every field access then costs a local-memory access; with the array outside, the
// fields stay in registers.
template<int STACK = (int)TRAVERSAL_STACK>
struct ray_state_t
{
    float ox, oy, oz, tmin, dx, dy, dz, tmax, ix, iy, iz;
    float best_t, bu, bv;
    uint32_t best;
    int sp;
    bool done;
    uint2 *st; // uint2[STACK] {node, entry distance (float bits)}: one 64-bit access per push / pop
};
using ray_state = ray_state_t<>;

template<int STACK>
__device__ __forceinline__ void ray_init(ray_state_t<STACK> &s, float ox, float oy, float oz, float tmin, float dx, float dy,
                                         float dz, float tmax)
{
    s.ox = ox;
    s.oy = oy;
    s.oz = oz;
    s.tmin = tmin;
    s.dx = dx;
    s.dy = dy;
    s.dz = dz;
    s.tmax = tmax;
    s.ix = safe_rcp(dx);
    s.iy = safe_rcp(dy);
    s.iz = safe_rcp(dz);
    s.best_t = tmax;
    s.bu = s.bv = 0.f;
    s.best = VKG_MISS;
    s.done = false;
    s.sp = 1;
    s.st[0] = make_uint2(0u, __float_as_uint(tmin));
}

// entry-distance keys of the children of node ni for a ray (origin o, reciprocal direction i,
// interval [tmin, tmax]): key = ordered entry distance with its low 3 bits replaced by the slot,
// 0xFFFFFFFF for a child the ray misses. Truncation only lowers the stored distance, so pruning with
// it stays conservative. w4 / w5 receive the node's child words.
// COUNT: also count the internal (non-leaf) children the ray hits into *n_int; POS: the key mode of a
// ray with tmin >= +0 (child_key)
template<bool COUNT = false, bool POS = false>
__device__ __forceinline__ void node_keys(const node8 *__restrict__ nodes, uint32_t ni, float ox, float oy, float oz,
                                          float ix, float iy, float iz, float tmin, float tmax, uint32_t (&key)[8],
                                          uint4 &w4, uint4 &w5, uint32_t *n_int = nullptr)
{
    uint32_t nint = 0;
    const uint4 *np = reinterpret_cast<const uint4 *>(nodes + ni);
    const uint4 w0 = __ldg(np), w1 = __ldg(np + 1), w2 = __ldg(np + 2);
    const uint4 w3 = __ldg(np + 3);
    w4 = __ldg(np + 4);
    w5 = __ldg(np + 5);
    const uint32_t meta = w0.w;
    const uint32_t nch = meta >> 24;
    const bool negx = ix < 0.f, negy = iy < 0.f, negz = iz < 0.f;
    const float tox = __fmul_rn(__fsub_rn(__uint_as_float(w0.x), ox), ix);
    const float toy = __fmul_rn(__fsub_rn(__uint_as_float(w0.y), oy), iy);
    const float toz = __fmul_rn(__fsub_rn(__uint_as_float(w0.z), oz), iz);
    const float sx = __fmul_rn(exp_scale(meta & 0xFFu), ix);
    const float sy = __fmul_rn(exp_scale((meta >> 8) & 0xFFu), iy);
    const float sz = __fmul_rn(exp_scale((meta >> 16) & 0xFFu), iz);
    const uint32_t nx0 = negx ? w2.z : w1.x, nx1 = negx ? w2.w : w1.y;
    const uint32_t fx0 = negx ? w1.x : w2.z, fx1 = negx ? w1.y : w2.w;
    const uint32_t ny0 = negy ? w3.x : w1.z, ny1 = negy ? w3.y : w1.w;
    const uint32_t fy0 = negy ? w1.z : w3.x, fy1 = negy ? w1.w : w3.y;
    const uint32_t nz0 = negz ? w3.z : w2.x, nz1 = negz ? w3.w : w2.y;
    const uint32_t fz0 = negz ? w2.x : w3.z, fz1 = negz ? w2.y : w3.w;
#pragma unroll
    for(int k = 0; k < 8; ++k)
    {
        key[k] = 0xFFFFFFFFu;
        if((uint32_t)k < nch)
        {
            const uint32_t wnx = k < 4 ? nx0 : nx1, wfx = k < 4 ? fx0 : fx1;
            const uint32_t wny = k < 4 ? ny0 : ny1, wfy = k < 4 ? fy0 : fy1;
            const uint32_t wnz = k < 4 ? nz0 : nz1, wfz = k < 4 ? fz0 : fz1;
            const float tnx = fmaf(qbyte(wnx, k), sx, tox), tfx = fmaf(qbyte(wfx, k), sx, tox);
            const float tny = fmaf(qbyte(wny, k), sy, toy), tfy = fmaf(qbyte(wfy, k), sy, toy);
            const float tnz = fmaf(qbyte(wnz, k), sz, toz), tfz = fmaf(qbyte(wfz, k), sz, toz);
            const float tn = fmaxf(fmaxf(tnx, tny), fmaxf(tnz, tmin));
            const float tf = fminf(fminf(tfx, tfy), fminf(tfz, tmax));
            if(tn <= tf)
            {
                key[k] = child_key<POS>(tn, (uint32_t)k);
                if(COUNT)
                {
                    const uint32_t c = k < 4 ? (k == 0 ? w4.x : k == 1 ? w4.y : k == 2 ? w4.z : w4.w)
                                             : (k == 4 ? w5.x : k == 5 ? w5.y : k == 6 ? w5.z : w5.w);
                    nint += (c & LEAF_BIT) ? 0u : 1u;
                }
            }
        }
    }
    if(COUNT) *n_int = nint;
}

// one node of the traversal; returns false once the ray is finished. POS: the ray's tmin is >= +0
// (key_pos); f: the candidate filter
template<bool ANY, bool STATS, int STACK, bool POS = false, class F = no_filter>
__device__ __forceinline__ bool ray_step(ray_state_t<STACK> &s, const node8 *__restrict__ nodes, const tri_rec *__restrict__ tris,
                                         int cull, unsigned long long &visits, unsigned long long &tests,
                                         unsigned long long *__restrict__ counters, const F &f = F())
{
    while(s.sp > 0 && !s.done)
    {
        --s.sp;
        const uint2 ent = s.st[s.sp];
        const uint32_t ni = ent.x;
        if(__uint_as_float(ent.y) > s.best_t) continue;
        if(STATS) ++visits;
        uint32_t key[8];
        uint4 w4, w5;
        uint32_t n_int;
        node_keys<true, POS>(nodes, ni, s.ox, s.oy, s.oz, s.ix, s.iy, s.iz, s.tmin, s.best_t, key, w4, w5, &n_int);
        sort8(key);
        // one pass over the hit children, near to far: leaves are intersected as they come, internal
        // children are written to the stack far-to-near (the r-th nearest at base + n_int - 1 - r) so
        // that the nearest is popped first -- the order two separate passes would give
        const int base = s.sp;
        int r = 0;
#pragma unroll
        for(int h = 0; h < 8; ++h)
        {
            if(key[h] == 0xFFFFFFFFu || s.done) break;
            const uint32_t k = key[h] & 7u;
            // the child word from L1 (the node's line was just read): one load instead of a select
            // over eight registers
            const uint32_t c = __ldg(&nodes[ni].child[k]);
            const float tentry = key_dist<POS>(key[h]);
            if(!(c & LEAF_BIT))
            {
                const int pos = base + (int)n_int - 1 - r;
                ++r;
                if(pos < STACK) s.st[pos] = make_uint2(c, __float_as_uint(tentry));
                else if(counters) { atomicOr(&counters[2], 1ull); }
                continue;
            }
            if(tentry > s.best_t) continue;
            const uint32_t start = c & 0x07FFFFFFu, cnt = ((c >> 27) & 0xFu) + 1u;
            for(uint32_t ti = start; ti < start + cnt; ++ti)
            {
                const float4 *tp = reinterpret_cast<const float4 *>(tris + ti);
                const float4 a = __ldg(tp), b = __ldg(tp + 1), cc = __ldg(tp + 2);
                if(STATS) ++tests;
                const int tcull = cull == CULL_BACK ||
                                  (cull == CULL_BACK_UNLESS_TWOSIDED && !(__float_as_uint(cc.z) & TRI_FLAG_TWOSIDED));
                float t, u, v;
                if(!tri_test(a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w, cc.x, s.ox, s.oy, s.oz, s.dx, s.dy, s.dz, tcull, t,
                             u, v))
                    continue;
                if(!(t > s.tmin && t < s.tmax)) continue;
                const uint32_t prim = __float_as_uint(cc.y);
                const bool tested = F::active && (__float_as_uint(cc.z) & TRI_FLAG_ALPHA);
                if(ANY)
                {
                    if(tested && !f.accept(0u, prim, u, v)) continue;
                    s.done = true;
                    break;
                }
                if(t < s.best_t || (t == s.best_t && prim < s.best))
                {
                    if(tested && !f.accept(0u, prim, u, v)) continue;
                    s.best_t = t;
                    s.best = prim;
                    s.bu = u;
                    s.bv = v;
                }
            }
        }
        if(s.done) break;
        s.sp = min(base + (int)n_int, STACK);
        return true; // one node processed
    }
    return false;
}

template<int STACK>
__device__ __forceinline__ trace_result ray_result(const ray_state_t<STACK> &s)
{
    trace_result r;
    r.occluded = s.done;
    r.prim = s.best;
    r.t = s.best == VKG_MISS ? 0.f : s.best_t;
    r.u = s.best == VKG_MISS ? 0.f : s.bu;
    r.v = s.best == VKG_MISS ? 0.f : s.bv;
    return r;
}

// transmittance of a segment (light-NEE visibility): one pass over every triangle the ray crosses in
// (tmin, tmax) (back faces culled when cull == CULL_BACK), in traversal order; false at the first
// triangle without TRI_FLAG_TRANSMISSIVE, else T is multiplied by tint(prim, t, front face) of each
// crossed transmissive triangle. A triangle that is not transmissive but flagged TRI_FLAG_ALPHA
// blocks only if the filter accepts it (transmittance_test tints transmissive candidates before it
// tests coverage, visibility_test.slang:116-152).
// Every triangle sits in one leaf and every node is visited at most once, so each crossing counts
// once; the children need no ordering.
template<int STACK, class Tint, class F = no_filter>
__device__ __forceinline__ bool trace_transmit(const node8 *__restrict__ nodes, const tri_rec *__restrict__ tris,
                                               float ox, float oy, float oz, float tmin, float dx, float dy, float dz,
                                               float tmax, int cull, float3 &T, Tint tint, const F &f = F())
{
    const float ix = safe_rcp(dx), iy = safe_rcp(dy), iz = safe_rcp(dz);
    uint32_t st[STACK];
    int sp = 1;
    st[0] = 0u;
    while(sp > 0)
    {
        const uint32_t ni = st[--sp];
        uint32_t key[8];
        uint4 w4, w5;
        node_keys(nodes, ni, ox, oy, oz, ix, iy, iz, tmin, tmax, key, w4, w5);
#pragma unroll
        for(int k = 0; k < 8; ++k)
        {
            if(key[k] == 0xFFFFFFFFu) continue;
            const uint32_t c = (k & 4) ? sel4(w5, k & 3) : sel4(w4, k & 3);
            if(!(c & LEAF_BIT))
            {
                if(sp < STACK) st[sp++] = c;
                continue;
            }
            const uint32_t start = c & 0x07FFFFFFu, cnt = ((c >> 27) & 0xFu) + 1u;
            for(uint32_t ti = start; ti < start + cnt; ++ti)
            {
                const float4 *tp = reinterpret_cast<const float4 *>(tris + ti);
                const float4 a = __ldg(tp), b = __ldg(tp + 1), cc = __ldg(tp + 2);
                float t, u, v;
                if(!tri_test(a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w, cc.x, ox, oy, oz, dx, dy, dz,
                             cull == CULL_BACK ? 1 : 0, t, u, v))
                    continue;
                if(!(t > tmin && t < tmax)) continue;
                const uint32_t fl = __float_as_uint(cc.z);
                if(!(fl & TRI_FLAG_TRANSMISSIVE))
                {
                    if(F::active && (fl & TRI_FLAG_ALPHA) && !f.accept(0u, __float_as_uint(cc.y), u, v)) continue;
                    return false;
                }
                // front face: the ray runs against the normal e1 x e2
                const float nx = b.x * cc.x - b.y * b.w, ny = b.y * b.z - a.w * cc.x, nz = a.w * b.w - b.x * b.z;
                const float3 m = tint(__float_as_uint(cc.y), t, nx * dx + ny * dy + nz * dz < 0.f);
                T.x *= m.x;
                T.y *= m.y;
                T.z *= m.z;
            }
        }
    }
    return true;
}

template<bool ANY, bool STATS, int STACK, bool POS, class F = no_filter>
__device__ __forceinline__ trace_result trace_ray_mode(const node8 *__restrict__ nodes, const tri_rec *__restrict__ tris,
                                                       float ox, float oy, float oz, float tmin, float dx, float dy,
                                                       float dz, float tmax, int cull, unsigned long long &visits,
                                                       unsigned long long &tests,
                                                       unsigned long long *__restrict__ counters, const F &f = F())
{
    ray_state_t<STACK> s;
    uint2 stack[STACK];
    s.st = stack;
    ray_init(s, ox, oy, oz, tmin, dx, dy, dz, tmax);
    while(ray_step<ANY, STATS, STACK, POS, F>(s, nodes, tris, cull, visits, tests, counters, f)) {}
    return ray_result(s);
}

// one ray, in the key mode its tmin allows
template<bool ANY, bool STATS, int STACK = (int)TRAVERSAL_STACK, class F = no_filter>
__device__ __forceinline__ trace_result trace_ray(const node8 *__restrict__ nodes, const tri_rec *__restrict__ tris,
                                                  float ox, float oy, float oz, float tmin, float dx, float dy,
                                                  float dz, float tmax, int cull,
                                                  unsigned long long &visits, unsigned long long &tests,
                                                  unsigned long long *__restrict__ counters, const F &f = F())
{
    if(key_pos(tmin))
        return trace_ray_mode<ANY, STATS, STACK, true, F>(nodes, tris, ox, oy, oz, tmin, dx, dy, dz, tmax, cull, visits,
                                                           tests, counters, f);
    return trace_ray_mode<ANY, STATS, STACK, false, F>(nodes, tris, ox, oy, oz, tmin, dx, dy, dz, tmax, cull, visits,
                                                        tests, counters, f);
}

// one node of a ray's traversal (ray_step) in the key mode its tmin allows
template<bool ANY, bool STATS, int STACK>
__device__ __forceinline__ bool ray_step_auto(ray_state_t<STACK> &s, const node8 *__restrict__ nodes,
                                              const tri_rec *__restrict__ tris, int cull, unsigned long long &visits,
                                              unsigned long long &tests, unsigned long long *__restrict__ counters)
{
    return key_pos(s.tmin) ? ray_step<ANY, STATS, STACK, true>(s, nodes, tris, cull, visits, tests, counters)
                           : ray_step<ANY, STATS, STACK, false>(s, nodes, tris, cull, visits, tests, counters);
}

}// namespace vkg
