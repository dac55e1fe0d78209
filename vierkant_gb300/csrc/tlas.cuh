// Two-level traversal: the top-level 8-wide BVH over instance boxes, and at every instance the ray in
// that instance's object space through its BLAS (the node test of traverse.cuh at both levels). The world -> object move is
// done row by row with separately rounded products and sums (x, y, z terms left to right,
// translation last), so a CPU restatement reproduces the object-space ray bit for bit. The direction
// is not renormalised, so object-space t equals world-space t.
#pragma once

#include "traverse.cuh"

namespace vkg
{

struct tlas_result
{
    uint32_t prim, inst;
    float t, u, v;
    bool occluded;
};

__device__ __forceinline__ void to_object(const float4 (&m)[3], float ox, float oy, float oz, float dx, float dy,
                                          float dz, float (&o)[3], float (&d)[3])
{
#pragma unroll
    for(int r = 0; r < 3; ++r)
    {
        const float4 w = m[r];
        o[r] = fadd(fadd(fadd(fmul(w.x, ox), fmul(w.y, oy)), fmul(w.z, oz)), w.w);
        d[r] = fadd(fadd(fmul(w.x, dx), fmul(w.y, dy)), fmul(w.z, dz));
    }
}


// One stack for both levels. Entries are top-level nodes, instance entries (INST_BIT | instance
// record) or, above a RETURN sentinel, BLAS nodes of the instance being traversed. Each step
// processes one node of either level, so the lanes of a warp stay in step whichever level they are
// in: entering an instance pushes RETURN and the BLAS root and switches the ray to object space;
// popping RETURN switches back to the world ray and the top level.
constexpr uint32_t TL_STACK = TLAS_STACK + TRAVERSAL_STACK + 1;
constexpr uint32_t INST_BIT = 0x80000000u, TL_RETURN = 0xFFFFFFFFu;

struct tl_state
{
    float wo[3], wd[3], wi[3]; // world ray and reciprocal direction
    float o[3], d[3], inv[3];  // current ray (world or object space)
    float tmin, tmax, best_t, bu, bv;
    uint32_t best_prim, best_inst, cur_inst;
    const node8 *nodes;
    const tri_rec *tris;
    int sp;
    bool in_blas, done;
    bool cur_alpha; // the current instance's material is tested by the candidate filter
    uint2 *st; // uint2[TL_STACK] {entry, entry distance (float bits)}, a separate local array so that
               // the fields stay in registers (see ray_state_t)
};

__device__ __forceinline__ void tl_init(tl_state &s, const node8 *tnodes, float ox, float oy, float oz, float tmin,
                                        float dx, float dy, float dz, float tmax)
{
    s.wo[0] = s.o[0] = ox;
    s.wo[1] = s.o[1] = oy;
    s.wo[2] = s.o[2] = oz;
    s.wd[0] = s.d[0] = dx;
    s.wd[1] = s.d[1] = dy;
    s.wd[2] = s.d[2] = dz;
    s.wi[0] = s.inv[0] = safe_rcp(dx);
    s.wi[1] = s.inv[1] = safe_rcp(dy);
    s.wi[2] = s.inv[2] = safe_rcp(dz);
    s.tmin = tmin;
    s.tmax = tmax;
    s.best_t = tmax;
    s.bu = s.bv = 0.f;
    s.best_prim = s.best_inst = VKG_MISS;
    s.cur_inst = VKG_MISS;
    s.nodes = tnodes;
    s.tris = nullptr;
    s.in_blas = false;
    s.done = false;
    s.cur_alpha = false;
    s.sp = 1;
    s.st[0] = make_uint2(0u, __float_as_uint(tmin));
}

// one node of the two-level traversal; false once the ray is finished. f: the candidate filter
// (no_filter, traverse.cuh), asked per instance whether its material is tested. POS: the ray's tmin
// is >= +0 (key_pos): the child keys are the entry distances' float bits
template<bool ANY, class F = no_filter, bool POS = false>
__device__ __forceinline__ bool tl_step(tl_state &s, const node8 *__restrict__ tnodes, const inst_rec *__restrict__ inst,
                                        const blas_ref *__restrict__ blas, int cull, const F &f = F())
{
    while(s.sp > 0 && !s.done)
    {
        --s.sp;
        const uint2 ent = s.st[s.sp];
        const uint32_t e = ent.x;
        if(e == TL_RETURN)
        {
            for(int a = 0; a < 3; ++a)
            {
                s.o[a] = s.wo[a];
                s.d[a] = s.wd[a];
                s.inv[a] = s.wi[a];
            }
            s.nodes = tnodes;
            s.in_blas = false;
            continue;
        }
        if(__uint_as_float(ent.y) > s.best_t) continue;
        if(!s.in_blas && (e & INST_BIT))
        {
            // enter an instance: object-space ray, RETURN marker, BLAS root
            const float4 *mp = reinterpret_cast<const float4 *>(inst + (e & ~INST_BIT));
            const uint4 meta = __ldg(reinterpret_cast<const uint4 *>(mp + 6));
            const blas_ref B = blas[meta.x];
            if(B.num_tris == 0 || s.sp + 2 > (int)TL_STACK) continue;
            const float4 m[3] = {__ldg(mp), __ldg(mp + 1), __ldg(mp + 2)};
            to_object(m, s.wo[0], s.wo[1], s.wo[2], s.wd[0], s.wd[1], s.wd[2], s.o, s.d);
            for(int a = 0; a < 3; ++a) s.inv[a] = safe_rcp(s.d[a]);
            s.nodes = B.nodes;
            s.tris = B.tris;
            s.cur_inst = meta.y;
            if(F::active) s.cur_alpha = f.tests_material(meta.z);
            s.in_blas = true;
            s.st[s.sp] = make_uint2(TL_RETURN, __float_as_uint(s.tmin));
            s.st[s.sp + 1] = make_uint2(0u, __float_as_uint(s.tmin));
            s.sp += 2;
            continue;
        }
        uint32_t key[8];
        uint4 w4, w5;
        node_keys<false, POS>(s.nodes, e, s.o[0], s.o[1], s.o[2], s.inv[0], s.inv[1], s.inv[2], s.tmin, s.best_t, key,
                              w4, w5);
        sort8(key);
        if(s.in_blas)
        {
            // triangle leaves at once, nearest first (as the single-level traversal)
#pragma unroll
            for(int h = 0; h < 8; ++h)
            {
                if(key[h] == 0xFFFFFFFFu || s.done) break;
                const uint32_t k = key[h] & 7u;
                const uint32_t c = (k & 4u) ? sel4(w5, k & 3u) : sel4(w4, k & 3u);
                if(!(c & LEAF_BIT)) continue;
                if(key_dist<POS>(key[h]) > s.best_t) continue;
                const uint32_t start = c & 0x07FFFFFFu, cnt = ((c >> 27) & 0xFu) + 1u;
                for(uint32_t ti = start; ti < start + cnt; ++ti)
                {
                    const float4 *tp = reinterpret_cast<const float4 *>(s.tris + ti);
                    const float4 a = __ldg(tp), b = __ldg(tp + 1), cc = __ldg(tp + 2);
                    const int tcull = cull == CULL_BACK ||
                                      (cull == CULL_BACK_UNLESS_TWOSIDED && !(__float_as_uint(cc.z) & TRI_FLAG_TWOSIDED));
                    float t, u, v;
                    if(!tri_test(a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w, cc.x, s.o[0], s.o[1], s.o[2], s.d[0], s.d[1],
                                 s.d[2], tcull, t, u, v))
                        continue;
                    if(!(t > s.tmin && t < s.tmax)) continue;
                    const uint32_t prim = __float_as_uint(cc.y);
                    const bool tested = F::active && s.cur_alpha;
                    if(ANY)
                    {
                        if(tested && !f.accept(s.cur_inst, prim, u, v)) continue;
                        s.done = true;
                        break;
                    }
                    if(s.best_prim == VKG_MISS || t < s.best_t ||
                       (t == s.best_t && (s.cur_inst < s.best_inst || (s.cur_inst == s.best_inst && prim < s.best_prim))))
                    {
                        if(tested && !f.accept(s.cur_inst, prim, u, v)) continue;
                        s.best_t = t;
                        s.best_prim = prim;
                        s.best_inst = s.cur_inst;
                        s.bu = u;
                        s.bv = v;
                    }
                }
            }
            if(s.done) break;
        }
        // push far-to-near: internal children, and at the top level the instance leaves as entries
#pragma unroll
        for(int h = 7; h >= 0; --h)
        {
            if(key[h] == 0xFFFFFFFFu) continue;
            const uint32_t k = key[h] & 7u;
            const uint32_t c = (k & 4u) ? sel4(w5, k & 3u) : sel4(w4, k & 3u);
            const float te = key_dist<POS>(key[h]);
            if(c & LEAF_BIT)
            {
                if(s.in_blas) continue;
                const uint32_t start = c & 0x07FFFFFFu, cnt = ((c >> 27) & 0xFu) + 1u;
                for(uint32_t q = cnt; q-- > 0;)
                    if(s.sp < (int)TL_STACK)
                    {
                        s.st[s.sp] = make_uint2(INST_BIT | (start + q), __float_as_uint(te));
                        ++s.sp;
                    }
                continue;
            }
            if(s.sp < (int)TL_STACK)
            {
                s.st[s.sp] = make_uint2(c, __float_as_uint(te));
                ++s.sp;
            }
        }
        return true;
    }
    return false;
}

template<bool ANY, class F = no_filter>
__device__ __forceinline__ tlas_result trace_tlas(const node8 *__restrict__ tnodes, const inst_rec *__restrict__ inst,
                                                  const blas_ref *__restrict__ blas, float ox, float oy, float oz,
                                                  float tmin, float dx, float dy, float dz, float tmax, int cull,
                                                  const F &f = F())
{
    tl_state s;
    uint2 stack[TL_STACK];
    s.st = stack;
    tl_init(s, tnodes, ox, oy, oz, tmin, dx, dy, dz, tmax);
    if(key_pos(tmin))
        while(tl_step<ANY, F, true>(s, tnodes, inst, blas, cull, f)) {}
    else
        while(tl_step<ANY, F, false>(s, tnodes, inst, blas, cull, f)) {}
    tlas_result R;
    R.occluded = s.done;
    R.prim = s.best_prim;
    R.inst = s.best_inst;
    R.t = s.best_prim == VKG_MISS ? 0.f : s.best_t;
    R.u = s.best_prim == VKG_MISS ? 0.f : s.bu;
    R.v = s.best_prim == VKG_MISS ? 0.f : s.bv;
    return R;
}

}// namespace vkg
