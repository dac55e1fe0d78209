// Two-level traversal: the top-level 8-wide BVH over instance boxes, and at every instance leaf the
// ray in that instance's object space through its BLAS (traverse.cuh). The world -> object move is
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

// smallest float above a finite positive t (the BLAS accepts t < tmax strictly, so equal-t hits in a
// later instance stay visible for the tie rule)
__device__ __forceinline__ float next_up(float t) { return __uint_as_float(__float_as_uint(t) + 1u); }

template<bool ANY>
__device__ __forceinline__ tlas_result trace_tlas(const node8 *__restrict__ tnodes, const inst_rec *__restrict__ inst,
                                                  const blas_ref *__restrict__ blas, float ox, float oy, float oz,
                                                  float tmin, float dx, float dy, float dz, float tmax, int cull)
{
    tlas_result R{VKG_MISS, VKG_MISS, 0.f, 0.f, 0.f, false};
    const float ix = safe_rcp(dx), iy = safe_rcp(dy), iz = safe_rcp(dz);
    uint32_t st_node[TLAS_STACK];
    float st_t[TLAS_STACK];
    int sp = 1;
    st_node[0] = 0;
    st_t[0] = tmin;
    float best_t = tmax;
    while(sp > 0)
    {
        --sp;
        const uint32_t ni = st_node[sp];
        if(st_t[sp] > best_t) continue;
        uint32_t key[8];
        uint4 w4, w5;
        node_keys(tnodes, ni, ox, oy, oz, ix, iy, iz, tmin, best_t, key, w4, w5);
        sort8(key);
#pragma unroll 1
        for(int h = 0; h < 8; ++h)
        {
            if(key[h] == 0xFFFFFFFFu) break;
            const uint32_t k = key[h] & 7u;
            const uint32_t c = (k & 4u) ? sel4(w5, k & 3u) : sel4(w4, k & 3u);
            if(!(c & LEAF_BIT)) continue;
            if(tdec(key[h] & ~7u) > best_t) continue;
            const uint32_t start = c & 0x07FFFFFFu, cnt = ((c >> 27) & 0xFu) + 1u;
            for(uint32_t ii = start; ii < start + cnt; ++ii)
            {
                const float4 *mp = reinterpret_cast<const float4 *>(inst + ii);
                const float4 m[3] = {__ldg(mp), __ldg(mp + 1), __ldg(mp + 2)};
                const uint4 meta = __ldg(reinterpret_cast<const uint4 *>(mp + 6));
                const blas_ref B = blas[meta.x];
                if(B.num_tris == 0) continue;
                float o[3], d[3];
                to_object(m, ox, oy, oz, dx, dy, dz, o, d);
                unsigned long long v = 0, t = 0;
                // before the first hit the interval is (tmin, tmax); after it (tmin, best_t] so that equal-t hits
                // of this instance still reach the tie rule
                const float tb = (ANY || R.prim == VKG_MISS) ? tmax : next_up(best_t);
                const trace_result r = trace_ray<ANY, false>(B.nodes, B.tris, o[0], o[1], o[2], tmin, d[0], d[1], d[2],
                                                             tb, cull, v, t, nullptr);
                if(ANY)
                {
                    if(r.occluded)
                    {
                        R.occluded = true;
                        return R;
                    }
                }
                else if(r.prim != VKG_MISS &&
                        (R.prim == VKG_MISS || r.t < best_t ||
                         (r.t == best_t && (meta.y < R.inst || (meta.y == R.inst && r.prim < R.prim)))))
                {
                    best_t = r.t;
                    R.prim = r.prim;
                    R.inst = meta.y;
                    R.u = r.u;
                    R.v = r.v;
                }
            }
        }
#pragma unroll
        for(int h = 7; h >= 0; --h)
        {
            if(key[h] == 0xFFFFFFFFu) continue;
            const uint32_t k = key[h] & 7u;
            const uint32_t c = (k & 4u) ? sel4(w5, k & 3u) : sel4(w4, k & 3u);
            if(c & LEAF_BIT) continue;
            if(sp < (int)TLAS_STACK)
            {
                st_node[sp] = c;
                st_t[sp] = tdec(key[h] & ~7u);
                ++sp;
            }
        }
    }
    R.t = R.prim == VKG_MISS ? 0.f : best_t;
    return R;
}

}// namespace vkg
