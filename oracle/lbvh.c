/*
 * LBVH -> 8-wide quantised BVH and its traversal. TEST INFRASTRUCTURE ONLY (CPU oracle).
 *
 * The reference has no BVH of its own (its acceleration structures are driver-built Vulkan
 * BLAS/TLAS, src/RayBuilder.cpp:98-300 / :386-760), so this file is the CPU statement of the
 * project's build, step for step what the CUDA kernels do, so Morton codes, the sorted order, the
 * BVH2 topology and the final 8-wide nodes can be compared bit-for-bit:
 *
 *  1. triangle boxes; scene box = union; margin = 2^-15 * max(scene extent, max |coordinate|)
 *  2. 30-bit Morton code of the box centre, 10 bits per axis over the scene box
 *     (q = (c - min) * (1024 / extent), truncated, clamped to 1023)
 *  3. stable sort of (code, triangle id) -- equal codes keep input order
 *  4. Karras 2012 binary radix tree over the sorted codes (equal codes split by index)
 *  5. bottom-up refit (min/max, order independent)
 *  6. collapse to 8-wide nodes in breadth-first order: starting from {left, right}, repeatedly
 *     open the openable slot (internal, > leaf_max triangles) with the largest surface area
 *     (ties: lowest slot) until 8 slots; slots with <= leaf_max triangles become leaf ranges
 *  7. quantise child boxes to 8 bits against the node origin with power-of-two scales, every
 *     child box first grown by the margin (conservative: a box never rejects a triangle whose
 *     Moeller-Trumbore hit lies inside it, for ray origins within ~16 scene extents)
 *
 * Traversal (closest hit): ordered by 32-bit keys (ordered entry distance with its low 3 bits
 * replaced by the slot), leaves first, internal children pushed far-to-near with the truncated
 * entry distance; slab tests evaluated as fmaf(q, s*inv_d, (o'-o)*inv_d) exactly as the kernels do. Triangle test = intersection.cpp:114-129 on precomputed v0/e1/e2.
 */
#include "oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stdlib.h>
#include <string.h>

int orc__run_threads(void *(*fn)(void *), void *arg, int nthreads);

#define LEAF_BIT 0x80000000u

static inline uint32_t expand10(uint32_t v)
{
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

static inline int clz32(uint32_t x) { return x ? __builtin_clz(x) : 32; }

static inline int delta(const uint32_t *codes, int64_t n, int64_t i, int64_t j)
{
    if(j < 0 || j >= n) return -1;
    uint32_t a = codes[i], b = codes[j];
    if(a == b) return 32 + clz32((uint32_t)i ^ (uint32_t)j);
    return clz32(a ^ b);
}

typedef struct { uint32_t code, prim; } kv;
static int kv_cmp(const void *a, const void *b)
{
    const kv *x = (const kv *)a, *y = (const kv *)b;
    if(x->code != y->code) return x->code < y->code ? -1 : 1;
    return x->prim < y->prim ? -1 : (x->prim > y->prim);
}

typedef struct { float lo[3], hi[3]; } box3;

static inline void box_union(box3 *a, const box3 *b)
{
    for(int i = 0; i < 3; ++i)
    {
        a->lo[i] = fminf(a->lo[i], b->lo[i]);
        a->hi[i] = fmaxf(a->hi[i], b->hi[i]);
    }
}

static inline float box_area(const box3 *b)
{
    float dx = b->hi[0] - b->lo[0], dy = b->hi[1] - b->lo[1], dz = b->hi[2] - b->lo[2];
    return (dx * dy + dy * dz) + dz * dx;
}

/* decode a power-of-two scale exponent byte (127 + e) into 2^e */
static inline float exp_scale(uint8_t e)
{
    uint32_t bits = (uint32_t)e << 23;
    float f;
    memcpy(&f, &bits, 4);
    return f;
}

typedef struct {
    uint32_t n;
    const uint32_t *left, *right, *first, *last;
    const box3 *ibox, *lbox;
} bvh2;

static inline uint32_t ref_count(const bvh2 *t, uint32_t r)
{
    if(r & LEAF_BIT) return 1;
    return t->last[r] - t->first[r] + 1;
}
static inline uint32_t ref_first(const bvh2 *t, uint32_t r) { return (r & LEAF_BIT) ? (r & ~LEAF_BIT) : t->first[r]; }
static inline const box3 *ref_box(const bvh2 *t, uint32_t r)
{
    return (r & LEAF_BIT) ? &t->lbox[r & ~LEAF_BIT] : &t->ibox[r];
}

int orc_bvh_build(const float *xyz, const uint32_t *idx, uint32_t ntri, uint32_t leaf_max, orc_bvh *out)
{
    memset(out, 0, sizeof(*out));
    out->num_tris = ntri;
    out->leaf_max = leaf_max;
    if(ntri == 0) return 0;
    if(leaf_max < 1 || leaf_max > 16) return -1;

    /* 1. boxes */
    box3 *tbox = (box3 *)malloc(sizeof(box3) * ntri);
    box3 scene = {{INFINITY, INFINITY, INFINITY}, {-INFINITY, -INFINITY, -INFINITY}};
    for(uint32_t i = 0; i < ntri; ++i)
    {
        box3 b = {{INFINITY, INFINITY, INFINITY}, {-INFINITY, -INFINITY, -INFINITY}};
        for(int k = 0; k < 3; ++k)
        {
            const float *p = xyz + 3 * (size_t)idx[3 * (size_t)i + k];
            for(int a = 0; a < 3; ++a)
            {
                b.lo[a] = fminf(b.lo[a], p[a]);
                b.hi[a] = fmaxf(b.hi[a], p[a]);
            }
        }
        tbox[i] = b;
        box_union(&scene, &b);
    }
    float ext_max = 0.f, abs_max = 0.f;
    for(int a = 0; a < 3; ++a)
    {
        out->scene_min[a] = scene.lo[a];
        out->scene_max[a] = scene.hi[a];
        ext_max = fmaxf(ext_max, scene.hi[a] - scene.lo[a]);
        abs_max = fmaxf(abs_max, fmaxf(fabsf(scene.lo[a]), fabsf(scene.hi[a])));
    }
    out->margin = fmaxf(ext_max, abs_max) * 0x1p-15f;

    /* 2. Morton codes */
    out->morton = (uint32_t *)malloc(4 * (size_t)ntri);
    float scale[3];
    for(int a = 0; a < 3; ++a)
    {
        float e = scene.hi[a] - scene.lo[a];
        scale[a] = e > 0.f ? 1024.0f / e : 0.f;
    }
    for(uint32_t i = 0; i < ntri; ++i)
    {
        uint32_t q[3];
        for(int a = 0; a < 3; ++a)
        {
            float c = (tbox[i].lo[a] + tbox[i].hi[a]) * 0.5f;
            float f = (c - scene.lo[a]) * scale[a];
            uint32_t v = f > 0.f ? (uint32_t)f : 0u;
            q[a] = v > 1023u ? 1023u : v;
        }
        out->morton[i] = (expand10(q[0]) << 2) | (expand10(q[1]) << 1) | expand10(q[2]);
    }

    /* 3. stable sort */
    kv *pairs = (kv *)malloc(sizeof(kv) * ntri);
    for(uint32_t i = 0; i < ntri; ++i) pairs[i] = (kv){out->morton[i], i};
    qsort(pairs, ntri, sizeof(kv), kv_cmp);
    uint32_t *codes = (uint32_t *)malloc(4 * (size_t)ntri);
    out->sorted_prim = (uint32_t *)malloc(4 * (size_t)ntri);
    for(uint32_t i = 0; i < ntri; ++i)
    {
        codes[i] = pairs[i].code;
        out->sorted_prim[i] = pairs[i].prim;
    }
    free(pairs);

    /* leaf boxes in sorted order */
    box3 *lbox = (box3 *)malloc(sizeof(box3) * ntri);
    for(uint32_t i = 0; i < ntri; ++i) lbox[i] = tbox[out->sorted_prim[i]];

    /* 4. Karras hierarchy */
    uint32_t ni = ntri - 1;
    uint32_t *left = (uint32_t *)malloc(4 * (size_t)(ni + 1)), *right = (uint32_t *)malloc(4 * (size_t)(ni + 1));
    uint32_t *first = (uint32_t *)malloc(4 * (size_t)(ni + 1)), *last = (uint32_t *)malloc(4 * (size_t)(ni + 1));
    uint32_t *iparent = (uint32_t *)malloc(4 * (size_t)(ni + 1)), *lparent = (uint32_t *)malloc(4 * (size_t)ntri);
    int64_t n = ntri;
    for(int64_t i = 0; i < (int64_t)ni; ++i)
    {
        int d = (delta(codes, n, i, i + 1) - delta(codes, n, i, i - 1)) >= 0 ? 1 : -1;
        int dmin = delta(codes, n, i, i - d);
        int64_t lmax = 2;
        while(delta(codes, n, i, i + lmax * d) > dmin) lmax *= 2;
        int64_t l = 0;
        for(int64_t t = lmax / 2; t >= 1; t /= 2)
            if(delta(codes, n, i, i + (l + t) * d) > dmin) l += t;
        int64_t j = i + l * d;
        int dnode = delta(codes, n, i, j);
        int64_t s = 0, t = l;
        do
        {
            t = (t + 1) / 2;
            if(delta(codes, n, i, i + (s + t) * d) > dnode) s += t;
        } while(t > 1);
        int64_t gamma = i + s * d + (d < 0 ? -1 : 0);
        int64_t lo = i < j ? i : j, hi = i < j ? j : i;
        left[i] = (lo == gamma) ? (LEAF_BIT | (uint32_t)gamma) : (uint32_t)gamma;
        right[i] = (hi == gamma + 1) ? (LEAF_BIT | (uint32_t)(gamma + 1)) : (uint32_t)(gamma + 1);
        first[i] = (uint32_t)lo;
        last[i] = (uint32_t)hi;
    }
    for(uint32_t i = 0; i < ni; ++i)
    {
        uint32_t c[2] = {left[i], right[i]};
        for(int k = 0; k < 2; ++k)
        {
            if(c[k] & LEAF_BIT) lparent[c[k] & ~LEAF_BIT] = i;
            else iparent[c[k]] = i;
        }
    }

    /* 5. refit */
    box3 *ibox = (box3 *)malloc(sizeof(box3) * (ni + 1));
    uint32_t *visits = (uint32_t *)calloc(ni + 1, 4);
    for(uint32_t leaf = 0; leaf < ntri && ni > 0; ++leaf)
    {
        uint32_t p = lparent[leaf];
        for(;;)
        {
            if(++visits[p] < 2) break;
            box3 b = *((left[p] & LEAF_BIT) ? &lbox[left[p] & ~LEAF_BIT] : &ibox[left[p]]);
            box_union(&b, (right[p] & LEAF_BIT) ? &lbox[right[p] & ~LEAF_BIT] : &ibox[right[p]]);
            ibox[p] = b;
            if(p == 0) break;
            p = iparent[p];
        }
    }
    free(visits);
    out->bvh2_left = left;
    out->bvh2_right = right;

    /* 6 + 7. collapse (breadth-first) and quantise */
    bvh2 T = {ntri, left, right, first, last, ibox, lbox};
    size_t cap = (size_t)ntri + 8;
    uint32_t *queue = (uint32_t *)malloc(4 * cap); /* BVH2 ref of each 8-wide node */
    uint32_t *level = (uint32_t *)malloc(4 * cap);
    orc_node8 *nodes = (orc_node8 *)calloc(cap, sizeof(orc_node8));
    uint32_t qn = 1;
    queue[0] = (ntri == 1) ? (LEAF_BIT | 0u) : 0u;
    level[0] = 1;
    uint32_t depth = 1;
    const float m = out->margin;
    for(uint32_t qi = 0; qi < qn; ++qi)
    {
        uint32_t r = queue[qi];
        uint32_t slots[8];
        uint32_t ns = 0;
        if((r & LEAF_BIT) || ref_count(&T, r) <= 1) { slots[ns++] = r; }
        else
        {
            slots[ns++] = left[r];
            slots[ns++] = right[r];
            while(ns < 8)
            {
                int best = -1;
                float best_area = -1.f;
                for(uint32_t k = 0; k < ns; ++k)
                {
                    uint32_t s = slots[k];
                    if((s & LEAF_BIT) || ref_count(&T, s) <= leaf_max) continue;
                    float a = box_area(&ibox[s]);
                    if(a > best_area)
                    {
                        best_area = a;
                        best = (int)k;
                    }
                }
                if(best < 0) break;
                uint32_t s = slots[best];
                slots[best] = left[s];
                slots[ns++] = right[s];
            }
        }
        orc_node8 *nd = &nodes[qi];
        nd->nchild = (uint8_t)ns;
        box3 gb[8];
        box3 nb = {{INFINITY, INFINITY, INFINITY}, {-INFINITY, -INFINITY, -INFINITY}};
        for(uint32_t k = 0; k < ns; ++k)
        {
            const box3 *b = ref_box(&T, slots[k]);
            for(int a = 0; a < 3; ++a)
            {
                gb[k].lo[a] = b->lo[a] - m;
                gb[k].hi[a] = b->hi[a] + m;
            }
            box_union(&nb, &gb[k]);
        }
        for(int a = 0; a < 3; ++a)
        {
            float range = nb.hi[a] - nb.lo[a];
            float x = range / 255.0f;
            uint32_t xb;
            memcpy(&xb, &x, 4);
            uint32_t e = ((xb >> 23) & 0xFFu) + 1u;
            if(e > 254u) e = 254u;
            nd->origin[a] = nb.lo[a];
            nd->exps[a] = (uint8_t)e;
            float inv_s = exp_scale((uint8_t)(254u - e));
            for(uint32_t k = 0; k < ns; ++k)
            {
                float ql = floorf((gb[k].lo[a] - nb.lo[a]) * inv_s);
                float qh = ceilf((gb[k].hi[a] - nb.lo[a]) * inv_s);
                nd->qlo[a][k] = (uint8_t)(ql < 0.f ? 0.f : (ql > 255.f ? 255.f : ql));
                nd->qhi[a][k] = (uint8_t)(qh < 0.f ? 0.f : (qh > 255.f ? 255.f : qh));
            }
        }
        for(uint32_t k = 0; k < ns; ++k)
        {
            uint32_t s = slots[k];
            uint32_t cnt = ref_count(&T, s);
            if(cnt <= leaf_max) { nd->child[k] = LEAF_BIT | ((cnt - 1u) << 27) | ref_first(&T, s); }
            else
            {
                nd->child[k] = qn;
                queue[qn] = s;
                level[qn] = level[qi] + 1;
                if(level[qn] > depth) depth = level[qn];
                ++qn;
            }
        }
    }
    out->num_nodes = qn;
    out->depth = depth;
    out->nodes = nodes;
    free(queue);
    free(level);

    /* triangle records in sorted order */
    out->tris = (orc_tri *)calloc(ntri, sizeof(orc_tri));
    for(uint32_t i = 0; i < ntri; ++i)
    {
        uint32_t p = out->sorted_prim[i];
        const float *v0 = xyz + 3 * (size_t)idx[3 * (size_t)p];
        const float *v1 = xyz + 3 * (size_t)idx[3 * (size_t)p + 1];
        const float *v2 = xyz + 3 * (size_t)idx[3 * (size_t)p + 2];
        float *r = out->tris[i].v;
        for(int a = 0; a < 3; ++a)
        {
            r[a] = v0[a];
            r[3 + a] = v1[a] - v0[a];
            r[6 + a] = v2[a] - v0[a];
        }
        memcpy(&r[9], &p, 4);
    }

    free(tbox);
    free(lbox);
    free(codes);
    free(first);
    free(last);
    free(iparent);
    free(lparent);
    free(ibox);
    return 0;
}

void orc_bvh_free(orc_bvh *b)
{
    free(b->morton);
    free(b->sorted_prim);
    free(b->bvh2_left);
    free(b->bvh2_right);
    free(b->nodes);
    free(b->tris);
    memset(b, 0, sizeof(*b));
}

/* ---- traversal ----------------------------------------------------------------------------- */
static inline uint32_t fenc_(float f)
{
    uint32_t b;
    memcpy(&b, &f, 4);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
static inline float fdec_(uint32_t u)
{
    uint32_t b = (u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u;
    float f;
    memcpy(&f, &b, 4);
    return f;
}
static inline uint32_t fbits_(float f)
{
    uint32_t b;
    memcpy(&b, &f, 4);
    return b;
}
static inline float fval_(uint32_t b)
{
    float f;
    memcpy(&f, &b, 4);
    return f;
}
#define STACK_CAP 256

typedef struct {
    const orc_bvh *b;
    const orc_ray *rays;
    uint32_t nray;
    orc_hit *hits;
    uint32_t *occluded;
    int cull;
    atomic_uint next;
    atomic_ullong visits, tests;
    orc_tri_fn tri_fn; /* NULL: the restated test on the precomputed record */
    void *tri_ctx;
} tr_job;

/* Moeller-Trumbore on the precomputed record (same ops as intersection.cpp:114-129) */
static inline int tri_test(const float *r, const float o[3], const float d[3], int cull, float *t, float *u,
                           float *v)
{
    const float *v0 = r, *e1 = r + 3, *e2 = r + 6;
    float pvec[3] = {d[1] * e2[2] - e2[1] * d[2], d[2] * e2[0] - e2[2] * d[0], d[0] * e2[1] - e2[0] * d[1]};
    float det = e1[0] * pvec[0] + e1[1] * pvec[1] + e1[2] * pvec[2];
    const float eps = 10.0e-10f;
    if(det > -eps && det < eps) return 0;
    if(cull && det < 0.f) return 0;
    float inv_det = 1.0f / det;
    float tv[3] = {o[0] - v0[0], o[1] - v0[1], o[2] - v0[2]};
    float uu = inv_det * (tv[0] * pvec[0] + tv[1] * pvec[1] + tv[2] * pvec[2]);
    if(uu < 0.0f || uu > 1.0f) return 0;
    float q[3] = {tv[1] * e1[2] - e1[1] * tv[2], tv[2] * e1[0] - e1[2] * tv[0], tv[0] * e1[1] - e1[0] * tv[1]};
    float vv = (d[0] * q[0] + d[1] * q[1] + d[2] * q[2]) * inv_det;
    if(vv < 0.0f || (uu + vv) > 1.0f) return 0;
    *t = (e2[0] * q[0] + e2[1] * q[1] + e2[2] * q[2]) * inv_det;
    *u = uu;
    *v = vv;
    return 1;
}

/* cull: 0 none, 1 every back face, 2 back faces of triangles not flagged in twosided[prim]; accept:
   candidate filter or NULL */
static void trace_one_ex(const orc_bvh *b, const orc_ray *ray, int cull, const uint8_t *twosided, int any,
                         orc_hit *hit, uint32_t *occ, uint64_t *nv, uint64_t *nt, orc_tri_fn fn, void *fn_ctx,
                         orc_accept_fn accept, const void *acc_ctx);
static void trace_one(const orc_bvh *b, const orc_ray *ray, int cull, int any, orc_hit *hit, uint32_t *occ,
                      uint64_t *nv, uint64_t *nt, orc_tri_fn fn, void *fn_ctx)
{
    trace_one_ex(b, ray, cull ? 1 : 0, NULL, any, hit, occ, nv, nt, fn, fn_ctx, NULL, NULL);
}

void orc_bvh_trace1_filter(const orc_bvh *b, const orc_ray *ray, int cull_mode, const uint8_t *twosided, int any,
                           orc_accept_fn accept, const void *ctx, orc_hit *hit, uint32_t *occ)
{
    uint64_t nv = 0, nt = 0;
    if(b->num_tris == 0)
    {
        if(hit) *hit = (orc_hit){ORC_MISS, 0.f, 0.f, 0.f};
        if(occ) *occ = 0;
        return;
    }
    trace_one_ex(b, ray, cull_mode, twosided, any, hit, occ, &nv, &nt, NULL, NULL, accept, ctx);
}

void orc_bvh_trace1(const orc_bvh *b, const orc_ray *ray, int cull_mode, const uint8_t *twosided, int any,
                    orc_hit *hit, uint32_t *occ)
{
    orc_bvh_trace1_filter(b, ray, cull_mode, twosided, any, NULL, NULL, hit, occ);
}

static void trace_one_ex(const orc_bvh *b, const orc_ray *ray, int cull_mode, const uint8_t *twosided, int any,
                         orc_hit *hit, uint32_t *occ, uint64_t *nv, uint64_t *nt, orc_tri_fn fn, void *fn_ctx,
                         orc_accept_fn accept, const void *acc_ctx)
{
    float inv_d[3];
    int neg[3];
    for(int a = 0; a < 3; ++a)
    {
        float dd = ray->d[a];
        if(fabsf(dd) < 1e-20f) dd = copysignf(1e-20f, dd);
        inv_d[a] = 1.0f / dd;
        neg[a] = inv_d[a] < 0.f;
    }
    float best_t = ray->tmax, bu = 0.f, bv = 0.f;
    const int pos = !(fbits_(ray->tmin) & 0x80000000u);
    uint32_t best = ORC_MISS;
    uint32_t st_node[STACK_CAP];
    float st_t[STACK_CAP];
    int sp = 0;
    st_node[sp] = 0;
    st_t[sp] = ray->tmin;
    ++sp;
    uint64_t visits = 0, tests = 0;
    int done = 0;
    while(sp > 0 && !done)
    {
        --sp;
        uint32_t ni = st_node[sp];
        if(st_t[sp] > best_t) continue;
        ++visits;
        const orc_node8 *nd = &b->nodes[ni];
        float torig[3], sinv[3];
        for(int a = 0; a < 3; ++a)
        {
            torig[a] = (nd->origin[a] - ray->o[a]) * inv_d[a];
            sinv[a] = exp_scale(nd->exps[a]) * inv_d[a];
        }
        float ht[8];
        int hk[8];
        uint32_t hkey[8];
        int nh = 0;
        for(int k = 0; k < nd->nchild; ++k)
        {
            float tn3[3], tf3[3];
            for(int a = 0; a < 3; ++a)
            {
                float ql = (float)nd->qlo[a][k], qh = (float)nd->qhi[a][k];
                float qn = neg[a] ? qh : ql, qf = neg[a] ? ql : qh;
                tn3[a] = fmaf(qn, sinv[a], torig[a]);
                tf3[a] = fmaf(qf, sinv[a], torig[a]);
            }
            float tn = fmaxf(fmaxf(tn3[0], tn3[1]), fmaxf(tn3[2], ray->tmin));
            float tf = fminf(fminf(tf3[0], tf3[1]), fminf(tf3[2], best_t));
            if(tn <= tf)
            {
                /* 32-bit key as in the kernels: ordered entry distance, low 3 bits = slot; a ray with
                   tmin >= +0 keys the distance's bits with the sign cleared */
                uint32_t key = pos ? ((fbits_(tn) & 0x7FFFFFF8u) | (uint32_t)k) : ((fenc_(tn) & ~7u) | (uint32_t)k);
                int p = nh++;
                while(p > 0 && hkey[p - 1] > key)
                {
                    hkey[p] = hkey[p - 1];
                    --p;
                }
                hkey[p] = key;
            }
        }
        for(int h = 0; h < nh; ++h)
        {
            ht[h] = pos ? fval_(hkey[h] & 0x7FFFFFF8u) : fdec_(hkey[h] & ~7u);
            hk[h] = (int)(hkey[h] & 7u);
        }
        for(int h = 0; h < nh && !done; ++h)
        {
            uint32_t c = nd->child[hk[h]];
            if(!(c & LEAF_BIT)) continue;
            if(ht[h] > best_t) continue;
            uint32_t start = c & 0x07FFFFFFu, cnt = ((c >> 27) & 0xFu) + 1u;
            for(uint32_t i = start; i < start + cnt; ++i)
            {
                const float *r = b->tris[i].v;
                uint32_t prim;
                memcpy(&prim, &r[9], 4);
                float t, u, v;
                ++tests;
                int cull = cull_mode == 1 || (cull_mode == 2 && !(twosided && twosided[prim]));
                if(fn)
                {
                    /* caller's triangle test on the original triangle (no culling on this path) */
                    float tuv[3];
                    if(fn(fn_ctx, prim, ray->o, ray->d, tuv) != 1) continue;
                    t = tuv[0];
                    u = tuv[1];
                    v = tuv[2];
                }
                else if(!tri_test(r, ray->o, ray->d, cull, &t, &u, &v)) continue;
                if(!(t > ray->tmin && t < ray->tmax)) continue;
                if(any)
                {
                    if(accept && !accept(acc_ctx, prim, u, v)) continue;
                    done = 1;
                    break;
                }
                if(t < best_t || (t == best_t && prim < best))
                {
                    if(accept && !accept(acc_ctx, prim, u, v)) continue;
                    best_t = t;
                    best = prim;
                    bu = u;
                    bv = v;
                }
            }
        }
        for(int h = nh - 1; h >= 0 && !done; --h)
        {
            uint32_t c = nd->child[hk[h]];
            if(c & LEAF_BIT) continue;
            if(sp < STACK_CAP)
            {
                st_node[sp] = c;
                st_t[sp] = ht[h];
                ++sp;
            }
        }
    }
    if(occ) *occ = (uint32_t)done;
    if(hit)
    {
        if(best == ORC_MISS) *hit = (orc_hit){ORC_MISS, 0.f, 0.f, 0.f};
        else *hit = (orc_hit){best, best_t, bu, bv};
    }
    *nv += visits;
    *nt += tests;
}

static void *tr_worker(void *arg)
{
    tr_job *j = (tr_job *)arg;
    uint64_t nv = 0, nt = 0;
    for(;;)
    {
        uint32_t begin = atomic_fetch_add(&j->next, 64u);
        if(begin >= j->nray) break;
        uint32_t end = begin + 64u < j->nray ? begin + 64u : j->nray;
        for(uint32_t r = begin; r < end; ++r)
            trace_one(j->b, &j->rays[r], j->cull, j->occluded != NULL, j->hits ? &j->hits[r] : NULL,
                      j->occluded ? &j->occluded[r] : NULL, &nv, &nt, j->tri_fn, j->tri_ctx);
    }
    atomic_fetch_add(&j->visits, nv);
    atomic_fetch_add(&j->tests, nt);
    return NULL;
}

int orc_bvh_closest_hit(const orc_bvh *b, const orc_ray *rays, uint32_t nray, orc_hit *hits, int nthreads,
                        int cull_back, uint64_t *stats)
{
    if(b->num_tris == 0)
    {
        for(uint32_t r = 0; r < nray; ++r) hits[r] = (orc_hit){ORC_MISS, 0.f, 0.f, 0.f};
        if(stats) stats[0] = stats[1] = 0;
        return 1;
    }
    tr_job j = {b, rays, nray, hits, NULL, cull_back, 0, 0, 0, NULL, NULL};
    int n = orc__run_threads(tr_worker, &j, nthreads);
    if(stats)
    {
        stats[0] = atomic_load(&j.visits);
        stats[1] = atomic_load(&j.tests);
    }
    return n;
}

int orc_bvh_closest_hit_fn(const orc_bvh *b, const orc_ray *rays, uint32_t nray, orc_hit *hits, int nthreads,
                           orc_tri_fn fn, void *fn_ctx, uint64_t *stats)
{
    if(b->num_tris == 0 || fn == NULL) return orc_bvh_closest_hit(b, rays, nray, hits, nthreads, 0, stats);
    tr_job j = {b, rays, nray, hits, NULL, 0, 0, 0, 0, fn, fn_ctx};
    int n = orc__run_threads(tr_worker, &j, nthreads);
    if(stats)
    {
        stats[0] = atomic_load(&j.visits);
        stats[1] = atomic_load(&j.tests);
    }
    return n;
}

int orc_bvh_any_hit(const orc_bvh *b, const orc_ray *rays, uint32_t nray, uint32_t *occluded, int nthreads,
                    int cull_back)
{
    if(b->num_tris == 0)
    {
        memset(occluded, 0, 4 * (size_t)nray);
        return 1;
    }
    tr_job j = {b, rays, nray, NULL, occluded, cull_back, 0, 0, 0, NULL, NULL};
    return orc__run_threads(tr_worker, &j, nthreads);
}
