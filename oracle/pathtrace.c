/*
 * Path tracer on the CPU. TEST INFRASTRUCTURE ONLY (CPU oracle).
 *
 *  - FP32 twin (fp64 = 0): the GPU kernels' estimator path for path: the same PCG32 stream per path
 *    (initseq = (batch << 40) ^ (sample * pixels + pixel), 2 jitter draws, 8 draws per segment), the
 *    oracle's float BVH traversal (bit-identical hits to the GPU's), and the GPU's own environment
 *    alias table as input. Differences come only from transcendental functions and fused
 *    multiply-adds, so most paths agree to a few ulps.
 *  - FP64 oracle (fp64 = 1): the same estimator in double precision with an independent
 *    environment sampler (FP64 CDF + binary search), double-precision ray casting over the same
 *    8-wide BVH (box tests in double, Moeller-Trumbore in double), and 32-bit uniforms.
 * The estimator itself is oracle/pt_core.inc (see its header for the reference lines it follows).
 */
#include "oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stdlib.h>
#include <string.h>

int orc__run_threads(void *(*fn)(void *), void *arg, int nthreads);

#define LEAF_BIT 0x80000000u

/* the medium a boundary material defines (raypipeline.slang:493-511), computed in float as the
   product's host code does; flags: 1 finite attenuation distance, 2 null surface */
typedef struct {
    float sigma_s[3], g, sigma_a[3], ior, emission[3];
    uint32_t flags;
} orc_medium;

static void orc_medium_from(const orc_pt_material *m, orc_medium *r)
{
    int vol = m->attenuation_distance > 0.f && m->attenuation_distance < 3.0e38f;
    for(int c = 0; c < 3; ++c)
    {
        float st = vol ? -logf(m->attenuation_color[c]) / m->attenuation_distance : 0.f;
        float ms = m->scatter_factor * m->scatter_color[c];
        float kc = 4.09712f + 4.20863f * ms - sqrtf(9.59217f + 41.6808f * ms + 17.7126f * ms * ms);
        float ss = 1.f - kc * kc;
        r->sigma_s[c] = ss * st;
        r->sigma_a[c] = (1.f - ss) * st;
        r->emission[c] = m->null_surface ? m->emission[c] : 0.f;
    }
    r->g = m->phase_g;
    r->ior = m->ior;
    r->flags = (vol ? 1u : 0u) | (m->null_surface ? 2u : 0u);
}

/* a medium given directly (media.hpp:26-49 converted as to_media, media.cpp:6-23): p = attenuation
   colour[3], distance, scatter factor, scatter colour[3], g, ior, emission colour[3], intensity */
static void orc_medium_from_params(const float *p, orc_medium *r)
{
    for(int c = 0; c < 3; ++c)
    {
        float st = -logf(p[c]) / p[3];
        float ms = p[4] * p[5 + c];
        float kc = 4.09712f + 4.20863f * ms - sqrtf(9.59217f + 41.6808f * ms + 17.7126f * ms * ms);
        float ss = 1.f - kc * kc;
        r->sigma_s[c] = ss * st;
        r->sigma_a[c] = (1.f - ss) * st;
        r->emission[c] = p[10 + c] * p[13];
    }
    r->g = p[8];
    r->ior = p[9];
    r->flags = 1u;
}

/* the medium table of a render: one record per material, plus the camera's medium as the last one;
   NULL when no material bounds a medium and the camera sits in vacuum */
static orc_medium *orc_media_table(const orc_pt_scene *scene, const orc_pt_settings *set, uint32_t *cam)
{
    int any = set->camera_medium != NULL || set->camera_material < scene->nmat;
    for(uint32_t i = 0; i < scene->nmat && !any; ++i)
    {
        const orc_pt_material *m = &scene->mats[i];
        any = m->null_surface || (m->attenuation_distance > 0.f && m->attenuation_distance < 3.0e38f);
    }
    *cam = 0xFFFFFFFFu;
    if(!any) return NULL;
    orc_medium *media = (orc_medium *)calloc(scene->nmat + 1, sizeof(orc_medium));
    for(uint32_t i = 0; i < scene->nmat; ++i) orc_medium_from(&scene->mats[i], &media[i]);
    if(set->camera_medium)
    {
        orc_medium_from_params(set->camera_medium, &media[scene->nmat]);
        *cam = scene->nmat;
    }
    else if(set->camera_material < scene->nmat)
    {
        media[scene->nmat] = media[set->camera_material];
        media[scene->nmat].flags = 1u;
        *cam = scene->nmat;
    }
    return media;
}

static uint32_t orc__any_dispersive(const orc_pt_scene *scene)
{
    for(uint32_t i = 0; i < scene->nmat; ++i)
        if(scene->mats[i].dispersion > 0.f && scene->mats[i].transmission > 0.f) return 1u;
    return 0u;
}

/* a material whose candidate hits are tested for coverage: alpha mask (2) or blend (1), not a null
   surface (raypipeline.slang:694-695) */
static int orc__alpha_tested(const orc_pt_material *m)
{
    return (m->blend_mode == 1u || m->blend_mode == 2u) && !m->null_surface;
}

static uint32_t orc__any_alpha(const orc_pt_scene *scene)
{
    for(uint32_t i = 0; i < scene->nmat; ++i)
        if(orc__alpha_tested(&scene->mats[i])) return 1u;
    return 0u;
}

typedef struct {
    const orc_pt_scene *scene;
    const orc_bvh *bvh;
    const orc_pt_env *env;
    const orc_camera *cam;
    const uint8_t *twosided; /* by triangle id */
    uint32_t seed, batch, spp, max_depth, rr_depth, mis_mode, disable_material, draw_skybox;
    float max_path_beta, environment;
    const orc_pt_light *lights;
    uint32_t num_lights, suppress_caustics;
    orc_pixel *pixels;
    float clip_near;
    const orc_medium *media; /* per material (+ the camera's), NULL: no media */
    uint32_t cam_medium;     /* index of the camera's medium, 0xFFFFFFFF: vacuum */
    uint32_t cx0, cy0, cw, ch;
    double *out, *sq;
    const orc_pt_instances *inst; /* NULL: single-level scene */
    const void *ibvh;             /* instance BVH of an instanced scene */
    atomic_uint next;
    atomic_ullong ext, shadow;
    int fp64;
    uint32_t dispersion; /* a transmissive material disperses: one more uniform per segment */
    uint32_t alpha;      /* a material is alpha-tested: candidate hits go through the coverage filter */
    uint32_t fork_depth; /* the variance split's fork segment (orc_pt_variance_split) */
    double *split;       /* [pixels][4] of orc_pt_variance_split */
} orc_pt_job;

/* ---- coverage of alpha-tested materials (any_hit, raypipeline.slang:686-720; visibility_test.slang:
   45-87, :131-152): alpha x the colour texture's alpha at level 0; MASK rejects alpha < cutoff, BLEND
   rejects alpha < xi. xi: for an extension ray the first uniform of the segment that shades the hit
   (the path's generator is not advanced); for shadow rays one uniform per candidate hashed from the
   path's generator state, the ray kind, the instance and the triangle (the GPU kernels' rule) */
typedef struct {
    const orc_pt_job *J;
    uint32_t inst;         /* instanced scenes: the instance being traced */
    double xi;             /* extension rays */
    uint64_t key;          /* shadow rays: the path's generator state */
    uint32_t salt;         /* 0: an extension ray; else the shadow ray's kind */
    int pass_transmissive; /* light-NEE rays: transmissive surfaces are tinted, not tested */
} orc_alpha_ctx;
#define ORC_SALT_SHADOW 0x9E3779B9u
#define ORC_SALT_LIGHT_SHADOW 0x7F4A7C15u

static float orc_alpha_uniform(uint64_t key, uint32_t salt, uint32_t inst, uint32_t prim)
{
    uint32_t h = orc_xxhash32((uint32_t)key ^ salt, (uint32_t)(key >> 32));
    h = orc_xxhash32(h, inst);
    h = orc_xxhash32(h, prim);
    return orc_u01(h);
}

/* defined after the estimator core (they sample textures) */
static int f_alpha_accept(const void *ctx, uint32_t prim, float u, float v);
static int d_alpha_accept(const orc_alpha_ctx *c, uint32_t prim, double u, double v);

/* ---- FP32 twin hooks ------------------------------------------------------------------------ */
static inline float f_draw_raw(orc_pcg32 *g) { return orc_u01(orc_pcg32_next(g)); }

static void f_hit_raw(const orc_pt_job *J, float ox, float oy, float oz, float tmin, float dx, float dy, float dz,
                      float xi, uint32_t *prim, uint32_t *inst, float *u, float *v, float *t)
{
    *inst = 0;
    orc_ray r = {{ox, oy, oz}, tmin, {dx, dy, dz}, 1e4f};
    orc_hit h;
    const orc_alpha_ctx ac = {J, 0u, (double)xi, 0u, 0u, 0};
    orc_bvh_trace1_filter(J->bvh, &r, 2, J->twosided, 0, J->alpha ? f_alpha_accept : NULL, &ac, &h, NULL);
    *prim = h.prim;
    *u = h.u;
    *v = h.v;
    *t = h.t;
}

/* light-NEE visibility (visibility_test.slang:94-131): 0 at the first opaque surface in (tmin, tmax),
   else transmission x base colour of every transmissive surface crossed, nearest first; null surfaces
   pass unattenuated */
static void f_transmit_raw(const orc_pt_job *J, float ox, float oy, float oz, float tmin, float dx, float dy, float dz,
                           float tmax, int cull, float T[3], uint64_t key)
{
    T[0] = T[1] = T[2] = 1.f;
    float od[3] = {0.f, 0.f, 0.f};
    const orc_alpha_ctx ac = {J, 0u, 0.0, key, ORC_SALT_LIGHT_SHADOW, 1};
    for(int k = 0;; ++k)
    {
        orc_ray r = {{ox, oy, oz}, tmin, {dx, dy, dz}, tmax};
        orc_hit h;
        orc_bvh_trace1_filter(J->bvh, &r, cull ? 1 : 0, NULL, 0, J->alpha ? f_alpha_accept : NULL, &ac, &h, NULL);
        if(h.prim == ORC_MISS) break;
        const uint32_t mi = J->scene->tri_mat[h.prim];
        const orc_pt_material *m = &J->scene->mats[mi];
        if(m->null_surface && k + 1 < 32)
        {
            tmin = h.t; /* null surfaces pass unattenuated (visibility_test.slang:113) */
            continue;
        }
        if(!(m->transmission > 0.f) || k + 1 >= 32)
        {
            T[0] = T[1] = T[2] = 0.f;
            return;
        }
        for(int c = 0; c < 3; ++c) T[c] = T[c] * m->base[c] * m->transmission;
        if(J->media && (J->media[mi].flags & 1u))
        {
            /* Beer-Lambert: -sigma_t t entering (front face), +sigma_t t leaving */
            const float *xyz = J->scene->xyz;
            const uint32_t *ix = J->scene->idx + 3 * (size_t)h.prim;
            const float *a = xyz + 3 * (size_t)ix[0], *b = xyz + 3 * (size_t)ix[1], *c2 = xyz + 3 * (size_t)ix[2];
            float e1[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]}, e2[3] = {c2[0] - a[0], c2[1] - a[1], c2[2] - a[2]};
            float n[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
            int front = n[0] * dx + n[1] * dy + n[2] * dz < 0.f;
            for(int c = 0; c < 3; ++c)
            {
                float st = J->media[mi].sigma_s[c] + J->media[mi].sigma_a[c];
                od[c] += st * (front ? -h.t : h.t);
            }
        }
        tmin = h.t;
    }
    if(J->media)
        for(int c = 0; c < 3; ++c) T[c] *= expf(-fmaxf(od[c], 0.f));
}

static int f_occluded_raw(const orc_pt_job *J, float ox, float oy, float oz, float tmin, float dx, float dy, float dz,
                          int cull, uint64_t key)
{
    orc_ray r = {{ox, oy, oz}, tmin, {dx, dy, dz}, 1e4f};
    uint32_t occ = 0;
    const orc_alpha_ctx ac = {J, 0u, 0.0, key, ORC_SALT_SHADOW, 0};
    orc_bvh_trace1_filter(J->bvh, &r, cull ? 1 : 0, NULL, 1, J->alpha ? f_alpha_accept : NULL, &ac, NULL, &occ);
    return (int)occ;
}

/* alias-table sample, as env_sample() in the GPU kernels */
static void f_env_sample_raw(const orc_pt_env *e, float u0, float u1, float u2, float u3, float *dx, float *dy,
                             float *dz, float *pdf, uint32_t *texel)
{
    const uint32_t n = e->w * e->h;
    uint32_t b = (uint32_t)(u0 * (float)n);
    if(b > n - 1u) b = n - 1u;
    uint32_t t = u1 < e->alias_prob[b] ? b : e->alias[b];
    uint32_t i = t % e->w, j = t / e->w;
    float u = ((float)i + u2) / (float)e->w, v = ((float)j + u3) / (float)e->h;
    const float PI = 3.14159265358979323846f;
    float phi = (u - 0.5f) * 2.f * PI, theta = v * PI;
    float st = sinf(theta);
    *dx = st * sinf(phi);
    *dy = cosf(theta);
    *dz = -st * cosf(phi);
    *pdf = st > 0.f ? e->weight[t] / (2.f * PI * PI * st) : 0.f;
    *texel = t;
}

/* ---- FP64 oracle hooks ---------------------------------------------------------------------- */
static inline double d_draw_raw(orc_pcg32 *g) { return (double)orc_pcg32_next(g) * 0x1p-32; }

static inline float exp_scale_f(uint8_t e)
{
    uint32_t bits = (uint32_t)e << 23;
    float f;
    memcpy(&f, &bits, 4);
    return f;
}

/* closest hit (any = 0) or occlusion (any = 1) in double precision over one 8-wide BVH, t in
   (tmin, tmax); two-sidedness per triangle (twosided[prim]) or for the whole mesh (all_twosided) */
static int d_trace_bvh(const orc_bvh *b, const uint8_t *twosided, int all_twosided, const double o[3], double tmin,
                       const double d[3], double tmax, int cull_mode, int any, uint32_t *prim_out, double *t_out,
                       double *u_out, double *v_out, const orc_alpha_ctx *ac)
{
    *prim_out = ORC_MISS;
    if(b->num_tris == 0) return 0;
    double inv[3];
    for(int a = 0; a < 3; ++a) inv[a] = d[a] != 0.0 ? 1.0 / d[a] : copysign(1e300, d[a]);
    double best_t = tmax, bu = 0, bv = 0;
    uint32_t best = ORC_MISS;
    uint32_t stack[512];
    int sp = 0;
    stack[sp++] = 0;
    while(sp > 0)
    {
        const orc_node8 *nd = &b->nodes[stack[--sp]];
        for(int k = 0; k < nd->nchild; ++k)
        {
            double tn = tmin, tf = best_t;
            for(int a = 0; a < 3; ++a)
            {
                double s = (double)exp_scale_f(nd->exps[a]);
                double lo = (double)nd->origin[a] + (double)nd->qlo[a][k] * s;
                double hi = (double)nd->origin[a] + (double)nd->qhi[a][k] * s;
                double t0 = (lo - o[a]) * inv[a], t1 = (hi - o[a]) * inv[a];
                if(t0 > t1)
                {
                    double tt = t0;
                    t0 = t1;
                    t1 = tt;
                }
                if(t0 > tn) tn = t0;
                if(t1 < tf) tf = t1;
            }
            if(tn > tf) continue;
            uint32_t c = nd->child[k];
            if(!(c & LEAF_BIT))
            {
                if(sp < 512) stack[sp++] = c;
                continue;
            }
            uint32_t start = c & 0x07FFFFFFu, cnt = ((c >> 27) & 0xFu) + 1u;
            for(uint32_t i = start; i < start + cnt; ++i)
            {
                const float *r = b->tris[i].v;
                uint32_t prim;
                memcpy(&prim, &r[9], 4);
                double v0[3] = {r[0], r[1], r[2]}, e1[3] = {r[3], r[4], r[5]}, e2[3] = {r[6], r[7], r[8]};
                double p[3] = {d[1] * e2[2] - e2[1] * d[2], d[2] * e2[0] - e2[2] * d[0], d[0] * e2[1] - e2[0] * d[1]};
                double det = e1[0] * p[0] + e1[1] * p[1] + e1[2] * p[2];
                if(det > -1e-12 && det < 1e-12) continue;
                int cull = cull_mode == 1 || (cull_mode == 2 && !all_twosided && !(twosided && twosided[prim]));
                if(cull && det < 0) continue;
                double id = 1.0 / det;
                double tv[3] = {o[0] - v0[0], o[1] - v0[1], o[2] - v0[2]};
                double uu = id * (tv[0] * p[0] + tv[1] * p[1] + tv[2] * p[2]);
                if(uu < 0.0 || uu > 1.0) continue;
                double q[3] = {tv[1] * e1[2] - e1[1] * tv[2], tv[2] * e1[0] - e1[2] * tv[0],
                               tv[0] * e1[1] - e1[0] * tv[1]};
                double vv = (d[0] * q[0] + d[1] * q[1] + d[2] * q[2]) * id;
                if(vv < 0.0 || uu + vv > 1.0) continue;
                double t = (e2[0] * q[0] + e2[1] * q[1] + e2[2] * q[2]) * id;
                if(!(t > tmin && t < tmax)) continue;
                if(any)
                {
                    if(ac && !d_alpha_accept(ac, prim, uu, vv)) continue;
                    return 1;
                }
                if(t < best_t)
                {
                    if(ac && !d_alpha_accept(ac, prim, uu, vv)) continue;
                    best_t = t;
                    best = prim;
                    bu = uu;
                    bv = vv;
                }
            }
        }
    }
    *prim_out = best;
    *t_out = best_t;
    *u_out = bu;
    *v_out = bv;
    return best != ORC_MISS;
}

static int d_trace(const orc_pt_job *J, const double o[3], double tmin, const double d[3], double tmax, int cull_mode,
                   int any, uint32_t *prim_out, double *t_out, double *u_out, double *v_out, const orc_alpha_ctx *ac)
{
    return d_trace_bvh(J->bvh, J->twosided, 0, o, tmin, d, tmax, cull_mode, any, prim_out, t_out, u_out, v_out,
                       J->alpha ? ac : NULL);
}

/* ---- instanced scenes (FP64) ----------------------------------------------------------------
   A binary BVH over the instances' exact world boxes (the 8 transformed corners of the mesh bounds,
   in double), split at the median centroid of the longest axis; an instance leaf moves the ray to
   object space with the inverse transform (computed in double) and traces the mesh BVH. */
typedef struct
{
    double lo[3], hi[3];
    uint32_t left, count; /* count > 0: leaf over order[left .. left + count) */
} ib_node;

typedef struct
{
    ib_node *nodes;
    uint32_t *order;
    double *w2o;  /* [n][12] */
    double *o2w;  /* [n][12] */
    double (*box)[6];
    uint8_t *mesh_unculled; /* [num_meshes]: two-sided, or used by an instance of a transmissive material */
} inst_bvh;

static void inv3x4(const double *m, double *r)
{
    const double a = m[0], b = m[1], c = m[2], d = m[4], e = m[5], f = m[6], g = m[8], h = m[9], i = m[10];
    const double A = e * i - f * h, B = f * g - d * i, C = d * h - e * g;
    const double det = a * A + b * B + c * C, q = 1.0 / det;
    const double M[9] = {A, c * h - b * i, b * f - c * e, B, a * i - c * g, c * d - a * f, C, b * g - a * h, a * e - b * d};
    for(int row = 0; row < 3; ++row)
    {
        double acc = 0;
        for(int k = 0; k < 3; ++k)
        {
            r[4 * row + k] = M[3 * row + k] * q;
            acc += r[4 * row + k] * m[4 * k + 3];
        }
        r[4 * row + 3] = -acc;
    }
}

typedef struct
{
    double c;
    uint32_t i;
} ib_key;

static int ib_key_cmp(const void *a, const void *b)
{
    const ib_key *x = (const ib_key *)a, *y = (const ib_key *)b;
    if(x->c < y->c) return -1;
    if(x->c > y->c) return 1;
    return x->i < y->i ? -1 : (x->i > y->i);
}

/* back faces are traced for two-sided surfaces and for objects rays enter and leave (transmission) */
static int orc_material_unculled(const orc_pt_material *m)
{
    return m->twosided != 0u || m->transmission > 0.f || m->diffuse_transmission > 0.f || m->null_surface != 0u ||
           (m->attenuation_distance > 0.f && m->attenuation_distance < 3.0e38f);
}

static inst_bvh *build_inst_bvh(const orc_pt_instances *I)
{
    const uint32_t n = I->num_instances;
    inst_bvh *B = (inst_bvh *)calloc(1, sizeof(inst_bvh));
    B->nodes = (ib_node *)calloc(2 * (size_t)n + 1, sizeof(ib_node));
    B->order = (uint32_t *)malloc(sizeof(uint32_t) * (n ? n : 1));
    B->w2o = (double *)malloc(sizeof(double) * 12 * (n ? n : 1));
    B->o2w = (double *)malloc(sizeof(double) * 12 * (n ? n : 1));
    B->box = (double(*)[6])malloc(sizeof(double[6]) * (n ? n : 1));
    B->mesh_unculled = (uint8_t *)calloc(I->num_meshes ? I->num_meshes : 1, 1);
    for(uint32_t m = 0; m < I->num_meshes; ++m) B->mesh_unculled[m] = I->mesh_twosided[m] ? 1 : 0;
    double (*mb)[6] = (double(*)[6])malloc(sizeof(double[6]) * (I->num_meshes ? I->num_meshes : 1));
    for(uint32_t m = 0; m < I->num_meshes; ++m)
    {
        for(int a = 0; a < 3; ++a)
        {
            mb[m][a] = 1e300;
            mb[m][3 + a] = -1e300;
        }
        for(uint32_t v = 0; v < I->mesh_nvert[m]; ++v)
            for(int a = 0; a < 3; ++a)
            {
                const double x = I->mesh_xyz[m][3 * (size_t)v + a];
                if(x < mb[m][a]) mb[m][a] = x;
                if(x > mb[m][3 + a]) mb[m][3 + a] = x;
            }
    }
    for(uint32_t k = 0; k < n; ++k)
    {
        double *o = B->o2w + 12 * (size_t)k;
        for(int j = 0; j < 12; ++j) o[j] = I->o2w[12 * (size_t)k + j];
        inv3x4(o, B->w2o + 12 * (size_t)k);
        const double *bb = mb[I->inst_mesh[k]];
        for(int a = 0; a < 3; ++a)
        {
            B->box[k][a] = 1e300;
            B->box[k][3 + a] = -1e300;
        }
        for(int c = 0; c < 8; ++c)
        {
            const double p[3] = {(c & 1) ? bb[3] : bb[0], (c & 2) ? bb[4] : bb[1], (c & 4) ? bb[5] : bb[2]};
            for(int a = 0; a < 3; ++a)
            {
                const double w = o[4 * a] * p[0] + o[4 * a + 1] * p[1] + o[4 * a + 2] * p[2] + o[4 * a + 3];
                if(w < B->box[k][a]) B->box[k][a] = w;
                if(w > B->box[k][3 + a]) B->box[k][3 + a] = w;
            }
        }
        B->order[k] = k;
    }
    free(mb);
    /* iterative median split */
    uint32_t used = 1;
    typedef struct { uint32_t node, lo, hi; } task;
    task *stack = (task *)malloc(sizeof(task) * (2 * (size_t)n + 2));
    int sp = 0;
    stack[sp++] = (task){0, 0, n};
    while(sp > 0)
    {
        task t = stack[--sp];
        ib_node *nd = &B->nodes[t.node];
        for(int a = 0; a < 3; ++a)
        {
            nd->lo[a] = 1e300;
            nd->hi[a] = -1e300;
        }
        for(uint32_t i = t.lo; i < t.hi; ++i)
            for(int a = 0; a < 3; ++a)
            {
                if(B->box[B->order[i]][a] < nd->lo[a]) nd->lo[a] = B->box[B->order[i]][a];
                if(B->box[B->order[i]][3 + a] > nd->hi[a]) nd->hi[a] = B->box[B->order[i]][3 + a];
            }
        if(t.hi - t.lo <= 2)
        {
            nd->left = t.lo;
            nd->count = t.hi - t.lo;
            continue;
        }
        int axis = 0;
        for(int a = 1; a < 3; ++a)
            if(nd->hi[a] - nd->lo[a] > nd->hi[axis] - nd->lo[axis]) axis = a;
        /* order the range by centroid along the axis; the median splits it */
        const uint32_t cnt = t.hi - t.lo, mid = (t.lo + t.hi) / 2;
        ib_key *keys = (ib_key *)malloc(sizeof(ib_key) * cnt);
        for(uint32_t i = 0; i < cnt; ++i)
        {
            const uint32_t k = B->order[t.lo + i];
            keys[i].c = B->box[k][axis] + B->box[k][3 + axis];
            keys[i].i = k;
        }
        qsort(keys, cnt, sizeof(ib_key), ib_key_cmp);
        for(uint32_t i = 0; i < cnt; ++i) B->order[t.lo + i] = keys[i].i;
        free(keys);
        nd->left = used;
        nd->count = 0;
        const uint32_t l = used, r = used + 1;
        used += 2;
        stack[sp++] = (task){l, t.lo, mid};
        stack[sp++] = (task){r, mid, t.hi};
    }
    free(stack);
    return B;
}

static void free_inst_bvh(inst_bvh *B)
{
    if(!B) return;
    free(B->nodes);
    free(B->order);
    free(B->w2o);
    free(B->o2w);
    free(B->box);
    free(B->mesh_unculled);
    free(B);
}

static int slab(const double lo[3], const double hi[3], const double o[3], const double inv[3], double tmin, double tmax)
{
    for(int a = 0; a < 3; ++a)
    {
        double t0 = (lo[a] - o[a]) * inv[a], t1 = (hi[a] - o[a]) * inv[a];
        if(t0 > t1)
        {
            double tt = t0;
            t0 = t1;
            t1 = tt;
        }
        if(t0 > tmin) tmin = t0;
        if(t1 < tmax) tmax = t1;
    }
    return tmin <= tmax;
}

static int d_trace_inst(const orc_pt_job *J, const double o[3], double tmin, const double d[3], double tmax,
                        int cull_mode, int any, uint32_t *prim_out, uint32_t *inst_out, double *t_out, double *u_out,
                        double *v_out, const orc_alpha_ctx *ac)
{
    const orc_pt_instances *I = J->inst;
    const inst_bvh *B = (const inst_bvh *)J->ibvh;
    *prim_out = *inst_out = ORC_MISS;
    if(I->num_instances == 0) return 0;
    double inv[3];
    for(int a = 0; a < 3; ++a) inv[a] = d[a] != 0.0 ? 1.0 / d[a] : copysign(1e300, d[a]);
    double best_t = tmax, bu = 0, bv = 0;
    uint32_t stack[256];
    int sp = 0;
    stack[sp++] = 0;
    while(sp > 0)
    {
        const ib_node *nd = &B->nodes[stack[--sp]];
        if(!slab(nd->lo, nd->hi, o, inv, tmin, best_t)) continue;
        if(nd->count == 0)
        {
            if(sp + 2 <= 256)
            {
                stack[sp++] = nd->left;
                stack[sp++] = nd->left + 1;
            }
            continue;
        }
        for(uint32_t i = nd->left; i < nd->left + nd->count; ++i)
        {
            const uint32_t k = B->order[i];
            const double *w = B->w2o + 12 * (size_t)k;
            double oo[3], dd[3];
            for(int r = 0; r < 3; ++r)
            {
                oo[r] = w[4 * r] * o[0] + w[4 * r + 1] * o[1] + w[4 * r + 2] * o[2] + w[4 * r + 3];
                dd[r] = w[4 * r] * d[0] + w[4 * r + 1] * d[1] + w[4 * r + 2] * d[2];
            }
            const uint32_t m = I->inst_mesh[k];
            uint32_t prim;
            double t, u, v;
            /* the coverage filter for an instance of an alpha-tested material */
            orc_alpha_ctx ik;
            const orc_alpha_ctx *iac = NULL;
            if(ac && J->alpha && orc__alpha_tested(&J->scene->mats[I->inst_mat[k]]))
            {
                ik = *ac;
                ik.inst = k;
                iac = &ik;
            }
            if(!d_trace_bvh(I->mesh_bvh[m], NULL, B->mesh_unculled[m], oo, tmin, dd, best_t, cull_mode, any, &prim, &t,
                            &u, &v, iac))
                continue;
            if(any) return 1;
            best_t = t;
            *prim_out = prim;
            *inst_out = k;
            bu = u;
            bv = v;
        }
    }
    *u_out = bu;
    *v_out = bv;
    *t_out = best_t;
    return *prim_out != ORC_MISS;
}

/* CDF inversion sample (independent of the GPU's alias table) */
static void d_env_sample_raw(const orc_pt_env *e, double u0, double u1, double u2, double u3, double *dx, double *dy,
                             double *dz, double *pdf, uint32_t *texel)
{
    (void)u1;
    const uint32_t n = e->w * e->h;
    uint32_t lo = 0, hi = n; /* largest t with cdf[t] <= u0 */
    while(hi - lo > 1)
    {
        uint32_t mid = (lo + hi) >> 1;
        if(e->cdf[mid] <= u0) lo = mid;
        else hi = mid;
    }
    uint32_t t = lo;
    uint32_t i = t % e->w, j = t / e->w;
    double u = ((double)i + u2) / (double)e->w, v = ((double)j + u3) / (double)e->h;
    const double PI = 3.14159265358979323846;
    double phi = (u - 0.5) * 2.0 * PI, theta = v * PI;
    double st = sin(theta);
    *dx = st * sin(phi);
    *dy = cos(theta);
    *dz = -st * cos(phi);
    *pdf = st > 0.0 ? (double)e->weight[t] / (2.0 * PI * PI * st) : 0.0;
    *texel = t;
}

static void d_hit_raw(const orc_pt_job *J, double ox, double oy, double oz, double tmin, double dx, double dy,
                      double dz, double xi, uint32_t *prim, uint32_t *inst, double *u, double *v, double *t)
{
    double o[3] = {ox, oy, oz}, d[3] = {dx, dy, dz};
    *u = *v = 0;
    *t = 1e4;
    *inst = 0;
    const orc_alpha_ctx ac = {J, 0u, xi, 0u, 0u, 0};
    if(J->inst) d_trace_inst(J, o, tmin, d, 1e4, 2, 0, prim, inst, t, u, v, &ac);
    else d_trace(J, o, tmin, d, 1e4, 2, 0, prim, t, u, v, &ac);
}

static int d_occluded_raw(const orc_pt_job *J, double ox, double oy, double oz, double tmin, double dx, double dy,
                          double dz, int cull, uint64_t key)
{
    double o[3] = {ox, oy, oz}, d[3] = {dx, dy, dz}, u, v, t;
    uint32_t prim, inst;
    const orc_alpha_ctx ac = {J, 0u, 0.0, key, ORC_SALT_SHADOW, 0};
    if(J->inst) return d_trace_inst(J, o, tmin, d, 1e4, cull ? 1 : 0, 1, &prim, &inst, &t, &u, &v, &ac);
    return d_trace(J, o, tmin, d, 1e4, cull ? 1 : 0, 1, &prim, &t, &u, &v, &ac);
}

static void d_transmit_raw(const orc_pt_job *J, double ox, double oy, double oz, double tmin, double dx, double dy,
                           double dz, double tmax, int cull, double T[3], uint64_t key)
{
    double o[3] = {ox, oy, oz}, d[3] = {dx, dy, dz}, od[3] = {0, 0, 0};
    T[0] = T[1] = T[2] = 1.0;
    const orc_alpha_ctx ac = {J, 0u, 0.0, key, ORC_SALT_LIGHT_SHADOW, 1};
    for(int k = 0;; ++k)
    {
        uint32_t prim, inst = 0;
        double t, u, v;
        int hit = J->inst ? d_trace_inst(J, o, tmin, d, tmax, cull ? 1 : 0, 0, &prim, &inst, &t, &u, &v, &ac)
                          : d_trace(J, o, tmin, d, tmax, cull ? 1 : 0, 0, &prim, &t, &u, &v, &ac);
        if(!hit) break;
        const uint32_t mat = J->inst ? J->inst->inst_mat[inst] : J->scene->tri_mat[prim];
        const orc_pt_material *m = &J->scene->mats[mat];
        if(m->null_surface && k + 1 < 32)
        {
            tmin = t;
            continue;
        }
        if(!(m->transmission > 0.f) || k + 1 >= 32)
        {
            T[0] = T[1] = T[2] = 0.0;
            return;
        }
        for(int c = 0; c < 3; ++c) T[c] = T[c] * (double)m->base[c] * (double)m->transmission;
        if(J->media && (J->media[mat].flags & 1u))
        {
            /* Beer-Lambert through transmissive volumes: the face from the triangle's normal against
               the ray, in object space for an instance (the world-to-object map of the direction) */
            const float *xyz;
            const uint32_t *ix;
            double dd[3] = {dx, dy, dz};
            if(!J->inst)
            {
                xyz = J->scene->xyz;
                ix = J->scene->idx + 3 * (size_t)prim;
            }
            else
            {
                const uint32_t m = J->inst->inst_mesh[inst];
                xyz = J->inst->mesh_xyz[m];
                ix = J->inst->mesh_idx[m] + 3 * (size_t)prim;
                const double *w = ((const inst_bvh *)J->ibvh)->w2o + 12 * (size_t)inst;
                for(int r = 0; r < 3; ++r) dd[r] = w[4 * r] * dx + w[4 * r + 1] * dy + w[4 * r + 2] * dz;
            }
            const float *a = xyz + 3 * (size_t)ix[0], *b = xyz + 3 * (size_t)ix[1], *c2 = xyz + 3 * (size_t)ix[2];
            double e1[3] = {(double)b[0] - a[0], (double)b[1] - a[1], (double)b[2] - a[2]};
            double e2[3] = {(double)c2[0] - a[0], (double)c2[1] - a[1], (double)c2[2] - a[2]};
            double n[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
            int front = n[0] * dd[0] + n[1] * dd[1] + n[2] * dd[2] < 0.0;
            for(int c = 0; c < 3; ++c)
            {
                double st = (double)J->media[mat].sigma_s[c] + (double)J->media[mat].sigma_a[c];
                od[c] += st * (front ? -t : t);
            }
        }
        tmin = t;
    }
    if(J->media)
        for(int c = 0; c < 3; ++c) T[c] *= exp(-(od[c] > 0 ? od[c] : 0));
}

/* ---- instantiate the estimator ------------------------------------------------------------- */
#define REAL float
#define SFX(n) f_##n
#define RSQRT(x) sqrtf(x)
#define RSIN(x) sinf(x)
#define RCOS(x) cosf(x)
#define RATAN2(y, x) atan2f(y, x)
#define RACOS(x) acosf(x)
#define RFMA(a, b, c) fmaf(a, b, c)
#define RABS(x) fabsf(x)
#define RPOW(x, y) powf(x, y)
#define HIT_RAW f_hit_raw
#define OCC_RAW f_occluded_raw
#define ENV_RAW f_env_sample_raw
#define DRAW_RAW f_draw_raw
#define TRANS_RAW f_transmit_raw
#define RASIN(x) asinf(x)
#define REXP(x) expf(x)
#define RLOG(x) logf(x)
#define RLOG2(x) log2f(x)
#define RFLOOR(x) floorf(x)
#define RATAN(x) atanf(x)
#include "pt_core.inc"
static int f_alpha_accept(const void *ctx, uint32_t prim, float u, float v)
{
    return f_alpha_core((const orc_alpha_ctx *)ctx, prim, u, v);
}
#undef REAL
#undef SFX
#undef RSQRT
#undef RSIN
#undef RCOS
#undef RATAN2
#undef RACOS
#undef RFMA
#undef RABS
#undef RPOW
#undef HIT_RAW
#undef OCC_RAW
#undef ENV_RAW
#undef DRAW_RAW
#undef TRANS_RAW
#undef RASIN
#undef REXP
#undef RLOG
#undef RLOG2
#undef RFLOOR
#undef RATAN

#define REAL double
#define SFX(n) d_##n
#define RSQRT(x) sqrt(x)
#define RSIN(x) sin(x)
#define RCOS(x) cos(x)
#define RATAN2(y, x) atan2(y, x)
#define RACOS(x) acos(x)
#define RFMA(a, b, c) fma(a, b, c)
#define RABS(x) fabs(x)
#define RPOW(x, y) pow(x, y)
#define HIT_RAW d_hit_raw
#define OCC_RAW d_occluded_raw
#define ENV_RAW d_env_sample_raw
#define DRAW_RAW d_draw_raw
#define TRANS_RAW d_transmit_raw
#define RASIN(x) asin(x)
#define REXP(x) exp(x)
#define RLOG(x) log(x)
#define RLOG2(x) log2(x)
#define RFLOOR(x) floor(x)
#define RATAN(x) atan(x)
#include "pt_core.inc"
static int d_alpha_accept(const orc_alpha_ctx *c, uint32_t prim, double u, double v) { return d_alpha_core(c, prim, u, v); }

void orc_sun_light(const float color[3], float intensity, const float spherical_coords[2], float angular_size,
                   orc_pt_light *out)
{
    memset(out, 0, sizeof(*out));
    out->type = 2;
    for(int c = 0; c < 3; ++c) out->color[c] = color[c];
    out->intensity = intensity;
    /* q = q_y(azimuth) q_x(elevation); direction = q (0,0,1) q^-1 = (cos el sin az, -sin el, cos el cos az) */
    double el = spherical_coords[0], az = spherical_coords[1];
    double d[3] = {cos(el) * sin(az), -sin(el), cos(el) * cos(az)};
    double len = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    for(int c = 0; c < 3; ++c) out->direction[c] = (float)(d[c] / len);
    out->range = INFINITY;
    out->angular_size = angular_size;
}

/* ---- single BSDF evaluations (FP64), for the sampling / evaluation consistency tests ---------- */
void orc_bsdf_sample(const orc_pt_material *mt, const double n[3], const double v[3], double eta, const double u[3],
                     double dir[3], double *pdf, double f[3], int *transmission)
{
    d_mat m;
    d_load_mat(mt, 0, &m);
    d_v3 d, fv;
    d_sample_bsdf(&m, d_mk(n[0], n[1], n[2]), d_mk(v[0], v[1], v[2]), eta, u[0], u[1], u[2], &d, pdf, &fv,
                  transmission);
    dir[0] = d.x, dir[1] = d.y, dir[2] = d.z;
    f[0] = fv.x, f[1] = fv.y, f[2] = fv.z;
}

/* one FP64 Henyey-Greenstein phase sample around +z (phase_function.slang:17-31): direction and pdf */
void orc_phase_hg_sample(double x, double y, double g, double dir[3], double *pdf)
{
    d_v3 d = d_sample_phase_hg(x, y, g, pdf);
    dir[0] = d.x, dir[1] = d.y, dir[2] = d.z;
}

double orc_phase_hg(double cos_theta, double g) { return d_phase_hg(cos_theta, g); }

/* chromatic dispersion (FP64): the Cauchy ior of a wavelength and its Rec.709 colour */
double orc_cauchy_ior(double ior, double dispersion, double lambda) { return d_cauchy_ior(ior, dispersion, lambda); }
void orc_lambda_rgb(double lambda, double out[3])
{
    d_v3 c = d_lambda_rgb(lambda);
    out[0] = c.x, out[1] = c.y, out[2] = c.z;
}

void orc_iridescent_fresnel(double outside, double film, const double f0[3], double thickness, double cos1,
                            double out[3])
{
    d_v3 r = d_iridescent_fresnel(outside, film, d_mk(f0[0], f0[1], f0[2]), thickness, cos1);
    out[0] = r.x, out[1] = r.y, out[2] = r.z;
}

double orc_bsdf_eval(const orc_pt_material *mt, const double l[3], const double n[3], const double v[3], double eta,
                     double f[3])
{
    d_mat m;
    d_load_mat(mt, 0, &m);
    double pdf;
    d_v3 fv = d_eval_bsdf(&m, d_mk(l[0], l[1], l[2]), d_mk(n[0], n[1], n[2]), d_mk(v[0], v[1], v[2]), eta, &pdf);
    f[0] = fv.x, f[1] = fv.y, f[2] = fv.z;
    return pdf;
}

/* ---- render ---------------------------------------------------------------------------------- */
static void *pt_worker(void *arg)
{
    orc_pt_job *J = (orc_pt_job *)arg;
    const uint32_t npix = J->cw * J->ch;
    uint64_t st[2] = {0, 0};
    for(;;)
    {
        uint32_t pix = atomic_fetch_add(&J->next, 1u);
        if(pix >= npix) break;
        uint32_t x = J->cx0 + pix % J->cw, y = J->cy0 + pix / J->cw;
        double acc[3] = {0, 0, 0}, sq = 0;
        int covered = 0;
        for(uint32_t s = 0; s < J->spp; ++s)
        {
            uint64_t seq = ((uint64_t)J->batch << 40) ^ ((uint64_t)s * npix + pix);
            double L[3];
            /* the pixel record: coverage from every sample, the G-buffer from the last one */
            orc_pixel *rec = (J->pixels && s + 1 == J->spp) ? &J->pixels[pix] : NULL;
            int hit0 = 0;
            if(J->fp64)
            {
                d_v3 r = d_trace_path(J, x, y, seq, st, rec, &hit0, NULL);
                L[0] = r.x;
                L[1] = r.y;
                L[2] = r.z;
            }
            else
            {
                f_v3 r = f_trace_path(J, x, y, seq, st, rec, &hit0, NULL);
                L[0] = r.x;
                L[1] = r.y;
                L[2] = r.z;
            }
            /* the FP32 twin sums in float like the GPU's accumulation kernel */
            for(int c = 0; c < 3; ++c) acc[c] = J->fp64 ? acc[c] + L[c] : (double)((float)acc[c] + (float)L[c]);
            double lum = 0.2126 * L[0] + 0.7152 * L[1] + 0.0722 * L[2];
            sq += lum * lum;
            covered = covered || hit0;
        }
        if(J->pixels) J->pixels[pix].alpha = covered ? 1.f : 0.f;
        for(int c = 0; c < 3; ++c)
            J->out[3 * (size_t)pix + c] = J->fp64 ? acc[c] / J->spp : (double)((float)acc[c] / (float)J->spp);
        if(J->sq) J->sq[pix] = sq / J->spp;
    }
    atomic_fetch_add(&J->ext, st[0]);
    atomic_fetch_add(&J->shadow, st[1]);
    return NULL;
}

int orc_pt_render(int fp64, const orc_pt_scene *scene, const orc_bvh *bvh, const orc_pt_env *env,
                  const orc_camera *cam, const orc_pt_settings *set, double *out, double *sq, uint64_t *stats,
                  int nthreads)
{
    uint8_t *ts = (uint8_t *)calloc(scene->ntri ? scene->ntri : 1, 1);
    for(uint32_t i = 0; i < scene->ntri; ++i)
    {
        uint32_t m = scene->tri_mat[i];
        ts[i] = (m < scene->nmat && orc_material_unculled(&scene->mats[m])) ? 1 : 0;
    }
    orc_pt_job J;
    memset(&J, 0, sizeof(J));
    J.scene = scene;
    J.dispersion = orc__any_dispersive(scene);
    J.alpha = orc__any_alpha(scene);
    J.bvh = bvh;
    J.env = env;
    J.cam = cam;
    J.twosided = ts;
    J.seed = set->seed;
    J.batch = set->batch;
    J.spp = set->spp;
    J.max_depth = set->max_depth;
    J.rr_depth = set->rr_depth;
    J.mis_mode = set->mis_mode;
    J.disable_material = set->disable_material;
    J.draw_skybox = set->draw_skybox;
    J.max_path_beta = set->max_path_beta;
    J.environment = set->environment;
    J.lights = set->lights;
    J.num_lights = set->lights ? set->num_lights : 0;
    J.suppress_caustics = set->suppress_caustics;
    J.pixels = set->pixels;
    J.clip_near = set->clip_near > 0.f ? set->clip_near : 0.1f;
    orc_medium *media = orc_media_table(scene, set, &J.cam_medium);
    J.media = media;
    J.cx0 = set->crop[0];
    J.cy0 = set->crop[1];
    J.cw = set->crop[2] ? set->crop[2] : cam->width;
    J.ch = set->crop[3] ? set->crop[3] : cam->height;
    J.out = out;
    J.sq = sq;
    J.fp64 = fp64;
    atomic_init(&J.next, 0u);
    atomic_init(&J.ext, 0ull);
    atomic_init(&J.shadow, 0ull);
    int n = orc__run_threads(pt_worker, &J, nthreads);
    if(stats)
    {
        stats[0] = atomic_load(&J.ext);
        stats[1] = atomic_load(&J.shadow);
    }
    free(ts);
    free(media);
    return n;
}

/* ---- variance split (FP64): how much of a pixel's variance a radiance cache could remove --------
   Each sample traces its path twice with the same random numbers up to the surface that segment
   fork_depth reaches, and with independent streams after it (d_fork). With L = prefix + tail:
     var_plain = Var(lum L)                      per-sample variance of the plain estimator
     var_tail  = E[(lum L_a - lum L_b)^2 / 2]    = E[Var(lum tail | prefix)], the part an exact cache
                                                  at that surface (zero variance) would remove
   split[pix] = {mean lum L_a, var_plain, var_tail, fraction of samples that reached the fork}. */
static void *pt_split_worker(void *arg)
{
    orc_pt_job *J = (orc_pt_job *)arg;
    const uint32_t npix = J->cw * J->ch;
    uint64_t st[2] = {0, 0};
    for(;;)
    {
        uint32_t pix = atomic_fetch_add(&J->next, 1u);
        if(pix >= npix) break;
        uint32_t x = J->cx0 + pix % J->cw, y = J->cy0 + pix / J->cw;
        double s1 = 0, s2 = 0, tail = 0, forks = 0;
        for(uint32_t s = 0; s < J->spp; ++s)
        {
            uint64_t seq = ((uint64_t)J->batch << 40) ^ ((uint64_t)s * npix + pix);
            uint64_t fseq = (1ull << 61) | (2ull * ((uint64_t)s * npix + pix));
            int hit0 = 0;
            d_fork fa = {fseq, {0, 0, 0}, 0}, fb = {fseq + 1, {0, 0, 0}, 0};
            d_v3 a = d_trace_path(J, x, y, seq, st, NULL, &hit0, &fa);
            d_v3 b = d_trace_path(J, x, y, seq, NULL, NULL, &hit0, &fb);
            double la = 0.2126 * a.x + 0.7152 * a.y + 0.0722 * a.z;
            double lb = 0.2126 * b.x + 0.7152 * b.y + 0.0722 * b.z;
            s1 += la;
            s2 += la * la;
            tail += 0.5 * (la - lb) * (la - lb);
            forks += fa.forked ? 1 : 0;
        }
        double n = (double)J->spp, m = s1 / n;
        double *o = J->split + 4 * (size_t)pix;
        o[0] = m;
        o[1] = n > 1 ? (s2 - n * m * m) / (n - 1) : 0;
        o[2] = tail / n;
        o[3] = forks / n;
    }
    atomic_fetch_add(&J->ext, st[0]);
    atomic_fetch_add(&J->shadow, st[1]);
    return NULL;
}

int orc_pt_variance_split(const orc_pt_scene *scene, const orc_bvh *bvh, const orc_pt_env *env, const orc_camera *cam,
                          const orc_pt_settings *set, uint32_t fork_depth, double *split, uint64_t *stats,
                          int nthreads)
{
    uint8_t *ts = (uint8_t *)calloc(scene->ntri ? scene->ntri : 1, 1);
    for(uint32_t i = 0; i < scene->ntri; ++i)
    {
        uint32_t m = scene->tri_mat[i];
        ts[i] = (m < scene->nmat && orc_material_unculled(&scene->mats[m])) ? 1 : 0;
    }
    orc_pt_job J;
    memset(&J, 0, sizeof(J));
    J.scene = scene;
    J.dispersion = orc__any_dispersive(scene);
    J.alpha = orc__any_alpha(scene);
    J.bvh = bvh;
    J.env = env;
    J.cam = cam;
    J.twosided = ts;
    J.seed = set->seed;
    J.batch = set->batch;
    J.spp = set->spp;
    J.max_depth = set->max_depth;
    J.rr_depth = set->rr_depth;
    J.mis_mode = set->mis_mode;
    J.disable_material = set->disable_material;
    J.draw_skybox = set->draw_skybox;
    J.max_path_beta = set->max_path_beta;
    J.environment = set->environment;
    J.lights = set->lights;
    J.num_lights = set->lights ? set->num_lights : 0;
    J.suppress_caustics = set->suppress_caustics;
    J.clip_near = set->clip_near > 0.f ? set->clip_near : 0.1f;
    orc_medium *media = orc_media_table(scene, set, &J.cam_medium);
    J.media = media;
    J.cx0 = set->crop[0];
    J.cy0 = set->crop[1];
    J.cw = set->crop[2] ? set->crop[2] : cam->width;
    J.ch = set->crop[3] ? set->crop[3] : cam->height;
    J.fp64 = 1;
    J.fork_depth = fork_depth;
    J.split = split;
    atomic_init(&J.next, 0u);
    atomic_init(&J.ext, 0ull);
    atomic_init(&J.shadow, 0ull);
    int n = orc__run_threads(pt_split_worker, &J, nthreads);
    if(stats)
    {
        stats[0] = atomic_load(&J.ext);
        stats[1] = atomic_load(&J.shadow);
    }
    free(ts);
    free(media);
    return n;
}

int orc_pt_render_instanced(const orc_pt_scene *scene, const orc_pt_instances *inst, const orc_pt_env *env,
                            const orc_camera *cam, const orc_pt_settings *set, double *out, double *sq,
                            uint64_t *stats, int nthreads)
{
    inst_bvh *B = build_inst_bvh(inst);
    for(uint32_t i = 0; i < inst->num_instances; ++i)
        if(inst->inst_mat[i] < scene->nmat && orc_material_unculled(&scene->mats[inst->inst_mat[i]]))
            B->mesh_unculled[inst->inst_mesh[i]] = 1;
    orc_pt_job J;
    memset(&J, 0, sizeof(J));
    J.scene = scene;
    J.dispersion = orc__any_dispersive(scene);
    J.alpha = orc__any_alpha(scene);
    J.inst = inst;
    J.ibvh = B;
    J.env = env;
    J.cam = cam;
    J.seed = set->seed;
    J.batch = set->batch;
    J.spp = set->spp;
    J.max_depth = set->max_depth;
    J.rr_depth = set->rr_depth;
    J.mis_mode = set->mis_mode;
    J.disable_material = set->disable_material;
    J.draw_skybox = set->draw_skybox;
    J.max_path_beta = set->max_path_beta;
    J.environment = set->environment;
    J.lights = set->lights;
    J.num_lights = set->lights ? set->num_lights : 0;
    J.suppress_caustics = set->suppress_caustics;
    J.pixels = set->pixels;
    J.clip_near = set->clip_near > 0.f ? set->clip_near : 0.1f;
    orc_medium *media = orc_media_table(scene, set, &J.cam_medium);
    J.media = media;
    J.cx0 = set->crop[0];
    J.cy0 = set->crop[1];
    J.cw = set->crop[2] ? set->crop[2] : cam->width;
    J.ch = set->crop[3] ? set->crop[3] : cam->height;
    J.out = out;
    J.sq = sq;
    J.fp64 = 1;
    atomic_init(&J.next, 0u);
    atomic_init(&J.ext, 0ull);
    atomic_init(&J.shadow, 0ull);
    int n = orc__run_threads(pt_worker, &J, nthreads);
    if(stats)
    {
        stats[0] = atomic_load(&J.ext);
        stats[1] = atomic_load(&J.shadow);
    }
    free_inst_bvh(B);
    free(media);
    return n;
}

/* the material record's size, checked by the Python binding against its own record */
uint32_t orc_pt_material_size(void) { return (uint32_t)sizeof(orc_pt_material); }

void orc_pt_env_tables(const float *rgb, uint32_t w, uint32_t h, float *weight, double *cdf)
{
    const size_t n = (size_t)w * h;
    double *wt = (double *)malloc(sizeof(double) * n);
    double total = 0;
    for(size_t t = 0; t < n; ++t)
    {
        uint32_t j = (uint32_t)(t / w);
        double theta = ((double)j + 0.5) * 3.14159265358979323846 / (double)h;
        double lum = 0.2126 * rgb[3 * t] + 0.7152 * rgb[3 * t + 1] + 0.0722 * rgb[3 * t + 2];
        wt[t] = lum > 0 ? lum * sin(theta) : 0;
        total += wt[t];
    }
    /* a black map: uniform weights (the GPU table builder's fallback), so pdfs stay finite */
    if(!(total > 0))
        for(size_t t = 0; t < n; ++t) wt[t] = 1.0;
    if(!(total > 0)) total = (double)n;
    double run = 0;
    for(size_t t = 0; t < n; ++t)
    {
        cdf[t] = run / total;
        run += wt[t];
        weight[t] = (float)(wt[t] * (double)n / total);
    }
    cdf[n] = 1.0;
    free(wt);
}

void orc_pt_env_procedural(uint32_t w, uint32_t h, const float sun_dir[3], double peak, double width, float *rgb)
{
    const double PI = 3.14159265358979323846;
    for(uint32_t j = 0; j < h; ++j)
        for(uint32_t i = 0; i < w; ++i)
        {
            double u = ((double)i + 0.5) / w, v = ((double)j + 0.5) / h;
            double phi = (u - 0.5) * 2.0 * PI, theta = v * PI;
            double st = sin(theta);
            double d[3] = {st * sin(phi), cos(theta), -st * cos(phi)};
            /* environment_white (procedural_environment.slang:7-11) */
            double sky = d[1] > 0 ? 0.6 + (1.3 - 0.6) * d[1] : 0.6 + (0.1 - 0.6) * (-d[1]);
            double cg = d[0] * sun_dir[0] + d[1] * sun_dir[1] + d[2] * sun_dir[2];
            double sun = peak * exp((cg - 1.0) / width);
            size_t t = (size_t)j * w + i;
            rgb[3 * t] = rgb[3 * t + 1] = rgb[3 * t + 2] = (float)(sky + sun);
        }
}

/* one texture sample (FP64 restatement), for the sampling pins */
void orc_tex_sample(const orc_tex_rec *rec, const uint32_t *texels, double u, double v, double lambda, double out[4])
{
    d_tsample(rec, texels, u, v, lambda, out);
}
