/*
 * Ray-primitive intersection restated from the reference. TEST INFRASTRUCTURE ONLY (CPU oracle).
 *
 *   orc_intersect_ray_triangle : src/intersection.cpp:114-129 (Moeller-Trumbore, two-sided,
 *                                |det| < 10e-10 rejected, no t-range test)
 *   orc_intersect_ray_aabb     : src/intersection.cpp:308-312 -> :219-227 (OBB(AABB, identity))
 *                                -> :152-184 (slab test, parallel threshold 1e-10)
 * The op order follows glm's scalar dot/cross (left-to-right sums, see ref_shim/glm_shim.hpp).
 *
 * Closest-hit contract on top (project-defined, mirrors the RT pipeline's closest-hit):
 * accept INTERSECT with t in (tmin, tmax), keep the smallest t, ties -> smaller triangle id.
 * Optional back-face culling: front face <=> det > 0 (counter-clockwise seen from the origin).
 */
#include "oracle.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stdlib.h>
#include <unistd.h>

static inline float dot3(const float a[3], const float b[3]) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

static inline void cross3(const float a[3], const float b[3], float r[3])
{
    r[0] = a[1] * b[2] - b[1] * a[2];
    r[1] = a[2] * b[0] - b[2] * a[0];
    r[2] = a[0] * b[1] - b[0] * a[1];
}

/* returns det through *det_out so callers can apply the facing rule without recomputing */
static int mt(const float o[3], const float d[3], const float *v0, const float *v1, const float *v2, float out[3],
              float *det_out)
{
    float e1[3] = {v1[0] - v0[0], v1[1] - v0[1], v1[2] - v0[2]};
    float e2[3] = {v2[0] - v0[0], v2[1] - v0[1], v2[2] - v0[2]};
    float pvec[3];
    cross3(d, e2, pvec);
    float det = dot3(e1, pvec);
    *det_out = det;
    const float epsilon = 10.0e-10f;
    if(det > -epsilon && det < epsilon) return 0;
    float inv_det = 1.0f / det;
    float tvec[3] = {o[0] - v0[0], o[1] - v0[1], o[2] - v0[2]};
    float u = inv_det * dot3(tvec, pvec);
    if(u < 0.0f || u > 1.0f) return 0;
    float qvec[3];
    cross3(tvec, e1, qvec);
    float v = dot3(d, qvec) * inv_det;
    if(v < 0.0f || (u + v) > 1.0f) return 0;
    out[0] = dot3(e2, qvec) * inv_det;
    out[1] = u;
    out[2] = v;
    return 1;
}

int orc_intersect_ray_triangle(const float o[3], const float d[3], const float tri[9], float out[3])
{
    float det;
    out[0] = out[1] = out[2] = 0.f;
    return mt(o, d, tri, tri + 3, tri + 6, out, &det);
}

int orc_intersect_ray_triangle_cull(const float o[3], const float d[3], const float tri[9], int cull_back,
                                    float out[3])
{
    float det;
    out[0] = out[1] = out[2] = 0.f;
    int r = mt(o, d, tri, tri + 3, tri + 6, out, &det);
    if(r && cull_back && det < 0.f) return 0;
    return r;
}

int orc_intersect_ray_aabb(const float o[3], const float d[3], const float bmin[3], const float bmax[3], float *t_out)
{
    /* OBB(aabb, mat4(1)): center, unit axes, half extents (intersection.cpp:219-227) */
    float center[3], half[3];
    for(int i = 0; i < 3; ++i)
    {
        float c = (bmax[i] + bmin[i]) / 2.f;
        /* (mat4(1) * vec4(c, 1)).xyz evaluates as ((1*c.x + 0*c.y) + 0*c.z) + 0*1 per row */
        center[i] = c;
        half[i] = ((bmax[i] - bmin[i]) / 2.f) * 1.0f;
    }
    float cx[3];
    for(int r = 0; r < 3; ++r)
    {
        float col[4][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {0, 0, 0}};
        cx[r] = col[0][r] * center[0] + col[1][r] * center[1] + col[2][r] * center[2] + col[3][r] * 1.0f;
    }
    const float axis[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    const float epsilon = 1e-10f;
    float t_min = -FLT_MAX, t_max = FLT_MAX;
    float p[3] = {cx[0] - o[0], cx[1] - o[1], cx[2] - o[2]};
    *t_out = 0.f;
    for(int i = 0; i < 3; i++)
    {
        float e = dot3(axis[i], p);
        float f = dot3(axis[i], d);
        if(fabsf(f) > epsilon)
        {
            float t1 = (e + half[i]) / f;
            float t2 = (e - half[i]) / f;
            if(t1 > t2)
            {
                float tmp = t1;
                t1 = t2;
                t2 = tmp;
            }
            if(t1 > t_min) t_min = t1;
            if(t2 < t_max) t_max = t2;
            if(t_min > t_max) return 0;
            if(t_max < 0) return 0;
        }
        else if((-e - half[i]) > 0 || (-e + half[i]) < 0) { return 0; }
    }
    *t_out = t_min > 0 ? t_min : t_max;
    return 1;
}

/* ---- brute force over host threads ----------------------------------------------------- */
typedef struct {
    const float *xyz;
    const uint32_t *idx;
    uint32_t ntri;
    const orc_ray *rays;
    uint32_t nray;
    orc_hit *hits;
    uint32_t *occluded;
    int cull;
    atomic_uint next;
} bf_job;

static void *bf_worker(void *arg)
{
    bf_job *j = (bf_job *)arg;
    for(;;)
    {
        uint32_t begin = atomic_fetch_add(&j->next, 16u);
        if(begin >= j->nray) break;
        uint32_t end = begin + 16u < j->nray ? begin + 16u : j->nray;
        for(uint32_t r = begin; r < end; ++r)
        {
            const orc_ray *ray = &j->rays[r];
            orc_hit best = {ORC_MISS, ray->tmax, 0.f, 0.f};
            int occ = 0;
            for(uint32_t i = 0; i < j->ntri && !occ; ++i)
            {
                const float *v0 = j->xyz + 3 * (size_t)j->idx[3 * (size_t)i];
                const float *v1 = j->xyz + 3 * (size_t)j->idx[3 * (size_t)i + 1];
                const float *v2 = j->xyz + 3 * (size_t)j->idx[3 * (size_t)i + 2];
                float tuv[3], det;
                if(!mt(ray->o, ray->d, v0, v1, v2, tuv, &det)) continue;
                if(j->cull && det < 0.f) continue;
                float t = tuv[0];
                if(!(t > ray->tmin && t < ray->tmax)) continue;
                if(j->occluded) { occ = 1; break; }
                if(t < best.t || (t == best.t && i < best.prim))
                {
                    best.prim = i;
                    best.t = t;
                    best.u = tuv[1];
                    best.v = tuv[2];
                }
            }
            if(j->occluded) { j->occluded[r] = (uint32_t)occ; }
            else
            {
                if(best.prim == ORC_MISS) { best.t = 0.f; }
                j->hits[r] = best;
            }
        }
    }
    return NULL;
}

static int run_threads(void *(*fn)(void *), void *arg, int nthreads)
{
    if(nthreads <= 0) nthreads = (int)sysconf(_SC_NPROCESSORS_ONLN);
    if(nthreads < 1) nthreads = 1;
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)nthreads);
    for(int i = 0; i < nthreads; ++i) pthread_create(&th[i], NULL, fn, arg);
    for(int i = 0; i < nthreads; ++i) pthread_join(th[i], NULL);
    free(th);
    return nthreads;
}

int orc_closest_hit_bruteforce(const float *xyz, const uint32_t *idx, uint32_t ntri, const orc_ray *rays,
                               uint32_t nray, orc_hit *hits, int nthreads, int cull_back)
{
    bf_job j = {xyz, idx, ntri, rays, nray, hits, NULL, cull_back, 0};
    return run_threads(bf_worker, &j, nthreads);
}

int orc_any_hit_bruteforce(const float *xyz, const uint32_t *idx, uint32_t ntri, const orc_ray *rays,
                           uint32_t nray, uint32_t *occluded, int nthreads, int cull_back)
{
    bf_job j = {xyz, idx, ntri, rays, nray, NULL, occluded, cull_back, 0};
    return run_threads(bf_worker, &j, nthreads);
}

/* shared with lbvh.c */
int orc__run_threads(void *(*fn)(void *), void *arg, int nthreads) { return run_threads(fn, arg, nthreads); }
int orc__mt(const float o[3], const float d[3], const float *v0, const float *v1, const float *v2, float out[3],
            float *det)
{
    return mt(o, d, v0, v1, v2, out, det);
}
