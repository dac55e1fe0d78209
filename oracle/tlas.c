/* Two-level ray queries on the CPU. TEST INFRASTRUCTURE ONLY (the checker of vkg_tlas_*).
 *
 * Every instance is visited in input order (no top-level tree): the world ray moves to object space
 * with the instance's world -> object 3x4 transform, row by row, with separately rounded float
 * operations (x, y, z terms left to right, translation last; -ffp-contract=off), and runs through
 * the instance's mesh BVH (orc_bvh_trace1, whose hits equal the reference's ray-triangle test). The
 * closest hit is the smallest t, then the smallest instance, then the smallest triangle; any hit
 * stops at the first occluding instance. */
#include "oracle.h"

#include <stdatomic.h>
#include <string.h>

int orc__run_threads(void *(*fn)(void *), void *arg, int nthreads);

typedef struct
{
    uint32_t prim, inst;
    float t, u, v;
    uint32_t pad[3];
} orc_inst_hit; /* 32 B, the layout of vkg_inst_hit */

typedef struct
{
    const orc_bvh *const *blas;
    const float *w2o;        /* [ninst][12] */
    const uint32_t *inst_blas;
    uint32_t ninst;
    const orc_ray *rays;
    uint32_t nray;
    int cull;
    orc_inst_hit *hits;
    uint32_t *occluded;
    atomic_uint next;
} tl_job;

static void to_object(const float *m, const float o[3], const float d[3], float oo[3], float dd[3])
{
    for(int r = 0; r < 3; ++r)
    {
        const float *w = m + 4 * r;
        oo[r] = ((w[0] * o[0] + w[1] * o[1]) + w[2] * o[2]) + w[3];
        dd[r] = (w[0] * d[0] + w[1] * d[1]) + w[2] * d[2];
    }
}

static void trace_two_level(const tl_job *J, const orc_ray *ray, orc_inst_hit *hit, uint32_t *occ)
{
    orc_inst_hit best = {ORC_MISS, ORC_MISS, 0.f, 0.f, 0.f, {0, 0, 0}};
    for(uint32_t i = 0; i < J->ninst; ++i)
    {
        const orc_bvh *b = J->blas[J->inst_blas[i]];
        if(b->num_tris == 0) continue;
        orc_ray o;
        to_object(J->w2o + 12 * (size_t)i, ray->o, ray->d, o.o, o.d);
        o.tmin = ray->tmin;
        o.tmax = ray->tmax;
        if(occ)
        {
            uint32_t oc = 0;
            orc_bvh_trace1(b, &o, J->cull, NULL, 1, NULL, &oc);
            if(oc)
            {
                *occ = 1;
                return;
            }
            continue;
        }
        orc_hit h;
        orc_bvh_trace1(b, &o, J->cull, NULL, 0, &h, NULL);
        if(h.prim == ORC_MISS) continue;
        if(best.prim == ORC_MISS || h.t < best.t || (h.t == best.t && (i < best.inst || (i == best.inst && h.prim < best.prim))))
        {
            best.prim = h.prim;
            best.inst = i;
            best.t = h.t;
            best.u = h.u;
            best.v = h.v;
        }
    }
    if(occ) *occ = 0;
    if(hit) *hit = best;
}

static void *tl_worker(void *arg)
{
    tl_job *J = (tl_job *)arg;
    for(;;)
    {
        uint32_t begin = atomic_fetch_add(&J->next, 16u);
        if(begin >= J->nray) break;
        uint32_t end = begin + 16u < J->nray ? begin + 16u : J->nray;
        for(uint32_t r = begin; r < end; ++r)
            trace_two_level(J, &J->rays[r], J->hits ? &J->hits[r] : NULL, J->occluded ? &J->occluded[r] : NULL);
    }
    return NULL;
}

/* cull: 0 none, 1 back faces (object-space facing) */
int orc_tlas_closest_hit(const orc_bvh *const *blas, const float *w2o, const uint32_t *inst_blas, uint32_t ninst,
                         const orc_ray *rays, uint32_t nray, int cull, void *hits, int nthreads)
{
    tl_job J = {blas, w2o, inst_blas, ninst, rays, nray, cull, (orc_inst_hit *)hits, NULL, 0};
    return orc__run_threads(tl_worker, &J, nthreads);
}

int orc_tlas_any_hit(const orc_bvh *const *blas, const float *w2o, const uint32_t *inst_blas, uint32_t ninst,
                     const orc_ray *rays, uint32_t nray, int cull, uint32_t *occluded, int nthreads)
{
    tl_job J = {blas, w2o, inst_blas, ninst, rays, nray, cull, NULL, occluded, 0};
    return orc__run_threads(tl_worker, &J, nthreads);
}
