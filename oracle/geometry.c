/*
 * Scene geometry restated / defined for the benchmark workloads. TEST INFRASTRUCTURE ONLY.
 *
 * orc_icosphere: src/Geometry.cpp:566-613 (Geometry::IcoSphere) with tessellate() from
 *   src/Geometry.cpp:141-192: every subdivided triangle appends 3 NEW (unshared) vertices
 *   ac = k, ab = k+1, bc = k+2 and emits {a,ab,ac, ab,b,bc, ac,bc,c, ac,ab,bc}; positions are
 *   re-projected as radius * normalize(va + vb) (the tessellation-control lambda :588-596).
 *   IcoSphere(1, 5) -> 20,472 vertices, 20,480 triangles.
 * orc_cubesphere: project-defined sphere mesh with 6 * n * n * 2 triangles (n = 16 -> 3,072),
 *   used because IcoSphere only yields 20 * 4^k triangles. Outward counter-clockwise faces.
 * orc_cornell_scene: 5-quad Cornell box spanning [-1,1]^3, open toward +z, faces pointing
 *   inward, followed by `nspheres` cube-spheres with PCG32-drawn radius / centre / material.
 */
#include "oracle.h"

#include <math.h>
#include <string.h>

static inline void normalize_scale(const float v[3], float radius, float out[3])
{
    /* radius * glm::normalize(v) == radius * (v * (1 / sqrt(dot(v, v)))) */
    float d = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
    float inv = 1.0f / sqrtf(d);
    for(int i = 0; i < 3; ++i) out[i] = radius * (v[i] * inv);
}

uint32_t orc_icosphere_counts(uint32_t tess, uint32_t *num_tris)
{
    uint32_t nv = 12, nt = 20;
    for(uint32_t i = 0; i < tess; ++i)
    {
        nv += 3 * nt;
        nt *= 4;
    }
    if(num_tris) *num_tris = nt;
    return nv;
}

void orc_icosphere(float radius, uint32_t tess, float *xyz, uint32_t *idx)
{
    const float phi = 1.61803398874989484820f; /* std::numbers::phi_v<float> */
    const float e1 = radius / sqrtf(1.f + phi * phi);
    const float e2 = phi * e1;
    const float base[12][3] = {{-e1, e2, 0},  {e1, e2, 0},  {-e1, -e2, 0}, {e1, -e2, 0}, {0, -e1, e2},  {0, e1, e2},
                               {0, -e1, -e2}, {0, e1, -e2}, {e2, 0, -e1},  {e2, 0, e1},  {-e2, 0, -e1}, {-e2, 0, e1}};
    const uint32_t faces[60] = {0, 11, 5, 0, 5,  1,  0,  1, 7, 0, 7,  10, 0, 10, 11, 1, 5, 9, 5, 11,
                                4, 11, 10, 2, 10, 7,  6,  7, 1, 8, 3,  9,  4, 3,  4, 2, 3, 2, 6,  3,
                                6, 8,  3,  8, 9,  4,  9,  5, 2, 4, 11, 6,  2, 10, 8, 6, 7, 9, 8,  1};
    uint32_t nt_final;
    orc_icosphere_counts(tess, &nt_final);
    memcpy(xyz, base, sizeof(base));
    uint32_t nv = 12, nt = 20;
    /* ping-pong the index list inside the output buffer's tail is awkward: keep two buffers on the
       caller's output by building each level into the front and copying */
    uint32_t *cur = idx;
    memcpy(cur, faces, sizeof(faces));
    for(uint32_t it = 0; it < tess; ++it)
    {
        /* new indices are 4x larger: build from the back so the input is never overwritten early */
        for(int64_t j = (int64_t)nt - 1; j >= 0; --j)
        {
            uint32_t a = cur[3 * j], b = cur[3 * j + 1], c = cur[3 * j + 2];
            uint32_t k = nv + 3 * (uint32_t)j;
            uint32_t *o = cur + 12 * j;
            const uint32_t ni[12] = {a, k + 1, k, k + 1, b, k + 2, k, k + 2, c, k, k + 1, k + 2};
            float va[3], vb[3], vc[3], s[3];
            memcpy(va, xyz + 3 * a, 12);
            memcpy(vb, xyz + 3 * b, 12);
            memcpy(vc, xyz + 3 * c, 12);
            /* ab = k+1, ac = k, bc = k+2 */
            for(int q = 0; q < 3; ++q) s[q] = va[q] + vb[q];
            normalize_scale(s, radius, xyz + 3 * (k + 1));
            for(int q = 0; q < 3; ++q) s[q] = va[q] + vc[q];
            normalize_scale(s, radius, xyz + 3 * k);
            for(int q = 0; q < 3; ++q) s[q] = vb[q] + vc[q];
            normalize_scale(s, radius, xyz + 3 * (k + 2));
            memcpy(o, ni, sizeof(ni));
        }
        nv += 3 * nt;
        nt *= 4;
    }
    (void)nt_final;
}

/* face frames (n, u) with v = n x u so that u x v = n: counter-clockwise (u,v) quads face outward */
static const float CS_N[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
static const float CS_U[6][3] = {{0, 0, -1}, {0, 0, 1}, {1, 0, 0}, {1, 0, 0}, {1, 0, 0}, {-1, 0, 0}};

void orc_cubesphere(float radius, const float center[3], uint32_t n, float *xyz, uint32_t *idx, uint32_t vbase)
{
    uint32_t vpf = (n + 1) * (n + 1);
    for(uint32_t f = 0; f < 6; ++f)
    {
        const float *N = CS_N[f], *U = CS_U[f];
        float V[3] = {N[1] * U[2] - U[1] * N[2], N[2] * U[0] - U[2] * N[0], N[0] * U[1] - U[0] * N[1]};
        for(uint32_t j = 0; j <= n; ++j)
            for(uint32_t i = 0; i <= n; ++i)
            {
                float a = (float)(2 * i) / (float)n - 1.0f;
                float b = (float)(2 * j) / (float)n - 1.0f;
                float q[3], p[3];
                for(int c = 0; c < 3; ++c) q[c] = (N[c] + a * U[c]) + b * V[c];
                normalize_scale(q, radius, p);
                float *dst = xyz + 3 * (size_t)(f * vpf + j * (n + 1) + i);
                for(int c = 0; c < 3; ++c) dst[c] = p[c] + center[c];
            }
        for(uint32_t j = 0; j < n; ++j)
            for(uint32_t i = 0; i < n; ++i)
            {
                uint32_t v00 = vbase + f * vpf + j * (n + 1) + i;
                uint32_t v10 = v00 + 1, v01 = v00 + (n + 1), v11 = v01 + 1;
                uint32_t *t = idx + 6 * (size_t)((f * n + j) * n + i);
                t[0] = v00; t[1] = v10; t[2] = v11;
                t[3] = v00; t[4] = v11; t[5] = v01;
            }
    }
}

void orc_cornell_sphere_params(uint64_t seed, uint64_t stream, uint32_t nspheres, orc_sphere_params *out)
{
    orc_pcg32 g;
    orc_pcg32_seed(&g, seed, stream);
    for(uint32_t s = 0; s < nspheres; ++s)
    {
        orc_sphere_params *p = &out[s];
        p->radius = 0.1f + 0.3f * orc_u01(orc_pcg32_next(&g));
        float lo = -1.0f + p->radius, hi = 1.0f - p->radius;
        for(int c = 0; c < 3; ++c) p->center[c] = lo + (hi - lo) * orc_u01(orc_pcg32_next(&g));
        p->roughness = 0.05f + 0.95f * orc_u01(orc_pcg32_next(&g));
        p->metalness = orc_u01(orc_pcg32_next(&g)) < 0.3f ? 1.0f : 0.0f;
        for(int c = 0; c < 3; ++c) p->base[c] = 0.1f + 0.8f * orc_u01(orc_pcg32_next(&g));
    }
}

/* 20 vertices, 10 triangles; materials 0 = white (back, floor, ceiling), 1 = red (left), 2 = green (right) */
static const float CB_V[20][3] = {
        {-1, -1, -1}, {1, -1, -1}, {1, 1, -1},  {-1, 1, -1},  /* back  z=-1, faces +z */
        {-1, -1, 1},  {1, -1, 1},  {1, -1, -1}, {-1, -1, -1}, /* floor y=-1, faces +y */
        {-1, 1, -1},  {1, 1, -1},  {1, 1, 1},   {-1, 1, 1},   /* ceiling y=+1, faces -y */
        {-1, -1, 1},  {-1, -1, -1}, {-1, 1, -1}, {-1, 1, 1},  /* left x=-1, faces +x */
        {1, -1, -1},  {1, -1, 1},  {1, 1, 1},   {1, 1, -1}};  /* right x=+1, faces -x */
static const uint32_t CB_MAT[5] = {0, 0, 0, 1, 2};

void orc_cornell_scene(uint64_t seed, uint64_t stream, uint32_t nspheres, uint32_t n, float *xyz, uint32_t *idx,
                       uint32_t *tri_material)
{
    memcpy(xyz, CB_V, sizeof(CB_V));
    for(uint32_t q = 0; q < 5; ++q)
    {
        uint32_t a = 4 * q;
        uint32_t *t = idx + 6 * q;
        t[0] = a; t[1] = a + 1; t[2] = a + 2;
        t[3] = a; t[4] = a + 2; t[5] = a + 3;
        if(tri_material) tri_material[2 * q] = tri_material[2 * q + 1] = CB_MAT[q];
    }
    orc_sphere_params p[1024];
    orc_sphere_params *pp = p;
    if(nspheres > 1024) return;
    orc_cornell_sphere_params(seed, stream, nspheres, pp);
    uint32_t vps = 6 * (n + 1) * (n + 1), tps = 12 * n * n;
    for(uint32_t s = 0; s < nspheres; ++s)
    {
        uint32_t vb = 20 + s * vps;
        orc_cubesphere(pp[s].radius, pp[s].center, n, xyz + 3 * (size_t)vb, idx + 3 * (size_t)(10 + s * tps), vb);
        if(tri_material)
            for(uint32_t t = 0; t < tps; ++t) tri_material[10 + s * tps + t] = 3 + s;
    }
}
