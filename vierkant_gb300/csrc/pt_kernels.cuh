// Wavefront path-tracer kernels shared by the single-scene tracer (pathtrace.cu) and the batch
// renderer (batch.cu). The queue kernels are templated on a scene resolver: `single_scene` (one
// scene per launch, its parameters in the kernel arguments) or `job_table` (every path carries the
// index of its job in a device table). Everything lives in an anonymous namespace: each translation
// unit instantiates its own kernels.
#pragma once

#include "nrc.cuh"
#include "light.cuh"
#include "medium.cuh"
#include "pathtrace.cuh"
#include "pixel.cuh"
#include "texture.cuh"
#include "tlas.cuh"
#include "traverse.cuh"

#include <cmath>
#include <limits>
#include <type_traits>
#include <vector>

namespace vkg
{
// vertex and index arrays of one mesh of an instanced scene (device)
struct mesh_ref
{
    const float *xyz;
    const uint32_t *idx;
    const float *nrm; // unit vertex normals (3 floats per vertex) or nullptr: shade with the face normal
    const float *uv;  // texture coordinates (2 floats per vertex) or nullptr: no textures
    const float *tng; // unit vertex tangents (3 floats per vertex) or nullptr: no normal maps
};
}// namespace vkg

// a scene: geometry, materials, its BVH and its environment tables
struct vkg_scene
{
    vkg_bvh *bvh = nullptr;         // single-level scenes
    float *xyz = nullptr;
    uint32_t *idx = nullptr;
    uint32_t *tri_mat = nullptr;
    vkg_material *mats = nullptr;
    uint32_t num_tris = 0, num_vertices = 0, num_materials = 0;
    vkg::env_tables env;
    // instanced scenes: meshes (owned copies + their BLASes) and the two-level BVH over the instances
    vkg_tlas *tlas = nullptr;
    std::vector<vkg_bvh *> blas;
    std::vector<float *> mesh_xyz;
    std::vector<uint32_t *> mesh_idx;
    std::vector<float *> mesh_nrm;       // per mesh: unit vertex normals or nullptr
    std::vector<uint32_t> mesh_vertices; // per mesh: vertex count
    std::vector<vkg::mesh_ref> h_meshes; // host copy of d_meshes
    std::vector<float *> mesh_uv, mesh_tng;
    float *nrm = nullptr;                // single-level scenes: unit vertex normals or nullptr
    float *uv = nullptr, *tng = nullptr; // single-level scenes: texture coordinates, tangents
    vkg::tex_rec *d_tex = nullptr;       // textures: records and all their levels' RGBA8 texels
    uint32_t *d_texels = nullptr;
    uint32_t num_textures = 0;
    vkg::mesh_ref *d_meshes = nullptr;
    uint32_t num_instances = 0;
    bool any_transmissive = false;  // a material with transmission > 0 or a null surface (light shadow rays pass)
    bool any_full = false;          // a material with a lobe beyond metal-roughness
    bool any_dispersion = false;    // a transmissive material with dispersion > 0
    bool any_alpha = false;         // an alpha-masked or blended material (material_alpha_tested)
    vkg::medium_rec *d_media = nullptr; // per-material medium records, when a material bounds a medium
    std::vector<vkg::medium_rec> h_media; // the same records for every material (host)
    std::vector<vkg_material> h_mats;     // host copy of the materials
    std::vector<vkg_instance> h_inst;     // host copy of the instances (instanced scenes)
    std::vector<vkg_light> lights;  // analytic lights (host copy; the tracer uploads them per render)
};

namespace vkg
{
namespace
{

constexpr int PT_THREADS = 128;

struct pt_params
{
    const node8 *nodes;
    const tri_rec *tris;
    // instanced scenes: two-level BVH (nodes, leaf-order and input-order instance records, BLASes)
    // and the meshes' vertex / index arrays; two_level selects them
    const node8 *tl_nodes;
    const inst_rec *tl_inst, *tl_by_id;
    const blas_ref *tl_blas;
    const mesh_ref *meshes;
    uint32_t two_level;
    const float *xyz;
    const uint32_t *idx;
    const float *nrm; // unit vertex normals of a single-level scene, or nullptr (face normals)
    const float *uv, *tng; // texture coordinates / tangents of a single-level scene, or nullptr
    // textures (num_textures 0: none) and the per-path ray-cone widths (nullptr: textures are not
    // sampled); cone_spread: the camera's pixel spread angle (raypipeline.slang:102)
    const tex_rec *tex;
    const uint32_t *texels;
    uint32_t num_textures;
    float cone_spread;
    float *cone;
    const uint32_t *tri_mat;
    const vkg_material *mats;
    env_view env;
    vkg_camera cam;
    uint32_t cx0, cy0, cw, ch, npix;
    uint32_t max_depth, rr_depth, mis_mode, disable_material, draw_skybox;
    float max_path_beta;
    uint64_t seed, batch;
    uint32_t s0; // first sample index of the wave
    uint32_t term_depth;  // with a cache: interaction at which rendering paths become cache queries
    uint32_t rec_depth;   // interactions recorded per training path
    uint32_t train_base;  // paths [train_base, train_base + train_paths) of the wave are training paths
    uint32_t train_paths;
    // analytic lights (the sun first) and the switches of their estimators
    const vkg_light *lights;
    uint32_t num_lights, suppress_caustics, transmissive;
    // per-pixel records of the traced window (nullptr: none): coverage from every sample, the
    // G-buffer fields from sample last_sample's primary hit; clip_near for the reversed-z depth
    vkg_pixel_data *gbuf;
    uint32_t last_sample;
    float clip_near;
    // homogeneous media: the per-material medium table (nullptr: no material bounds a medium) and
    // the per-path medium stacks
    const medium_rec *media;
    uint4 *mstack;
    uint32_t cam_medium; // medium table index of the camera's medium (0xFFFFFFFF: vacuum)
    uint32_t dispersion; // a material disperses: every segment draws one more uniform (the wavelength)
    // the reference's random streams (VKG_RNG_REFERENCE, one sample per pixel and wave): the batch
    // seed, the full-resolution width and samples per batch, and per window pixel the chain state
    // between samples and the sub-pixel offset of the batch
    uint32_t ref_rng, ref_seed, ref_width, ref_samples;
    uint32_t *ref_chain;
    float *ref_offset;
    // diagnostics: the drawn random numbers (vkg_diag_tracer_uniforms), records of dbg_stride floats
    float *dbg_u;
    uint32_t dbg_stride, dbg_segments;
};

constexpr uint32_t DBG_U_PER_SEGMENT = 16;

// the shade kernel's two modes
enum : int
{
    MODE_PLAIN = 0,
    MODE_CACHE = 1
};

struct cache_io
{
    float *q_feat;
    float4 *q_beta;
    uint32_t *q_count;
    float4 *rec;
    uint32_t *vcount;
};

constexpr int REC_F4 = 5; // float4 per training record

// the light-NEE shadow queue (count == nullptr: the scene has no lights)
struct light_queue
{
    vkg_ray *ray;
    uint32_t *pid;
    float4 *contrib;
    uint32_t *count;
};

__device__ __forceinline__ uint64_t path_seq(const pt_params &P, uint32_t pid)
{
    if(pid >= P.train_base) return ((P.batch << 40) ^ (uint64_t)(pid - P.train_base)) ^ (1ull << 62);
    const uint64_t g = (uint64_t)P.s0 * P.npix + pid; // = sample * npix + pixel
    return (P.batch << 40) ^ g;
}

__device__ __forceinline__ uint32_t warp_push(uint32_t *count, bool pred)
{
    const uint32_t lane = threadIdx.x & 31u;
    const unsigned m = __ballot_sync(0xffffffffu, pred);
    if(m == 0) return 0;
    const uint32_t leader = __ffs(m) - 1;
    uint32_t base = 0;
    if(lane == leader) base = atomicAdd(count, (uint32_t)__popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
    return base + __popc(m & ((1u << lane) - 1u));
}

// scene parameters and PCG32 increment of a queued path: one scene per launch (the tracer) ...
struct single_scene
{
    pt_params P;
    static constexpr bool per_path = false;
    __device__ __forceinline__ const pt_params &params(uint32_t) const { return P; }
    __device__ __forceinline__ uint64_t inc(uint32_t pid) const { return (path_seq(P, pid) << 1u) | 1u; }
};

// ... or one job per path (the batch renderer): a job table plus per-path job index and increment
struct job_table
{
    const pt_params *jobs;
    const uint32_t *pjob;
    const uint64_t *pinc;
    static constexpr bool per_path = true;
    __device__ __forceinline__ const pt_params &params(uint32_t pid) const { return jobs[pjob[pid]]; }
    __device__ __forceinline__ uint64_t inc(uint32_t pid) const { return pinc[pid]; }
};

// Coverage of alpha-masked / blended materials at a candidate hit: the traversal's candidate filter
// (no_filter, traverse.cuh) for the path tracer's queries. The reference tests coverage in its any-hit
// stages (raypipeline.slang:686-720 for the closest-hit trace, visibility_test.slang:45-87 and
// :131-152 for shadow rays): alpha = the material's alpha times the colour texture's alpha sampled at
// level 0 at the candidate's texture coordinates; MASK rejects alpha < alpha_cutoff, BLEND rejects
// alpha < xi. xi: for an extension ray the first uniform of the segment that will shade the hit,
// drawn from a copy of the path's generator (any_hit reads a copy of the payload's stream, so every
// candidate of the ray sees the same value and the path's stream does not move); for shadow rays,
// whose reference stream advances once per tested candidate in the hardware's traversal order, an
// independent uniform per candidate hashed from the path's generator state, the ray kind, the
// instance and the triangle, so that the answer does not depend on the order of the traversal.
constexpr uint32_t ALPHA_SALT_SHADOW = 0x9E3779B9u;      // the environment-NEE shadow queue
constexpr uint32_t ALPHA_SALT_LIGHT_SHADOW = 0x7F4A7C15u; // the light-NEE shadow queue

__device__ __forceinline__ float alpha_uniform(uint64_t key, uint32_t salt, uint32_t inst, uint32_t prim)
{
    uint32_t h = xxhash32((uint32_t)key ^ salt, (uint32_t)(key >> 32));
    h = xxhash32(h, inst);
    h = xxhash32(h, prim);
    return u01(h);
}

// the first uniform the shade kernel will draw for segment `depth` of a path whose generator state is
// `state` (PCG32, or the reference's chained streams), without advancing it
__device__ __forceinline__ float peek_uniform(const pt_params &P, uint64_t state, uint64_t inc, uint32_t depth)
{
    if(P.ref_rng)
    {
        uint32_t l = xxhash32((uint32_t)state, depth);
        return rnd(l);
    }
    pcg32 g{state, inc};
    return u01(pcg32_next(g));
}

struct alpha_filter
{
    static constexpr bool active = true;
    const pt_params *P;
    uint64_t key;     // shadow rays: the path's generator state
    float xi;         // extension rays: the segment's first uniform
    uint32_t salt;    // 0: an extension ray (xi, and disable_material applies); else the shadow ray's kind
    bool pass_transmissive; // light-NEE rays: transmissive surfaces are tinted, never tested

    __device__ __forceinline__ bool tests_material(uint32_t mat) const { return material_alpha_tested(P->mats[mat]); }

    __device__ bool accept(uint32_t inst, uint32_t prim, float bu, float bv) const
    {
        const pt_params &Q = *P;
        uint32_t mat;
        const float *tuv = Q.uv;
        const uint32_t *idx = Q.idx;
        if(Q.two_level)
        {
            const inst_rec *R = Q.tl_by_id + inst;
            mat = __ldg(&R->material);
            const mesh_ref &M = Q.meshes[__ldg(&R->blas)];
            tuv = M.uv;
            idx = M.idx;
        }
        else
            mat = __ldg(&Q.tri_mat[prim]);
        const vkg_material &m = Q.mats[mat];
        if(!material_alpha_tested(m) || (pass_transmissive && m.transmission > 0.f)) return true;
        float a;
        if(salt == 0u && Q.disable_material) a = 1.f; // the closest-hit stage's grey override
        else
        {
            a = m.alpha;
            if(m.tex_color < Q.num_textures && tuv)
            {
                const uint32_t i0 = __ldg(&idx[3 * (size_t)prim]), i1 = __ldg(&idx[3 * (size_t)prim + 1]),
                               i2 = __ldg(&idx[3 * (size_t)prim + 2]);
                const float w0 = 1.f - bu - bv;
                const float u = __ldg(&tuv[2 * (size_t)i0]) * w0 + __ldg(&tuv[2 * (size_t)i1]) * bu +
                                __ldg(&tuv[2 * (size_t)i2]) * bv;
                const float v = __ldg(&tuv[2 * (size_t)i0 + 1]) * w0 + __ldg(&tuv[2 * (size_t)i1 + 1]) * bu +
                                __ldg(&tuv[2 * (size_t)i2 + 1]) * bv;
                a *= tex_bilinear(Q.tex[m.tex_color], Q.texels, 0u, u, v).w;
            }
        }
        if(m.blend_mode == VKG_BLEND_MASK) return !(a < m.alpha_cutoff);
        return !(a < (salt ? alpha_uniform(key, salt, Q.two_level ? inst : 0u, prim) : xi));
    }
};

// camera ray through pixel (x, y) jittered by (jx, jy): PBRPathTracer's pinhole (raypipeline.slang:58-89)
__device__ __forceinline__ void camera_ray(const vkg_camera &c, uint32_t x, uint32_t y, float jx, float jy,
                                           float4 *o)
{
    const float sx = fdiv(fadd((float)x, jx), (float)c.width);
    const float sy = fdiv(fadd((float)y, jy), (float)c.height);
    const float nx = fsub(fmul(2.0f, sx), 1.0f), ny = fsub(fmul(2.0f, sy), 1.0f);
    const float cx = fmul(nx, fmul(c.tan_half_fovy, c.aspect));
    const float cy = -fmul(ny, c.tan_half_fovy);
    float d[3];
    for(int a = 0; a < 3; ++a) d[a] = fadd(fadd(fmul(c.right[a], cx), fmul(c.up[a], cy)), fmul(c.back[a], -1.0f));
    const float inv = frcp(fsqrt(dot3(d[0], d[1], d[2], d[0], d[1], d[2])));
    o[0] = make_float4(c.eye[0], c.eye[1], c.eye[2], PT_EPS);
    o[1] = make_float4(fmul(d[0], inv), fmul(d[1], inv), fmul(d[2], inv), PT_TMAX);
}

__global__ void __launch_bounds__(PT_THREADS)
        k_pt_generate(pt_params P, uint32_t n, vkg_ray *__restrict__ q_ray, uint32_t *__restrict__ q_pid,
                      uint64_t *__restrict__ rng, float4 *__restrict__ beta_pdf, float4 *__restrict__ radiance,
                      uint32_t *__restrict__ counters, uint32_t *__restrict__ vcount)
{
    const uint32_t stride = gridDim.x * blockDim.x;
    for(uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += stride)
    {
        pcg32 g = pcg32_seed(P.seed, path_seq(P, p));
        uint32_t pix = p % P.npix;
        if(p >= P.train_base)
        {
            // training path k: a random pixel of the k-th of train_paths equal runs of the window
            // (stratified, so neighbouring lanes trace neighbouring pixels)
            const uint64_t k = p - P.train_base, lo = k * P.npix / P.train_paths,
                           hi = (k + 1) * P.npix / P.train_paths;
            pix = (uint32_t)(lo + (hi > lo ? pcg32_next(g) % (uint32_t)(hi - lo) : 0u));
            vcount[k] = 0;
        }
        const uint32_t x = P.cx0 + pix % P.cw, y = P.cy0 + pix / P.cw;
        float jx, jy;
        if(P.ref_rng)
        {
            // the reference's raygen streams (raypipeline.slang:95-108): the pixel's chain runs through
            // the batch's samples, one sample per wave
            uint32_t chain;
            float off;
            if(P.s0 == 0)
            {
                chain = xxhash32(P.ref_seed, P.ref_width * y + x);
                off = fsub(fmul(2.0f, rnd(chain)), 1.0f);
                P.ref_offset[pix] = off;
            }
            else
            {
                chain = P.ref_chain[pix];
                off = P.ref_offset[pix];
            }
            rnd(chain); // Xi, the lens sample: a pinhole camera does not use it
            rnd(chain);
            // frac(Hammersley(s, N) + offset), Hammersley(i, N) = (i / N, reversebits(i) 2^-32)
            const float hx = fdiv((float)P.s0, (float)P.ref_samples);
            const float hy = fmul((float)__brev(P.s0), 2.3283064365386963e-10f);
            const float ax = fadd(hx, off), ay = fadd(hy, off);
            jx = fsub(ax, floorf(ax));
            jy = fsub(ay, floorf(ay));
            g.state = chain;
        }
        else
        {
            jx = u01(pcg32_next(g));
            jy = u01(pcg32_next(g));
        }
        if(P.dbg_u)
        {
            float *d = P.dbg_u + ((size_t)P.s0 * P.npix + p) * P.dbg_stride;
            d[0] = jx;
            d[1] = jy;
        }
        camera_ray(P.cam, x, y, jx, jy, reinterpret_cast<float4 *>(q_ray + p));
        q_pid[p] = p;
        rng[p] = g.state;
        beta_pdf[p] = make_float4(1.f, 1.f, 1.f, 0.f);
        radiance[p] = make_float4(0.f, 0.f, 0.f, 0.f);
        if(P.cone) P.cone[p] = 0.f; // the ray cone starts at width 0 (raypipeline.slang:112-114)
        // the camera's medium seeds the stack (raypipeline.slang:128-135)
        if(P.mstack)
            P.mstack[p] = P.cam_medium != 0xFFFFFFFFu ? make_uint4(1u, P.cam_medium, 0u, 0u) : make_uint4(0u, 0u, 0u, 0u);
    }
    if(blockIdx.x == 0 && threadIdx.x == 0) counters[0] = n;
}

// ALPHA: the scene has alpha-tested materials (alpha_filter); rng and depth then give each ray its
// segment's first uniform
template<class J, int STACK = (int)TRAVERSAL_STACK, bool ALPHA = false>
__global__ void __launch_bounds__(PT_THREADS, STACK <= 64 ? 8 : 6) // 64 / 85 registers
        k_pt_extend(J S, const vkg_ray *__restrict__ q_ray, const uint32_t *__restrict__ q_pid,
                    const uint32_t *__restrict__ count, vkg_hit *__restrict__ hits, uint32_t *__restrict__ hit_inst,
                    const uint32_t *__restrict__ perm = nullptr, const uint32_t *__restrict__ reordered = nullptr,
                    const uint64_t *__restrict__ rng = nullptr, uint32_t depth = 0)
{
    const uint32_t n = *count;
    const uint32_t stride = gridDim.x * blockDim.x;
    // a binned queue (bin_rays): position j traces entry perm[j]; results stay in the entry's slot
    if(perm && *reordered == 0u) perm = nullptr;
    for(uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += stride)
    {
        const uint32_t i = perm ? __ldg(perm + j) : j;
        const uint32_t pid = (J::per_path || ALPHA) ? q_pid[i] : 0u;
        const pt_params &P = S.params(J::per_path ? pid : 0u);
        const float4 *rp = reinterpret_cast<const float4 *>(q_ray + i);
        const float4 r0 = __ldg(rp), r1 = __ldg(rp + 1);
        using F = std::conditional_t<ALPHA, alpha_filter, no_filter>;
        F f{};
        if constexpr(ALPHA) f = alpha_filter{&P, 0ull, peek_uniform(P, rng[pid], S.inc(pid), depth), 0u, false};
        if(P.two_level)
        {
            const tlas_result r = trace_tlas<false, F>(P.tl_nodes, P.tl_inst, P.tl_blas, r0.x, r0.y, r0.z, r0.w, r1.x,
                                                       r1.y, r1.z, r1.w, CULL_BACK_UNLESS_TWOSIDED, f);
            reinterpret_cast<uint4 *>(hits)[i] =
                    make_uint4(r.prim, __float_as_uint(r.t), __float_as_uint(r.u), __float_as_uint(r.v));
            hit_inst[i] = r.inst;
            continue;
        }
        unsigned long long v = 0, t = 0;
        trace_result r = trace_ray<false, false, STACK, F>(P.nodes, P.tris, r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, r1.z,
                                                           r1.w, CULL_BACK_UNLESS_TWOSIDED, v, t, nullptr, f);
        reinterpret_cast<uint4 *>(hits)[i] =
                make_uint4(r.prim, __float_as_uint(r.t), __float_as_uint(r.u), __float_as_uint(r.v));
    }
}

// surface point, unit geometric normal (world space) and material of a hit: the triangle's vertices,
// the barycentric point; for an instanced scene both moved to world space (point by the
// object -> world transform, normal by the transpose of world -> object). ns (when not null): the
// unit shading normal, the vertex normals interpolated with the barycentric weights (1 - u - v, u, v)
// and normalised as interpolate_vertex does (raypipeline.slang:336-360), moved like the face normal;
// the face normal itself when the mesh has no vertex normals
__device__ __forceinline__ void hit_surface(const pt_params &P, uint32_t prim, uint32_t inst, float bu, float bv,
                                            float3 &p, float3 &ng, uint32_t &mat, float3 *ns = nullptr)
{
    const float *xyz = P.xyz;
    const uint32_t *idx = P.idx;
    const float *nrm = P.nrm;
    const inst_rec *R = nullptr;
    if(P.two_level)
    {
        R = P.tl_by_id + inst;
        const mesh_ref M = P.meshes[__ldg(&R->blas)];
        xyz = M.xyz;
        idx = M.idx;
        nrm = M.nrm;
    }
    const uint32_t i0 = __ldg(&idx[3 * (size_t)prim]), i1 = __ldg(&idx[3 * (size_t)prim + 1]),
                   i2 = __ldg(&idx[3 * (size_t)prim + 2]);
    const float3 v0 = f3(__ldg(&xyz[3 * (size_t)i0]), __ldg(&xyz[3 * (size_t)i0 + 1]), __ldg(&xyz[3 * (size_t)i0 + 2]));
    const float3 v1 = f3(__ldg(&xyz[3 * (size_t)i1]), __ldg(&xyz[3 * (size_t)i1 + 1]), __ldg(&xyz[3 * (size_t)i1 + 2]));
    const float3 v2 = f3(__ldg(&xyz[3 * (size_t)i2]), __ldg(&xyz[3 * (size_t)i2 + 1]), __ldg(&xyz[3 * (size_t)i2 + 2]));
    const float3 e1 = v1 - v0, e2 = v2 - v0;
    p = v0 + e1 * bu + e2 * bv;
    float3 n = cross(e1, e2);
    const bool smooth = ns && nrm;
    float3 sn = f3(0.f, 0.f, 0.f);
    if(smooth)
    {
        auto vn = [&](uint32_t k) {
            return f3(__ldg(&nrm[3 * (size_t)k]), __ldg(&nrm[3 * (size_t)k + 1]), __ldg(&nrm[3 * (size_t)k + 2]));
        };
        sn = vn(i0) * (1.f - bu - bv) + vn(i1) * bu + vn(i2) * bv;
    }
    if(R)
    {
        float o[12], w[12];
        for(int k = 0; k < 12; ++k)
        {
            o[k] = __ldg(&R->o2w[k]);
            w[k] = __ldg(&R->w2o[k]);
        }
        p = f3(o[0] * p.x + o[1] * p.y + o[2] * p.z + o[3], o[4] * p.x + o[5] * p.y + o[6] * p.z + o[7],
               o[8] * p.x + o[9] * p.y + o[10] * p.z + o[11]);
        n = f3(w[0] * n.x + w[4] * n.y + w[8] * n.z, w[1] * n.x + w[5] * n.y + w[9] * n.z,
               w[2] * n.x + w[6] * n.y + w[10] * n.z);
        if(smooth)
            sn = f3(w[0] * sn.x + w[4] * sn.y + w[8] * sn.z, w[1] * sn.x + w[5] * sn.y + w[9] * sn.z,
                    w[2] * sn.x + w[6] * sn.y + w[10] * sn.z);
        mat = __ldg(&R->material);
    }
    else
        mat = __ldg(&P.tri_mat[prim]);
    ng = normalize(n);
    if(ns) *ns = smooth ? normalize(sn) : ng;
}

// FULL = false: a scene without lights whose materials are metal-roughness only; the light terms and
// the other lobes compile away. MEDIA = true (with FULL): the homogeneous-media terms
// texture coordinates of a hit (the vertices' interpolated with the barycentric weights), the
// triangle's texture-LOD constant 0.5 log2(uv area / world area) (lod_constant,
// raypipeline.slang:299-310; the world area after the instance's object -> world transform) and,
// when asked for and present, the unit tangent (interpolated, moved by the object -> world
// transform). false: the mesh has no texture coordinates.
__device__ __forceinline__ bool hit_texcoords(const pt_params &P, uint32_t prim, uint32_t inst, float bu, float bv,
                                              bool want_tangent, float2 &uv, float &lod, float3 &tangent, bool &has_tangent)
{
    const float *xyz = P.xyz, *tuv = P.uv, *tng = P.tng;
    const uint32_t *idx = P.idx;
    const inst_rec *R = nullptr;
    if(P.two_level)
    {
        R = P.tl_by_id + inst;
        const mesh_ref M = P.meshes[__ldg(&R->blas)];
        xyz = M.xyz;
        idx = M.idx;
        tuv = M.uv;
        tng = M.tng;
    }
    if(!tuv) return false;
    const uint32_t i0 = __ldg(&idx[3 * (size_t)prim]), i1 = __ldg(&idx[3 * (size_t)prim + 1]),
                   i2 = __ldg(&idx[3 * (size_t)prim + 2]);
    auto vtx = [&](uint32_t k) {
        return f3(__ldg(&xyz[3 * (size_t)k]), __ldg(&xyz[3 * (size_t)k + 1]), __ldg(&xyz[3 * (size_t)k + 2]));
    };
    const float2 t0 = make_float2(__ldg(&tuv[2 * (size_t)i0]), __ldg(&tuv[2 * (size_t)i0 + 1]));
    const float2 t1 = make_float2(__ldg(&tuv[2 * (size_t)i1]), __ldg(&tuv[2 * (size_t)i1 + 1]));
    const float2 t2 = make_float2(__ldg(&tuv[2 * (size_t)i2]), __ldg(&tuv[2 * (size_t)i2 + 1]));
    const float w0 = 1.f - bu - bv;
    uv = make_float2(t0.x * w0 + t1.x * bu + t2.x * bv, t0.y * w0 + t1.y * bu + t2.y * bv);
    const float3 v0 = vtx(i0);
    float3 e1 = vtx(i1) - v0, e2 = vtx(i2) - v0;
    float3 T = f3(0.f, 0.f, 0.f);
    has_tangent = want_tangent && tng != nullptr;
    if(has_tangent)
    {
        auto tv = [&](uint32_t k) {
            return f3(__ldg(&tng[3 * (size_t)k]), __ldg(&tng[3 * (size_t)k + 1]), __ldg(&tng[3 * (size_t)k + 2]));
        };
        T = tv(i0) * w0 + tv(i1) * bu + tv(i2) * bv;
    }
    if(R)
    {
        float o[9];
        for(int r = 0; r < 3; ++r)
            for(int c = 0; c < 3; ++c) o[3 * r + c] = __ldg(&R->o2w[4 * r + c]);
        auto lin = [&](float3 a) {
            return f3(o[0] * a.x + o[1] * a.y + o[2] * a.z, o[3] * a.x + o[4] * a.y + o[5] * a.z,
                      o[6] * a.x + o[7] * a.y + o[8] * a.z);
        };
        e1 = lin(e1);
        e2 = lin(e2);
        if(has_tangent) T = lin(T);
    }
    const float3 c = cross(e1, e2);
    const float p_a = sqrtf(dot(c, c));
    const float t_a = fabsf((t1.x - t0.x) * (t2.y - t0.y) - (t2.x - t0.x) * (t1.y - t0.y));
    lod = 0.5f * log2f(t_a / p_a);
    if(has_tangent) tangent = normalize(T);
    return true;
}

// the material's textures at a surface hit (raypipeline.slang:526-606): every sample at level
// lod + log2|cone width| + 0.5 log2(w h) - log2|N.V| (sample_texture_lod, :312-320) with N the
// shading normal before the normal map; base colour, normal map (tangent frame (T, +-B, N),
// B = normalize(N x T) negated for back faces, hemisphere clamp), emission, roughness / metalness,
// transmission and the diffuse-transmission terms
__device__ __forceinline__ void apply_textures(const pt_params &P, const vkg_material &q, float2 uv, float lod,
                                               float cone_w, float3 V, bool back_face, bool has_tangent,
                                               float3 tangent, material_view &m, float3 &emit, float3 &N)
{
    const float base_lambda = lod + log2f(fabsf(cone_w)) - log2f(fabsf(dot(V, N)));
    auto ok = [&](uint32_t t) { return t < P.num_textures; };
    auto S = [&](uint32_t t) {
        const tex_rec &T = P.tex[t];
        return tex_sample(T, P.texels, uv.x, uv.y, base_lambda + 0.5f * log2f((float)T.width * (float)T.height));
    };
    if(ok(q.tex_color) && !P.disable_material)
    {
        const float4 c = S(q.tex_color);
        m.base = m.base * f3(c.x, c.y, c.z);
    }
    if(ok(q.tex_normal) && has_tangent)
    {
        const float4 t = S(q.tex_normal);
        const float nx = 2.f * (t.x - 0.5f), ny = 2.f * (t.y - 0.5f);
        const float nz = sqrtf(fmaxf(0.f, 1.f - nx * nx - ny * ny));
        const float3 b = normalize(cross(N, tangent));
        const float3 n = normalize(tangent * nx + (back_face ? -b : b) * ny + N * nz);
        N = normalize(n + N * fmaxf(0.f, -dot(n, N) + 1e-3f));
    }
    if(ok(q.tex_emission))
    {
        const float4 e = S(q.tex_emission);
        const float3 te = f3(e.x, e.y, e.z);
        emit = (emit.x > 0.f || emit.y > 0.f || emit.z > 0.f) ? emit * te : te;
    }
    if(ok(q.tex_ao_rough_metal))
    {
        const float4 a = S(q.tex_ao_rough_metal);
        m.roughness *= a.y;
        m.metalness *= a.z;
    }
    if(ok(q.tex_transmission)) m.transmission *= S(q.tex_transmission).x;
    if(ok(q.tex_diffuse_transmission)) m.diffuse_transmission *= S(q.tex_diffuse_transmission).w;
    if(ok(q.tex_diffuse_transmission_color))
    {
        const float4 c = S(q.tex_diffuse_transmission_color);
        m.dt_color = m.dt_color * f3(c.x, c.y, c.z);
    }
}

// material classes of a queue entry for shading coherence: 0 miss, then by the costliest lobe the
// material takes (thin film, dielectric, medium boundary / null surface, clearcoat, sheen, diffuse
// transmission, metal-roughness only)
constexpr uint32_t PT_BIN_CLASSES = 8;
__device__ __forceinline__ uint32_t material_class(const vkg_material &m)
{
    if(m.iridescence > 0.f) return 1;
    if(m.transmission > 0.f) return 2;
    if(m.null_surface || (m.attenuation_distance > 0.f && m.attenuation_distance < 3.0e38f)) return 3;
    if(m.clearcoat > 0.f) return 4;
    if(m.sheen_color[0] > 0.f || m.sheen_color[1] > 0.f || m.sheen_color[2] > 0.f) return 5;
    if(m.diffuse_transmission > 0.f) return 6;
    return 7;
}
template<class J>
__device__ __forceinline__ uint32_t entry_class(const J &S, const uint32_t *__restrict__ in_pid,
                                                const vkg_hit *__restrict__ hits, const uint32_t *__restrict__ hit_inst,
                                                uint32_t i)
{
    const uint32_t prim = __ldg(&hits[i].prim);
    if(prim == VKG_MISS) return 0;
    const pt_params &P = S.params(__ldg(&in_pid[i]));
    const uint32_t mat = P.two_level ? __ldg(&P.tl_by_id[__ldg(&hit_inst[i])].material) : __ldg(&P.tri_mat[prim]);
    return material_class(P.mats[mat]);
}
// counts per class of the queue (bins[0..7]; zero at launch)
template<class J>
__global__ void __launch_bounds__(PT_THREADS)
        k_pt_bin_count(J S, const uint32_t *__restrict__ in_pid, const vkg_hit *__restrict__ hits,
                       const uint32_t *__restrict__ hit_inst, const uint32_t *__restrict__ in_count,
                       uint32_t *__restrict__ bins)
{
    __shared__ uint32_t h[PT_BIN_CLASSES];
    if(threadIdx.x < PT_BIN_CLASSES) h[threadIdx.x] = 0u;
    __syncthreads();
    const uint32_t n = *in_count;
    for(uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        atomicAdd(&h[entry_class(S, in_pid, hits, hit_inst, i)], 1u);
    __syncthreads();
    if(threadIdx.x < PT_BIN_CLASSES && h[threadIdx.x]) atomicAdd(&bins[threadIdx.x], h[threadIdx.x]);
}
// order[k] = queue entry of the k-th slot, classes in ascending order (bins[8..15] are the classes'
// fill cursors, zero at launch); within a class the order is arbitrary — each path's result does not
// depend on its slot
template<class J>
__global__ void __launch_bounds__(PT_THREADS)
        k_pt_bin_scatter(J S, const uint32_t *__restrict__ in_pid, const vkg_hit *__restrict__ hits,
                         const uint32_t *__restrict__ hit_inst, const uint32_t *__restrict__ in_count,
                         uint32_t *__restrict__ bins, uint32_t *__restrict__ order)
{
    __shared__ uint32_t start[PT_BIN_CLASSES];
    if(threadIdx.x == 0)
    {
        uint32_t acc = 0;
        for(uint32_t c = 0; c < PT_BIN_CLASSES; ++c)
        {
            start[c] = acc;
            acc += bins[c];
        }
    }
    __syncthreads();
    const uint32_t n = *in_count;
    const uint32_t lane = threadIdx.x & 31u;
    for(uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x)
    {
        const uint32_t i = base + threadIdx.x;
        const bool active = i < n;
        const uint32_t c = active ? entry_class(S, in_pid, hits, hit_inst, i) : PT_BIN_CLASSES;
        // one atomic per class present in the warp
        const uint32_t peers = __match_any_sync(0xFFFFFFFFu, c);
        const uint32_t leader = __ffs(peers) - 1u;
        uint32_t pos = 0;
        if(active && lane == leader) pos = atomicAdd(&bins[PT_BIN_CLASSES + c], (uint32_t)__popc(peers));
        pos = __shfl_sync(0xFFFFFFFFu, pos, (int)leader);
        if(active) order[start[c] + pos + (uint32_t)__popc(peers & ((1u << lane) - 1u))] = i;
    }
}

// TEX: the scene has textures (P.cone set); the untextured variant carries no texture code, which
// keeps its register budget
template<int MODE, class J, bool FULL = true, bool MEDIA = false, bool TEX = false>
__global__ void __launch_bounds__(PT_THREADS)
        k_pt_shade(J S, uint32_t depth, const vkg_ray *__restrict__ in_ray,
                   const uint32_t *__restrict__ in_pid, const vkg_hit *__restrict__ hits,
                   const uint32_t *__restrict__ hit_inst,
                   const uint32_t *__restrict__ in_count, vkg_ray *__restrict__ out_ray,
                   uint32_t *__restrict__ out_pid, uint32_t *__restrict__ out_count, vkg_ray *__restrict__ s_ray,
                   uint32_t *__restrict__ s_pid, float4 *__restrict__ s_contrib, uint32_t *__restrict__ s_count,
                   uint64_t *__restrict__ rng, float4 *__restrict__ beta_pdf, float4 *__restrict__ radiance,
                   cache_io io, light_queue lq, const uint32_t *__restrict__ order)
{
    const uint32_t n = *in_count;
    const uint32_t stride = gridDim.x * blockDim.x;
    for(uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride)
    {
        // order (may be null): queue entries grouped by material class, so that a warp's lanes take
        // the same lobes (k_pt_bin_count / k_pt_bin_scatter)
        const uint32_t j = base + threadIdx.x;
        const bool active = j < n;
        const uint32_t i = active && order ? __ldg(&order[j]) : j;
        bool push_ext = false, push_shadow = false, push_query = false, push_light = false;
        bool cull_back_shadow = false; // shadow rays from inside a medium leave it through back faces
        float3 P0 = f3(0.f, 0.f, 0.f), ndir = P0, sdir = P0, N = P0;
        float3 contrib = P0, qbeta = P0, albedo = P0, vq = P0, ldir_s = P0, lcontrib = P0;
        float rough = 0.f, ldist = 0.f;
        uint32_t pid = 0;
        if(active)
        {
            pid = in_pid[i];
            const pt_params &P = S.params(pid);
            const float4 *rp = reinterpret_cast<const float4 *>(in_ray + i);
            const float4 r1 = rp[1];
            const float3 dir = f3(r1.x, r1.y, r1.z);
            const uint4 h = reinterpret_cast<const uint4 *>(hits)[i];
            pcg32 g{rng[pid], S.inc(pid)};
            // 8 draws per segment; 3 more (light pick, point on the light) when the scene has lights,
            // 4 more (channel, distance, phase direction) when it has media
            const uint32_t num_lights = FULL ? P.num_lights : 0u;
            const bool media = FULL && MEDIA && P.media;
            // one more (the wavelength) when a material disperses, after the others
            float u[16];
            const bool disp = FULL && P.dispersion;
            const int nu = (media ? 15 : (num_lights ? 11 : 8)) + (disp ? 1 : 0);
            if(P.ref_rng)
            {
                // the reference's per-segment stream: chain = xxhash32(chain, i) (raypipeline.slang:150),
                // the hit shader's rnd() LCG started at it (random.slang:27-36)
                const uint32_t chain = xxhash32((uint32_t)g.state, depth);
                uint32_t l = chain;
                for(int k = 0; k < 16; ++k) u[k] = k < nu ? rnd(l) : 0.f;
                g.state = chain;
            }
            else
                for(int k = 0; k < 16; ++k) u[k] = k < nu ? u01(pcg32_next(g)) : 0.f;
            const float u_lambda = media ? u[15] : (num_lights ? u[11] : u[8]);
            if(P.dbg_u && depth < P.dbg_segments)
            {
                float *d = P.dbg_u + ((size_t)P.s0 * P.npix + pid) * P.dbg_stride + 2 + DBG_U_PER_SEGMENT * depth;
                for(int k = 0; k < nu; ++k) d[k] = u[k];
            }
            const float4 bp = beta_pdf[pid];
            float3 beta = f3(bp.x, bp.y, bp.z);
            const float3 seg_beta = beta;
            float prev_pdf = bp.w;
            const float4 lr = radiance[pid];
            float3 L = f3(lr.x, lr.y, lr.z);
            uint32_t flags = __float_as_uint(lr.w); // PATH_REGULARIZE | PATH_CAUSTIC
            const float4 r0 = rp[0];
            float t_end = h.x == VKG_MISS ? r1.w : __uint_as_float(h.y);
            // the medium the segment runs through (raypipeline.slang:388-474, homogeneous branch)
            uint4 mst = make_uint4(0u, 0u, 0u, 0u);
            bool scattered = false;
            float scatter_g = 0.f;
            if(media)
            {
                // only a segment that ends on a surface runs through a medium: the reference samples it
                // in the closest-hit stage, an escaping ray goes straight to the miss stage
                mst = P.mstack[pid];
                const uint32_t top = stack_top(mst);
                if(top != 0xFFFFFFFFu && h.x != VKG_MISS)
                {
                    const medium_rec &M = P.media[top];
                    const float3 ss = f3(M.sigma_s[0], M.sigma_s[1], M.sigma_s[2]);
                    const float3 sa = f3(M.sigma_a[0], M.sigma_a[1], M.sigma_a[2]);
                    const float3 st = ss + sa;
                    if(st.x > 0.f || st.y > 0.f || st.z > 0.f)
                    {
                        const float T = t_end;
                        const float3 le = f3(M.emission[0], M.emission[1], M.emission[2]);
                        if(le.x > 0.f || le.y > 0.f || le.z > 0.f)
                        {
                            // emission over the segment: sigma_a Le (1 - exp(-sigma_t T)) / sigma_t
                            const float3 ti = f3((1.f - expf(-st.x * T)) / fmaxf(st.x, PT_EPS),
                                                 (1.f - expf(-st.y * T)) / fmaxf(st.y, PT_EPS),
                                                 (1.f - expf(-st.z * T)) / fmaxf(st.z, PT_EPS));
                            L = L + beta * sa * le * ti;
                        }
                        const int ch = (int)fminf(u[11] * 3.f, 2.f);
                        const float stc = ch == 0 ? st.x : (ch == 1 ? st.y : st.z);
                        const float t = fminf(-logf(1.f - u[12]) / fmaxf(stc, PT_EPS), T);
                        scattered = t < T;
                        const float3 tr = f3(expf(-st.x * t), expf(-st.y * t), expf(-st.z * t));
                        const float3 dens = scattered ? tr * st : tr;
                        const float pdf = fmaxf((dens.x + dens.y + dens.z) / 3.f, PT_PDF_EPS);
                        beta = scattered ? beta * (ss * tr * (1.f / pdf)) : beta * (tr * (1.f / pdf));
                        if(scattered)
                        {
                            t_end = t;
                            scatter_g = M.g;
                        }
                    }
                }
            }
            const bool light_hits = num_lights && !(P.suppress_caustics && (flags & PATH_CAUSTIC));
            if(light_hits)
            {
                // light bodies the segment passed (raypipeline.slang:196-224): additive emitters,
                // MIS-weighted against their NEE strategy, with the throughput at the segment's start
                const float3 o = f3(r0.x, r0.y, r0.z);
                const float inv_n = 1.f / (float)num_lights;
                for(uint32_t li = 0; li < num_lights; ++li)
                {
                    const vkg_light &l = P.lights[li];
                    const float2 lh = intersect_light(l, o, dir);
                    if(lh.x <= r0.w || lh.x >= t_end) continue;
                    const float w = mis_weight_hit(P.mis_mode, prev_pdf, light_pdf(l, o, dir) * inv_n);
                    L = L + seg_beta * lv3(l.color) * (w * l.intensity);
                }
            }
            if(scattered)
            {
                // a scattering event: NEE toward one light with the phase function (nee_volume,
                // direct_lighting.slang:334-366), then a phase-function bounce. The environment gets no
                // NEE sample here (as in the reference): a shadow ray would not see the medium's
                // attenuation, so the environment is left to the phase-sampled path, whose miss then
                // takes MIS weight 1 (PATH_NO_ENV_NEE)
                P0 = f3(r0.x, r0.y, r0.z) + dir * t_end;
                cull_back_shadow = true;
                flags |= PATH_NO_ENV_NEE;
                if(num_lights)
                {
                    const uint32_t nl = num_lights;
                    const uint32_t li = nl > 1 ? min((uint32_t)(u[8] * (float)nl), nl - 1u) : 0u;
                    const vkg_light &l = P.lights[li];
                    const light_sample ls = sample_light(l, P0, u[9], u[10]);
                    if(max3(ls.radiance) > 0.f)
                    {
                        const float ph = phase_hg(dot(dir, ls.dir), scatter_g);
                        const float w = bsdf_reachable(l) ? mis_weight_nee(P.mis_mode, ls.pdf / (float)nl, ph) : 1.f;
                        lcontrib = beta * ls.radiance * (w * (float)nl * ph / ls.pdf);
                        if(max3(lcontrib) > 0.f)
                        {
                            push_light = true;
                            ldir_s = ls.dir;
                            ldist = ls.dist;
                        }
                    }
                }
                float ppdf;
                const float3 loc = sample_phase_hg(u[13], u[14], scatter_g, ppdf);
                ndir = to_world(local_frame(dir), loc);
                prev_pdf = ppdf;
                if(ppdf < PT_REGULARIZE_PDF_THRESHOLD) flags |= PATH_REGULARIZE;
                bool alive = true;
                if(P.rr_depth == 0)
                {
                    if(max3(beta) <= 0.05f * (float)depth)
                    {
                        const float q = 1.f - max3(beta);
                        if(u[7] < q) alive = false;
                        else beta = beta * (1.f / (1.f - q));
                    }
                }
                else if(depth + 1 >= P.rr_depth)
                {
                    const float q = fmaxf(0.f, 1.f - max3(beta));
                    if(u[7] < q) alive = false;
                    else beta = beta * (1.f / (1.f - q));
                }
                push_ext = alive && depth + 1 < P.max_depth && max3(beta) > 0.f;
            }
            // the pixel record of a camera ray (raypipeline.slang:224-236, :250-268)
            const bool record = depth == 0 && P.gbuf && pid < P.train_base &&
                                P.s0 + pid / P.npix == P.last_sample;
            if(record && h.x == VKG_MISS && !scattered)
            {
                vkg_pixel_data &px = P.gbuf[pid % P.npix];
                px.depth = 0.f;
                px.normal = 0u;
                px.object_id = 0xFFFFu;
                px.albedo = pack_rgba8(0.f, 0.f, 0.f, 1.f);
            }
            if(scattered) {}
            else if(h.x == VKG_MISS)
            {
                if(light_hits)
                {
                    // sun discs seen by the ray (eval_distant_lights, raypipeline.slang:728-744)
                    const float inv_n = 1.f / (float)num_lights;
                    for(uint32_t li = 0; li < num_lights; ++li)
                    {
                        const vkg_light &l = P.lights[li];
                        if(l.type != VKG_LIGHT_DIRECTIONAL) continue;
                        const float pdf = light_pdf(l, f3(0.f, 0.f, 0.f), dir);
                        if(pdf <= 0.f) continue;
                        const float w = mis_weight_hit(P.mis_mode, prev_pdf, pdf * inv_n);
                        L = L + beta * lv3(l.color) * (w * l.intensity);
                    }
                }
                // miss_environment (raypipeline.slang:764-781) with the hit-side MIS weight
                const uint32_t t = env_texel(dir, P.env.w, P.env.h);
                float3 le = env_radiance(P.env, t);
                if(depth == 0 && !P.draw_skybox) le = f3(0.f, 0.f, 0.f);
                float w = 1.f;
                if(prev_pdf > 0.f && !(flags & PATH_NO_ENV_NEE))
                {
                    if(P.mis_mode == 1) w = 0.f;
                    else if(P.mis_mode == 0) w = power_heuristic(prev_pdf, env_pdf(P.env, dir, t));
                }
                L = L + beta * le * w;
            }
            else
            {
                float3 ng, sn;
                uint32_t mat;
                hit_surface(P, h.x, P.two_level ? hit_inst[i] : 0u, __uint_as_float(h.z), __uint_as_float(h.w), P0,
                            ng, mat, &sn);
                // the side comes from the face (HitKind); the shading normal -- the interpolated vertex
                // normal where the mesh has them -- is turned to that side (raypipeline.slang:359)
                const bool back_face = !(dot(ng, dir) < 0.f);
                N = back_face ? -sn : sn;
                const float3 V = -dir;
                // media: a boundary pushes its medium on a transmission through a front face and pops
                // on one through a back face (raypipeline.slang:516-523, :656-664)
                const bool boundary = media && ((P.media[mat].flags & MEDIUM_VOLUME) || P.mats[mat].transmission > 0.f);
                if(media && (P.media[mat].flags & MEDIUM_NULL))
                {
                    // a null surface: no interaction, the path crosses it (raypipeline.slang:478, :524);
                    // it enters / leaves a medium only when it bounds one
                    if(boundary)
                    {
                        if(back_face) stack_pop(mst);
                        else stack_push(mst, mat);
                    }
                    bool alive = true;
                    if(P.rr_depth == 0)
                    {
                        if(max3(beta) <= 0.05f * (float)depth)
                        {
                            const float q = 1.f - max3(beta);
                            if(u[7] < q) alive = false;
                            else beta = beta * (1.f / (1.f - q));
                        }
                    }
                    else if(depth + 1 >= P.rr_depth)
                    {
                        const float q = fmaxf(0.f, 1.f - max3(beta));
                        if(u[7] < q) alive = false;
                        else beta = beta * (1.f / (1.f - q));
                    }
                    push_ext = alive && depth + 1 < P.max_depth;
                    ndir = dir;
                    goto done;
                }
                {
                material_view m = load_material<FULL>(P.mats, mat, P.disable_material);
                const float *em = P.mats[mat].emission;
                float3 emit = f3(em[0], em[1], em[2]);
                if(TEX && P.cone)
                {
                    // textures sampled with the ray cone as it reached this surface, which then grows
                    // by the segment (propagate with no surface spread, raypipeline.slang:608)
                    const float cone_w = P.cone[pid];
                    const vkg_material &q = P.mats[mat];
                    const bool want_t = q.tex_normal < P.num_textures;
                    float2 tuv;
                    float lod;
                    float3 tangent;
                    bool has_t = false;
                    if((q.tex_color & q.tex_normal & q.tex_emission & q.tex_ao_rough_metal & q.tex_transmission &
                        q.tex_diffuse_transmission & q.tex_diffuse_transmission_color) != VKG_NO_TEXTURE &&
                       hit_texcoords(P, h.x, P.two_level ? hit_inst[i] : 0u, __uint_as_float(h.z),
                                     __uint_as_float(h.w), want_t, tuv, lod, tangent, has_t))
                    {
                        // the texture-coordinate transform (raypipeline.slang:350); the LOD keeps the
                        // untransformed coordinates' constant
                        if(q.has_uv_transform)
                        {
                            const float *t6 = q.uv_transform;
                            tuv = make_float2(t6[0] * tuv.x + t6[1] * tuv.y + t6[2], t6[3] * tuv.x + t6[4] * tuv.y + t6[5]);
                        }
                        apply_textures(P, q, tuv, lod, cone_w, V, back_face, has_t, tangent, m, emit, N);
                    }
                    P.cone[pid] = cone_w + P.cone_spread * __uint_as_float(h.y);
                }
                // path regularisation (raypipeline.slang:611): after a non-peaked bounce, later vertices
                // shade (sample and NEE) with roughness >= 0.25
                if(flags & PATH_REGULARIZE) m.roughness = fmaxf(m.roughness, PT_REGULARIZE_MIN_ROUGHNESS);
                // chromatic dispersion (raypipeline.slang:485-488): a wavelength, locked by the path's
                // first transmission through a dispersive surface (bits 16..31 of the path flags, FP16
                // as the reference's payload keeps it) or drawn here, and the surface's Cauchy ior
                const bool dispersive = disp && material_dispersive(P.mats[mat]);
                const bool lambda_locked = (flags >> 16) != 0u;
                float lambda = 0.f, surf_ior = FULL ? P.mats[mat].ior : 1.f;
                if(dispersive)
                {
                    lambda = lambda_locked ? __half2float(__ushort_as_half((unsigned short)(flags >> 16)))
                                           : fadd(400.0f, fmul(u_lambda, 300.0f));
                    surf_ior = cauchy_ior(P.mats[mat].ior, P.mats[mat].dispersion, lambda);
                }
                float eta = FULL ? (dispersive ? hit_eta_ior(surf_ior, back_face) : hit_eta(P.mats, mat, back_face)) : 1.f;
                if(media && P.mats[mat].transmission > 0.f)
                {
                    // eta from the media stack: the current medium's ior over the surface's entering,
                    // the surface's over the enclosing medium's leaving (raypipeline.slang:489-491)
                    const float ior = surf_ior;
                    eta = (back_face ? ior / stack_ior(P.media, mst, mst.x ? mst.x - 1 : 0)
                                     : stack_ior(P.media, mst, mst.x) / ior) + PT_EPS;
                }
                L = L + beta * emit;
                if(depth == 0 && P.gbuf && pid < P.train_base)
                {
                    vkg_pixel_data &px = P.gbuf[pid % P.npix];
                    px.alpha = 1.f; // coverage: any sample of the batch hit geometry
                    if(record)
                    {
                        // reversed-z depth near / (distance along the view axis); normal and albedo
                        // of the primary hit
                        const float3 fwd = f3(-P.cam.back[0], -P.cam.back[1], -P.cam.back[2]);
                        const float3 rel = P0 - f3(P.cam.eye[0], P.cam.eye[1], P.cam.eye[2]);
                        px.depth = P.clip_near / dot(rel, fwd);
                        const float2 oc = oct_encode(N.x, N.y, N.z);
                        px.normal = pack_snorm_2x16(oc.x, oc.y);
                        px.object_id = P.two_level ? hit_inst[i] : 0u;
                        px.albedo = pack_rgba8(m.base.x, m.base.y, m.base.z, 1.f);
                    }
                }
                if constexpr(MODE == MODE_CACHE)
                {
                    if(pid < P.train_base && depth == P.term_depth)
                    {
                        push_query = true;
                        qbeta = beta;
                        vq = V;
                        albedo = m.base;
                        rough = m.roughness;
                    }
                }
                if constexpr(MODE == MODE_CACHE)
                {
                    if(pid >= P.train_base && depth < P.rec_depth)
                    {
                        const uint32_t k = pid - P.train_base;
                        float4 *r = io.rec + ((size_t)k * P.rec_depth + depth) * REC_F4;
                        r[0] = make_float4(P0.x, P0.y, P0.z, V.x);
                        r[1] = make_float4(V.y, V.z, N.x, N.y);
                        r[2] = make_float4(N.z, m.roughness, m.base.x, m.base.y);
                        r[3] = make_float4(m.base.z, beta.x, beta.y, beta.z);
                        r[4] = make_float4(L.x, L.y, L.z, 0.f);
                        io.vcount[k] = depth + 1;
                    }
                }
                // next-event estimation against the environment (mis_weight_nee, direct_lighting.slang:239-244)
                if(!push_query && P.mis_mode != 2)
                {
                    float pdf_env;
                    uint32_t texel;
                    const float3 ld = env_sample(P.env, u[3], u[4], u[5], u[6], pdf_env, texel);
                    const float cosl = dot(N, ld);
                    if(pdf_env > 0.f && cosl > 0.f)
                    {
                        float pdf_b;
                        const float3 f = FULL ? eval_bsdf_ool(m, ld, N, V, eta, pdf_b) : eval_bsdf(m, ld, N, V, eta, pdf_b);
                        if(pdf_b > 0.f)
                        {
                            const float w = P.mis_mode == 1 ? 1.f : power_heuristic(pdf_env, pdf_b);
                            contrib = beta * f * env_radiance(P.env, texel) * (w * cosl / pdf_env);
                            if(max3(contrib) > 0.f)
                            {
                                push_shadow = true;
                                sdir = ld;
                            }
                        }
                    }
                }
                // next-event estimation against one uniformly picked light (nee_surface,
                // direct_lighting.slang:297-332); its shadow ray passes transmissive surfaces
                if(!push_query && num_lights)
                {
                    const uint32_t nl = num_lights;
                    const uint32_t li = nl > 1 ? min((uint32_t)(u[8] * (float)nl), nl - 1u) : 0u;
                    const vkg_light &l = P.lights[li];
                    const light_sample ls = sample_light(l, P0, u[9], u[10]);
                    if(max3(ls.radiance) > 0.f)
                    {
                        const float cosl = fmaxf(dot(N, ls.dir), 0.f);
                        float pdf_b = 0.f;
                        const float3 f = FULL ? eval_bsdf_ool(m, ls.dir, N, V, eta, pdf_b) : eval_bsdf(m, ls.dir, N, V, eta, pdf_b);
                        const float w = bsdf_reachable(l) ? mis_weight_nee(P.mis_mode, ls.pdf / (float)nl, pdf_b) : 1.f;
                        lcontrib = beta * f * ls.radiance * (w * (float)nl * cosl / ls.pdf);
                        if(max3(lcontrib) > 0.f)
                        {
                            push_light = true;
                            ldir_s = ls.dir;
                            ldist = ls.dist;
                        }
                    }
                }
                // BSDF sample (sample_disney) and throughput
                const bsdf_sample bs = sample_bsdf(m, N, V, eta, u[0], u[1], u[2]);
                bool alive = bs.pdf > 0.f && !push_query;
                if(alive)
                {
                    // raypipeline.slang:632-637: a bounce with pdf below the threshold turns
                    // regularisation on; the refractive-caustic marker follows the same test
                    const bool below = bs.pdf < PT_REGULARIZE_PDF_THRESHOLD;
                    const bool caustic = below && ((flags & PATH_CAUSTIC) || bs.transmission);
                    flags = (flags | (below ? PATH_REGULARIZE : 0u)) & ~(PATH_CAUSTIC | PATH_NO_ENV_NEE);
                    if(caustic) flags |= PATH_CAUSTIC;
                    const float cost = fabsf(dot(N, bs.dir));
                    float3 tp = bs.f * (cost / fmaxf(bs.pdf, PT_PDF_EPS));
                    if(depth >= 1 && P.max_path_beta > 0.f)
                        tp = f3(fminf(tp.x, P.max_path_beta), fminf(tp.y, P.max_path_beta), fminf(tp.z, P.max_path_beta));
                    beta = beta * tp;
                    // the first transmission through a dispersive surface locks the wavelength and tints
                    // the throughput by its white-balanced colour (raypipeline.slang:651-659)
                    if(dispersive && bs.transmission && !lambda_locked)
                    {
                        flags |= (uint32_t)__half_as_ushort(__float2half_rn(lambda)) << 16;
                        const float3 c = lambda_to_rgb(lambda);
                        beta = beta * f3(fmul(LAMBDA_RGB_NORM_R, c.x), fmul(LAMBDA_RGB_NORM_G, c.y),
                                         fmul(LAMBDA_RGB_NORM_B, c.z));
                    }
                    // MIS pdf of the bounce for an environment hit: the mixture pdf where the
                    // environment sampler competes (directions above the surface), 0 below it
                    float pdf_mix = 0.f;
                    if(dot(N, bs.dir) > 0.f)
                    {
                        if constexpr(FULL) pdf_mix = pdf_bsdf_ool(m, bs.dir, N, V, eta);
                        else eval_bsdf<false>(m, bs.dir, N, V, eta, pdf_mix);
                    }
                    prev_pdf = pdf_mix;
                    // Russian roulette
                    if(P.rr_depth == 0)
                    {
                        if(max3(beta) <= 0.05f * (float)depth)
                        {
                            const float q = 1.f - max3(beta);
                            if(u[7] < q) alive = false;
                            else beta = beta * (1.f / (1.f - q));
                        }
                    }
                    else if(depth + 1 >= P.rr_depth)
                    {
                        const float q = fmaxf(0.f, 1.f - max3(beta));
                        if(u[7] < q) alive = false;
                        else beta = beta * (1.f / (1.f - q));
                    }
                    if(alive && depth + 1 < P.max_depth)
                    {
                        push_ext = true;
                        ndir = bs.dir;
                    }
                    if(boundary && bs.transmission)
                    {
                        if(back_face) stack_pop(mst);
                        else stack_push(mst, mat);
                    }
                }
                }
            }
        done:
            if(media) P.mstack[pid] = mst;
            rng[pid] = g.state;
            // the reference's chain of a finished path continues with the pixel's next sample
            if(P.ref_rng && !push_ext) P.ref_chain[pid] = (uint32_t)g.state;
            beta_pdf[pid] = make_float4(beta.x, beta.y, beta.z, prev_pdf);
            radiance[pid] = make_float4(L.x, L.y, L.z, __uint_as_float(flags));
        }
        const uint32_t pe = warp_push(out_count, push_ext);
        if(push_ext)
        {
            float4 *o = reinterpret_cast<float4 *>(out_ray + pe);
            o[0] = make_float4(P0.x, P0.y, P0.z, PT_EPS);
            o[1] = make_float4(ndir.x, ndir.y, ndir.z, PT_TMAX);
            out_pid[pe] = pid;
        }
        const uint32_t ps = warp_push(s_count, push_shadow);
        if(push_shadow)
        {
            // from a surface: offset along the normal, tmin 0; from inside a medium: the scattering
            // point, tmin EPS, back faces culled (flag in the contribution's w)
            const float3 so = cull_back_shadow ? P0 : P0 + N * PT_EPS;
            float4 *o = reinterpret_cast<float4 *>(s_ray + ps);
            o[0] = make_float4(so.x, so.y, so.z, cull_back_shadow ? PT_EPS : 0.f);
            o[1] = make_float4(sdir.x, sdir.y, sdir.z, PT_TMAX);
            s_pid[ps] = pid;
            s_contrib[ps] = make_float4(contrib.x, contrib.y, contrib.z, cull_back_shadow ? 1.f : 0.f);
        }
        if(FULL && lq.count)
        {
            const uint32_t pl = warp_push(lq.count, push_light);
            if(push_light)
            {
                const float3 so = cull_back_shadow ? P0 : P0 + N * PT_EPS;
                float4 *o = reinterpret_cast<float4 *>(lq.ray + pl);
                o[0] = make_float4(so.x, so.y, so.z, cull_back_shadow ? PT_EPS : 0.f);
                o[1] = make_float4(ldir_s.x, ldir_s.y, ldir_s.z, ldist);
                lq.pid[pl] = pid;
                lq.contrib[pl] = make_float4(lcontrib.x, lcontrib.y, lcontrib.z, cull_back_shadow ? 1.f : 0.f);
            }
        }
        if constexpr(MODE == MODE_CACHE)
        {
            const uint32_t pq = warp_push(io.q_count, push_query);
            if(push_query)
            {
                // feature record: position, outgoing direction, normal, roughness, albedo
                float *f = io.q_feat + (size_t)nrc::FEAT * pq;
                const float3 V = vq;
                f[0] = P0.x; f[1] = P0.y; f[2] = P0.z;
                f[3] = V.x; f[4] = V.y; f[5] = V.z;
                f[6] = N.x; f[7] = N.y; f[8] = N.z;
                f[9] = rough;
                f[10] = albedo.x; f[11] = albedo.y; f[12] = albedo.z;
                io.q_beta[pq] = make_float4(qbeta.x, qbeta.y, qbeta.z, __uint_as_float(pid));
            }
        }
    }
}

// ALPHA: alpha-tested materials (alpha_filter), each candidate's uniform hashed from rng[path]
template<class J, int STACK = (int)TRAVERSAL_STACK, bool ALPHA = false>
__global__ void __launch_bounds__(PT_THREADS, STACK <= 64 ? 8 : 6) // 64 / 85 registers
        k_pt_shadow(J S, const vkg_ray *__restrict__ s_ray, const uint32_t *__restrict__ s_pid,
                    const float4 *__restrict__ s_contrib, const uint32_t *__restrict__ count,
                    float4 *__restrict__ radiance, const uint32_t *__restrict__ perm = nullptr,
                    const uint32_t *__restrict__ reordered = nullptr, const uint64_t *__restrict__ rng = nullptr)
{
    const uint32_t n = *count;
    const uint32_t stride = gridDim.x * blockDim.x;
    // a binned queue (bin_rays): position j tests entry perm[j] (each path has one entry per launch)
    if(perm && *reordered == 0u) perm = nullptr;
    for(uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += stride)
    {
        const uint32_t i = perm ? __ldg(perm + j) : j;
        const pt_params &P = S.params(J::per_path ? s_pid[i] : 0u);
        const float4 *rp = reinterpret_cast<const float4 *>(s_ray + i);
        const float4 r0 = __ldg(rp), r1 = __ldg(rp + 1);
        const float4 c = s_contrib[i];
        const int cull = c.w != 0.f ? CULL_BACK : CULL_NONE; // from inside a medium: back faces culled
        using F = std::conditional_t<ALPHA, alpha_filter, no_filter>;
        F f{};
        if constexpr(ALPHA) f = alpha_filter{&P, rng[s_pid[i]], 0.f, ALPHA_SALT_SHADOW, false};
        bool occluded;
        if(P.two_level)
            occluded = trace_tlas<true, F>(P.tl_nodes, P.tl_inst, P.tl_blas, r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, r1.z,
                                           r1.w, cull, f)
                               .occluded;
        else
        {
            unsigned long long v = 0, t = 0;
            occluded = trace_ray<true, false, STACK, F>(P.nodes, P.tris, r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, r1.z, r1.w,
                                                        cull, v, t, nullptr, f)
                               .occluded;
        }
        if(!occluded)
        {
            const uint32_t pid = s_pid[i];
            float4 L = radiance[pid];
            L.x += c.x;
            L.y += c.y;
            L.z += c.z;
            radiance[pid] = L;
        }
    }
}

// light-NEE visibility (transmittance_test, visibility_test.slang:94-131): 0 at the first opaque
// surface on the segment, else the product of transmission x base colour over the transmissive
// surfaces it crosses; null surfaces pass unattenuated. Scenes without transmissive materials take one any-hit query; single-level
// scenes one pass over the crossed triangles (trace_transmit); instanced scenes repeated closest-hit
// queries from the last crossing (at most PT_MAX_CROSSINGS; more count as blocked). Runs after the
// environment shadow kernel, so each path's radiance has one writer at a time.
constexpr int PT_MAX_CROSSINGS = 32;

template<class J, int STACK = (int)TRAVERSAL_STACK, bool ALPHA = false>
__global__ void __launch_bounds__(PT_THREADS, STACK <= 64 ? 8 : 6) // 64 / 85 registers
        k_pt_light_shadow(J S, light_queue lq, float4 *__restrict__ radiance, const uint64_t *__restrict__ rng = nullptr)
{
    const uint32_t n = *lq.count;
    const uint32_t stride = gridDim.x * blockDim.x;
    for(uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    {
        const uint32_t pid = lq.pid[i];
        const pt_params &P = S.params(J::per_path ? pid : 0u);
        const float4 *rp = reinterpret_cast<const float4 *>(lq.ray + i);
        const float4 r0 = __ldg(rp), r1 = __ldg(rp + 1);
        const float4 cc = lq.contrib[i];
        // rays from inside a medium cull back faces (nee_volume, direct_lighting.slang:348-354)
        const int cull = cc.w != 0.f ? CULL_BACK : CULL_NONE;
        float3 T = f3(1.f, 1.f, 1.f);
        unsigned long long v = 0, c = 0;
        using F = std::conditional_t<ALPHA, alpha_filter, no_filter>;
        F f{};
        if constexpr(ALPHA) f = alpha_filter{&P, rng[pid], 0.f, ALPHA_SALT_LIGHT_SHADOW, true};
        if(!P.transmissive)
        {
            const bool occ = P.two_level ? trace_tlas<true, F>(P.tl_nodes, P.tl_inst, P.tl_blas, r0.x, r0.y, r0.z, r0.w,
                                                               r1.x, r1.y, r1.z, r1.w, cull, f)
                                                   .occluded
                                         : trace_ray<true, false, STACK, F>(P.nodes, P.tris, r0.x, r0.y, r0.z, r0.w,
                                                                            r1.x, r1.y, r1.z, r1.w, cull, v, c, nullptr,
                                                                            f)
                                                   .occluded;
            if(occ) T = f3(0.f, 0.f, 0.f);
        }
        else if(!P.two_level)
        {
            // Beer-Lambert through transmissive volumes: optical depth -sigma_t t at an entry (front
            // face), +sigma_t t at an exit, clamped at 0 (visibility_test.slang:123-129, :161-162)
            float3 od = f3(0.f, 0.f, 0.f);
            const bool open = trace_transmit<STACK>(
                    P.nodes, P.tris, r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, r1.z, r1.w, cull, T,
                    [&](uint32_t prim, float t, bool front) {
                        const uint32_t mi = __ldg(&P.tri_mat[prim]);
                        const vkg_material &q = P.mats[mi];
                        if(q.null_surface) return f3(1.f, 1.f, 1.f); // null surfaces pass unattenuated
                        if(P.media && (P.media[mi].flags & MEDIUM_VOLUME))
                        {
                            const medium_rec &M = P.media[mi];
                            const float3 st = f3(M.sigma_s[0] + M.sigma_a[0], M.sigma_s[1] + M.sigma_a[1],
                                                 M.sigma_s[2] + M.sigma_a[2]);
                            od = od + st * (front ? -t : t);
                        }
                        return f3(q.base_color[0], q.base_color[1], q.base_color[2]) * q.transmission;
                    },
                    f);
            if(!open) T = f3(0.f, 0.f, 0.f);
            else if(P.media)
                T = T * f3(expf(-fmaxf(od.x, 0.f)), expf(-fmaxf(od.y, 0.f)), expf(-fmaxf(od.z, 0.f)));
        }
        else
        {
            // instanced scenes: a material per instance, so crossings are found one closest hit at a time;
            // Beer-Lambert optical depth as in the single-level pass, the face taken from the hit's
            // world-space geometric normal
            float tmin = r0.w;
            float3 od = f3(0.f, 0.f, 0.f);
            for(int k = 0;; ++k)
            {
                uint32_t prim, mat, inst = 0;
                float t, hu = 0.f, hv = 0.f;
                if(P.two_level)
                {
                    const tlas_result r = trace_tlas<false, F>(P.tl_nodes, P.tl_inst, P.tl_blas, r0.x, r0.y, r0.z,
                                                               tmin, r1.x, r1.y, r1.z, r1.w, cull, f);
                    prim = r.prim;
                    t = r.t;
                    inst = r.inst;
                    hu = r.u;
                    hv = r.v;
                    mat = prim == VKG_MISS ? 0u : __ldg(&P.tl_by_id[r.inst].material);
                }
                else
                {
                    const trace_result r = trace_ray<false, false, STACK, F>(P.nodes, P.tris, r0.x, r0.y, r0.z, tmin,
                                                                             r1.x, r1.y, r1.z, r1.w, cull, v, c,
                                                                             nullptr, f);
                    prim = r.prim;
                    t = r.t;
                    hu = r.u;
                    hv = r.v;
                    mat = prim == VKG_MISS ? 0u : __ldg(&P.tri_mat[prim]);
                }
                if(prim == VKG_MISS) break;
                const vkg_material &q = P.mats[mat];
                if(q.null_surface && k + 1 < PT_MAX_CROSSINGS)
                {
                    tmin = t;
                    continue;
                }
                if(!(q.transmission > 0.f) || k + 1 >= PT_MAX_CROSSINGS)
                {
                    T = f3(0.f, 0.f, 0.f);
                    break;
                }
                T = T * f3(q.base_color[0], q.base_color[1], q.base_color[2]) * q.transmission;
                if(P.media && (P.media[mat].flags & MEDIUM_VOLUME))
                {
                    float3 hp, ng;
                    uint32_t hm;
                    hit_surface(P, prim, inst, hu, hv, hp, ng, hm);
                    const medium_rec &M = P.media[mat];
                    const float3 st = f3(M.sigma_s[0] + M.sigma_a[0], M.sigma_s[1] + M.sigma_a[1],
                                         M.sigma_s[2] + M.sigma_a[2]);
                    od = od + st * (dot(ng, f3(r1.x, r1.y, r1.z)) < 0.f ? -t : t);
                }
                tmin = t;
            }
            if(P.media && max3(T) > 0.f)
                T = T * f3(expf(-fmaxf(od.x, 0.f)), expf(-fmaxf(od.y, 0.f)), expf(-fmaxf(od.z, 0.f)));
        }
        if(max3(T) > 0.f)
        {
            float4 L = radiance[pid];
            L.x += T.x * cc.x;
            L.y += T.y * cc.y;
            L.z += T.z * cc.z;
            radiance[pid] = L;
        }
    }
}

// persistent queue tracer: each warp refills its finished lanes from the queue with one atomic
// (work stealing), so rays of cheap and expensive scenes balance across the machine. SHADOW: any-hit
// visibility of NEE rays, adding the contribution of unoccluded ones; else closest hit of extension
// rays. Single-level scenes only (instanced scenes use k_pt_tl_persistent or the grid-stride
// kernels). `work` must be zero at launch.
template<bool SHADOW, class J, int STACK = (int)TRAVERSAL_STACK>
__global__ void __launch_bounds__(PT_THREADS)
        k_pt_trace_persistent(J S, const vkg_ray *__restrict__ q_ray, const uint32_t *__restrict__ q_pid,
                              const uint32_t *__restrict__ count, vkg_hit *__restrict__ hits,
                              uint32_t *__restrict__ hit_inst, const float4 *__restrict__ s_contrib,
                              float4 *__restrict__ radiance, uint32_t *__restrict__ work)
{
    const uint32_t n = *count;
    const uint32_t lane = threadIdx.x & 31u, lt = (1u << lane) - 1u;
    unsigned long long v = 0, t = 0;
    ray_state_t<STACK> s;
    uint2 stack[STACK];
    s.st = stack;
    const node8 *nodes = nullptr;
    const tri_rec *tris = nullptr;
    uint32_t cur = 0xFFFFFFFFu;
    bool exhausted = false;
    for(;;)
    {
        const bool need = cur == 0xFFFFFFFFu && !exhausted;
        const unsigned m = __ballot_sync(0xffffffffu, need);
        if(m)
        {
            const uint32_t leader = __ffs(m) - 1;
            uint32_t base = 0;
            if(lane == leader) base = atomicAdd(work, (uint32_t)__popc(m));
            base = __shfl_sync(0xffffffffu, base, leader);
            if(need)
            {
                const uint32_t idx = base + __popc(m & lt);
                if(idx < n)
                {
                    const pt_params &P = S.params(J::per_path ? q_pid[idx] : 0u);
                    const float4 *rp = reinterpret_cast<const float4 *>(q_ray + idx);
                    const float4 r0 = __ldg(rp), r1 = __ldg(rp + 1);
                    nodes = P.nodes;
                    tris = P.tris;
                    ray_init(s, r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, r1.z, r1.w);
                    cur = idx;
                }
                else
                    exhausted = true;
            }
        }
        const bool active = cur != 0xFFFFFFFFu;
        if(!__any_sync(0xffffffffu, active)) break;
        if(active &&
           !ray_step_auto<SHADOW, false>(s, nodes, tris, SHADOW ? CULL_NONE : CULL_BACK_UNLESS_TWOSIDED, v, t, nullptr))
        {
            const trace_result r = ray_result(s);
            if constexpr(SHADOW)
            {
                if(!r.occluded)
                {
                    const uint32_t pid = q_pid[cur];
                    const float4 c = s_contrib[cur];
                    float4 L = radiance[pid];
                    L.x += c.x;
                    L.y += c.y;
                    L.z += c.z;
                    radiance[pid] = L;
                }
            }
            else
                reinterpret_cast<uint4 *>(hits)[cur] =
                        make_uint4(r.prim, __float_as_uint(r.t), __float_as_uint(r.u), __float_as_uint(r.v));
            cur = 0xFFFFFFFFu;
        }
    }
}

// the same persistent refilling for instanced scenes: one two-level node per step (tl_step), so a
// lane whose ray finished takes the next ray of the queue at once instead of idling until the slowest
// lane of its warp is done. One scene per launch. `work` must be zero at launch.
template<bool SHADOW>
__global__ void __launch_bounds__(PT_THREADS)
        k_pt_tl_persistent(single_scene S, const vkg_ray *__restrict__ q_ray, const uint32_t *__restrict__ q_pid,
                           const uint32_t *__restrict__ count, vkg_hit *__restrict__ hits,
                           uint32_t *__restrict__ hit_inst, const float4 *__restrict__ s_contrib,
                           float4 *__restrict__ radiance, uint32_t *__restrict__ work)
{
    const pt_params &P = S.P;
    const uint32_t n = *count;
    const uint32_t lane = threadIdx.x & 31u, lt = (1u << lane) - 1u;
    const int cull = SHADOW ? CULL_NONE : CULL_BACK_UNLESS_TWOSIDED;
    tl_state s;
    uint2 stack[TL_STACK];
    s.st = stack;
    uint32_t cur = 0xFFFFFFFFu;
    bool exhausted = false;
    for(;;)
    {
        const bool need = cur == 0xFFFFFFFFu && !exhausted;
        const unsigned m = __ballot_sync(0xffffffffu, need);
        if(m)
        {
            const uint32_t leader = __ffs(m) - 1;
            uint32_t base = 0;
            if(lane == leader) base = atomicAdd(work, (uint32_t)__popc(m));
            base = __shfl_sync(0xffffffffu, base, leader);
            if(need)
            {
                const uint32_t idx = base + __popc(m & lt);
                if(idx < n)
                {
                    const float4 *rp = reinterpret_cast<const float4 *>(q_ray + idx);
                    const float4 r0 = __ldg(rp), r1 = __ldg(rp + 1);
                    tl_init(s, P.tl_nodes, r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, r1.z, r1.w);
                    cur = idx;
                }
                else
                    exhausted = true;
            }
        }
        const bool active = cur != 0xFFFFFFFFu;
        if(!__any_sync(0xffffffffu, active)) break;
        if(active && !tl_step<SHADOW>(s, P.tl_nodes, P.tl_inst, P.tl_blas, cull))
        {
            if constexpr(SHADOW)
            {
                if(!s.done)
                {
                    const uint32_t pid = q_pid[cur];
                    const float4 c = s_contrib[cur];
                    float4 L = radiance[pid];
                    L.x += c.x;
                    L.y += c.y;
                    L.z += c.z;
                    radiance[pid] = L;
                }
            }
            else
            {
                const bool hit = s.best_prim != VKG_MISS;
                reinterpret_cast<uint4 *>(hits)[cur] =
                        make_uint4(s.best_prim, __float_as_uint(hit ? s.best_t : 0.f), __float_as_uint(hit ? s.bu : 0.f),
                                   __float_as_uint(hit ? s.bv : 0.f));
                hit_inst[cur] = s.best_inst;
            }
            cur = 0xFFFFFFFFu;
        }
    }
}

__global__ void k_fill_miss_queue(const uint32_t *__restrict__ count, vkg_hit *__restrict__ hits)
{
    const uint32_t n = *count;
    for(uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        reinterpret_cast<uint4 *>(hits)[i] = make_uint4(VKG_MISS, 0u, 0u, 0u);
}

__global__ void k_pt_tally(const uint32_t *__restrict__ ext_count, const uint32_t *__restrict__ s_count,
                           const uint32_t *__restrict__ l_count, unsigned long long *__restrict__ totals)
{
    totals[0] += *ext_count;
    totals[1] += *s_count + (l_count ? *l_count : 0u);
}

// rendering with a cache: path radiance += throughput x prediction (negative outputs clamped)
__global__ void k_cache_resolve(const float4 *__restrict__ q_beta, const float *__restrict__ Y,
                                const uint32_t *__restrict__ count, float4 *__restrict__ radiance,
                                unsigned long long *__restrict__ totals)
{
    const uint32_t n = *count;
    if(blockIdx.x == 0 && threadIdx.x == 0) totals[2] += n;
    for(uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        const float4 b = q_beta[i];
        const uint32_t pid = __float_as_uint(b.w);
        float4 L = radiance[pid];
        L.x += b.x * fmaxf(Y[3 * (size_t)i], 0.f);
        L.y += b.y * fmaxf(Y[3 * (size_t)i + 1], 0.f);
        L.z += b.z * fmaxf(Y[3 * (size_t)i + 2], 0.f);
        radiance[pid] = L;
    }
}

// training wave done: one (features, target) pair per recorded interaction, compacted in path order
__global__ void __launch_bounds__(PT_THREADS)
        k_cache_targets(const float4 *__restrict__ rec, const uint32_t *__restrict__ vcount, uint32_t paths,
                        uint32_t rec_depth, const float4 *__restrict__ radiance, float *__restrict__ t_feat,
                        float *__restrict__ t_target, uint32_t *__restrict__ t_count)
{
    const uint32_t n = paths * rec_depth;
    for(uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x)
    {
        const uint32_t i = base + threadIdx.x;
        bool ok = false;
        float f[nrc::FEAT], tg[3];
        if(i < n)
        {
            const uint32_t p = i / rec_depth, k = i - p * rec_depth;
            if(k < vcount[p])
            {
                const float4 *r = rec + (size_t)i * REC_F4;
                const float4 r0 = r[0], r1 = r[1], r2 = r[2], r3 = r[3], r4 = r[4];
                const float4 Lf = radiance[p];
                const float beta[3] = {r3.y, r3.z, r3.w}, Lk[3] = {r4.x, r4.y, r4.z}, Lp[3] = {Lf.x, Lf.y, Lf.z};
                ok = true;
                for(int c = 0; c < 3; ++c)
                {
                    tg[c] = beta[c] > 0.f ? fmaxf(Lp[c] - Lk[c], 0.f) / beta[c] : 0.f;
                    ok = ok && isfinite(tg[c]);
                }
                const float v[nrc::FEAT] = {r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, r1.z, r1.w, r2.x, r2.y, r2.z, r2.w, r3.x};
                for(int c = 0; c < nrc::FEAT; ++c) f[c] = v[c];
            }
        }
        const uint32_t o = warp_push(t_count, ok);
        if(ok)
        {
            for(int c = 0; c < nrc::FEAT; ++c) t_feat[(size_t)o * nrc::FEAT + c] = f[c];
            for(int c = 0; c < 3; ++c) t_target[(size_t)o * 3 + c] = tg[c];
        }
    }
}

// optimiser step k of the frame trains on the window [k * B, (k + 1) * B) of the compacted records
__global__ void k_cache_window(const uint32_t *__restrict__ t_count, uint32_t k, uint32_t B,
                               uint32_t *__restrict__ b_count)
{
    const uint64_t cnt = *t_count, lo = (uint64_t)k * B;
    *b_count = cnt > lo ? (uint32_t)std::min<uint64_t>(cnt - lo, B) : 0u;
}

__global__ void k_pt_accumulate(uint32_t npix, uint32_t ns, const float4 *__restrict__ radiance, float *__restrict__ sum)
{
    uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
    if(pix >= npix) return;
    float sx = sum[3 * (size_t)pix], sy = sum[3 * (size_t)pix + 1], sz = sum[3 * (size_t)pix + 2];
    for(uint32_t k = 0; k < ns; ++k)
    {
        const float4 L = radiance[(size_t)k * npix + pix];
        sx += L.x;
        sy += L.y;
        sz += L.z;
    }
    sum[3 * (size_t)pix] = sx;
    sum[3 * (size_t)pix + 1] = sy;
    sum[3 * (size_t)pix + 2] = sz;
}

__global__ void k_pt_finalize(uint32_t npix, uint32_t spp, uint32_t batch, const float *__restrict__ sum,
                              float *__restrict__ accum, float *__restrict__ out)
{
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if(k >= 3 * npix) return;
    const float mean = sum[k] / (float)spp;
    const float a = batch == 0 ? mean : (mean + (float)batch * accum[k]) / (float)(batch + 1);
    accum[k] = a;
    if(out) out[k] = a;
}

// the accumulated radiance into the pixel records
__global__ void k_pixel_radiance(const float *__restrict__ accum, uint32_t npix, vkg_pixel_data *__restrict__ px)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= npix) return;
    px[i].radiance[0] = accum[3 * (size_t)i];
    px[i].radiance[1] = accum[3 * (size_t)i + 1];
    px[i].radiance[2] = accum[3 * (size_t)i + 2];
}

__global__ void k_tri_flags(tri_rec *__restrict__ tris, uint32_t n, const uint32_t *__restrict__ tri_mat,
                            const vkg_material *__restrict__ mats, uint32_t num_mats)
{
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= n) return;
    const uint32_t m = tri_mat[tris[i].prim];
    tris[i].pad[0] = (m < num_mats && material_unculled(mats[m]) ? TRI_FLAG_TWOSIDED : 0u) |
                     (m < num_mats && (mats[m].transmission > 0.f || mats[m].null_surface) ? TRI_FLAG_TRANSMISSIVE : 0u) |
                     (m < num_mats && material_alpha_tested(mats[m]) ? TRI_FLAG_ALPHA : 0u);
}

__global__ void k_check_materials(const uint32_t *__restrict__ tri_mat, uint32_t n, uint32_t num_mats,
                                  uint32_t *__restrict__ bad)
{
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i < n && tri_mat[i] >= num_mats) atomicOr(bad, 1u);
}

}// namespace

// settings checks shared by the tracer and the batch renderer (pathtrace.cu)
vkg_status check_tracer_settings(vkg_ctx *ctx, const vkg_settings *s);

// the crop window of a settings block: (x0, y0, width, height); the whole image if no crop is set
inline void crop_window(const vkg_settings &S, uint32_t &x0, uint32_t &y0, uint32_t &w, uint32_t &h)
{
    const bool crop = S.crop[2] && S.crop[3];
    x0 = crop ? S.crop[0] : 0;
    y0 = crop ? S.crop[1] : 0;
    w = crop ? S.crop[2] : S.resolution[0];
    h = crop ? S.crop[3] : S.resolution[1];
}

// the per-launch parameters of one scene, camera and settings block (no radiance cache)
inline pt_params make_params(const vkg_scene *sc, const vkg_camera &cam, const vkg_settings &S, uint32_t seed,
                             uint32_t batch)
{
    pt_params P{};
    P.nodes = sc->bvh ? sc->bvh->d_nodes : nullptr;
    P.tris = sc->bvh ? sc->bvh->d_tris : nullptr;
    if(sc->tlas)
    {
        P.two_level = 1;
        P.tl_nodes = sc->tlas->top.d_nodes;
        P.tl_inst = sc->tlas->d_inst;
        P.tl_by_id = sc->tlas->d_inst_by_id;
        P.tl_blas = sc->tlas->d_blas;
        P.meshes = sc->d_meshes;
    }
    P.xyz = sc->xyz;
    P.nrm = sc->nrm;
    P.uv = sc->uv;
    P.tng = sc->tng;
    P.tex = sc->d_tex;
    P.texels = sc->d_texels;
    P.num_textures = sc->num_textures;
    P.cone_spread = atanf(2.f * cam.tan_half_fovy / (float)cam.height);
    P.cone = nullptr;
    P.idx = sc->idx;
    P.tri_mat = sc->tri_mat;
    P.mats = sc->mats;
    P.env = env_view{sc->env.rgb, sc->env.pdf_w, sc->env.alias, sc->env.w, sc->env.h, S.environment};
    P.cam = cam;
    crop_window(S, P.cx0, P.cy0, P.cw, P.ch);
    P.npix = P.cw * P.ch;
    P.max_depth = S.max_trace_depth;
    P.rr_depth = S.rr_start_depth;
    P.mis_mode = S.mis_mode;
    P.disable_material = S.disable_material;
    P.draw_skybox = S.draw_skybox;
    P.max_path_beta = S.max_path_beta;
    P.seed = seed;
    P.batch = batch;
    P.dispersion = sc->any_dispersion ? 1u : 0u;
    P.term_depth = 0xFFFFFFFFu;
    P.rec_depth = 0;
    P.train_base = 0xFFFFFFFFu;
    P.train_paths = 0;
    P.lights = nullptr;
    P.num_lights = 0;
    P.suppress_caustics = S.suppress_refractive_caustics;
    P.transmissive = sc->any_transmissive ? 1u : 0u;
    P.gbuf = nullptr;
    P.media = sc->d_media;
    P.mstack = nullptr;
    P.cam_medium = 0xFFFFFFFFu;
    P.last_sample = S.num_samples ? S.num_samples - 1 : 0u;
    P.clip_near = S.clip_near > 0.f ? S.clip_near : 0.1f;
    return P;
}

// the light list of a render: the settings' sun (PBRPathTracer.cpp:610-624) first, then the scene's
inline std::vector<vkg_light> render_lights(const vkg_scene *sc, const vkg_settings &S)
{
    std::vector<vkg_light> out;
    if(S.sun_intensity > 0.f)
    {
        vkg_light sun{};
        sun.type = VKG_LIGHT_DIRECTIONAL;
        for(int c = 0; c < 3; ++c) sun.color[c] = S.sun_color[c];
        sun.intensity = S.sun_intensity;
        // the propagation direction: +z rotated by the quaternion of the Euler angles
        // (elevation, azimuth, 0), normalised
        const float hx = 0.5f * S.sun_spherical_coords[0], hy = 0.5f * S.sun_spherical_coords[1];
        const float cx = std::cos(hx), sx = std::sin(hx), cy = std::cos(hy), sy = std::sin(hy);
        const float qw = cx * cy, qx = sx * cy, qy = cx * sy, qz = -sx * sy;
        // v' = v + 2 w (q x v) + 2 q x (q x v) for v = (0, 0, 1)
        const float ax = qy, ay = -qx, az = 0.f;                                  // q x v
        const float bx = qy * az - qz * ay, by = qz * ax - qx * az, bz = qx * ay - qy * ax; // q x (q x v)
        float d[3] = {2.f * qw * ax + 2.f * bx, 2.f * qw * ay + 2.f * by, 1.f + 2.f * qw * az + 2.f * bz};
        const float len2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
        if(len2 > 0.f)
        {
            const float inv = 1.f / std::sqrt(len2);
            for(float &x: d) x *= inv;
        }
        for(int c = 0; c < 3; ++c) sun.direction[c] = d[c];
        sun.range = std::numeric_limits<float>::infinity();
        sun.angular_size = S.sun_angular_size;
        out.push_back(sun);
    }
    out.insert(out.end(), sc->lights.begin(), sc->lights.end());
    return out;
}
}// namespace vkg
