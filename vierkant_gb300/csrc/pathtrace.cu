// Wavefront plain path tracer: the multi-bounce radiance estimator of vierkant's PBRPathTracer
// (raygen / closest-hit / miss of shaders/slang/raypipeline.slang:91-270, :361-680, :747-781)
// restated as queue kernels, with next-event estimation against the importance-sampled
// environment added (the reference only reaches the environment through BSDF-sampled misses).
//
// Per wave (pixels x samples_per_wave paths in flight), per segment:
//   k_pt_extend   closest hit of every queued ray (back faces culled unless the triangle is two-sided,
//                 raypipeline.slang:165 + RayBuilder.cpp:521-522)
//   k_pt_shade    miss: environment radiance with the hit-side MIS weight; hit: emission, one
//                 environment NEE sample (pushed to the shadow queue with its MIS-weighted
//                 contribution), BSDF sample, throughput update F*cos/max(pdf, 1e-3)
//                 (raypipeline.slang:639-648), Russian roulette, next ray pushed to the other queue.
//                 Queues are compacted with warp ballots (one atomic per warp).
//   k_pt_shadow   any-hit visibility of the NEE rays (no culling, visibility_test.slang:45-87);
//                 visible contributions are added to the path radiance
// then k_pt_accumulate sums the wave's samples per pixel, and k_pt_finalize blends the batch into
// the running mean (raypipeline.slang:258-266). No host synchronisation inside a render: queue
// lengths live in device memory and every queue kernel is a grid-stride loop over them.
//
// RNG: PCG32 per path, initstate = create-info seed, initseq = (batch << 40) ^ (sample * pixels +
// pixel); the camera jitter takes 2 draws, every segment exactly 8 (lobe, 2 BSDF, 4 environment,
// roulette) whatever branch is taken.
//
// With a radiance cache attached (vkg_tracer_attach_cache) the same kernels run in two more modes:
//   rendering  the shade kernel turns the terminate_depth-th interaction of every path into a cache
//              query (features + throughput); one batched inference resolves all queries of the wave;
//   training   train_paths paths through random pixels (initseq tagged with bit 62, first draw picks
//              the pixel) run the plain estimator and record their first train_depth interactions
//              (features, throughput on arrival, radiance gathered so far including the emission
//              there); afterwards target_k = (L_path - L_k) / throughput_k, the radiance that left
//              interaction k towards the previous vertex, feeds train_steps optimiser steps.
#include "nrc.cuh"
#include "pathtrace.cuh"
#include "traverse.cuh"

#include <algorithm>
#include <cstring>

struct vkg_scene
{
    vkg_bvh *bvh = nullptr;
    float *xyz = nullptr;
    uint32_t *idx = nullptr;
    uint32_t *tri_mat = nullptr;
    vkg_material *mats = nullptr;
    uint32_t num_tris = 0, num_vertices = 0, num_materials = 0;
    vkg::env_tables env;
};

struct vkg_tracer
{
    vkg_ctx *ctx = nullptr;
    uint32_t seed = 0;
    vkg_settings settings{};
    uint32_t batch = 0;
    // buffers sized for `capacity` paths and `npix` pixels
    size_t capacity = 0, npix_cap = 0;
    vkg_ray *q_ray[2] = {nullptr, nullptr};
    uint32_t *q_pid[2] = {nullptr, nullptr};
    vkg_hit *hits = nullptr;
    vkg_ray *s_ray = nullptr;
    uint32_t *s_pid = nullptr;
    float4 *s_contrib = nullptr;
    uint64_t *rng = nullptr;
    float4 *beta_pdf = nullptr;
    float4 *radiance = nullptr;
    float *sum = nullptr;
    float *accum = nullptr;
    uint32_t *counters = nullptr;           // [0..1] queue lengths, [2] shadow queue length, [3] cache queries,
                                            // [4] training records, [5] training batch length
    unsigned long long *totals = nullptr;   // [0] extension rays, [1] shadow rays, [2] cache queries
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev_train = nullptr;
    uint64_t last_paths = 0;
    bool rendered = false;
    bool trained = false;
    // radiance cache
    vkg_nrc *cache = nullptr;
    size_t q_cap = 0, rec_cap = 0;
    float *q_feat = nullptr;       // cache queries: q_cap x 13
    float4 *q_beta = nullptr;      // throughput xyz, path id in w
    uint32_t *q_x = nullptr;       // encoded queries
    float *q_y = nullptr;          // predictions q_cap x 3
    float4 *rec = nullptr;         // training records: rec_cap x 5 float4, path-major
    uint32_t *vcount = nullptr;    // recorded interactions per training path
    float *t_feat = nullptr, *t_target = nullptr; // compacted training set: rec_cap x 13, rec_cap x 3
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
    const float *xyz;
    const uint32_t *idx;
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
};

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
        const float jx = u01(pcg32_next(g)), jy = u01(pcg32_next(g));
        const vkg_camera &c = P.cam;
        const float sx = fdiv(fadd((float)x, jx), (float)c.width);
        const float sy = fdiv(fadd((float)y, jy), (float)c.height);
        const float nx = fsub(fmul(2.0f, sx), 1.0f), ny = fsub(fmul(2.0f, sy), 1.0f);
        const float cx = fmul(nx, fmul(c.tan_half_fovy, c.aspect));
        const float cy = -fmul(ny, c.tan_half_fovy);
        float d[3];
        for(int a = 0; a < 3; ++a) d[a] = fadd(fadd(fmul(c.right[a], cx), fmul(c.up[a], cy)), fmul(c.back[a], -1.0f));
        const float inv = frcp(fsqrt(dot3(d[0], d[1], d[2], d[0], d[1], d[2])));
        float4 *o = reinterpret_cast<float4 *>(q_ray + p);
        o[0] = make_float4(c.eye[0], c.eye[1], c.eye[2], PT_EPS);
        o[1] = make_float4(fmul(d[0], inv), fmul(d[1], inv), fmul(d[2], inv), PT_TMAX);
        q_pid[p] = p;
        rng[p] = g.state;
        beta_pdf[p] = make_float4(1.f, 1.f, 1.f, 0.f);
        radiance[p] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    if(blockIdx.x == 0 && threadIdx.x == 0) counters[0] = n;
}

__global__ void __launch_bounds__(PT_THREADS)
        k_pt_extend(const node8 *__restrict__ nodes, const tri_rec *__restrict__ tris,
                    const vkg_ray *__restrict__ q_ray, const uint32_t *__restrict__ count, vkg_hit *__restrict__ hits)
{
    const uint32_t n = *count;
    const uint32_t stride = gridDim.x * blockDim.x;
    for(uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    {
        const float4 *rp = reinterpret_cast<const float4 *>(q_ray + i);
        const float4 r0 = __ldg(rp), r1 = __ldg(rp + 1);
        unsigned long long v = 0, t = 0;
        trace_result r = trace_ray<false, false>(nodes, tris, r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, r1.z, r1.w,
                                                 CULL_BACK_UNLESS_TWOSIDED, v, t, nullptr);
        reinterpret_cast<uint4 *>(hits)[i] =
                make_uint4(r.prim, __float_as_uint(r.t), __float_as_uint(r.u), __float_as_uint(r.v));
    }
}

template<int MODE>
__global__ void __launch_bounds__(PT_THREADS)
        k_pt_shade(pt_params P, uint32_t depth, const vkg_ray *__restrict__ in_ray,
                   const uint32_t *__restrict__ in_pid, const vkg_hit *__restrict__ hits,
                   const uint32_t *__restrict__ in_count, vkg_ray *__restrict__ out_ray,
                   uint32_t *__restrict__ out_pid, uint32_t *__restrict__ out_count, vkg_ray *__restrict__ s_ray,
                   uint32_t *__restrict__ s_pid, float4 *__restrict__ s_contrib, uint32_t *__restrict__ s_count,
                   uint64_t *__restrict__ rng, float4 *__restrict__ beta_pdf, float4 *__restrict__ radiance,
                   cache_io io)
{
    const uint32_t n = *in_count;
    const uint32_t stride = gridDim.x * blockDim.x;
    for(uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride)
    {
        const uint32_t i = base + threadIdx.x;
        const bool active = i < n;
        bool push_ext = false, push_shadow = false, push_query = false;
        float3 P0 = f3(0.f, 0.f, 0.f), ndir = P0, sdir = P0, N = P0;
        float3 contrib = P0, qbeta = P0, albedo = P0, vq = P0;
        float rough = 0.f;
        uint32_t pid = 0;
        if(active)
        {
            pid = in_pid[i];
            const float4 *rp = reinterpret_cast<const float4 *>(in_ray + i);
            const float4 r1 = rp[1];
            const float3 dir = f3(r1.x, r1.y, r1.z);
            const uint4 h = reinterpret_cast<const uint4 *>(hits)[i];
            pcg32 g{rng[pid], (path_seq(P, pid) << 1u) | 1u};
            float u[8];
            for(int k = 0; k < 8; ++k) u[k] = u01(pcg32_next(g));
            const float4 bp = beta_pdf[pid];
            float3 beta = f3(bp.x, bp.y, bp.z);
            float prev_pdf = bp.w;
            const float4 lr = radiance[pid];
            float3 L = f3(lr.x, lr.y, lr.z);
            if(h.x == VKG_MISS)
            {
                // miss_environment (raypipeline.slang:764-781) with the hit-side MIS weight
                const uint32_t t = env_texel(dir, P.env.w, P.env.h);
                float3 le = env_radiance(P.env, t);
                if(depth == 0 && !P.draw_skybox) le = f3(0.f, 0.f, 0.f);
                float w = 1.f;
                if(prev_pdf > 0.f)
                {
                    if(P.mis_mode == 1) w = 0.f;
                    else if(P.mis_mode == 0) w = power_heuristic(prev_pdf, env_pdf(P.env, dir, t));
                }
                L = L + beta * le * w;
            }
            else
            {
                const uint32_t prim = h.x;
                const float bu = __uint_as_float(h.z), bv = __uint_as_float(h.w);
                const uint32_t i0 = __ldg(&P.idx[3 * (size_t)prim]), i1 = __ldg(&P.idx[3 * (size_t)prim + 1]),
                               i2 = __ldg(&P.idx[3 * (size_t)prim + 2]);
                const float3 v0 = f3(__ldg(&P.xyz[3 * (size_t)i0]), __ldg(&P.xyz[3 * (size_t)i0 + 1]),
                                     __ldg(&P.xyz[3 * (size_t)i0 + 2]));
                const float3 v1 = f3(__ldg(&P.xyz[3 * (size_t)i1]), __ldg(&P.xyz[3 * (size_t)i1 + 1]),
                                     __ldg(&P.xyz[3 * (size_t)i1 + 2]));
                const float3 v2 = f3(__ldg(&P.xyz[3 * (size_t)i2]), __ldg(&P.xyz[3 * (size_t)i2 + 1]),
                                     __ldg(&P.xyz[3 * (size_t)i2 + 2]));
                const float3 e1 = v1 - v0, e2 = v2 - v0;
                P0 = v0 + e1 * bu + e2 * bv;
                const float3 ng = normalize(cross(e1, e2));
                N = dot(ng, dir) < 0.f ? ng : -ng; // shading normal faces the incoming ray
                const float3 V = -dir;
                const vkg_material mt = P.mats[__ldg(&P.tri_mat[prim])];
                material_view m;
                m.base = P.disable_material ? f3(0.8f, 0.8f, 0.8f) : f3(mt.base_color[0], mt.base_color[1], mt.base_color[2]);
                m.roughness = mt.roughness;
                m.metalness = mt.metalness;
                L = L + beta * f3(mt.emission[0], mt.emission[1], mt.emission[2]);
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
                        const float3 f = eval_bsdf(m, ld, N, V, pdf_b);
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
                // BSDF sample (sample_disney) and throughput
                const bsdf_sample bs = sample_bsdf(m, N, V, u[0], u[1], u[2]);
                bool alive = bs.pdf > 0.f && !push_query;
                if(alive)
                {
                    const float cost = fabsf(dot(N, bs.dir));
                    float3 tp = bs.f * (cost / fmaxf(bs.pdf, PT_PDF_EPS));
                    if(depth >= 1 && P.max_path_beta > 0.f)
                        tp = f3(fminf(tp.x, P.max_path_beta), fminf(tp.y, P.max_path_beta), fminf(tp.z, P.max_path_beta));
                    beta = beta * tp;
                    float pdf_mix = 0.f;
                    eval_bsdf(m, bs.dir, N, V, pdf_mix);
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
                }
            }
            rng[pid] = g.state;
            beta_pdf[pid] = make_float4(beta.x, beta.y, beta.z, prev_pdf);
            radiance[pid] = make_float4(L.x, L.y, L.z, 0.f);
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
            const float3 so = P0 + N * PT_EPS;
            float4 *o = reinterpret_cast<float4 *>(s_ray + ps);
            o[0] = make_float4(so.x, so.y, so.z, 0.f);
            o[1] = make_float4(sdir.x, sdir.y, sdir.z, PT_TMAX);
            s_pid[ps] = pid;
            s_contrib[ps] = make_float4(contrib.x, contrib.y, contrib.z, 0.f);
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

__global__ void __launch_bounds__(PT_THREADS)
        k_pt_shadow(const node8 *__restrict__ nodes, const tri_rec *__restrict__ tris, const vkg_ray *__restrict__ s_ray,
                    const uint32_t *__restrict__ s_pid, const float4 *__restrict__ s_contrib,
                    const uint32_t *__restrict__ count, float4 *__restrict__ radiance)
{
    const uint32_t n = *count;
    const uint32_t stride = gridDim.x * blockDim.x;
    for(uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    {
        const float4 *rp = reinterpret_cast<const float4 *>(s_ray + i);
        const float4 r0 = __ldg(rp), r1 = __ldg(rp + 1);
        unsigned long long v = 0, t = 0;
        trace_result r = trace_ray<true, false>(nodes, tris, r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, r1.z, r1.w, CULL_NONE,
                                                v, t, nullptr);
        if(!r.occluded)
        {
            const uint32_t pid = s_pid[i];
            const float4 c = s_contrib[i];
            float4 L = radiance[pid];
            L.x += c.x;
            L.y += c.y;
            L.z += c.z;
            radiance[pid] = L;
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
                           unsigned long long *__restrict__ totals)
{
    totals[0] += *ext_count;
    totals[1] += *s_count;
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

__global__ void k_tri_flags(tri_rec *__restrict__ tris, uint32_t n, const uint32_t *__restrict__ tri_mat,
                            const vkg_material *__restrict__ mats, uint32_t num_mats)
{
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= n) return;
    const uint32_t m = tri_mat[tris[i].prim];
    tris[i].pad[0] = (m < num_mats && mats[m].twosided) ? TRI_FLAG_TWOSIDED : 0u;
}

__global__ void k_check_materials(const uint32_t *__restrict__ tri_mat, uint32_t n, uint32_t num_mats,
                                  uint32_t *__restrict__ bad)
{
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i < n && tri_mat[i] >= num_mats) atomicOr(bad, 1u);
}

void tracer_free_buffers(vkg_tracer *t)
{
    for(void *p: {(void *)t->q_ray[0], (void *)t->q_ray[1], (void *)t->q_pid[0], (void *)t->q_pid[1], (void *)t->hits,
                  (void *)t->s_ray, (void *)t->s_pid, (void *)t->s_contrib, (void *)t->rng, (void *)t->beta_pdf,
                  (void *)t->radiance, (void *)t->sum, (void *)t->accum})
        cudaFree(p);
    t->q_ray[0] = t->q_ray[1] = nullptr;
    t->q_pid[0] = t->q_pid[1] = nullptr;
    t->hits = nullptr;
    t->s_ray = nullptr;
    t->s_pid = nullptr;
    t->s_contrib = nullptr;
    t->rng = nullptr;
    t->beta_pdf = t->radiance = nullptr;
    t->sum = t->accum = nullptr;
    t->capacity = t->npix_cap = 0;
}

void tracer_free_cache_buffers(vkg_tracer *t)
{
    for(void *p: {(void *)t->q_feat, (void *)t->q_beta, (void *)t->q_x, (void *)t->q_y, (void *)t->rec,
                  (void *)t->vcount, (void *)t->t_feat, (void *)t->t_target})
        cudaFree(p);
    t->q_feat = nullptr;
    t->q_beta = nullptr;
    t->q_x = nullptr;
    t->q_y = nullptr;
    t->rec = nullptr;
    t->vcount = nullptr;
    t->t_feat = t->t_target = nullptr;
    t->q_cap = t->rec_cap = 0;
}

// query buffers for `queries` rendering paths, training buffers for the cache's configuration
vkg_status tracer_ensure_cache(vkg_tracer *t, size_t queries)
{
    const vkg_nrc_config &cfg = nrc::nrc_config(t->cache);
    const size_t recs = (size_t)cfg.train_paths * cfg.train_depth;
    if(queries <= t->q_cap && recs <= t->rec_cap && (t->q_cap || !queries)) return VKG_OK;
    queries = std::max(queries, t->q_cap);
    tracer_free_cache_buffers(t);
    cudaError_t e = cudaSuccess;
    auto al = [&](void **p, size_t bytes) {
        if(e == cudaSuccess && bytes) e = cudaMalloc(p, bytes);
    };
    al((void **)&t->q_feat, queries * nrc::FEAT * sizeof(float));
    al((void **)&t->q_beta, queries * sizeof(float4));
    al((void **)&t->q_x, queries * nrc::ENCODED_BYTES);
    al((void **)&t->q_y, queries * 3 * sizeof(float));
    al((void **)&t->rec, std::max<size_t>(recs, 1) * REC_F4 * sizeof(float4));
    al((void **)&t->vcount, std::max<size_t>(cfg.train_paths, 1) * sizeof(uint32_t));
    al((void **)&t->t_feat, std::max<size_t>(recs, 1) * nrc::FEAT * sizeof(float));
    al((void **)&t->t_target, std::max<size_t>(recs, 1) * 3 * sizeof(float));
    if(e != cudaSuccess)
    {
        tracer_free_cache_buffers(t);
        return cuda_check(t->ctx, e, "radiance cache buffers");
    }
    t->q_cap = queries;
    t->rec_cap = recs;
    return VKG_OK;
}

// (re)allocates the wave buffers; a new pixel count also restarts the accumulation
vkg_status tracer_ensure(vkg_tracer *t, size_t paths, size_t npix)
{
    if(paths <= t->capacity && npix == t->npix_cap) return VKG_OK;
    paths = std::max(paths, t->npix_cap == npix ? t->capacity : size_t(0));
    tracer_free_buffers(t);
    cudaError_t e = cudaSuccess;
    auto al = [&](void **p, size_t bytes) {
        if(e == cudaSuccess) e = cudaMalloc(p, bytes);
    };
    for(int q = 0; q < 2; ++q)
    {
        al((void **)&t->q_ray[q], paths * sizeof(vkg_ray));
        al((void **)&t->q_pid[q], paths * sizeof(uint32_t));
    }
    al((void **)&t->hits, paths * sizeof(vkg_hit));
    al((void **)&t->s_ray, paths * sizeof(vkg_ray));
    al((void **)&t->s_pid, paths * sizeof(uint32_t));
    al((void **)&t->s_contrib, paths * sizeof(float4));
    al((void **)&t->rng, paths * sizeof(uint64_t));
    al((void **)&t->beta_pdf, paths * sizeof(float4));
    al((void **)&t->radiance, paths * sizeof(float4));
    al((void **)&t->sum, npix * 3 * sizeof(float));
    al((void **)&t->accum, npix * 3 * sizeof(float));
    if(e != cudaSuccess)
    {
        tracer_free_buffers(t);
        return cuda_check(t->ctx, e, "path tracer buffers");
    }
    t->capacity = paths;
    t->npix_cap = npix;
    t->batch = 0;
    return VKG_OK;
}

}// namespace
}// namespace vkg

using namespace vkg;

extern "C" {

vkg_status vkg_scene_create(vkg_ctx *ctx, const vkg_scene_desc *d, vkg_scene **out, void *stream)
{
    if(!ctx) return VKG_ERR_INVALID_ARGUMENT;
    if(!d || !out) return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_scene_create: NULL argument");
    *out = nullptr;
    if(!d->d_tri_material || !d->d_materials || d->num_materials == 0)
        return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_scene_create: materials are required");
    if(!d->d_env_rgb || d->env_width == 0 || d->env_height == 0)
        return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_scene_create: an environment map is required");
    if(vkg_status s = bind_device(ctx); s != VKG_OK) return s;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    auto *sc = new vkg_scene();
    sc->num_tris = d->num_tris;
    sc->num_vertices = d->num_vertices;
    sc->num_materials = d->num_materials;
    cudaError_t e = cudaSuccess;
    auto chk = [&](cudaError_t x) {
        if(e == cudaSuccess) e = x;
    };
    const size_t nt = std::max<size_t>(d->num_tris, 1), nv = std::max<size_t>(d->num_vertices, 1);
    chk(cudaMalloc(&sc->xyz, nv * 3 * sizeof(float)));
    chk(cudaMalloc(&sc->idx, nt * 3 * sizeof(uint32_t)));
    chk(cudaMalloc(&sc->tri_mat, nt * sizeof(uint32_t)));
    chk(cudaMalloc(&sc->mats, d->num_materials * sizeof(vkg_material)));
    if(d->num_tris)
    {
        chk(cudaMemcpyAsync(sc->xyz, d->d_xyz, (size_t)d->num_vertices * 3 * sizeof(float), cudaMemcpyDeviceToDevice, st));
        chk(cudaMemcpyAsync(sc->idx, d->d_indices, (size_t)d->num_tris * 3 * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st));
        chk(cudaMemcpyAsync(sc->tri_mat, d->d_tri_material, (size_t)d->num_tris * sizeof(uint32_t),
                            cudaMemcpyDeviceToDevice, st));
    }
    chk(cudaMemcpyAsync(sc->mats, d->d_materials, d->num_materials * sizeof(vkg_material), cudaMemcpyDeviceToDevice, st));
    if(e != cudaSuccess)
    {
        vkg_scene_destroy(ctx, sc);
        return cuda_check(ctx, e, "vkg_scene_create");
    }
    vkg_bvh_build_options opt{d->leaf_max};
    vkg_status s = vkg_bvh_build(ctx, sc->xyz, d->num_vertices, sc->idx, d->num_tris, &opt, &sc->bvh, stream);
    if(s != VKG_OK)
    {
        vkg_scene_destroy(ctx, sc);
        return s;
    }
    if(d->num_tris)
    {
        uint32_t *bad = nullptr, hbad = 0;
        chk(cudaMallocAsync(&bad, sizeof(uint32_t), st));
        chk(cudaMemsetAsync(bad, 0, sizeof(uint32_t), st));
        k_check_materials<<<(d->num_tris + 255) / 256, 256, 0, st>>>(sc->tri_mat, d->num_tris, d->num_materials, bad);
        k_tri_flags<<<(d->num_tris + 255) / 256, 256, 0, st>>>(sc->bvh->d_tris, d->num_tris, sc->tri_mat, sc->mats,
                                                               d->num_materials);
        chk(cudaMemcpyAsync(&hbad, bad, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        chk(cudaFreeAsync(bad, st));
        chk(cudaStreamSynchronize(st));
        if(e == cudaSuccess && hbad)
        {
            vkg_scene_destroy(ctx, sc);
            return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_scene_create: a material id >= num_materials");
        }
    }
    if(e == cudaSuccess) s = env_build(ctx, d->d_env_rgb, d->env_width, d->env_height, sc->env, st);
    if(e == cudaSuccess) chk(cudaStreamSynchronize(st));
    if(e != cudaSuccess || s != VKG_OK)
    {
        vkg_scene_destroy(ctx, sc);
        return e != cudaSuccess ? cuda_check(ctx, e, "vkg_scene_create") : s;
    }
    *out = sc;
    return VKG_OK;
}

vkg_status vkg_scene_destroy(vkg_ctx *ctx, vkg_scene *sc)
{
    if(!sc) return VKG_OK;
    if(ctx) bind_device(ctx);
    vkg_bvh_destroy(ctx, sc->bvh);
    cudaFree(sc->xyz);
    cudaFree(sc->idx);
    cudaFree(sc->tri_mat);
    cudaFree(sc->mats);
    env_free(sc->env);
    delete sc;
    return VKG_OK;
}

vkg_status vkg_scene_bvh(const vkg_scene *sc, const vkg_bvh **out)
{
    if(!sc || !out) return VKG_ERR_INVALID_ARGUMENT;
    *out = sc->bvh;
    return VKG_OK;
}

vkg_status vkg_scene_env_tables(const vkg_scene *sc, const float **w, const void **alias, uint32_t *width,
                                uint32_t *height)
{
    if(!sc) return VKG_ERR_INVALID_ARGUMENT;
    if(w) *w = sc->env.pdf_w;
    if(alias) *alias = sc->env.alias;
    if(width) *width = sc->env.w;
    if(height) *height = sc->env.h;
    return VKG_OK;
}

vkg_status vkg_settings_default(vkg_settings *s)
{
    if(!s) return VKG_ERR_INVALID_ARGUMENT;
    *s = vkg_settings{};
    s->resolution[0] = 1280;
    s->resolution[1] = 720;
    s->max_num_batches = 0;
    s->num_samples = 1;
    s->max_trace_depth = 6;
    s->max_path_beta = 0.f;
    s->suspend_trace_when_done = 1;
    s->disable_material = 0;
    s->mis_mode = 0;
    s->draw_skybox = 1;
    s->environment = 1.f;
    s->rr_start_depth = 0;
    return VKG_OK;
}

static vkg_status check_settings(vkg_ctx *ctx, const vkg_settings *s)
{
    if(s->resolution[0] == 0 || s->resolution[1] == 0)
        return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "settings: zero resolution");
    if(s->num_samples == 0) return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "settings: num_samples == 0");
    if(s->max_trace_depth == 0 || s->max_trace_depth > 64)
        return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "settings: max_trace_depth must be 1..64");
    if(s->mis_mode > 2) return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "settings: mis_mode must be 0, 1 or 2");
    if(s->crop[2] && s->crop[3] &&
       ((uint64_t)s->crop[0] + s->crop[2] > s->resolution[0] || (uint64_t)s->crop[1] + s->crop[3] > s->resolution[1]))
        return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "settings: crop window outside the resolution");
    return VKG_OK;
}

vkg_status vkg_tracer_create(vkg_ctx *ctx, const vkg_tracer_create_info *info, vkg_tracer **out)
{
    if(!ctx) return VKG_ERR_INVALID_ARGUMENT;
    if(!info || !out) return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_tracer_create: NULL argument");
    *out = nullptr;
    if(vkg_status s = check_settings(ctx, &info->settings); s != VKG_OK) return s;
    if(vkg_status s = bind_device(ctx); s != VKG_OK) return s;
    auto *t = new vkg_tracer();
    t->ctx = ctx;
    t->seed = info->seed;
    t->settings = info->settings;
    if(cudaMalloc(&t->counters, 8 * sizeof(uint32_t)) != cudaSuccess ||
       cudaMalloc(&t->totals, 3 * sizeof(unsigned long long)) != cudaSuccess ||
       cudaEventCreate(&t->ev0) != cudaSuccess || cudaEventCreate(&t->ev1) != cudaSuccess ||
       cudaEventCreate(&t->ev_train) != cudaSuccess)
    {
        vkg_tracer_destroy(t);
        return set_error(ctx, VKG_ERR_CUDA, "vkg_tracer_create: allocation failed");
    }
    *out = t;
    return VKG_OK;
}

vkg_status vkg_tracer_set_settings(vkg_tracer *t, const vkg_settings *s)
{
    if(!t || !s) return VKG_ERR_INVALID_ARGUMENT;
    if(vkg_status r = check_settings(t->ctx, s); r != VKG_OK) return r;
    t->settings = *s;
    return VKG_OK;
}

vkg_status vkg_tracer_get_settings(const vkg_tracer *t, vkg_settings *out)
{
    if(!t || !out) return VKG_ERR_INVALID_ARGUMENT;
    *out = t->settings;
    return VKG_OK;
}

vkg_status vkg_tracer_reset_accumulator(vkg_tracer *t)
{
    if(!t) return VKG_ERR_INVALID_ARGUMENT;
    t->batch = 0;
    return VKG_OK;
}

vkg_status vkg_tracer_current_batch(const vkg_tracer *t, uint32_t *out)
{
    if(!t || !out) return VKG_ERR_INVALID_ARGUMENT;
    *out = t->batch;
    return VKG_OK;
}

vkg_status vkg_tracer_render(vkg_tracer *t, const vkg_scene *sc, const vkg_camera *cam, float *d_rgb_out, void *stream)
{
    if(!t) return VKG_ERR_INVALID_ARGUMENT;
    vkg_ctx *ctx = t->ctx;
    if(!sc || !cam) return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_tracer_render: NULL scene or camera");
    const vkg_settings &S = t->settings;
    if(cam->width != S.resolution[0] || cam->height != S.resolution[1])
        return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_tracer_render: camera size %ux%u != resolution %ux%u",
                         cam->width, cam->height, S.resolution[0], S.resolution[1]);
    if(S.max_num_batches && S.suspend_trace_when_done && t->batch >= S.max_num_batches) return VKG_OK;
    if(vkg_status s = bind_device(ctx); s != VKG_OK) return s;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const uint32_t cx0 = (S.crop[2] && S.crop[3]) ? S.crop[0] : 0, cy0 = (S.crop[2] && S.crop[3]) ? S.crop[1] : 0;
    const uint32_t cw = (S.crop[2] && S.crop[3]) ? S.crop[2] : S.resolution[0];
    const uint32_t ch = (S.crop[2] && S.crop[3]) ? S.crop[3] : S.resolution[1];
    const uint32_t npix = cw * ch;
    uint32_t spw = S.samples_per_wave;
    if(spw == 0) spw = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(S.num_samples, (8u << 20) / npix));
    spw = std::min(spw, S.num_samples);
    const size_t paths = (size_t)npix * spw;
    if(paths >= (1ull << 31)) return set_error(ctx, VKG_ERR_CAPACITY, "vkg_tracer_render: too many paths per wave");
    const vkg_nrc_config *ccfg = t->cache ? &nrc::nrc_config(t->cache) : nullptr;
    const bool cache_render = ccfg && ccfg->terminate_depth < S.max_trace_depth;
    const uint32_t rec_depth = ccfg ? std::min(ccfg->train_depth, S.max_trace_depth) : 0u;
    const uint32_t train_paths = ccfg && rec_depth ? ccfg->train_paths : 0u;
    if(paths + train_paths >= (1ull << 31))
        return set_error(ctx, VKG_ERR_CAPACITY, "vkg_tracer_render: too many paths per wave");
    const bool same_pixels = t->npix_cap == npix;
    const uint32_t old_batch = t->batch;
    if(vkg_status s = tracer_ensure(t, paths + train_paths, npix); s != VKG_OK) return s;
    t->batch = same_pixels ? old_batch : 0u; // growing the wave keeps the accumulation of the same window
    if(ccfg)
        if(vkg_status s = tracer_ensure_cache(t, cache_render ? paths : 0u); s != VKG_OK) return s;

    pt_params P{};
    P.nodes = sc->bvh->d_nodes;
    P.tris = sc->bvh->d_tris;
    P.xyz = sc->xyz;
    P.idx = sc->idx;
    P.tri_mat = sc->tri_mat;
    P.mats = sc->mats;
    P.env = env_view{sc->env.rgb, sc->env.pdf_w, sc->env.alias, sc->env.w, sc->env.h, S.environment};
    P.cam = *cam;
    P.cx0 = cx0;
    P.cy0 = cy0;
    P.cw = cw;
    P.ch = ch;
    P.npix = npix;
    P.max_depth = S.max_trace_depth;
    P.rr_depth = S.rr_start_depth;
    P.mis_mode = S.mis_mode;
    P.disable_material = S.disable_material;
    P.draw_skybox = S.draw_skybox;
    P.max_path_beta = S.max_path_beta;
    P.seed = t->seed;
    P.batch = t->batch;
    P.term_depth = cache_render ? ccfg->terminate_depth : 0xFFFFFFFFu;
    P.rec_depth = rec_depth;
    P.train_paths = train_paths;

    const bool empty = sc->num_tris == 0;
    uint32_t *cnt_q = t->counters + 3, *cnt_rec = t->counters + 4, *cnt_b = t->counters + 5;
    cache_io io{t->q_feat, t->q_beta, cnt_q, t->rec, t->vcount};

    VKG_TRY_CUDA(ctx, cudaMemsetAsync(t->sum, 0, (size_t)npix * 3 * sizeof(float), st));
    VKG_TRY_CUDA(ctx, cudaMemsetAsync(t->totals, 0, 3 * sizeof(unsigned long long), st));
    VKG_TRY_CUDA(ctx, cudaEventRecord(t->ev0, st));
    for(uint32_t s0 = 0; s0 < S.num_samples; s0 += spw)
    {
        const uint32_t ns = std::min(spw, S.num_samples - s0);
        const uint32_t n_render = npix * ns;
        // the training paths ride along with the last wave of rendering paths
        const bool last = s0 + ns >= S.num_samples;
        const uint32_t n = n_render + (last ? train_paths : 0u);
        const int mode = ccfg ? MODE_CACHE : MODE_PLAIN;
        const uint32_t depths = (!cache_render || (last && train_paths)) ? S.max_trace_depth : ccfg->terminate_depth + 1;
        P.s0 = s0;
        P.train_base = last && train_paths ? n_render : 0xFFFFFFFFu;
        const uint32_t grid = (uint32_t)std::min<size_t>((n + PT_THREADS - 1) / PT_THREADS, (size_t)ctx->num_sms * 16);
        if(cache_render) VKG_TRY_CUDA(ctx, cudaMemsetAsync(cnt_q, 0, sizeof(uint32_t), st));
        k_pt_generate<<<grid, PT_THREADS, 0, st>>>(P, n, t->q_ray[0], t->q_pid[0], t->rng, t->beta_pdf, t->radiance,
                                                   t->counters, t->vcount);
        int a = 0;
        for(uint32_t depth = 0; depth < depths; ++depth)
        {
            uint32_t *cnt_in = t->counters + a, *cnt_out = t->counters + (1 - a), *cnt_s = t->counters + 2;
            if(empty)
                k_fill_miss_queue<<<grid, PT_THREADS, 0, st>>>(cnt_in, t->hits);
            else
                k_pt_extend<<<grid, PT_THREADS, 0, st>>>(P.nodes, P.tris, t->q_ray[a], cnt_in, t->hits);
            VKG_TRY_CUDA(ctx, cudaMemsetAsync(cnt_out, 0, sizeof(uint32_t), st));
            VKG_TRY_CUDA(ctx, cudaMemsetAsync(cnt_s, 0, sizeof(uint32_t), st));
#define VKG_SHADE(M)                                                                                                   \
    k_pt_shade<M><<<grid, PT_THREADS, 0, st>>>(P, depth, t->q_ray[a], t->q_pid[a], t->hits, cnt_in, t->q_ray[1 - a],    \
                                               t->q_pid[1 - a], cnt_out, t->s_ray, t->s_pid, t->s_contrib, cnt_s,         \
                                               t->rng, t->beta_pdf, t->radiance, io)
            if(mode == MODE_PLAIN) VKG_SHADE(MODE_PLAIN);
            else VKG_SHADE(MODE_CACHE);
#undef VKG_SHADE
            if(!empty)
                k_pt_shadow<<<grid, PT_THREADS, 0, st>>>(P.nodes, P.tris, t->s_ray, t->s_pid, t->s_contrib, cnt_s,
                                                         t->radiance);
            k_pt_tally<<<1, 1, 0, st>>>(cnt_in, cnt_s, t->totals);
            a = 1 - a;
        }
        if(cache_render)
        {
            if(vkg_status s = nrc::nrc_predict(t->cache, t->q_feat, n_render, cnt_q, t->q_x, t->q_y, st); s != VKG_OK)
                return s;
            const uint32_t rg = (uint32_t)std::min<size_t>((n_render + 255) / 256, (size_t)ctx->num_sms * 8);
            k_cache_resolve<<<rg, 256, 0, st>>>(t->q_beta, t->q_y, cnt_q, t->radiance, t->totals);
        }
        k_pt_accumulate<<<(npix + 255) / 256, 256, 0, st>>>(npix, ns, t->radiance, t->sum);
        if(last && train_paths)
        {
            VKG_TRY_CUDA(ctx, cudaEventRecord(t->ev_train, st));
            VKG_TRY_CUDA(ctx, cudaMemsetAsync(cnt_rec, 0, sizeof(uint32_t), st));
            const uint32_t nrec = train_paths * rec_depth;
            const uint32_t tg = (uint32_t)std::min<size_t>((nrec + PT_THREADS - 1) / PT_THREADS, (size_t)ctx->num_sms * 16);
            k_cache_targets<<<tg, PT_THREADS, 0, st>>>(t->rec, t->vcount, train_paths, rec_depth, t->radiance + n_render,
                                                       t->t_feat, t->t_target, cnt_rec);
            // train_steps windows of batch_size records (0: as many as the record capacity needs); a
            // window past the frame's record count takes no optimiser step
            const uint32_t B = std::min(ccfg->batch_size, nrec);
            const uint32_t windows = (uint32_t)((nrec + (uint64_t)B - 1) / B);
            const uint32_t steps = ccfg->train_steps ? std::min(ccfg->train_steps, windows) : windows;
            for(uint32_t k = 0; k < steps; ++k)
            {
                k_cache_window<<<1, 1, 0, st>>>(cnt_rec, k, B, cnt_b);
                const size_t lo = (size_t)k * B;
                const uint32_t cap = (uint32_t)std::min<size_t>(B, nrec - lo);
                if(vkg_status s = nrc::nrc_train(t->cache, t->t_feat + lo * nrc::FEAT, t->t_target + lo * 3, cap, cnt_b, st);
                   s != VKG_OK)
                    return s;
            }
        }
    }
    if(!train_paths) VKG_TRY_CUDA(ctx, cudaEventRecord(t->ev_train, st));
    t->trained = train_paths > 0;
    k_pt_finalize<<<(3 * npix + 255) / 256, 256, 0, st>>>(npix, S.num_samples, t->batch, t->sum, t->accum, d_rgb_out);
    VKG_TRY_CUDA(ctx, cudaEventRecord(t->ev1, st));
    VKG_TRY_CUDA(ctx, cudaGetLastError());
    t->last_paths = (uint64_t)npix * S.num_samples;
    t->rendered = true;
    t->batch += 1;
    return VKG_OK;
}

vkg_status vkg_tracer_statistics(vkg_tracer *t, vkg_tracer_stats *out)
{
    if(!t || !out) return VKG_ERR_INVALID_ARGUMENT;
    *out = vkg_tracer_stats{};
    out->batch = t->batch;
    if(!t->rendered) return VKG_OK;
    if(vkg_status s = bind_device(t->ctx); s != VKG_OK) return s;
    VKG_TRY_CUDA(t->ctx, cudaEventSynchronize(t->ev1));
    float ms = 0.f, render_ms = 0.f;
    cudaEventElapsedTime(&ms, t->ev0, t->ev1);
    cudaEventElapsedTime(&render_ms, t->ev0, t->ev_train);
    unsigned long long tot[3] = {0, 0, 0};
    VKG_TRY_CUDA(t->ctx, cudaMemcpy(tot, t->totals, sizeof(tot), cudaMemcpyDeviceToHost));
    uint32_t recs = 0;
    if(t->trained) VKG_TRY_CUDA(t->ctx, cudaMemcpy(&recs, t->counters + 4, sizeof(recs), cudaMemcpyDeviceToHost));
    out->raytrace_ms = render_ms;
    out->total_ms = ms;
    out->train_ms = ms - render_ms;
    out->paths = t->last_paths;
    out->extension_rays = tot[0];
    out->shadow_rays = tot[1];
    out->cache_queries = tot[2];
    out->train_records = recs;
    return VKG_OK;
}

vkg_status vkg_tracer_attach_cache(vkg_tracer *t, vkg_nrc *cache)
{
    if(!t) return VKG_ERR_INVALID_ARGUMENT;
    if(cache != t->cache)
    {
        if(vkg_status s = bind_device(t->ctx); s != VKG_OK) return s;
        cudaDeviceSynchronize(); // buffers of the previous cache may still be in use
        tracer_free_cache_buffers(t);
    }
    t->cache = cache;
    return VKG_OK;
}

vkg_status vkg_tracer_destroy(vkg_tracer *t)
{
    if(!t) return VKG_OK;
    if(t->ctx) bind_device(t->ctx);
    tracer_free_buffers(t);
    tracer_free_cache_buffers(t);
    cudaFree(t->counters);
    cudaFree(t->totals);
    if(t->ev0) cudaEventDestroy(t->ev0);
    if(t->ev1) cudaEventDestroy(t->ev1);
    if(t->ev_train) cudaEventDestroy(t->ev_train);
    delete t;
    return VKG_OK;
}

}// extern "C"
