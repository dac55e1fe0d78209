// Batched uneven rendering: many (scene, camera, settings) jobs traced through one set of wavefront
// queues and launched as one CUDA graph per render.
//
// Planning (host, once per tuning): every job contributes npix x num_samples paths. Waves are packed
// greedily from chunks of whole samples of the jobs (job order, then sample order), at most
// wave_paths paths per wave, so every pixel of a job meets its samples in increasing order and the
// per-pixel running sums are formed exactly as the single-scene tracer forms them.
//
// Per wave (device): k_batch_generate maps wave path p -> (chunk, job, sample, pixel) with a binary
// search over the wave's chunk table, seeds PCG32 with the job's seed and sequence
// (batch << 40) ^ (sample * pixels + pixel) (the tracer's streams) and writes the camera ray, the
// job index and the PCG32 increment. The queue kernels of pt_kernels.cuh run with the job_table
// resolver (BVH, materials, environment and settings of the path's own job); depths run to the
// largest max_trace_depth in the wave. k_batch_accumulate adds the wave's radiance to the job
// pixels' sums; after the last wave k_batch_finalize blends every job into its running mean.
//
// The render is recorded once into a CUDA graph (the batch index lives in device memory, so the
// same graph serves every render) and replayed. The autotuner times the candidate tunings
// (grid-stride vs persistent work-stealing queue tracers, grid size, wave size, block size, traversal
// stack depth) on a one-sample render and keeps the fastest; tunings change timing only, never the
// images.
//
// Analytic lights and the settings' sun: every job's light list in one device array, the light-NEE
// shadow queue per wave and the light-shadow launch after the environment shadow launch, as the
// tracer does. One shade variant serves all jobs of a batch: the full one when any job needs it
// (materials beyond metal-roughness or lights), so a metal-rough job in such a batch equals its
// tracer render up to the rounding of the out-of-line BSDF evaluation. Media are refused.
//
// Textures and alpha coverage: when a job's scene has textures the batch keeps one ray-cone width
// per wave path (the jobs with textures point at it, the others leave their cone null) and shades
// with the textured variant; when a job's scene has alpha-tested materials the grid-stride queue
// kernels run with the coverage filter (the persistent tracers are then not used).
#include "pt_kernels.cuh"

#include <algorithm>
#include <vector>

namespace vkg
{
namespace
{

struct batch_chunk
{
    uint32_t job, s0, ns, path_base, pix_base, npix;
};

struct batch_job_dev
{
    uint32_t npix, spp, pix_off;
    float *out;
};

__global__ void __launch_bounds__(PT_THREADS)
        k_batch_generate(const pt_params *__restrict__ jobs, const batch_chunk *__restrict__ chunks, uint32_t nchunks,
                         uint32_t n, const uint32_t *__restrict__ d_batch, vkg_ray *__restrict__ q_ray,
                         uint32_t *__restrict__ q_pid, uint64_t *__restrict__ rng, uint64_t *__restrict__ pinc,
                         uint32_t *__restrict__ pjob, float4 *__restrict__ beta_pdf, float4 *__restrict__ radiance,
                         uint32_t *__restrict__ counters)
{
    const uint64_t batch = *d_batch;
    const uint32_t stride = gridDim.x * blockDim.x;
    for(uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += stride)
    {
        uint32_t lo = 0, hi = nchunks;
        while(hi - lo > 1)
        {
            const uint32_t mid = (lo + hi) / 2;
            if(chunks[mid].path_base <= p) lo = mid;
            else hi = mid;
        }
        const batch_chunk c = chunks[lo];
        const pt_params &P = jobs[c.job];
        const uint32_t li = p - c.path_base, s = c.s0 + li / c.npix, pix = li % c.npix;
        const uint64_t seq = (batch << 40) ^ ((uint64_t)s * P.npix + pix);
        pcg32 g = pcg32_seed(P.seed, seq);
        const uint32_t x = P.cx0 + pix % P.cw, y = P.cy0 + pix / P.cw;
        const float jx = u01(pcg32_next(g)), jy = u01(pcg32_next(g));
        camera_ray(P.cam, x, y, jx, jy, reinterpret_cast<float4 *>(q_ray + p));
        if(P.cone) P.cone[p] = 0.f; // the ray cone starts at width 0 (raypipeline.slang:112-114)
        q_pid[p] = p;
        rng[p] = g.state;
        pinc[p] = (seq << 1u) | 1u;
        pjob[p] = c.job;
        beta_pdf[p] = make_float4(1.f, 1.f, 1.f, 0.f);
        radiance[p] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    if(blockIdx.x == 0 && threadIdx.x == 0) counters[0] = n;
}

// the wave's radiance into the job pixels' sums: one thread per (chunk, pixel), samples in order
__global__ void k_batch_accumulate(const batch_chunk *__restrict__ chunks, uint32_t nchunks, uint32_t npix_wave,
                                   const batch_job_dev *__restrict__ jd, const float4 *__restrict__ radiance,
                                   float *__restrict__ sum)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if(t >= npix_wave) return;
    uint32_t lo = 0, hi = nchunks;
    while(hi - lo > 1)
    {
        const uint32_t mid = (lo + hi) / 2;
        if(chunks[mid].pix_base <= t) lo = mid;
        else hi = mid;
    }
    const batch_chunk c = chunks[lo];
    const uint32_t pix = t - c.pix_base;
    float *o = sum + 3 * ((size_t)jd[c.job].pix_off + pix);
    float sx = o[0], sy = o[1], sz = o[2];
    for(uint32_t k = 0; k < c.ns; ++k)
    {
        const float4 L = radiance[c.path_base + (size_t)k * c.npix + pix];
        sx += L.x;
        sy += L.y;
        sz += L.z;
    }
    o[0] = sx;
    o[1] = sy;
    o[2] = sz;
}

// every job's batch mean into its running mean (the tracer's k_pt_finalize per job)
__global__ void k_batch_finalize(const batch_job_dev *__restrict__ jd, uint32_t njobs, uint32_t total_pix,
                                 const uint32_t *__restrict__ d_batch, const float *__restrict__ sum,
                                 float *__restrict__ accum)
{
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if(e >= 3 * total_pix) return;
    const uint32_t pix = e / 3;
    uint32_t lo = 0, hi = njobs;
    while(hi - lo > 1)
    {
        const uint32_t mid = (lo + hi) / 2;
        if(jd[mid].pix_off <= pix) lo = mid;
        else hi = mid;
    }
    const batch_job_dev j = jd[lo];
    const uint32_t batch = *d_batch;
    const float mean = sum[e] / (float)j.spp;
    const float a = batch == 0 ? mean : (mean + (float)batch * accum[e]) / (float)(batch + 1);
    accum[e] = a;
    if(j.out) j.out[e - 3 * j.pix_off] = a;
}

__global__ void k_batch_advance(uint32_t *__restrict__ d_batch) { *d_batch += 1u; }

}// namespace
}// namespace vkg

using namespace vkg;

struct vkg_batch
{
    vkg_ctx *ctx = nullptr;
    std::vector<vkg_batch_job> jobs;
    std::vector<pt_params> params;
    std::vector<batch_job_dev> jdev;
    uint32_t njobs = 0, total_pix = 0, max_depth = 0;
    bool any_instanced = false;
    bool any_full = false; // a job scene with materials beyond metal-roughness
    bool any_textures = false; // a job scene with textures: the textured shade variant, per-path cone widths
    bool any_alpha = false;    // a job scene with alpha-tested materials: the coverage-testing queue kernels
    float *cone = nullptr;     // ray-cone width per path of a wave (jobs with textures)
    uint32_t max_bvh_depth = 0;
    uint64_t total_paths = 0;
    vkg_batch_tuning tuning{};
    pt_params *d_params = nullptr;
    batch_job_dev *d_jd = nullptr;
    float *sum = nullptr, *accum = nullptr;
    uint32_t *d_batch = nullptr;
    uint32_t *counters = nullptr; // [0..1] queues, [2] shadow queue, [3] persistent work counter
    unsigned long long *totals = nullptr;
    // plan for the current tuning
    struct wave
    {
        uint32_t paths, chunk_off, nchunks, npix, depths;
    };
    std::vector<wave> waves;
    std::vector<batch_chunk> chunks;
    batch_chunk *d_chunks = nullptr;
    size_t cap = 0; // wave buffers' capacity in paths
    vkg_ray *q_ray[2] = {nullptr, nullptr};
    uint32_t *q_pid[2] = {nullptr, nullptr};
    vkg_hit *hits = nullptr;
    uint32_t *hit_inst = nullptr;
    vkg_ray *s_ray = nullptr;
    uint32_t *s_pid = nullptr;
    float4 *s_contrib = nullptr;
    uint64_t *rng = nullptr, *pinc = nullptr;
    uint32_t *pjob = nullptr;
    float4 *beta_pdf = nullptr, *radiance = nullptr;
    // analytic lights: every job's light list (the settings' sun first) in one array, and the
    // light-NEE shadow queue of a wave (allocated when a job has lights)
    bool any_lights = false;
    vkg_light *d_lights = nullptr;
    vkg_ray *l_ray = nullptr;
    uint32_t *l_pid = nullptr;
    float4 *l_contrib = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    uint32_t batch = 0;
    bool rendered = false;
};

namespace
{

void free_waves(vkg_batch *b)
{
    for(void *p: {(void *)b->q_ray[0], (void *)b->q_ray[1], (void *)b->q_pid[0], (void *)b->q_pid[1], (void *)b->hits,
                  (void *)b->hit_inst,
                  (void *)b->s_ray, (void *)b->s_pid, (void *)b->s_contrib, (void *)b->rng, (void *)b->pinc,
                  (void *)b->pjob, (void *)b->beta_pdf, (void *)b->radiance, (void *)b->d_chunks, (void *)b->l_ray,
                  (void *)b->l_pid, (void *)b->l_contrib, (void *)b->cone})
        cudaFree(p);
    b->cone = nullptr;
    b->l_ray = nullptr;
    b->l_pid = nullptr;
    b->l_contrib = nullptr;
    b->q_ray[0] = b->q_ray[1] = nullptr;
    b->q_pid[0] = b->q_pid[1] = nullptr;
    b->hits = nullptr;
    b->hit_inst = nullptr;
    b->s_ray = nullptr;
    b->s_pid = nullptr;
    b->s_contrib = nullptr;
    b->rng = b->pinc = nullptr;
    b->pjob = nullptr;
    b->beta_pdf = b->radiance = nullptr;
    b->d_chunks = nullptr;
    b->cap = 0;
}

void drop_graph(vkg_batch *b)
{
    if(b->exec) cudaGraphExecDestroy(b->exec);
    if(b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
}

// waves of whole samples of the jobs for `spp_cap` samples per job (0: each job's num_samples)
void plan(vkg_batch *b, uint32_t spp_cap, std::vector<vkg_batch::wave> &waves, std::vector<batch_chunk> &chunks)
{
    waves.clear();
    chunks.clear();
    const uint64_t W = std::max<uint64_t>(b->tuning.wave_paths, 1);
    vkg_batch::wave cur{0, 0, 0, 0, 0};
    auto close = [&]() {
        if(cur.nchunks) waves.push_back(cur);
        cur = vkg_batch::wave{0, (uint32_t)chunks.size(), 0, 0, 0};
    };
    for(uint32_t j = 0; j < b->njobs; ++j)
    {
        const uint32_t npix = b->jdev[j].npix;
        const uint32_t spp = spp_cap ? std::min(spp_cap, b->jobs[j].settings.num_samples) : b->jobs[j].settings.num_samples;
        uint32_t s = 0;
        while(s < spp)
        {
            uint64_t room = W > cur.paths ? (W - cur.paths) / npix : 0;
            if(room == 0 && cur.paths == 0) room = 1; // one sample of a job larger than a wave
            if(room == 0)
            {
                close();
                continue;
            }
            const uint32_t ns = (uint32_t)std::min<uint64_t>(room, spp - s);
            chunks.push_back(batch_chunk{j, s, ns, cur.paths, cur.npix, npix});
            cur.paths += ns * npix;
            cur.npix += npix;
            cur.nchunks += 1;
            cur.depths = std::max(cur.depths, b->jobs[j].settings.max_trace_depth);
            s += ns;
        }
    }
    close();
}

vkg_status ensure_waves(vkg_batch *b, const std::vector<vkg_batch::wave> &waves, const std::vector<batch_chunk> &chunks)
{
    size_t need = 0;
    for(const auto &w: waves) need = std::max<size_t>(need, w.paths);
    cudaFree(b->d_chunks);
    b->d_chunks = nullptr;
    if(need > b->cap)
    {
        free_waves(b);
        cudaError_t e = cudaSuccess;
        auto al = [&](void **p, size_t bytes) {
            if(e == cudaSuccess) e = cudaMalloc(p, bytes);
        };
        for(int q = 0; q < 2; ++q)
        {
            al((void **)&b->q_ray[q], need * sizeof(vkg_ray));
            al((void **)&b->q_pid[q], need * sizeof(uint32_t));
        }
        al((void **)&b->hits, need * sizeof(vkg_hit));
        al((void **)&b->hit_inst, need * sizeof(uint32_t));
        al((void **)&b->s_ray, need * sizeof(vkg_ray));
        al((void **)&b->s_pid, need * sizeof(uint32_t));
        al((void **)&b->s_contrib, need * sizeof(float4));
        al((void **)&b->rng, need * sizeof(uint64_t));
        al((void **)&b->pinc, need * sizeof(uint64_t));
        al((void **)&b->pjob, need * sizeof(uint32_t));
        al((void **)&b->beta_pdf, need * sizeof(float4));
        al((void **)&b->radiance, need * sizeof(float4));
        if(b->any_lights)
        {
            al((void **)&b->l_ray, need * sizeof(vkg_ray));
            al((void **)&b->l_pid, need * sizeof(uint32_t));
            al((void **)&b->l_contrib, need * sizeof(float4));
        }
        if(b->any_textures) al((void **)&b->cone, need * sizeof(float));
        // the jobs with textures sample them through the wave's cone widths
        if(b->any_textures && e == cudaSuccess)
        {
            for(uint32_t j = 0; j < b->njobs; ++j) b->params[j].cone = b->jobs[j].scene->num_textures ? b->cone : nullptr;
            e = cudaMemcpy(b->d_params, b->params.data(), b->njobs * sizeof(pt_params), cudaMemcpyHostToDevice);
        }
        if(e != cudaSuccess)
        {
            free_waves(b);
            return cuda_check(b->ctx, e, "batch wave buffers");
        }
        b->cap = need;
    }
    if(cudaMalloc(&b->d_chunks, std::max<size_t>(chunks.size(), 1) * sizeof(batch_chunk)) != cudaSuccess)
        return set_error(b->ctx, VKG_ERR_CUDA, "batch chunk table");
    VKG_TRY_CUDA(b->ctx, cudaMemcpy(b->d_chunks, chunks.data(), chunks.size() * sizeof(batch_chunk),
                                    cudaMemcpyHostToDevice));
    return VKG_OK;
}

// records one render (all waves) on stream st
vkg_status enqueue(vkg_batch *b, const std::vector<vkg_batch::wave> &waves, cudaStream_t st)
{
    vkg_ctx *ctx = b->ctx;
    vkg_batch_tuning T = b->tuning;
    // the persistent tracers handle single-level scenes without alpha-tested materials only
    if(b->any_instanced || b->any_alpha) T.extend_kernel = 1;
    // a 64-entry stack serves BVHs of depth <= 10 (7 (depth - 1) + 1 entries at most)
    if(b->max_bvh_depth > 10) T.stack_depth = 128;
    const job_table J{b->d_params, b->pjob, b->pinc};
    uint32_t *cnt_l = b->any_lights ? b->counters + 4 : nullptr;
    const light_queue lq{b->l_ray, b->l_pid, b->l_contrib, cnt_l};
    VKG_TRY_CUDA(ctx, cudaMemsetAsync(b->sum, 0, (size_t)b->total_pix * 3 * sizeof(float), st));
    cache_io io{};
    const uint32_t bs = T.block_size;
    for(const auto &w: waves)
    {
        const batch_chunk *ch = b->d_chunks + w.chunk_off;
        const uint32_t n = w.paths;
        const uint32_t grid = (uint32_t)std::min<size_t>((n + bs - 1) / bs,
                                                         (size_t)ctx->num_sms * std::max(1u, T.ctas_per_sm));
        k_batch_generate<<<grid, bs, 0, st>>>(b->d_params, ch, w.nchunks, n, b->d_batch, b->q_ray[0], b->q_pid[0], b->rng,
                                             b->pinc, b->pjob, b->beta_pdf, b->radiance, b->counters);
        int a = 0;
        for(uint32_t depth = 0; depth < w.depths; ++depth)
        {
            uint32_t *cnt_in = b->counters + a, *cnt_out = b->counters + (1 - a), *cnt_s = b->counters + 2;
            if(T.extend_kernel == 2)
            {
                VKG_TRY_CUDA(ctx, cudaMemsetAsync(b->counters + 3, 0, sizeof(uint32_t), st));
                if(T.stack_depth == 64)
                    k_pt_trace_persistent<false, job_table, 64><<<grid, bs, 0, st>>>(
                            J, b->q_ray[a], b->q_pid[a], cnt_in, b->hits, b->hit_inst, nullptr, nullptr, b->counters + 3);
                else
                    k_pt_trace_persistent<false, job_table><<<grid, bs, 0, st>>>(
                            J, b->q_ray[a], b->q_pid[a], cnt_in, b->hits, b->hit_inst, nullptr, nullptr, b->counters + 3);
            }
            else if(b->any_alpha && T.stack_depth == 64)
                k_pt_extend<job_table, 64, true><<<grid, bs, 0, st>>>(J, b->q_ray[a], b->q_pid[a], cnt_in, b->hits,
                                                                       b->hit_inst, nullptr, nullptr, b->rng, depth);
            else if(b->any_alpha)
                k_pt_extend<job_table, (int)TRAVERSAL_STACK, true><<<grid, bs, 0, st>>>(
                        J, b->q_ray[a], b->q_pid[a], cnt_in, b->hits, b->hit_inst, nullptr, nullptr, b->rng, depth);
            else if(T.stack_depth == 64)
                k_pt_extend<job_table, 64><<<grid, bs, 0, st>>>(J, b->q_ray[a], b->q_pid[a], cnt_in, b->hits, b->hit_inst);
            else
                k_pt_extend<<<grid, bs, 0, st>>>(J, b->q_ray[a], b->q_pid[a], cnt_in, b->hits, b->hit_inst);
            VKG_TRY_CUDA(ctx, cudaMemsetAsync(cnt_out, 0, sizeof(uint32_t), st));
            VKG_TRY_CUDA(ctx, cudaMemsetAsync(cnt_s, 0, sizeof(uint32_t), st));
            if(cnt_l) VKG_TRY_CUDA(ctx, cudaMemsetAsync(cnt_l, 0, sizeof(uint32_t), st));
            // the shade variant: the full material set and the lights or metal-roughness only, each
            // with the texture terms when a job has textures
#define VKG_BATCH_SHADE(F, TX, LQ)                                                                                     \
    k_pt_shade<MODE_PLAIN, job_table, F, false, TX><<<grid, bs, 0, st>>>(                                              \
            J, depth, b->q_ray[a], b->q_pid[a], b->hits, b->hit_inst, cnt_in, b->q_ray[1 - a], b->q_pid[1 - a],       \
            cnt_out, b->s_ray, b->s_pid, b->s_contrib, cnt_s, b->rng, b->beta_pdf, b->radiance, io, LQ, nullptr)
            const bool full = b->any_full || b->any_lights;
            if(full && b->any_textures) VKG_BATCH_SHADE(true, true, lq);
            else if(full) VKG_BATCH_SHADE(true, false, lq);
            else if(b->any_textures) VKG_BATCH_SHADE(false, true, light_queue{});
            else VKG_BATCH_SHADE(false, false, light_queue{});
#undef VKG_BATCH_SHADE
            if(T.extend_kernel == 2)
            {
                VKG_TRY_CUDA(ctx, cudaMemsetAsync(b->counters + 3, 0, sizeof(uint32_t), st));
                if(T.stack_depth == 64)
                    k_pt_trace_persistent<true, job_table, 64><<<grid, bs, 0, st>>>(
                            J, b->s_ray, b->s_pid, cnt_s, nullptr, nullptr, b->s_contrib, b->radiance, b->counters + 3);
                else
                    k_pt_trace_persistent<true, job_table><<<grid, bs, 0, st>>>(
                            J, b->s_ray, b->s_pid, cnt_s, nullptr, nullptr, b->s_contrib, b->radiance, b->counters + 3);
            }
            else if(b->any_alpha && T.stack_depth == 64)
                k_pt_shadow<job_table, 64, true><<<grid, bs, 0, st>>>(J, b->s_ray, b->s_pid, b->s_contrib, cnt_s,
                                                                       b->radiance, nullptr, nullptr, b->rng);
            else if(b->any_alpha)
                k_pt_shadow<job_table, (int)TRAVERSAL_STACK, true><<<grid, bs, 0, st>>>(
                        J, b->s_ray, b->s_pid, b->s_contrib, cnt_s, b->radiance, nullptr, nullptr, b->rng);
            else if(T.stack_depth == 64)
                k_pt_shadow<job_table, 64><<<grid, bs, 0, st>>>(J, b->s_ray, b->s_pid, b->s_contrib, cnt_s, b->radiance);
            else
                k_pt_shadow<<<grid, bs, 0, st>>>(J, b->s_ray, b->s_pid, b->s_contrib, cnt_s, b->radiance);
            // light NEE after the environment shadow launch: one writer per path at a time
            if(cnt_l && b->any_alpha && T.stack_depth == 64)
                k_pt_light_shadow<job_table, 64, true><<<grid, bs, 0, st>>>(J, lq, b->radiance, b->rng);
            else if(cnt_l && b->any_alpha)
                k_pt_light_shadow<job_table, (int)TRAVERSAL_STACK, true><<<grid, bs, 0, st>>>(J, lq, b->radiance, b->rng);
            else if(cnt_l && T.stack_depth == 64)
                k_pt_light_shadow<job_table, 64><<<grid, bs, 0, st>>>(J, lq, b->radiance);
            else if(cnt_l)
                k_pt_light_shadow<job_table><<<grid, bs, 0, st>>>(J, lq, b->radiance);
            k_pt_tally<<<1, 1, 0, st>>>(cnt_in, cnt_s, cnt_l, b->totals);
            a = 1 - a;
        }
        k_batch_accumulate<<<(w.npix + 255) / 256, 256, 0, st>>>(ch, w.nchunks, w.npix, b->d_jd, b->radiance, b->sum);
    }
    k_batch_finalize<<<(3 * b->total_pix + 255) / 256, 256, 0, st>>>(b->d_jd, b->njobs, b->total_pix, b->d_batch,
                                                                     b->sum, b->accum);
    k_batch_advance<<<1, 1, 0, st>>>(b->d_batch);
    return cuda_check(ctx, cudaGetLastError(), "batch render");
}

vkg_status replan(vkg_batch *b)
{
    drop_graph(b);
    plan(b, 0, b->waves, b->chunks);
    return ensure_waves(b, b->waves, b->chunks);
}

vkg_status run(vkg_batch *b, cudaStream_t st)
{
    vkg_ctx *ctx = b->ctx;
    VKG_TRY_CUDA(ctx, cudaMemsetAsync(b->totals, 0, 2 * sizeof(unsigned long long), st));
    VKG_TRY_CUDA(ctx, cudaEventRecord(b->ev0, st));
    if(b->tuning.use_graph)
    {
        if(!b->exec)
        {
            // a render is recorded on a private stream (capture needs a non-default stream) and replayed
            cudaStream_t cap = nullptr;
            VKG_TRY_CUDA(ctx, cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
            cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
            vkg_status s = e == cudaSuccess ? enqueue(b, b->waves, cap) : cuda_check(ctx, e, "graph capture");
            cudaGraph_t g = nullptr;
            const cudaError_t e2 = cudaStreamEndCapture(cap, &g);
            cudaStreamDestroy(cap);
            if(s != VKG_OK)
            {
                if(g) cudaGraphDestroy(g);
                return s;
            }
            if(e2 != cudaSuccess) return cuda_check(ctx, e2, "graph capture");
            b->graph = g;
            VKG_TRY_CUDA(ctx, cudaGraphInstantiate(&b->exec, b->graph, 0));
        }
        VKG_TRY_CUDA(ctx, cudaGraphLaunch(b->exec, st));
    }
    else if(vkg_status s = enqueue(b, b->waves, st); s != VKG_OK)
        return s;
    VKG_TRY_CUDA(ctx, cudaEventRecord(b->ev1, st));
    b->batch += 1;
    b->rendered = true;
    return VKG_OK;
}

}// namespace

extern "C" {

vkg_status vkg_batch_tuning_default(vkg_batch_tuning *out)
{
    if(!out) return VKG_ERR_INVALID_ARGUMENT;
    out->extend_kernel = 1;
    out->ctas_per_sm = 16;
    out->wave_paths = 8u << 20;
    out->use_graph = 1;
    out->block_size = 128;
    out->stack_depth = 128;
    return VKG_OK;
}

static vkg_status check_tuning(vkg_ctx *ctx, const vkg_batch_tuning *t)
{
    if(t->extend_kernel < 1 || t->extend_kernel > 2)
        return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "batch tuning: extend_kernel must be 1 or 2");
    if(t->ctas_per_sm == 0 || t->ctas_per_sm > 64)
        return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "batch tuning: ctas_per_sm must be 1..64");
    if(t->wave_paths < 1024 || t->wave_paths > (1u << 30))
        return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "batch tuning: wave_paths must be 1024..2^30");
    if(t->block_size != 64 && t->block_size != 128)
        return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "batch tuning: block_size must be 64 or 128");
    if(t->stack_depth != 64 && t->stack_depth != 128)
        return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "batch tuning: stack_depth must be 64 or 128");
    return VKG_OK;
}

vkg_status vkg_batch_create(vkg_ctx *ctx, const vkg_batch_job *jobs, uint32_t njobs, const vkg_batch_tuning *tuning,
                            vkg_batch **out)
{
    if(!ctx) return VKG_ERR_INVALID_ARGUMENT;
    if(!out || (!jobs && njobs)) return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_batch_create: NULL argument");
    *out = nullptr;
    if(njobs == 0) return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_batch_create: no jobs");
    vkg_batch_tuning T{};
    vkg_batch_tuning_default(&T);
    if(tuning) T = *tuning;
    if(vkg_status s = check_tuning(ctx, &T); s != VKG_OK) return s;
    uint64_t pix = 0;
    for(uint32_t j = 0; j < njobs; ++j)
    {
        const vkg_batch_job &jb = jobs[j];
        if(!jb.scene) return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_batch_create: job %u has no scene", j);
        if(vkg_status s = check_tracer_settings(ctx, &jb.settings); s != VKG_OK) return s;
        if(jb.settings.rng_mode != VKG_RNG_PCG32)
            return set_error(ctx, VKG_ERR_NOT_SUPPORTED, "vkg_batch_create: job %u: VKG_RNG_REFERENCE is a tracer mode",
                             (unsigned)j);
        if(jb.scene->d_media || jb.settings.camera_medium_mode != VKG_CAMERA_MEDIUM_DETECT)
            return set_error(ctx, VKG_ERR_INVALID_ARGUMENT,
                             "vkg_batch_create: job %u: media are rendered by vkg_tracer_render", j);
        if(jb.camera.width != jb.settings.resolution[0] || jb.camera.height != jb.settings.resolution[1])
            return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_batch_create: job %u camera size != resolution", j);
        uint32_t x0, y0, w, h;
        crop_window(jb.settings, x0, y0, w, h);
        pix += (uint64_t)w * h;
    }
    if(pix >= (1ull << 31)) return set_error(ctx, VKG_ERR_CAPACITY, "vkg_batch_create: too many pixels");
    if(vkg_status s = bind_device(ctx); s != VKG_OK) return s;
    auto *b = new vkg_batch();
    b->ctx = ctx;
    b->tuning = T;
    b->njobs = njobs;
    b->jobs.assign(jobs, jobs + njobs);
    uint32_t off = 0;
    std::vector<vkg_light> all_lights;
    std::vector<uint32_t> light_off;
    for(uint32_t j = 0; j < njobs; ++j)
    {
        const vkg_batch_job &jb = jobs[j];
        b->params.push_back(make_params(jb.scene, jb.camera, jb.settings, jb.seed, 0));
        const std::vector<vkg_light> jl = render_lights(jb.scene, jb.settings);
        light_off.push_back((uint32_t)all_lights.size());
        b->params.back().num_lights = (uint32_t)jl.size();
        all_lights.insert(all_lights.end(), jl.begin(), jl.end());
        b->any_instanced = b->any_instanced || jb.scene->tlas != nullptr;
        b->any_full = b->any_full || jb.scene->any_full;
        b->any_textures = b->any_textures || jb.scene->num_textures > 0;
        b->any_alpha = b->any_alpha || jb.scene->any_alpha;
        if(jb.scene->bvh) b->max_bvh_depth = std::max(b->max_bvh_depth, jb.scene->bvh->depth);
        const uint32_t npix = b->params.back().npix;
        b->jdev.push_back(batch_job_dev{npix, jb.settings.num_samples, off, jb.d_rgb_out});
        off += npix;
        b->total_paths += (uint64_t)npix * jb.settings.num_samples;
        b->max_depth = std::max(b->max_depth, jb.settings.max_trace_depth);
    }
    b->total_pix = off;
    cudaError_t e = cudaSuccess;
    auto al = [&](void **p, size_t bytes) {
        if(e == cudaSuccess) e = cudaMalloc(p, bytes);
    };
    al((void **)&b->d_params, njobs * sizeof(pt_params));
    al((void **)&b->d_jd, njobs * sizeof(batch_job_dev));
    al((void **)&b->sum, (size_t)off * 3 * sizeof(float));
    al((void **)&b->accum, (size_t)off * 3 * sizeof(float));
    al((void **)&b->d_batch, sizeof(uint32_t));
    al((void **)&b->counters, 5 * sizeof(uint32_t));
    al((void **)&b->totals, 2 * sizeof(unsigned long long));
    b->any_lights = !all_lights.empty();
    if(b->any_lights)
    {
        al((void **)&b->d_lights, all_lights.size() * sizeof(vkg_light));
        if(e == cudaSuccess)
            e = cudaMemcpy(b->d_lights, all_lights.data(), all_lights.size() * sizeof(vkg_light), cudaMemcpyHostToDevice);
        for(uint32_t j = 0; j < njobs; ++j)
            b->params[j].lights = b->params[j].num_lights ? b->d_lights + light_off[j] : nullptr;
    }
    if(e == cudaSuccess) e = cudaMemcpy(b->d_params, b->params.data(), njobs * sizeof(pt_params), cudaMemcpyHostToDevice);
    if(e == cudaSuccess) e = cudaMemcpy(b->d_jd, b->jdev.data(), njobs * sizeof(batch_job_dev), cudaMemcpyHostToDevice);
    if(e == cudaSuccess) e = cudaMemset(b->d_batch, 0, sizeof(uint32_t));
    if(e == cudaSuccess) e = cudaEventCreate(&b->ev0);
    if(e == cudaSuccess) e = cudaEventCreate(&b->ev1);
    if(e != cudaSuccess)
    {
        vkg_batch_destroy(b);
        return cuda_check(ctx, e, "vkg_batch_create");
    }
    if(vkg_status s = replan(b); s != VKG_OK)
    {
        vkg_batch_destroy(b);
        return s;
    }
    *out = b;
    return VKG_OK;
}

vkg_status vkg_batch_set_tuning(vkg_batch *b, const vkg_batch_tuning *t)
{
    if(!b || !t) return VKG_ERR_INVALID_ARGUMENT;
    if(vkg_status s = check_tuning(b->ctx, t); s != VKG_OK) return s;
    if(vkg_status s = bind_device(b->ctx); s != VKG_OK) return s;
    VKG_TRY_CUDA(b->ctx, cudaDeviceSynchronize());
    b->tuning = *t;
    return replan(b);
}

vkg_status vkg_batch_render(vkg_batch *b, void *stream)
{
    if(!b) return VKG_ERR_INVALID_ARGUMENT;
    if(vkg_status s = bind_device(b->ctx); s != VKG_OK) return s;
    return run(b, static_cast<cudaStream_t>(stream));
}

vkg_status vkg_batch_autotune(vkg_batch *b, void *stream, vkg_batch_tuning *chosen)
{
    if(!b) return VKG_ERR_INVALID_ARGUMENT;
    if(vkg_status s = bind_device(b->ctx); s != VKG_OK) return s;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    vkg_ctx *ctx = b->ctx;
    const vkg_batch_tuning keep = b->tuning;
    vkg_batch_tuning best = keep;
    float best_ms = 3.4e38f;
    std::vector<vkg_batch::wave> waves;
    std::vector<batch_chunk> chunks;
    const bool small_stack = b->max_bvh_depth <= 10;
    for(uint32_t ek: {1u, 2u})
        for(uint32_t cps: {8u, 16u})
            for(uint32_t wp: {8u << 20, 16u << 20})
                for(uint32_t bs: {64u, 128u})
                    for(uint32_t sd: {64u, 128u})
                    {
                        if(sd == 64 && !small_stack) continue;
                        b->tuning = vkg_batch_tuning{ek, cps, wp, 0, bs, sd};
                        plan(b, 1, waves, chunks);
                        drop_graph(b);
                        if(vkg_status s = ensure_waves(b, waves, chunks); s != VKG_OK) return s;
                        float ms = 0.f;
                        for(int rep = 0; rep < 2; ++rep) // the first run warms the caches
                        {
                            VKG_TRY_CUDA(ctx, cudaEventRecord(b->ev0, st));
                            if(vkg_status s = enqueue(b, waves, st); s != VKG_OK) return s;
                            VKG_TRY_CUDA(ctx, cudaEventRecord(b->ev1, st));
                            VKG_TRY_CUDA(ctx, cudaEventSynchronize(b->ev1));
                            VKG_TRY_CUDA(ctx, cudaEventElapsedTime(&ms, b->ev0, b->ev1));
                        }
                        if(ms < best_ms)
                        {
                            best_ms = ms;
                            best = b->tuning;
                        }
                    }
    best.use_graph = keep.use_graph;
    b->tuning = best;
    if(chosen) *chosen = best;
    if(vkg_status s = replan(b); s != VKG_OK) return s;
    return vkg_batch_reset_accumulator(b);
}

vkg_status vkg_batch_reset_accumulator(vkg_batch *b)
{
    if(!b) return VKG_ERR_INVALID_ARGUMENT;
    if(vkg_status s = bind_device(b->ctx); s != VKG_OK) return s;
    VKG_TRY_CUDA(b->ctx, cudaDeviceSynchronize());
    VKG_TRY_CUDA(b->ctx, cudaMemset(b->d_batch, 0, sizeof(uint32_t)));
    b->batch = 0;
    return VKG_OK;
}

vkg_status vkg_batch_statistics(vkg_batch *b, vkg_batch_stats *out)
{
    if(!b || !out) return VKG_ERR_INVALID_ARGUMENT;
    *out = vkg_batch_stats{};
    out->waves = (uint32_t)b->waves.size();
    out->batch = b->batch;
    out->paths = b->total_paths;
    if(!b->rendered) return VKG_OK;
    if(vkg_status s = bind_device(b->ctx); s != VKG_OK) return s;
    VKG_TRY_CUDA(b->ctx, cudaEventSynchronize(b->ev1));
    float ms = 0.f;
    VKG_TRY_CUDA(b->ctx, cudaEventElapsedTime(&ms, b->ev0, b->ev1));
    unsigned long long tot[2] = {0, 0};
    VKG_TRY_CUDA(b->ctx, cudaMemcpy(tot, b->totals, sizeof(tot), cudaMemcpyDeviceToHost));
    out->render_ms = ms;
    out->extension_rays = tot[0];
    out->shadow_rays = tot[1];
    return VKG_OK;
}

vkg_status vkg_batch_destroy(vkg_batch *b)
{
    if(!b) return VKG_OK;
    if(b->ctx) bind_device(b->ctx);
    drop_graph(b);
    free_waves(b);
    for(void *p: {(void *)b->d_params, (void *)b->d_jd, (void *)b->sum, (void *)b->accum, (void *)b->d_batch,
                  (void *)b->counters, (void *)b->totals, (void *)b->d_lights})
        cudaFree(p);
    if(b->ev0) cudaEventDestroy(b->ev0);
    if(b->ev1) cudaEventDestroy(b->ev1);
    delete b;
    return VKG_OK;
}

}// extern "C"
