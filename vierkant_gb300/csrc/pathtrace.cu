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
#include "pt_kernels.cuh"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <random>


struct vkg_tracer
{
    vkg_ctx *ctx = nullptr;
    uint32_t seed = 0;
    // VKG_RNG_REFERENCE: the batch seeds (std::default_random_engine(seed), PBRPathTracer.cpp:32) and
    // per window pixel the chain state and sub-pixel offset carried from sample to sample
    std::minstd_rand0 ref_engine;
    uint32_t *ref_chain = nullptr;
    float *ref_offset = nullptr;
    size_t ref_cap = 0;
    // vkg_diag_tracer_uniforms
    float *dbg_u = nullptr;
    uint32_t dbg_segments = 0;
    vkg_settings settings{};
    uint32_t batch = 0;
    // buffers sized for `capacity` paths and `npix` pixels
    size_t capacity = 0, npix_cap = 0;
    vkg_ray *q_ray[2] = {nullptr, nullptr};
    uint32_t *q_pid[2] = {nullptr, nullptr};
    vkg_hit *hits = nullptr;
    uint32_t *hit_inst = nullptr; // instance of each hit (instanced scenes)
    vkg_ray *s_ray = nullptr;
    uint32_t *s_pid = nullptr;
    float4 *s_contrib = nullptr;
    uint64_t *rng = nullptr;
    float4 *beta_pdf = nullptr;
    float4 *radiance = nullptr;
    float *sum = nullptr;
    float *accum = nullptr;
    vkg_pixel_data *gbuf = nullptr; // pixel records of the traced window
    uint32_t *order = nullptr;      // queue slots grouped by material class (full material set)
    uint32_t *bins = nullptr;       // class counts [0..7] and fill cursors [8..15]
    uint4 *mstack = nullptr;        // per-path medium stacks (scenes with media)
    size_t mstack_cap = 0;
    float *cone = nullptr;          // per-path ray-cone widths (scenes with textures)
    size_t cone_cap = 0;
    uint32_t *counters = nullptr;           // [0..1] queue lengths, [2] shadow queue length, [3] cache queries,
                                            // [4] training records, [5] training batch length, [6] work
                                            // counter, [7] light shadow queue length
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
    // analytic lights: the light list of the last render and the light-NEE shadow queue
    vkg_light *d_lights = nullptr;
    size_t lights_cap = 0, lq_cap = 0;
    vkg_ray *l_ray = nullptr;
    uint32_t *l_pid = nullptr;
    float4 *l_contrib = nullptr;
    // medium table of renders with a camera medium: the scene's records + the camera's (last upload kept)
    vkg::medium_rec *d_media_cam = nullptr;
    std::vector<vkg::medium_rec> media_cam;
};

namespace vkg
{
vkg_status denoise_run(vkg_ctx *ctx, const vkg_pixel_data *px, uint32_t w, uint32_t h, float *out_rgba,
                       float *out_rgb, float *out_depth, cudaStream_t st);
namespace
{

// the camera medium of PBRPathTracer.cpp:471-525: of the instances whose world box (the mesh's box
// under the instance transform: an oriented box) contains the eye and whose material has a finite
// attenuation distance, the one with the smallest box volume (the first on ties); single-level
// scenes have no objects and start in vacuum
uint32_t detect_camera_medium(const vkg_scene *sc, const float eye[3])
{
    uint32_t best = 0xFFFFFFFFu;
    double best_volume = std::numeric_limits<double>::max();
    if(!sc->tlas) return best;
    for(const vkg_instance &in: sc->h_inst)
    {
        if(in.material >= sc->h_mats.size() || in.blas >= sc->blas.size()) continue;
        if(!material_has_volume(sc->h_mats[in.material])) continue;
        const vkg_bvh *b = sc->blas[in.blas];
        const float *M = in.transform;
        // object-space eye: solve A x = eye - t for the 3x3 part A (Cramer's rule in double)
        const double a[9] = {M[0], M[1], M[2], M[4], M[5], M[6], M[8], M[9], M[10]};
        const double r[3] = {eye[0] - (double)M[3], eye[1] - (double)M[7], eye[2] - (double)M[11]};
        const double det = a[0] * (a[4] * a[8] - a[5] * a[7]) - a[1] * (a[3] * a[8] - a[5] * a[6]) +
                           a[2] * (a[3] * a[7] - a[4] * a[6]);
        if(!(std::fabs(det) > 0.0)) continue;
        double x[3];
        for(int k = 0; k < 3; ++k)
        {
            double c[9];
            std::memcpy(c, a, sizeof(c));
            for(int row = 0; row < 3; ++row) c[3 * row + k] = r[row];
            x[k] = (c[0] * (c[4] * c[8] - c[5] * c[7]) - c[1] * (c[3] * c[8] - c[5] * c[6]) +
                    c[2] * (c[3] * c[7] - c[4] * c[6])) / det;
        }
        bool inside = true;
        double volume = 8.0;
        for(int k = 0; k < 3; ++k)
        {
            inside = inside && x[k] >= b->scene_min[k] && x[k] <= b->scene_max[k];
            const double col = std::sqrt(a[k] * a[k] + a[3 + k] * a[3 + k] + a[6 + k] * a[6 + k]);
            volume *= 0.5 * ((double)b->scene_max[k] - b->scene_min[k]) * col;
        }
        if(!inside || volume >= best_volume) continue;
        best_volume = volume;
        best = in.material;
    }
    return best;
}

// shading-coherence binning of the full material set (on unless VKG_PT_BINNING=0)
bool pt_binning_selected()
{
    static int v = -1;
    if(v < 0)
    {
        const char *s = std::getenv("VKG_PT_BINNING");
        v = (s && std::strcmp(s, "0") == 0) ? 0 : 1;
    }
    return v == 1;
}

bool tl_persistent_selected()
{
    static int v = -1;
    if(v < 0)
    {
        const char *e = std::getenv("VKG_TL_KERNEL");
        v = (e && std::strcmp(e, "persistent") == 0) ? 1 : 0;
    }
    return v == 1;
}

__global__ void k_set_tri_flags(tri_rec *__restrict__ tris, uint32_t n, uint32_t flags)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i < n) tris[i].pad[0] |= flags;
}

// flags instances whose material index is out of range (bad), and the meshes that an instance with an
// unculled material (two-sided or transmissive) references (mesh_unculled)
__global__ void k_check_instance_materials(const vkg_instance *__restrict__ inst, uint32_t n,
                                           const vkg_material *__restrict__ mats, uint32_t num_mats,
                                           uint32_t num_meshes, uint32_t *__restrict__ bad,
                                           uint32_t *__restrict__ mesh_unculled)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= n) return;
    const uint32_t m = inst[i].material, b = inst[i].blas;
    if(m >= num_mats) atomicOr(bad, 1u);
    else if(b < num_meshes && material_unculled(mats[m])) mesh_unculled[b] = 1u;
}

// the material fields the BSDF divides by or takes as probabilities must be in range
vkg_status check_material_values(vkg_ctx *ctx, const vkg_material *d_mats, uint32_t n, cudaStream_t st,
                                 const char *fn, bool *any_transmissive, bool *any_full, medium_rec **d_media,
                                 std::vector<medium_rec> *h_media, std::vector<vkg_material> *h_mats)
{
    *any_transmissive = false;
    *any_full = false;
    *d_media = nullptr;
    std::vector<medium_rec> media(n);
    bool any_medium = false;
    std::vector<vkg_material> h(n);
    cudaError_t e = cudaMemcpyAsync(h.data(), d_mats, n * sizeof(vkg_material), cudaMemcpyDeviceToHost, st);
    if(e == cudaSuccess) e = cudaStreamSynchronize(st);
    if(e != cudaSuccess) return cuda_check(ctx, e, fn);
    auto unit = [](float x) { return x >= 0.f && x <= 1.f; };
    for(uint32_t i = 0; i < n; ++i)
    {
        const vkg_material &m = h[i];
        if(!unit(m.transmission) || !unit(m.diffuse_transmission) || !unit(m.metalness))
            return set_error(ctx, VKG_ERR_INVALID_ARGUMENT,
                             "%s: material %u: metalness, transmission and diffuse_transmission must be in [0, 1]", fn, i);
        if(!unit(m.iridescence) ||
           (m.iridescence > 0.f && (!(m.iridescence_ior > 0.f) || !(m.iridescence_thickness >= 0.f) ||
                                    !std::isfinite(m.iridescence_ior) || !std::isfinite(m.iridescence_thickness))))
            return set_error(ctx, VKG_ERR_INVALID_ARGUMENT,
                             "%s: material %u: iridescence in [0, 1] needs an ior > 0 and a thickness >= 0", fn, i);
        if(m.transmission > 0.f && !(m.ior > 0.f && std::isfinite(m.ior)))
            return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "%s: material %u: a transmissive material needs ior > 0",
                             fn, i);
        if(!(m.dispersion >= 0.f) || !std::isfinite(m.dispersion))
            return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "%s: material %u: dispersion must be finite and >= 0", fn, i);
        if(!(m.clearcoat >= 0.f) || !(m.clearcoat_roughness >= 0.f) || !(m.sheen_roughness >= 0.f) ||
           !std::isfinite(m.clearcoat))
            return set_error(ctx, VKG_ERR_INVALID_ARGUMENT,
                             "%s: material %u: clearcoat, clearcoat_roughness and sheen_roughness must be >= 0", fn, i);
        const bool vol = material_has_volume(m);
        auto unit_open = [](float x) { return x > 0.f && x <= 1.f; };
        if((vol && (!unit_open(m.attenuation_color[0]) || !unit_open(m.attenuation_color[1]) ||
                    !unit_open(m.attenuation_color[2]))) ||
           !unit(m.scatter_factor) || !unit(m.scatter_color[0]) || !unit(m.scatter_color[1]) ||
           !unit(m.scatter_color[2]) || !(m.phase_g > -1.f && m.phase_g < 1.f))
            return set_error(ctx, VKG_ERR_INVALID_ARGUMENT,
                             "%s: material %u: attenuation colour in (0, 1], scatter factor / colour in [0, 1], "
                             "phase g in (-1, 1)", fn, i);
        if(m.blend_mode > VKG_BLEND_MASK ||
           (material_alpha_tested(m) && !(std::isfinite(m.alpha) && std::isfinite(m.alpha_cutoff))))
            return set_error(ctx, VKG_ERR_INVALID_ARGUMENT,
                             "%s: material %u: blend_mode must be VKG_BLEND_OPAQUE / _BLEND / _MASK, alpha and "
                             "alpha_cutoff finite", fn, i);
        *any_transmissive = *any_transmissive || m.transmission > 0.f || m.null_surface;
        *any_full = *any_full || material_full(m);
        media[i] = medium_from_material(m);
        any_medium = any_medium || vol || m.null_surface;
    }
    if(any_medium)
    {
        e = cudaMalloc(d_media, n * sizeof(medium_rec));
        if(e == cudaSuccess)
            e = cudaMemcpyAsync(*d_media, media.data(), n * sizeof(medium_rec), cudaMemcpyHostToDevice, st);
        if(e == cudaSuccess) e = cudaStreamSynchronize(st);
        if(e != cudaSuccess) return cuda_check(ctx, e, fn);
    }
    *h_media = std::move(media);
    *h_mats = std::move(h);
    return VKG_OK;
}

void tracer_free_buffers(vkg_tracer *t)
{
    for(void *p: {(void *)t->q_ray[0], (void *)t->q_ray[1], (void *)t->q_pid[0], (void *)t->q_pid[1], (void *)t->hits,
                  (void *)t->hit_inst,
                  (void *)t->s_ray, (void *)t->s_pid, (void *)t->s_contrib, (void *)t->rng, (void *)t->beta_pdf,
                  (void *)t->radiance, (void *)t->sum, (void *)t->accum, (void *)t->gbuf, (void *)t->order,
                  (void *)t->bins})
        cudaFree(p);
    t->order = t->bins = nullptr;
    t->q_ray[0] = t->q_ray[1] = nullptr;
    t->q_pid[0] = t->q_pid[1] = nullptr;
    t->hits = nullptr;
    t->hit_inst = nullptr;
    t->s_ray = nullptr;
    t->s_pid = nullptr;
    t->s_contrib = nullptr;
    t->rng = nullptr;
    t->beta_pdf = t->radiance = nullptr;
    t->gbuf = nullptr;
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
    al((void **)&t->hit_inst, paths * sizeof(uint32_t));
    al((void **)&t->s_ray, paths * sizeof(vkg_ray));
    al((void **)&t->s_pid, paths * sizeof(uint32_t));
    al((void **)&t->s_contrib, paths * sizeof(float4));
    al((void **)&t->rng, paths * sizeof(uint64_t));
    al((void **)&t->beta_pdf, paths * sizeof(float4));
    al((void **)&t->radiance, paths * sizeof(float4));
    al((void **)&t->sum, npix * 3 * sizeof(float));
    al((void **)&t->accum, npix * 3 * sizeof(float));
    al((void **)&t->gbuf, npix * sizeof(vkg_pixel_data));
    al((void **)&t->order, paths * sizeof(uint32_t));
    al((void **)&t->bins, 2 * PT_BIN_CLASSES * sizeof(uint32_t));
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

// the light list on the device and a light-NEE shadow queue for `paths` paths
vkg_status tracer_ensure_lights(vkg_tracer *t, const std::vector<vkg_light> &lights, size_t paths, cudaStream_t st)
{
    if(lights.empty()) return VKG_OK;
    cudaError_t e = cudaSuccess;
    if(lights.size() > t->lights_cap)
    {
        cudaFree(t->d_lights);
        t->d_lights = nullptr;
        t->lights_cap = 0;
        e = cudaMalloc(&t->d_lights, lights.size() * sizeof(vkg_light));
        if(e != cudaSuccess) return cuda_check(t->ctx, e, "light list");
        t->lights_cap = lights.size();
    }
    if(paths > t->lq_cap)
    {
        for(void *p: {(void *)t->l_ray, (void *)t->l_pid, (void *)t->l_contrib}) cudaFree(p);
        t->l_ray = nullptr;
        t->l_pid = nullptr;
        t->l_contrib = nullptr;
        t->lq_cap = 0;
        if(e == cudaSuccess) e = cudaMalloc(&t->l_ray, paths * sizeof(vkg_ray));
        if(e == cudaSuccess) e = cudaMalloc(&t->l_pid, paths * sizeof(uint32_t));
        if(e == cudaSuccess) e = cudaMalloc(&t->l_contrib, paths * sizeof(float4));
        if(e != cudaSuccess) return cuda_check(t->ctx, e, "light shadow queue");
        t->lq_cap = paths;
    }
    // pageable source: the copy is staged before the call returns
    e = cudaMemcpyAsync(t->d_lights, lights.data(), lights.size() * sizeof(vkg_light), cudaMemcpyHostToDevice, st);
    return e == cudaSuccess ? VKG_OK : cuda_check(t->ctx, e, "light list");
}

}// namespace
}// namespace vkg

using namespace vkg;

vkg_status vkg::check_tracer_settings(vkg_ctx *ctx, const vkg_settings *s)
{
    if(s->resolution[0] == 0 || s->resolution[1] == 0)
        return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "settings: zero resolution");
    if(s->num_samples == 0) return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "settings: num_samples == 0");
    if(s->max_trace_depth == 0 || s->max_trace_depth > 64)
        return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "settings: max_trace_depth must be 1..64");
    if(s->mis_mode > 2) return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "settings: mis_mode must be 0, 1 or 2");
    if(s->rng_mode > VKG_RNG_REFERENCE)
        return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "settings: rng_mode must be VKG_RNG_PCG32 or VKG_RNG_REFERENCE");
    if(s->crop[2] && s->crop[3] &&
       ((uint64_t)s->crop[0] + s->crop[2] > s->resolution[0] || (uint64_t)s->crop[1] + s->crop[3] > s->resolution[1]))
        return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "settings: crop window outside the resolution");
    if(!std::isfinite(s->sun_intensity) || s->sun_intensity < 0.f || !std::isfinite(s->sun_angular_size) ||
       s->sun_angular_size < 0.f || !std::isfinite(s->sun_spherical_coords[0]) ||
       !std::isfinite(s->sun_spherical_coords[1]))
        return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "settings: invalid sun parameters");
    return VKG_OK;
}

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
    if(vkg_status s = check_material_values(ctx, sc->mats, d->num_materials, st, "vkg_scene_create",
                                                 &sc->any_transmissive, &sc->any_full, &sc->d_media,
                                                 &sc->h_media, &sc->h_mats);
       s != VKG_OK)
    {
        vkg_scene_destroy(ctx, sc);
        return s;
    }
    for(const vkg_material &m: sc->h_mats)
    {
        sc->any_dispersion = sc->any_dispersion || material_dispersive(m);
        sc->any_alpha = sc->any_alpha || material_alpha_tested(m);
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

vkg_status vkg_scene_set_lights(vkg_ctx *ctx, vkg_scene *sc, const vkg_light *lights, uint32_t n)
{
    if(!ctx) return VKG_ERR_INVALID_ARGUMENT;
    if(!sc || (n && !lights)) return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_scene_set_lights: NULL argument");
    std::vector<vkg_light> v(lights, lights + n);
    auto finite = [](const float *p, int k) {
        for(int i = 0; i < k; ++i)
            if(!std::isfinite(p[i])) return false;
        return true;
    };
    auto unit = [](float *p) {
        const float l2 = p[0] * p[0] + p[1] * p[1] + p[2] * p[2];
        if(!(l2 > 0.f) || !std::isfinite(l2)) return false;
        const float inv = 1.f / std::sqrt(l2);
        for(int i = 0; i < 3; ++i) p[i] *= inv;
        return true;
    };
    for(uint32_t i = 0; i < n; ++i)
    {
        vkg_light &l = v[i];
        const uint32_t ty = l.type;
        if(ty > VKG_LIGHT_DISK || ty == VKG_LIGHT_AREA)
            return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_scene_set_lights: light %u: unsupported type %u", i, ty);
        if(!finite(l.position, 3) || !finite(l.color, 3) || !std::isfinite(l.intensity) || l.intensity < 0.f ||
           !(l.range > 0.f) || !std::isfinite(l.spot_angle_scale) || !std::isfinite(l.spot_angle_offset) ||
           !std::isfinite(l.angular_size) || l.angular_size < 0.f)
            return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_scene_set_lights: light %u: invalid parameters", i);
        const bool area = ty >= VKG_LIGHT_RECT;
        if(ty != VKG_LIGHT_OMNI && ty != VKG_LIGHT_SPHERE && !unit(l.direction))
            return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_scene_set_lights: light %u: zero direction", i);
        if(ty == VKG_LIGHT_RECT && !unit(l.tangent))
            return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_scene_set_lights: light %u: zero tangent", i);
        if(area && (!(l.size_x > 0.f) || !std::isfinite(l.size_x) ||
                    ((ty == VKG_LIGHT_RECT || ty == VKG_LIGHT_TUBE) && (!(l.size_y > 0.f) || !std::isfinite(l.size_y)))))
            return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_scene_set_lights: light %u: area lights need sizes > 0", i);
    }
    sc->lights = std::move(v);
    return VKG_OK;
}

namespace vkg
{
namespace
{
// per-vertex attributes from the caller's records: unit vectors from three floats or from the
// octahedral snorm16 pair of the reference's packed_vertex_t (packed_vertex.slang:17-23, unpacked
// as utils::unpack does with octahedral_map.slang:28-49); texture coordinates from two floats or
// two fp16
enum attr_kind : uint32_t
{
    ATTR_UNIT_F32X3,
    ATTR_UNIT_OCT16,
    ATTR_UV_F32X2,
    ATTR_UV_F16X2
};

__global__ void k_vertex_attr(const uint8_t *__restrict__ src, uint32_t stride, uint32_t kind, uint32_t n,
                              float *__restrict__ out)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if(k >= n) return;
    const uint8_t *r = src + (size_t)k * stride;
    if(kind == ATTR_UV_F32X2 || kind == ATTR_UV_F16X2)
    {
        float2 t;
        if(kind == ATTR_UV_F16X2)
        {
            const __half2 h = *reinterpret_cast<const __half2 *>(r);
            t = __half22float2(h);
        }
        else
            t = make_float2(reinterpret_cast<const float *>(r)[0], reinterpret_cast<const float *>(r)[1]);
        out[2 * (size_t)k] = t.x;
        out[2 * (size_t)k + 1] = t.y;
        return;
    }
    float3 v;
    if(kind == ATTR_UNIT_OCT16)
    {
        const float2 e = unpack_snorm_2x16(*reinterpret_cast<const uint32_t *>(r));
        v = oct_decode(e.x, e.y);
    }
    else
    {
        const float *f = reinterpret_cast<const float *>(r);
        v = normalize(f3(f[0], f[1], f[2]));
    }
    out[3 * (size_t)k] = v.x;
    out[3 * (size_t)k + 1] = v.y;
    out[3 * (size_t)k + 2] = v.z;
}

// which attribute a setter fills: the single-level slot and the per-mesh slots
enum attr_slot
{
    SLOT_NORMAL,
    SLOT_TANGENT,
    SLOT_UV
};

vkg_status set_vertex_attr(vkg_ctx *ctx, vkg_scene *sc, uint32_t mesh, const void *d_src, uint32_t stride,
                           uint32_t format, attr_slot slot, const char *fn, void *stream)
{
    if(!ctx) return VKG_ERR_INVALID_ARGUMENT;
    if(!sc) return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "%s: NULL scene", fn);
    if(vkg_status s = bind_device(ctx); s != VKG_OK) return s;
    const bool instanced = sc->bvh == nullptr; // an instanced scene has per-mesh BVHs instead
    if(instanced ? mesh >= sc->mesh_nrm.size() : mesh != 0)
        return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "%s: mesh %u out of range", fn, mesh);
    uint32_t kind, comps, min_stride;
    if(slot == SLOT_UV)
    {
        if(format != VKG_TEXCOORD_FLOAT2 && format != VKG_TEXCOORD_HALF2)
            return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "%s: unknown format %u", fn, format);
        kind = format == VKG_TEXCOORD_FLOAT2 ? ATTR_UV_F32X2 : ATTR_UV_F16X2;
        comps = 2;
        min_stride = format == VKG_TEXCOORD_FLOAT2 ? 8u : 4u;
    }
    else
    {
        if(format != VKG_NORMALS_FLOAT3 && format != VKG_NORMALS_OCT_SNORM16)
            return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "%s: unknown format %u", fn, format);
        kind = format == VKG_NORMALS_FLOAT3 ? ATTR_UNIT_F32X3 : ATTR_UNIT_OCT16;
        comps = 3;
        min_stride = format == VKG_NORMALS_FLOAT3 ? 12u : 4u;
    }
    if(stride == 0) stride = min_stride;
    if(stride < min_stride || stride % 4u || (reinterpret_cast<uintptr_t>(d_src) & 3u))
        return set_error(ctx, VKG_ERR_INVALID_ARGUMENT,
                         "%s: stride must be 0 or a multiple of 4 >= %u, the source 4-byte aligned", fn, min_stride);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    std::vector<float *> &per_mesh = slot == SLOT_NORMAL ? sc->mesh_nrm : slot == SLOT_TANGENT ? sc->mesh_tng : sc->mesh_uv;
    float *&single = slot == SLOT_NORMAL ? sc->nrm : slot == SLOT_TANGENT ? sc->tng : sc->uv;
    float *&ptr = instanced ? per_mesh[mesh] : single;
    const uint32_t nv = instanced ? sc->mesh_vertices[mesh] : sc->num_vertices;
    // the renders queued before keep reading the old array until they finish
    VKG_TRY_CUDA(ctx, cudaStreamSynchronize(st));
    VKG_TRY_CUDA(ctx, cudaDeviceSynchronize());
    cudaFree(ptr);
    ptr = nullptr;
    if(d_src && nv)
    {
        VKG_TRY_CUDA(ctx, cudaMalloc(&ptr, (size_t)nv * comps * sizeof(float)));
        k_vertex_attr<<<(nv + 255) / 256, 256, 0, st>>>(static_cast<const uint8_t *>(d_src), stride, kind, nv, ptr);
        VKG_TRY_CUDA(ctx, cudaGetLastError());
    }
    if(instanced)
    {
        mesh_ref &r = sc->h_meshes[mesh];
        (slot == SLOT_NORMAL ? r.nrm : slot == SLOT_TANGENT ? r.tng : r.uv) = ptr;
        VKG_TRY_CUDA(ctx, cudaMemcpyAsync(sc->d_meshes + mesh, &r, sizeof(mesh_ref), cudaMemcpyHostToDevice, st));
    }
    VKG_TRY_CUDA(ctx, cudaStreamSynchronize(st));
    return VKG_OK;
}
}// namespace
}// namespace vkg

extern "C" vkg_status vkg_scene_set_normals(vkg_ctx *ctx, vkg_scene *sc, uint32_t mesh, const void *d_src,
                                            uint32_t stride, uint32_t format, void *stream)
{
    return set_vertex_attr(ctx, sc, mesh, d_src, stride, format, SLOT_NORMAL, "vkg_scene_set_normals", stream);
}

extern "C" vkg_status vkg_scene_set_tangents(vkg_ctx *ctx, vkg_scene *sc, uint32_t mesh, const void *d_src,
                                             uint32_t stride, uint32_t format, void *stream)
{
    return set_vertex_attr(ctx, sc, mesh, d_src, stride, format, SLOT_TANGENT, "vkg_scene_set_tangents", stream);
}

extern "C" vkg_status vkg_scene_set_texcoords(vkg_ctx *ctx, vkg_scene *sc, uint32_t mesh, const void *d_src,
                                              uint32_t stride, uint32_t format, void *stream)
{
    return set_vertex_attr(ctx, sc, mesh, d_src, stride, format, SLOT_UV, "vkg_scene_set_texcoords", stream);
}

extern "C" vkg_status vkg_scene_set_textures(vkg_ctx *ctx, vkg_scene *sc, const vkg_texture_desc *textures, uint32_t n,
                                             void *stream)
{
    if(!ctx) return VKG_ERR_INVALID_ARGUMENT;
    if(!sc || (n && !textures)) return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_scene_set_textures: NULL argument");
    if(vkg_status s = bind_device(ctx); s != VKG_OK) return s;
    // records and every level on the host: level k + 1 = rounded mean of 2 x 2 texels of level k
    // (the last row / column repeated for odd sizes)
    std::vector<tex_rec> recs(n);
    std::vector<uint32_t> texels;
    for(uint32_t i = 0; i < n; ++i)
    {
        const vkg_texture_desc &d = textures[i];
        if(!d.h_rgba8 || d.width == 0 || d.height == 0 || d.width > 32768 || d.height > 32768)
            return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_scene_set_textures: texture %u: empty or larger than 32768", i);
        if(d.wrap_s > VKG_WRAP_MIRRORED_REPEAT || d.wrap_t > VKG_WRAP_MIRRORED_REPEAT)
            return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_scene_set_textures: texture %u: unknown wrap mode", i);
        tex_rec &r = recs[i];
        r = tex_rec{};
        r.width = d.width;
        r.height = d.height;
        r.wrap = d.wrap_s | (d.wrap_t << 8);
        uint32_t w = d.width, h = d.height, levels = 1;
        while((w > 1 || h > 1) && levels < TEX_MAX_LEVELS)
        {
            w = std::max(1u, w / 2);
            h = std::max(1u, h / 2);
            ++levels;
        }
        r.levels = levels;
        if(texels.size() + (size_t)d.width * d.height * 2 > 0xFFFFFFFFull)
            return set_error(ctx, VKG_ERR_CAPACITY, "vkg_scene_set_textures: more than 2^32 texels");
        r.offset[0] = (uint32_t)texels.size();
        const uint8_t *src = d.h_rgba8;
        for(size_t k = 0; k < (size_t)d.width * d.height; ++k)
            texels.push_back((uint32_t)src[4 * k] | ((uint32_t)src[4 * k + 1] << 8) | ((uint32_t)src[4 * k + 2] << 16) |
                             ((uint32_t)src[4 * k + 3] << 24));
        w = d.width;
        h = d.height;
        for(uint32_t l = 1; l < levels; ++l)
        {
            const uint32_t pw = w, ph = h, pbase = r.offset[l - 1];
            w = std::max(1u, w / 2);
            h = std::max(1u, h / 2);
            r.offset[l] = (uint32_t)texels.size();
            for(uint32_t y = 0; y < h; ++y)
                for(uint32_t x = 0; x < w; ++x)
                {
                    const uint32_t x0 = std::min(2 * x, pw - 1), x1 = std::min(2 * x + 1, pw - 1);
                    const uint32_t y0 = std::min(2 * y, ph - 1), y1 = std::min(2 * y + 1, ph - 1);
                    const uint32_t a = texels[pbase + y0 * pw + x0], b = texels[pbase + y0 * pw + x1];
                    const uint32_t c = texels[pbase + y1 * pw + x0], e = texels[pbase + y1 * pw + x1];
                    uint32_t out = 0;
                    for(int ch = 0; ch < 4; ++ch)
                    {
                        const uint32_t sh = 8u * (uint32_t)ch;
                        const uint32_t sum = ((a >> sh) & 0xFFu) + ((b >> sh) & 0xFFu) + ((c >> sh) & 0xFFu) +
                                             ((e >> sh) & 0xFFu);
                        out |= ((sum + 2u) >> 2) << sh;
                    }
                    texels.push_back(out);
                }
        }
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    VKG_TRY_CUDA(ctx, cudaStreamSynchronize(st));
    VKG_TRY_CUDA(ctx, cudaDeviceSynchronize());
    cudaFree(sc->d_tex);
    cudaFree(sc->d_texels);
    sc->d_tex = nullptr;
    sc->d_texels = nullptr;
    sc->num_textures = 0;
    if(n)
    {
        VKG_TRY_CUDA(ctx, cudaMalloc(&sc->d_tex, n * sizeof(tex_rec)));
        VKG_TRY_CUDA(ctx, cudaMalloc(&sc->d_texels, texels.size() * sizeof(uint32_t)));
        VKG_TRY_CUDA(ctx, cudaMemcpyAsync(sc->d_tex, recs.data(), n * sizeof(tex_rec), cudaMemcpyHostToDevice, st));
        VKG_TRY_CUDA(ctx, cudaMemcpyAsync(sc->d_texels, texels.data(), texels.size() * sizeof(uint32_t),
                                          cudaMemcpyHostToDevice, st));
        VKG_TRY_CUDA(ctx, cudaStreamSynchronize(st));
        sc->num_textures = n;
    }
    return VKG_OK;
}

vkg_status vkg_scene_destroy(vkg_ctx *ctx, vkg_scene *sc)
{
    if(!sc) return VKG_OK;
    if(ctx) bind_device(ctx);
    vkg_bvh_destroy(ctx, sc->bvh);
    vkg_tlas_destroy(ctx, sc->tlas);
    for(vkg_bvh *b: sc->blas) vkg_bvh_destroy(ctx, b);
    for(float *p: sc->mesh_xyz) cudaFree(p);
    for(uint32_t *p: sc->mesh_idx) cudaFree(p);
    for(float *p: sc->mesh_nrm) cudaFree(p);
    for(float *p: sc->mesh_uv) cudaFree(p);
    for(float *p: sc->mesh_tng) cudaFree(p);
    cudaFree(sc->d_meshes);
    cudaFree(sc->nrm);
    cudaFree(sc->uv);
    cudaFree(sc->tng);
    cudaFree(sc->d_tex);
    cudaFree(sc->d_texels);
    cudaFree(sc->xyz);
    cudaFree(sc->idx);
    cudaFree(sc->tri_mat);
    cudaFree(sc->mats);
    cudaFree(sc->d_media);
    env_free(sc->env);
    delete sc;
    return VKG_OK;
}

vkg_status vkg_scene_create_instanced(vkg_ctx *ctx, const vkg_instanced_scene_desc *d, vkg_scene **out, void *stream)
{
    if(!ctx) return VKG_ERR_INVALID_ARGUMENT;
    if(!d || !out) return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_scene_create_instanced: NULL argument");
    *out = nullptr;
    if(!d->d_materials || d->num_materials == 0)
        return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_scene_create_instanced: materials are required");
    if(!d->d_env_rgb || d->env_width == 0 || d->env_height == 0)
        return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_scene_create_instanced: an environment map is required");
    if((d->num_meshes && !d->meshes) || (d->num_instances && (!d->d_instances || d->num_meshes == 0)))
        return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_scene_create_instanced: NULL meshes or instances");
    if(vkg_status s = bind_device(ctx); s != VKG_OK) return s;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    auto *sc = new vkg_scene();
    sc->num_materials = d->num_materials;
    sc->num_instances = d->num_instances;
    cudaError_t e = cudaSuccess;
    auto chk = [&](cudaError_t x) {
        if(e == cudaSuccess) e = x;
    };
    auto fail = [&](vkg_status s) {
        vkg_scene_destroy(ctx, sc);
        return s;
    };
    chk(cudaMalloc(&sc->mats, d->num_materials * sizeof(vkg_material)));
    chk(cudaMemcpyAsync(sc->mats, d->d_materials, d->num_materials * sizeof(vkg_material), cudaMemcpyDeviceToDevice, st));
    if(e != cudaSuccess) return fail(cuda_check(ctx, e, "vkg_scene_create_instanced"));
    if(vkg_status s = check_material_values(ctx, sc->mats, d->num_materials, st, "vkg_scene_create_instanced",
                                                 &sc->any_transmissive, &sc->any_full, &sc->d_media,
                                                 &sc->h_media, &sc->h_mats);
       s != VKG_OK)
        return fail(s);
    for(const vkg_material &m: sc->h_mats)
    {
        sc->any_dispersion = sc->any_dispersion || material_dispersive(m);
        sc->any_alpha = sc->any_alpha || material_alpha_tested(m);
    }
    std::vector<mesh_ref> refs(d->num_meshes);
    uint64_t tris = 0;
    for(uint32_t m = 0; m < d->num_meshes && e == cudaSuccess; ++m)
    {
        const vkg_mesh_desc &M = d->meshes[m];
        if(M.num_tris && (!M.d_xyz || !M.d_indices || M.num_vertices == 0))
            return fail(set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_scene_create_instanced: mesh %u has no geometry", m));
        const size_t stride = M.vertex_stride ? M.vertex_stride : 12u;
        if(stride < 12u || stride % 4u)
            return fail(set_error(ctx, VKG_ERR_INVALID_ARGUMENT,
                                  "vkg_scene_create_instanced: mesh %u: vertex_stride must be 0 or a multiple of 4 >= 12", m));
        float *xyz = nullptr;
        uint32_t *idx = nullptr;
        chk(cudaMalloc(&xyz, std::max<size_t>(M.num_vertices, 1) * 3 * sizeof(float)));
        chk(cudaMalloc(&idx, std::max<size_t>(M.num_tris, 1) * 3 * sizeof(uint32_t)));
        sc->mesh_xyz.push_back(xyz);
        sc->mesh_idx.push_back(idx);
        if(M.num_tris)
        {
            if(stride == 12u)
                chk(cudaMemcpyAsync(xyz, M.d_xyz, (size_t)M.num_vertices * 3 * sizeof(float), cudaMemcpyDeviceToDevice, st));
            else // positions out of interleaved vertex records
                chk(cudaMemcpy2DAsync(xyz, 12, M.d_xyz, stride, 12, M.num_vertices, cudaMemcpyDeviceToDevice, st));
            chk(cudaMemcpyAsync(idx, M.d_indices, (size_t)M.num_tris * 3 * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st));
        }
        if(e != cudaSuccess) break;
        vkg_bvh_build_options opt{d->leaf_max};
        vkg_bvh *b = nullptr;
        if(vkg_status s = vkg_bvh_build(ctx, xyz, M.num_vertices, idx, M.num_tris, &opt, &b, stream); s != VKG_OK)
            return fail(s);
        sc->blas.push_back(b);
        if(M.twosided && M.num_tris)
            k_set_tri_flags<<<(M.num_tris + 255) / 256, 256, 0, st>>>(b->d_tris, M.num_tris, TRI_FLAG_TWOSIDED);
        refs[m] = mesh_ref{xyz, idx, nullptr, nullptr, nullptr};
        sc->mesh_nrm.push_back(nullptr);
        sc->mesh_uv.push_back(nullptr);
        sc->mesh_tng.push_back(nullptr);
        sc->mesh_vertices.push_back(M.num_vertices);
        tris += M.num_tris;
    }
    sc->h_meshes = refs;
    if(e == cudaSuccess && d->num_meshes)
    {
        chk(cudaMalloc(&sc->d_meshes, d->num_meshes * sizeof(mesh_ref)));
        chk(cudaMemcpyAsync(sc->d_meshes, refs.data(), d->num_meshes * sizeof(mesh_ref), cudaMemcpyHostToDevice, st));
    }
    if(e != cudaSuccess) return fail(cuda_check(ctx, e, "vkg_scene_create_instanced"));
    if(d->num_instances)
    {
        // word 0: bad material index; words 1..num_meshes: the mesh is used with an unculled material
        uint32_t *flags = nullptr;
        std::vector<uint32_t> hf(1 + d->num_meshes, 0u);
        chk(cudaMallocAsync(&flags, hf.size() * sizeof(uint32_t), st));
        chk(cudaMemsetAsync(flags, 0, hf.size() * sizeof(uint32_t), st));
        k_check_instance_materials<<<(d->num_instances + 255) / 256, 256, 0, st>>>(
                d->d_instances, d->num_instances, sc->mats, d->num_materials, d->num_meshes, flags, flags + 1);
        chk(cudaMemcpyAsync(hf.data(), flags, hf.size() * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        chk(cudaFreeAsync(flags, st));
        chk(cudaStreamSynchronize(st));
        if(e != cudaSuccess) return fail(cuda_check(ctx, e, "vkg_scene_create_instanced"));
        if(hf[0]) return fail(set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_scene_create_instanced: an instance material >= num_materials"));
        sc->h_inst.resize(d->num_instances);
        chk(cudaMemcpyAsync(sc->h_inst.data(), d->d_instances, d->num_instances * sizeof(vkg_instance),
                            cudaMemcpyDeviceToHost, st));
        chk(cudaStreamSynchronize(st));
        if(e != cudaSuccess) return fail(cuda_check(ctx, e, "vkg_scene_create_instanced"));
        // rays enter and leave transmissive instances through back faces: their meshes are not culled
        for(uint32_t m = 0; m < d->num_meshes; ++m)
            if(hf[1 + m] && !d->meshes[m].twosided && d->meshes[m].num_tris)
                k_set_tri_flags<<<(d->meshes[m].num_tris + 255) / 256, 256, 0, st>>>(sc->blas[m]->d_tris,
                                                                                   d->meshes[m].num_tris,
                                                                                   TRI_FLAG_TWOSIDED);
        chk(cudaGetLastError());
    }
    std::vector<const vkg_bvh *> bl(sc->blas.begin(), sc->blas.end());
    vkg_bvh_build_options topt{1}; // one instance per top-level leaf: its own quantised box culls it
    if(vkg_status s = vkg_tlas_build(ctx, bl.data(), (uint32_t)bl.size(), d->d_instances, d->num_instances, &topt,
                                     &sc->tlas, stream);
       s != VKG_OK)
        return fail(s);
    // an empty scene (no instances or no triangles) traces misses only
    sc->num_tris = d->num_instances ? (uint32_t)std::min<uint64_t>(tris, 0xFFFFFFFFu) : 0u;
    if(vkg_status s = env_build(ctx, d->d_env_rgb, d->env_width, d->env_height, sc->env, st); s != VKG_OK) return fail(s);
    chk(cudaStreamSynchronize(st));
    if(e != cudaSuccess) return fail(cuda_check(ctx, e, "vkg_scene_create_instanced"));
    *out = sc;
    return VKG_OK;
}

vkg_status vkg_scene_tlas(const vkg_scene *sc, const vkg_tlas **out)
{
    if(!sc || !out) return VKG_ERR_INVALID_ARGUMENT;
    *out = sc->tlas;
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
    s->denoising = 0;
    s->clip_near = 0.1f; // camera_params.hpp:37
    s->camera_medium_mode = VKG_CAMERA_MEDIUM_DETECT;
    vkg_medium_params_default(&s->camera_medium);
    return VKG_OK;
}

vkg_status vkg_medium_params_default(vkg_medium_params *p)
{
    if(!p) return VKG_ERR_INVALID_ARGUMENT;
    *p = vkg_medium_params{}; // media.hpp:26-49
    for(int c = 0; c < 3; ++c)
    {
        p->attenuation_color[c] = 0.7f;
        p->scatter_color[c] = 1.f;
        p->emission_color[c] = 1.f;
    }
    p->attenuation_distance = 1.f;
    p->ior = 1.f;
    return VKG_OK;
}

vkg_status vkg_scene_camera_medium(const vkg_scene *scene, const float eye[3], uint32_t *material)
{
    if(!scene || !eye || !material) return VKG_ERR_INVALID_ARGUMENT;
    *material = detect_camera_medium(scene, eye);
    return VKG_OK;
}


vkg_status vkg_tracer_create(vkg_ctx *ctx, const vkg_tracer_create_info *info, vkg_tracer **out)
{
    if(!ctx) return VKG_ERR_INVALID_ARGUMENT;
    if(!info || !out) return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_tracer_create: NULL argument");
    *out = nullptr;
    if(vkg_status s = check_tracer_settings(ctx, &info->settings); s != VKG_OK) return s;
    if(vkg_status s = bind_device(ctx); s != VKG_OK) return s;
    auto *t = new vkg_tracer();
    t->ctx = ctx;
    t->seed = info->seed;
    t->ref_engine.seed(info->seed);
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
    if(vkg_status r = check_tracer_settings(t->ctx, s); r != VKG_OK) return r;
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
    // the reference's streams chain a pixel's samples: one sample per pixel and wave
    const bool ref_rng = S.rng_mode == VKG_RNG_REFERENCE;
    if(ref_rng) spw = 1;
    if(ref_rng && t->cache)
        return set_error(ctx, VKG_ERR_NOT_SUPPORTED, "vkg_tracer_render: VKG_RNG_REFERENCE with a radiance cache");
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

    const std::vector<vkg_light> lights = render_lights(sc, S);
    if(vkg_status s = tracer_ensure_lights(t, lights, paths + train_paths, st); s != VKG_OK) return s;
    pt_params P = make_params(sc, *cam, S, t->seed, t->batch);
    if(ref_rng)
    {
        if(t->ref_cap < npix)
        {
            cudaFree(t->ref_chain);
            cudaFree(t->ref_offset);
            t->ref_chain = nullptr;
            t->ref_offset = nullptr;
            t->ref_cap = 0;
            VKG_TRY_CUDA(ctx, cudaMalloc(&t->ref_chain, npix * sizeof(uint32_t)));
            VKG_TRY_CUDA(ctx, cudaMalloc(&t->ref_offset, npix * sizeof(float)));
            t->ref_cap = npix;
        }
        P.ref_rng = 1;
        P.ref_seed = (uint32_t)t->ref_engine(); // trace_params.random_seed = m_random_engine() (PBRPathTracer.cpp:588)
        P.ref_width = S.resolution[0];
        P.ref_samples = S.num_samples;
        P.ref_chain = t->ref_chain;
        P.ref_offset = t->ref_offset;
    }
    P.dbg_u = t->dbg_u;
    P.dbg_segments = t->dbg_segments;
    P.dbg_stride = 2 + DBG_U_PER_SEGMENT * t->dbg_segments;
    P.lights = lights.empty() ? nullptr : t->d_lights;
    P.num_lights = (uint32_t)lights.size();
    uint32_t *cnt_l = lights.empty() ? nullptr : t->counters + 7;
    const light_queue lq{t->l_ray, t->l_pid, t->l_contrib, cnt_l};
    // the camera's medium (raypipeline.slang:128-135, PBRPathTracer.cpp:598-605): given, or the
    // medium of the smallest volume instance around the eye; its record follows the scene's
    uint32_t cam_mat = 0xFFFFFFFFu;
    medium_rec cam_rec{};
    if(S.camera_medium_mode == VKG_CAMERA_MEDIUM_GIVEN)
    {
        if(!medium_params_valid(S.camera_medium))
            return set_error(ctx, VKG_ERR_INVALID_ARGUMENT,
                             "vkg_tracer_render: camera medium: attenuation colour in (0, 1], finite distance > 0, "
                             "scatter factor / colour in [0, 1], phase g in (-1, 1), ior > 0, emission >= 0");
        cam_rec = medium_from_params(S.camera_medium);
        cam_mat = 0u;
    }
    else if(S.camera_medium_mode != VKG_CAMERA_MEDIUM_DETECT)
        return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_tracer_render: unknown camera_medium_mode %u",
                         S.camera_medium_mode);
    else if((cam_mat = detect_camera_medium(sc, cam->eye)) != 0xFFFFFFFFu)
    {
        cam_rec = sc->h_media[cam_mat];
        cam_rec.flags = MEDIUM_VOLUME; // keeps its own ior, also for a null-surface material
    }
    const bool cam_medium = cam_mat != 0xFFFFFFFFu;
    const bool has_media = sc->d_media || cam_medium;
    if(cam_medium)
    {
        const size_t n = sc->h_media.size();
        std::vector<medium_rec> table(sc->h_media);
        table.push_back(cam_rec);
        const bool same = t->media_cam.size() == table.size() &&
                          std::memcmp(t->media_cam.data(), table.data(), table.size() * sizeof(medium_rec)) == 0;
        if(!same)
        {
            if(t->media_cam.size() < table.size())
            {
                cudaFree(t->d_media_cam);
                t->d_media_cam = nullptr;
                t->media_cam.clear();
                VKG_TRY_CUDA(ctx, cudaMalloc(&t->d_media_cam, table.size() * sizeof(medium_rec)));
            }
            VKG_TRY_CUDA(ctx, cudaMemcpyAsync(t->d_media_cam, table.data(), table.size() * sizeof(medium_rec),
                                              cudaMemcpyHostToDevice, st));
            VKG_TRY_CUDA(ctx, cudaStreamSynchronize(st));
            t->media_cam = std::move(table);
        }
        P.media = t->d_media_cam;
        P.cam_medium = (uint32_t)n;
    }
    // the shade variant: the full Disney model and the light terms, or metal-roughness only
    const bool full = sc->any_full || !lights.empty() || has_media;
    P.gbuf = t->gbuf;
    if(has_media)
    {
        if(ccfg) return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_tracer_render: media with a radiance cache");
        if(t->mstack_cap < paths + train_paths)
        {
            cudaFree(t->mstack);
            t->mstack = nullptr;
            t->mstack_cap = 0;
            VKG_TRY_CUDA(ctx, cudaMalloc(&t->mstack, (paths + train_paths) * sizeof(uint4)));
            t->mstack_cap = paths + train_paths;
        }
        P.mstack = t->mstack;
    }
    if(sc->num_textures)
    {
        if(t->cone_cap < paths + train_paths)
        {
            cudaFree(t->cone);
            t->cone = nullptr;
            t->cone_cap = 0;
            VKG_TRY_CUDA(ctx, cudaMalloc(&t->cone, (paths + train_paths) * sizeof(float)));
            t->cone_cap = paths + train_paths;
        }
        P.cone = t->cone;
    }
    P.term_depth = cache_render ? ccfg->terminate_depth : 0xFFFFFFFFu;
    P.rec_depth = rec_depth;
    P.train_paths = train_paths;

    const bool empty = sc->num_tris == 0;
    uint32_t *cnt_q = t->counters + 3, *cnt_rec = t->counters + 4, *cnt_b = t->counters + 5, *cnt_work = t->counters + 6;
    // instanced scenes: grid-stride two-level tracers (faster on the stress scene: 274 vs 252 Mrays/s);
    // VKG_TL_KERNEL=persistent selects the refilling persistent ones
    const bool tl_persistent = sc->tlas && tl_persistent_selected() && !has_media && !sc->any_alpha;
    // alpha-tested materials: the queue tracers with the coverage filter (alpha_filter)
    const bool alpha = sc->any_alpha;
    const bool bin_materials = pt_binning_selected();
    // a 64-entry traversal stack serves BVHs up to 10 levels deep (7 (depth - 1) + 1 entries)
    const bool small_stack = sc->bvh && sc->bvh->depth <= 10;
    uint32_t tl_grid = 0;
    if(tl_persistent)
    {
        int per_sm = 0;
        VKG_TRY_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pt_tl_persistent<false>, PT_THREADS, 0));
        tl_grid = (uint32_t)ctx->num_sms * (uint32_t)std::max(1, per_sm);
    }
    cache_io io{t->q_feat, t->q_beta, cnt_q, t->rec, t->vcount};

    VKG_TRY_CUDA(ctx, cudaMemsetAsync(t->sum, 0, (size_t)npix * 3 * sizeof(float), st));
    VKG_TRY_CUDA(ctx, cudaMemsetAsync(t->gbuf, 0, (size_t)npix * sizeof(vkg_pixel_data), st));
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
        const single_scene SS{P};
        if(cache_render) VKG_TRY_CUDA(ctx, cudaMemsetAsync(cnt_q, 0, sizeof(uint32_t), st));
        k_pt_generate<<<grid, PT_THREADS, 0, st>>>(P, n, t->q_ray[0], t->q_pid[0], t->rng, t->beta_pdf, t->radiance,
                                                   t->counters, t->vcount);
        int a = 0;
        for(uint32_t depth = 0; depth < depths; ++depth)
        {
            uint32_t *cnt_in = t->counters + a, *cnt_out = t->counters + (1 - a), *cnt_s = t->counters + 2;
            if(empty)
                k_fill_miss_queue<<<grid, PT_THREADS, 0, st>>>(cnt_in, t->hits);
            else if(tl_persistent)
            {
                VKG_TRY_CUDA(ctx, cudaMemsetAsync(cnt_work, 0, sizeof(uint32_t), st));
                k_pt_tl_persistent<false><<<tl_grid, PT_THREADS, 0, st>>>(SS, t->q_ray[a], t->q_pid[a], cnt_in, t->hits,
                                                                         t->hit_inst, nullptr, nullptr, cnt_work);
            }
            else
            {
                // the first bounce's rays (the longest incoherent queue) are traced in bins of origin
                // cell x direction; the camera rays of depth 0 are coherent as they are, and the later
                // queues, shortened by Russian roulette and escapes, gain less than binning costs
                // (720p 64 spp: 69.1 ms binning depth 1, 69.3 ms binning every depth >= 1, 71.0 ms none)
                const uint32_t *reordered = nullptr;
                // (an instanced scene bins by the top level's box, its second bounce too, where the
                // costlier two-level traversal still gains: the stress frame 1,334 -> 1,268 ms with the
                // shadow queues below, 1,233 -> 1,215 ms with the second bounce)
                const vkg_bvh *bounds = sc->bvh ? sc->bvh : (sc->tlas ? &sc->tlas->top : nullptr);
                const bool bin_queue = depth == 1 || (sc->tlas && depth == 2);
                const uint32_t *perm =
                        bin_queue ? bin_rays(ctx, bounds, t->q_ray[a], n, cnt_in, 0u, st, &reordered) : nullptr;
                if(alpha && small_stack)
                    k_pt_extend<single_scene, 64, true><<<grid, PT_THREADS, 0, st>>>(
                            SS, t->q_ray[a], t->q_pid[a], cnt_in, t->hits, t->hit_inst, perm, reordered, t->rng, depth);
                else if(alpha)
                    k_pt_extend<single_scene, (int)TRAVERSAL_STACK, true><<<grid, PT_THREADS, 0, st>>>(
                            SS, t->q_ray[a], t->q_pid[a], cnt_in, t->hits, t->hit_inst, perm, reordered, t->rng, depth);
                else if(small_stack)
                    k_pt_extend<single_scene, 64><<<grid, PT_THREADS, 0, st>>>(SS, t->q_ray[a], t->q_pid[a], cnt_in,
                                                                                t->hits, t->hit_inst, perm, reordered);
                else
                    k_pt_extend<<<grid, PT_THREADS, 0, st>>>(SS, t->q_ray[a], t->q_pid[a], cnt_in, t->hits, t->hit_inst,
                                                             perm, reordered);
                if(perm) bin_rays_done(ctx, st);
            }
            VKG_TRY_CUDA(ctx, cudaMemsetAsync(cnt_out, 0, sizeof(uint32_t), st));
            VKG_TRY_CUDA(ctx, cudaMemsetAsync(cnt_s, 0, sizeof(uint32_t), st));
            if(cnt_l) VKG_TRY_CUDA(ctx, cudaMemsetAsync(cnt_l, 0, sizeof(uint32_t), st));
            // the full material set: group the queue by material class first, so that warps shade
            // coherently (k_pt_bin_count / k_pt_bin_scatter, two light passes over the hits)
            const uint32_t *order = nullptr;
            if(full && bin_materials)
            {
                VKG_TRY_CUDA(ctx, cudaMemsetAsync(t->bins, 0, 2 * PT_BIN_CLASSES * sizeof(uint32_t), st));
                k_pt_bin_count<<<grid, PT_THREADS, 0, st>>>(SS, t->q_pid[a], t->hits, t->hit_inst, cnt_in, t->bins);
                k_pt_bin_scatter<<<grid, PT_THREADS, 0, st>>>(SS, t->q_pid[a], t->hits, t->hit_inst, cnt_in, t->bins,
                                                              t->order);
                order = t->order;
            }
#define VKG_SHADE(M, F, MD, TX)                                                                                        \
    k_pt_shade<M, single_scene, F, MD, TX><<<grid, PT_THREADS, 0, st>>>(SS, depth, t->q_ray[a], t->q_pid[a], t->hits, t->hit_inst, cnt_in,    \
                                               t->q_ray[1 - a],                                                          \
                                               t->q_pid[1 - a], cnt_out, t->s_ray, t->s_pid, t->s_contrib, cnt_s,         \
                                               t->rng, t->beta_pdf, t->radiance, io, lq, order)
#define VKG_SHADE_T(M, F, MD)                                                                                          \
    do                                                                                                                 \
    {                                                                                                                  \
        if(P.cone) VKG_SHADE(M, F, MD, true);                                                                          \
        else VKG_SHADE(M, F, MD, false);                                                                               \
    } while(0)
            if(mode == MODE_PLAIN && has_media) VKG_SHADE_T(MODE_PLAIN, true, true);
            else if(mode == MODE_PLAIN && full) VKG_SHADE_T(MODE_PLAIN, true, false);
            else if(mode == MODE_PLAIN) VKG_SHADE_T(MODE_PLAIN, false, false);
            else if(full) VKG_SHADE_T(MODE_CACHE, true, false);
            else VKG_SHADE_T(MODE_CACHE, false, false);
#undef VKG_SHADE_T
#undef VKG_SHADE
            if(!empty && tl_persistent)
            {
                VKG_TRY_CUDA(ctx, cudaMemsetAsync(cnt_work, 0, sizeof(uint32_t), st));
                k_pt_tl_persistent<true><<<tl_grid, PT_THREADS, 0, st>>>(SS, t->s_ray, t->s_pid, cnt_s, nullptr, nullptr,
                                                                        t->s_contrib, t->radiance, cnt_work);
            }
            else if(!empty)
            {
                // the first two environment-shadow queues of a plain render are traced in bins too
                // (720p 64 spp: 68.5 -> 67.5 ms; the radiance-cache frames gain nothing from it)
                const uint32_t *s_reordered = nullptr;
                const vkg_bvh *s_bounds = sc->bvh ? sc->bvh : (sc->tlas ? &sc->tlas->top : nullptr);
                const uint32_t *s_perm = (mode == MODE_PLAIN && depth <= 1)
                                                 ? bin_rays(ctx, s_bounds, t->s_ray, n, cnt_s, 0u, st, &s_reordered)
                                                 : nullptr;
                if(alpha && small_stack)
                    k_pt_shadow<single_scene, 64, true><<<grid, PT_THREADS, 0, st>>>(
                            SS, t->s_ray, t->s_pid, t->s_contrib, cnt_s, t->radiance, s_perm, s_reordered, t->rng);
                else if(alpha)
                    k_pt_shadow<single_scene, (int)TRAVERSAL_STACK, true><<<grid, PT_THREADS, 0, st>>>(
                            SS, t->s_ray, t->s_pid, t->s_contrib, cnt_s, t->radiance, s_perm, s_reordered, t->rng);
                else if(small_stack)
                    k_pt_shadow<single_scene, 64><<<grid, PT_THREADS, 0, st>>>(SS, t->s_ray, t->s_pid, t->s_contrib,
                                                                                cnt_s, t->radiance, s_perm, s_reordered);
                else
                    k_pt_shadow<<<grid, PT_THREADS, 0, st>>>(SS, t->s_ray, t->s_pid, t->s_contrib, cnt_s, t->radiance,
                                                             s_perm, s_reordered);
                if(s_perm) bin_rays_done(ctx, st);
            }
            if(cnt_l && !empty)
            {
                if(alpha && small_stack)
                    k_pt_light_shadow<single_scene, 64, true><<<grid, PT_THREADS, 0, st>>>(SS, lq, t->radiance, t->rng);
                else if(alpha)
                    k_pt_light_shadow<single_scene, (int)TRAVERSAL_STACK, true>
                            <<<grid, PT_THREADS, 0, st>>>(SS, lq, t->radiance, t->rng);
                else if(small_stack)
                    k_pt_light_shadow<single_scene, 64><<<grid, PT_THREADS, 0, st>>>(SS, lq, t->radiance);
                else
                    k_pt_light_shadow<<<grid, PT_THREADS, 0, st>>>(SS, lq, t->radiance);
            }
            k_pt_tally<<<1, 1, 0, st>>>(cnt_in, cnt_s, cnt_l, t->totals);
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
    k_pixel_radiance<<<(npix + 255) / 256, 256, 0, st>>>(t->accum, npix, t->gbuf);
    if(S.denoising && d_rgb_out)
        if(vkg_status s = denoise_run(ctx, t->gbuf, cw, ch, nullptr, d_rgb_out, nullptr, st); s != VKG_OK) return s;
    VKG_TRY_CUDA(ctx, cudaEventRecord(t->ev1, st));
    VKG_TRY_CUDA(ctx, cudaGetLastError());
    t->last_paths = (uint64_t)npix * S.num_samples;
    t->rendered = true;
    t->batch += 1;
    return VKG_OK;
}

vkg_status vkg_tracer_pixel_data(vkg_tracer *t, vkg_pixel_data *d_out, void *stream)
{
    if(!t) return VKG_ERR_INVALID_ARGUMENT;
    if(!d_out) return set_error(t->ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_tracer_pixel_data: NULL buffer");
    if(!t->rendered) return set_error(t->ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_tracer_pixel_data: nothing rendered yet");
    if(vkg_status s = bind_device(t->ctx); s != VKG_OK) return s;
    VKG_TRY_CUDA(t->ctx, cudaMemcpyAsync(d_out, t->gbuf, t->npix_cap * sizeof(vkg_pixel_data), cudaMemcpyDeviceToDevice,
                                         static_cast<cudaStream_t>(stream)));
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

vkg_status vkg_diag_tracer_uniforms(vkg_tracer *t, float *d_buf, uint32_t max_segments)
{
    if(!t || (d_buf && (max_segments == 0 || max_segments > 64))) return VKG_ERR_INVALID_ARGUMENT;
    t->dbg_u = d_buf;
    t->dbg_segments = d_buf ? max_segments : 0u;
    return VKG_OK;
}

vkg_status vkg_tracer_destroy(vkg_tracer *t)
{
    if(!t) return VKG_OK;
    if(t->ctx) bind_device(t->ctx);
    tracer_free_buffers(t);
    tracer_free_cache_buffers(t);
    cudaFree(t->counters);
    for(void *p: {(void *)t->d_lights, (void *)t->l_ray, (void *)t->l_pid, (void *)t->l_contrib, (void *)t->mstack,
                  (void *)t->d_media_cam, (void *)t->ref_chain, (void *)t->ref_offset, (void *)t->cone})
        cudaFree(p);
    cudaFree(t->totals);
    if(t->ev0) cudaEventDestroy(t->ev0);
    if(t->ev1) cudaEventDestroy(t->ev1);
    if(t->ev_train) cudaEventDestroy(t->ev_train);
    delete t;
    return VKG_OK;
}

}// extern "C"
