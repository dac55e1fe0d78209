// Internal host-side state shared by the libvkg translation units (not part of the C ABI).
#pragma once

#include "../../include/vkg.h"
#include "../../include/vkg_diag.h"
#include "vkg_common.cuh"

#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <string>

struct vkg_ctx
{
    int device = 0;
    int num_sms = 0;
    std::string last_error;
    // device counters: [0] node visits, [1] triangle tests, [2] error flags (bit0 stack overflow)
    unsigned long long *d_counters = nullptr;
    // ray index counter of the persistent traversal kernels
    uint32_t *d_work = nullptr;
    // host-variant staging (grown on demand)
    void *d_stage_rays = nullptr;
    void *d_stage_hits = nullptr;
    size_t stage_rays_bytes = 0, stage_hits_bytes = 0;
    // the host variant's copy / trace pipeline (created on first use): streams [0], [1] trace
    // alternate chunks, [2] uploads, [3] downloads; events: [0] fork, [1..4] joins, [5] a chunk's
    // upload done, [6] a chunk's trace done
    cudaStream_t pipe[4] = {nullptr, nullptr, nullptr, nullptr};
    cudaEvent_t pipe_ev[7] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    // ray-binning scratch of the bulk queries (calls on different streams are ordered by `done`). keys: bin | rank in its tile << 16 per ray; perm: traced position -> ray
    // index (its first half holds the 16-bit bins before that); tile_counts: rays per (tile, bin);
    // bin_totals: rays per bin and the bins' first positions; done: recorded after the last use,
    // waited for by the next
    struct ray_bins
    {
        uint32_t *keys = nullptr;
        uint32_t *perm = nullptr;
        uint32_t *tile_counts = nullptr;
        uint32_t *bin_totals = nullptr;
        size_t cap = 0;
        uint32_t tiles_cap = 0;
        cudaEvent_t done = nullptr;
    } bins;
};

struct vkg_bvh
{
    uint32_t num_tris = 0, num_nodes = 0, depth = 0, leaf_max = 4;
    float scene_min[3] = {0, 0, 0}, scene_max[3] = {0, 0, 0}, margin = 0.f;
    vkg::node8 *d_nodes = nullptr;
    vkg::tri_rec *d_tris = nullptr;
    uint32_t *d_morton = nullptr; // input order
    uint32_t *d_sorted = nullptr; // sorted order -> triangle id
    size_t bytes = 0;
    float build_ms = 0.f;
};

namespace vkg
{
// instance record of a two-level BVH (128 B): world->object and object->world 3x4 row-major
// transforms, the BLAS the instance refers to, its input index and material
struct alignas(16) inst_rec
{
    float w2o[12];
    float o2w[12];
    uint32_t blas, instance, material, pad0;
    uint32_t pad1[4];
};
static_assert(sizeof(inst_rec) == 128, "inst_rec layout");

// top-level traversal stack; the build rejects top levels deeper than it supports
constexpr uint32_t TLAS_STACK = 64;
constexpr uint32_t TLAS_MAX_DEPTH = (TLAS_STACK - 1) / 7 + 1;

// a bottom-level BVH as the top level sees it
struct alignas(16) blas_ref
{
    const node8 *nodes;
    const tri_rec *tris;
    uint32_t num_tris, pad;
};
}// namespace vkg

struct vkg_tlas
{
    vkg_bvh top;                       // 8-wide BVH over the instances' world boxes (no triangle records)
    vkg::inst_rec *d_inst = nullptr;   // instance records in sorted (leaf) order
    vkg::inst_rec *d_inst_by_id = nullptr; // the same records in input order
    vkg::blas_ref *d_blas = nullptr;
    uint32_t num_instances = 0, num_blas = 0;
};

namespace vkg
{
// record an error message on ctx and return `status`
vkg_status set_error(vkg_ctx *ctx, vkg_status status, const char *fmt, ...);
// map a CUDA error to VKG_ERR_CUDA with location info; VKG_OK if err == cudaSuccess
vkg_status cuda_check(vkg_ctx *ctx, cudaError_t err, const char *what);
// ensure the context's device is current on this thread
vkg_status bind_device(vkg_ctx *ctx);

// traversal stack capacity (entries) of the traversal kernels; the build rejects deeper BVHs
constexpr uint32_t TRAVERSAL_STACK = 128;

// Ray binning (traverse.cu): the order in which to trace the rays d_rays[0, n) -- or [0, *d_n) when
// d_n is a device-side count <= n -- so that neighbouring threads follow similar paths through bvh:
// perm[position] = ray, valid when *reordered_out (a device word) is non-zero; otherwise the rays
// are to be traced as given. Returns nullptr (trace as given) for VKG_RAY_KEEP_ORDER, batches below
// 2^19 rays, a stream being captured, or scratch that cannot be allocated. The scratch is the
// context's; calls on different streams are ordered by an event recorded by bin_rays_done().
const uint32_t *bin_rays(vkg_ctx *ctx, const vkg_bvh *bvh, const vkg_ray *d_rays, uint32_t n, const uint32_t *d_n,
                         uint32_t flags, cudaStream_t st, const uint32_t **reordered_out);
// after the launch that reads the order: the scratch may be reused once the stream reaches here
inline void bin_rays_done(vkg_ctx *ctx, cudaStream_t st) { cudaEventRecord(ctx->bins.done, st); }
}// namespace vkg

#define VKG_TRY_CUDA(ctx, expr)                                                                                      \
    do                                                                                                               \
    {                                                                                                                \
        vkg_status s_ = vkg::cuda_check((ctx), (expr), #expr);                                                       \
        if(s_ != VKG_OK) return s_;                                                                                  \
    } while(0)
