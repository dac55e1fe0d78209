// GPU LBVH build collapsed to an 8-wide quantised BVH.
//
// Replaces the reference's driver-built bottom-level acceleration structure
// (RayBuilder::create_mesh_structures, src/RayBuilder.cpp:98-300, vkCmdBuildAccelerationStructuresKHR
// at :274) and its compaction copy (:305-356). The reference's BVH is opaque; this one is fully
// specified so that every stage can be compared bit-for-bit with the CPU statement of the same
// algorithm:
//   k_tri_boxes    triangle boxes + scene box (order-independent min/max atomics)
//   k_morton       30-bit Morton code of each box centre over the scene box
//   k_radix_*      stable LSD radix sort of (code, triangle id), 8 bits per pass
//   k_karras       Karras 2012 radix tree (equal codes split by index)
//   k_refit        bottom-up boxes, second arriving child finishes the parent
//   k_collapse     breadth-first collapse to 8-wide nodes + 8-bit box quantisation (one CTA)
//   k_tri_records  48-byte triangle records (v0, e1, e2, id) in sorted order
// Data layout in HBM: nodes (96 B each) and triangle records (48 B each) are contiguous arrays read
// with 16-byte vector loads by the traversal kernels.
#include "internal.hpp"
#include "radix_sort.cuh"

#include <algorithm>
#include <cstring>
#include <mutex>
#include <vector>

namespace vkg
{
namespace
{


struct box6
{
    float lo[3], hi[3];
};

// ordered-uint encoding: monotone for every float, so min/max atomics on it are exact
__device__ __forceinline__ uint32_t fenc(float f)
{
    uint32_t b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float fdec(uint32_t u) { return __uint_as_float((u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u); }

// errors reported by the build kernels
enum : uint32_t
{
    BUILD_ERR_INDEX = 1u,    // an index >= num_vertices (triangles) / a BLAS index >= num_blas (instances)
    BUILD_ERR_CAPACITY = 2u, // node capacity exceeded
    BUILD_ERR_SINGULAR = 4u, // an instance transform that cannot be inverted
};

__global__ void k_tri_boxes(const float *__restrict__ xyz, uint32_t nv, const uint32_t *__restrict__ idx, uint32_t n,
                            box6 *__restrict__ tbox, uint32_t *__restrict__ scene_enc, uint32_t *__restrict__ err)
{
    __shared__ uint32_t s_lo[3], s_hi[3];
    if(threadIdx.x < 3)
    {
        s_lo[threadIdx.x] = fenc(__int_as_float(0x7f800000));  // +inf
        s_hi[threadIdx.x] = fenc(__int_as_float(0xff800000));  // -inf
    }
    __syncthreads();
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i < n)
    {
        box6 b;
        for(int a = 0; a < 3; ++a)
        {
            b.lo[a] = __int_as_float(0x7f800000);
            b.hi[a] = __int_as_float(0xff800000);
        }
        for(int k = 0; k < 3; ++k)
        {
            uint32_t vi = __ldg(&idx[3 * (size_t)i + k]);
            if(vi >= nv)
            {
                atomicOr(err, BUILD_ERR_INDEX);
                vi = 0;
            }
            for(int a = 0; a < 3; ++a)
            {
                float p = __ldg(&xyz[3 * (size_t)vi + a]);
                b.lo[a] = fminf(b.lo[a], p);
                b.hi[a] = fmaxf(b.hi[a], p);
            }
        }
        tbox[i] = b;
        for(int a = 0; a < 3; ++a)
        {
            atomicMin(&s_lo[a], fenc(b.lo[a]));
            atomicMax(&s_hi[a], fenc(b.hi[a]));
        }
    }
    __syncthreads();
    if(threadIdx.x < 3)
    {
        atomicMin(&scene_enc[threadIdx.x], s_lo[threadIdx.x]);
        atomicMax(&scene_enc[3 + threadIdx.x], s_hi[threadIdx.x]);
    }
}

__device__ __forceinline__ void scene_box(const uint32_t *scene_enc, float lo[3], float hi[3])
{
    for(int a = 0; a < 3; ++a)
    {
        lo[a] = fdec(scene_enc[a]);
        hi[a] = fdec(scene_enc[3 + a]);
    }
}

__global__ void k_morton(const box6 *__restrict__ tbox, uint32_t n, const uint32_t *__restrict__ scene_enc,
                         uint32_t *__restrict__ keys, uint32_t *__restrict__ vals, uint32_t *__restrict__ morton_out)
{
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= n) return;
    float lo[3], hi[3];
    scene_box(scene_enc, lo, hi);
    box6 b = tbox[i];
    uint32_t q[3];
    for(int a = 0; a < 3; ++a)
    {
        float e = fsub(hi[a], lo[a]);
        float scale = e > 0.f ? fdiv(1024.0f, e) : 0.f;
        float c = fmul(fadd(b.lo[a], b.hi[a]), 0.5f);
        float f = fmul(fsub(c, lo[a]), scale);
        uint32_t v = f > 0.f ? __float2uint_rz(f) : 0u;
        q[a] = v > 1023u ? 1023u : v;
    }
    uint32_t code = (expand10(q[0]) << 2) | (expand10(q[1]) << 1) | expand10(q[2]);
    keys[i] = code;
    vals[i] = i;
    morton_out[i] = code;
}

__global__ void k_karras(const uint32_t *__restrict__ codes, uint32_t n, uint32_t *__restrict__ left,
                         uint32_t *__restrict__ right, uint32_t *__restrict__ first, uint32_t *__restrict__ last,
                         uint32_t *__restrict__ iparent, uint32_t *__restrict__ lparent)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= (int64_t)n - 1) return;
    const int64_t nn = n;
    int d = (kdelta(codes, nn, i, i + 1) - kdelta(codes, nn, i, i - 1)) >= 0 ? 1 : -1;
    int dmin = kdelta(codes, nn, i, i - d);
    int64_t lmax = 2;
    while(kdelta(codes, nn, i, i + lmax * d) > dmin) lmax *= 2;
    int64_t l = 0;
    for(int64_t t = lmax / 2; t >= 1; t /= 2)
        if(kdelta(codes, nn, i, i + (l + t) * d) > dmin) l += t;
    int64_t j = i + l * d;
    int dnode = kdelta(codes, nn, i, j);
    int64_t s = 0, t = l;
    do
    {
        t = (t + 1) / 2;
        if(kdelta(codes, nn, i, i + (s + t) * d) > dnode) s += t;
    } while(t > 1);
    int64_t gamma = i + s * d + (d < 0 ? -1 : 0);
    int64_t lo = i < j ? i : j, hi = i < j ? j : i;
    uint32_t lc = (lo == gamma) ? (LEAF_BIT | (uint32_t)gamma) : (uint32_t)gamma;
    uint32_t rc = (hi == gamma + 1) ? (LEAF_BIT | (uint32_t)(gamma + 1)) : (uint32_t)(gamma + 1);
    left[i] = lc;
    right[i] = rc;
    first[i] = (uint32_t)lo;
    last[i] = (uint32_t)hi;
    if(lc & LEAF_BIT) lparent[lc & ~LEAF_BIT] = (uint32_t)i;
    else iparent[lc] = (uint32_t)i;
    if(rc & LEAF_BIT) lparent[rc & ~LEAF_BIT] = (uint32_t)i;
    else iparent[rc] = (uint32_t)i;
}

__global__ void k_gather_leaf_boxes(const box6 *__restrict__ tbox, const uint32_t *__restrict__ sorted, uint32_t n,
                                    box6 *__restrict__ lbox)
{
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i < n) lbox[i] = tbox[sorted[i]];
}

__device__ __forceinline__ box6 load_box_cg(const box6 *p)
{
    const float *f = reinterpret_cast<const float *>(p);
    box6 b;
    for(int a = 0; a < 3; ++a)
    {
        b.lo[a] = __ldcg(f + a);
        b.hi[a] = __ldcg(f + 3 + a);
    }
    return b;
}

__global__ void k_refit(const uint32_t *__restrict__ lparent, const uint32_t *__restrict__ iparent,
                        const uint32_t *__restrict__ left, const uint32_t *__restrict__ right, const box6 *lbox,
                        box6 *ibox, uint32_t *visits, uint32_t n)
{
    uint32_t leaf = blockIdx.x * blockDim.x + threadIdx.x;
    if(leaf >= n || n < 2) return;
    uint32_t p = lparent[leaf];
    // bounded: a path to the root has at most n - 1 internal nodes
    for(uint32_t guard = 0; guard < n; ++guard)
    {
        __threadfence();
        if(atomicAdd(&visits[p], 1u) == 0u) return; // first arrival: the sibling finishes p
        __threadfence();                            // acquire: the sibling's box is visible now
        uint32_t l = left[p], r = right[p];
        box6 a = (l & LEAF_BIT) ? load_box_cg(&lbox[l & ~LEAF_BIT]) : load_box_cg(&ibox[l]);
        box6 b = (r & LEAF_BIT) ? load_box_cg(&lbox[r & ~LEAF_BIT]) : load_box_cg(&ibox[r]);
        box6 u;
        for(int k = 0; k < 3; ++k)
        {
            u.lo[k] = fminf(a.lo[k], b.lo[k]);
            u.hi[k] = fmaxf(a.hi[k], b.hi[k]);
        }
        float *dst = reinterpret_cast<float *>(&ibox[p]);
        for(int k = 0; k < 3; ++k)
        {
            __stcg(dst + k, u.lo[k]);
            __stcg(dst + 3 + k, u.hi[k]);
        }
        if(p == 0) return;
        p = iparent[p];
    }
}

// ---- breadth-first collapse to 8-wide nodes (one CTA, deterministic numbering) ----------------
struct collapse_args
{
    const uint32_t *left, *right, *first, *last;
    const box6 *ibox, *lbox;
    uint32_t n, leaf_max, capacity;
    const uint32_t *scene_enc;
    uint32_t *node_ref; // [capacity] BVH2 reference of each 8-wide node
    node8 *nodes;       // [capacity]
    uint32_t *out_info; // [0] num_nodes, [1] depth, [2] error flags
    float *out_margin;
};

__device__ __forceinline__ uint32_t ref_count(const collapse_args &A, uint32_t r)
{
    return (r & LEAF_BIT) ? 1u : (A.last[r] - A.first[r] + 1u);
}
__device__ __forceinline__ uint32_t ref_first(const collapse_args &A, uint32_t r)
{
    return (r & LEAF_BIT) ? (r & ~LEAF_BIT) : A.first[r];
}
__device__ __forceinline__ box6 ref_box(const collapse_args &A, uint32_t r)
{
    return (r & LEAF_BIT) ? A.lbox[r & ~LEAF_BIT] : A.ibox[r];
}
__device__ __forceinline__ float box_area(const box6 &b)
{
    float dx = fsub(b.hi[0], b.lo[0]), dy = fsub(b.hi[1], b.lo[1]), dz = fsub(b.hi[2], b.lo[2]);
    return fadd(fadd(fmul(dx, dy), fmul(dy, dz)), fmul(dz, dx));
}

constexpr int COLLAPSE_THREADS = 1024;

__global__ void __launch_bounds__(COLLAPSE_THREADS) k_collapse(collapse_args A)
{
    __shared__ uint32_t s_warp[32];
    __shared__ uint32_t s_level_end, s_next, s_err;
    __shared__ float s_margin;
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    if(tid == 0)
    {
        float lo[3], hi[3];
        scene_box(A.scene_enc, lo, hi);
        float ext = 0.f, amax = 0.f;
        for(int a = 0; a < 3; ++a)
        {
            ext = fmaxf(ext, fsub(hi[a], lo[a]));
            amax = fmaxf(amax, fmaxf(fabsf(lo[a]), fabsf(hi[a])));
        }
        s_margin = fmul(fmaxf(ext, amax), 3.0517578125e-05f); // 2^-15
        *A.out_margin = s_margin;
        A.node_ref[0] = (A.n == 1) ? (LEAF_BIT | 0u) : 0u;
        s_next = 1;
        s_err = 0;
    }
    __syncthreads();
    const float m = s_margin;
    uint32_t begin = 0, end = 1, depth = 0;
    while(begin < end)
    {
        ++depth;
        if(tid == 0) s_level_end = end;
        __syncthreads();
        for(uint32_t cbase = begin; cbase < end; cbase += COLLAPSE_THREADS)
        {
            uint32_t ni = cbase + tid;
            bool active = ni < end;
            uint32_t slots[8];
            uint32_t ns = 0, nint = 0;
            if(active)
            {
                uint32_t r = A.node_ref[ni];
                if((r & LEAF_BIT) || ref_count(A, r) <= 1u) { slots[ns++] = r; }
                else
                {
                    slots[ns++] = A.left[r];
                    slots[ns++] = A.right[r];
                    while(ns < 8)
                    {
                        int best = -1;
                        float best_area = -1.f;
                        for(uint32_t k = 0; k < ns; ++k)
                        {
                            uint32_t s = slots[k];
                            if((s & LEAF_BIT) || ref_count(A, s) <= A.leaf_max) continue;
                            float a = box_area(A.ibox[s]);
                            if(a > best_area)
                            {
                                best_area = a;
                                best = (int)k;
                            }
                        }
                        if(best < 0) break;
                        uint32_t s = slots[best];
                        slots[best] = A.left[s];
                        slots[ns++] = A.right[s];
                    }
                }
                for(uint32_t k = 0; k < ns; ++k) nint += ref_count(A, slots[k]) > A.leaf_max ? 1u : 0u;
            }
            // block exclusive scan of nint
            uint32_t x = nint;
            for(int o = 1; o < 32; o <<= 1)
            {
                uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
                if(lane >= (uint32_t)o) x += y;
            }
            if(lane == 31) s_warp[warp] = x;
            __syncthreads();
            if(warp == 0)
            {
                uint32_t w = s_warp[lane];
                for(int o = 1; o < 32; o <<= 1)
                {
                    uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
                    if(lane >= (uint32_t)o) w += y;
                }
                s_warp[lane] = w;
            }
            __syncthreads();
            uint32_t prefix = (warp ? s_warp[warp - 1] : 0u) + x - nint;
            uint32_t chunk_total = s_warp[31];
            uint32_t child_base = s_next + prefix;
            if(active)
            {
                node8 nd;
                nd.nchild = (uint8_t)ns;
                box6 gb[8];
                box6 nb;
                for(int a = 0; a < 3; ++a)
                {
                    nb.lo[a] = __int_as_float(0x7f800000);
                    nb.hi[a] = __int_as_float(0xff800000);
                }
                for(uint32_t k = 0; k < 8; ++k)
                {
                    if(k >= ns) break;
                    box6 b = ref_box(A, slots[k]);
                    for(int a = 0; a < 3; ++a)
                    {
                        gb[k].lo[a] = fsub(b.lo[a], m);
                        gb[k].hi[a] = fadd(b.hi[a], m);
                        nb.lo[a] = fminf(nb.lo[a], gb[k].lo[a]);
                        nb.hi[a] = fmaxf(nb.hi[a], gb[k].hi[a]);
                    }
                }
                for(int a = 0; a < 3; ++a)
                {
                    float range = fsub(nb.hi[a], nb.lo[a]);
                    float xq = fdiv(range, 255.0f);
                    uint32_t e = ((__float_as_uint(xq) >> 23) & 0xFFu) + 1u;
                    if(e > 254u) e = 254u;
                    nd.origin[a] = nb.lo[a];
                    nd.exps[a] = (uint8_t)e;
                    float inv_s = exp_scale(254u - e);
                    for(uint32_t k = 0; k < 8; ++k)
                    {
                        uint8_t ql = 0, qh = 0;
                        if(k < ns)
                        {
                            float fl = floorf(fmul(fsub(gb[k].lo[a], nb.lo[a]), inv_s));
                            float fh = ceilf(fmul(fsub(gb[k].hi[a], nb.lo[a]), inv_s));
                            ql = (uint8_t)(fl < 0.f ? 0.f : (fl > 255.f ? 255.f : fl));
                            qh = (uint8_t)(fh < 0.f ? 0.f : (fh > 255.f ? 255.f : fh));
                        }
                        nd.qlo[a][k] = ql;
                        nd.qhi[a][k] = qh;
                    }
                }
                uint32_t c = child_base;
                for(uint32_t k = 0; k < 8; ++k)
                {
                    uint32_t word = 0u;
                    if(k < ns)
                    {
                        uint32_t s = slots[k];
                        uint32_t cnt = ref_count(A, s);
                        if(cnt <= A.leaf_max) { word = LEAF_BIT | ((cnt - 1u) << 27) | ref_first(A, s); }
                        else
                        {
                            if(c < A.capacity) A.node_ref[c] = s;
                            else atomicOr(&s_err, BUILD_ERR_CAPACITY);
                            word = c++;
                        }
                    }
                    nd.child[k] = word;
                }
                A.nodes[ni] = nd;
            }
            __syncthreads();
            if(tid == 0) s_next += chunk_total;
            __syncthreads();
        }
        __threadfence_block();
        __syncthreads();
        begin = end;
        end = s_next;
        if(s_err) break;
        __syncthreads();
    }
    if(tid == 0)
    {
        A.out_info[0] = s_next;
        A.out_info[1] = depth;
        A.out_info[2] = s_err;
    }
}

__global__ void k_tri_records(const float *__restrict__ xyz, uint32_t nv, const uint32_t *__restrict__ idx,
                              const uint32_t *__restrict__ sorted, uint32_t n, tri_rec *__restrict__ out)
{
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= n) return;
    uint32_t p = sorted[i];
    float v[3][3];
    for(int k = 0; k < 3; ++k)
    {
        uint32_t vi = idx[3 * (size_t)p + k];
        if(vi >= nv) vi = 0;
        for(int a = 0; a < 3; ++a) v[k][a] = xyz[3 * (size_t)vi + a];
    }
    tri_rec r;
    for(int a = 0; a < 3; ++a)
    {
        r.v[a] = v[0][a];
        r.v[3 + a] = fsub(v[1][a], v[0][a]);
        r.v[6 + a] = fsub(v[2][a], v[0][a]);
    }
    r.prim = p;
    r.pad[0] = r.pad[1] = 0u;
    out[i] = r;
}

template<typename T>
cudaError_t dalloc(T **p, size_t count, cudaStream_t s)
{
    return cudaMallocAsync(reinterpret_cast<void **>(p), count * sizeof(T) + 16, s);
}

// ---- instances (two-level BVH) -------------------------------------------------------------------
struct blas_box
{
    float lo[3], hi[3];
    uint32_t num_tris, pad;
    const node8 *nodes; // the BLAS's nodes: its upper levels give a tighter instance box than its bounds
};

// child box k of a node, dequantised (the quantised boxes contain their geometry)
__device__ __forceinline__ void node_child_box(const node8 *nd, int k, double lo[3], double hi[3])
{
    const uint32_t *w = reinterpret_cast<const uint32_t *>(nd);
    const float ox = __uint_as_float(w[0]), oy = __uint_as_float(w[1]), oz = __uint_as_float(w[2]);
    const uint32_t meta = w[3];
    const double sx = exp_scale(meta & 0xFFu), sy = exp_scale((meta >> 8) & 0xFFu), sz = exp_scale((meta >> 16) & 0xFFu);
    auto q = [&](int word, int kk) { return (double)((w[word + (kk >> 2)] >> (8 * (kk & 3))) & 0xFFu); };
    // layout (traverse.cuh, node_keys): lo x / y / z in words 4-5 / 6-7 / 8-9, hi x / y / z in 10-11 / 12-13 / 14-15
    lo[0] = ox + q(4, k) * sx;
    lo[1] = oy + q(6, k) * sy;
    lo[2] = oz + q(8, k) * sz;
    hi[0] = ox + q(10, k) * sx;
    hi[1] = oy + q(12, k) * sy;
    hi[2] = oz + q(14, k) * sz;
}

__device__ __forceinline__ void grow_transformed(const float *T, const double lo[3], const double hi[3], double wlo[3],
                                                 double whi[3])
{
    for(int c = 0; c < 8; ++c)
    {
        const double p[3] = {(c & 1) ? hi[0] : lo[0], (c & 2) ? hi[1] : lo[1], (c & 4) ? hi[2] : lo[2]};
        for(int a = 0; a < 3; ++a)
        {
            const double w = (double)T[4 * a] * p[0] + (double)T[4 * a + 1] * p[1] + (double)T[4 * a + 2] * p[2] +
                             (double)T[4 * a + 3];
            wlo[a] = fmin(wlo[a], w);
            whi[a] = fmax(whi[a], w);
        }
    }
}

// world -> object transform of an object -> world 3x4 transform: inverse of the 3x3 part by the
// adjugate in double precision, translation -A^-1 t, rounded to float once. false if singular.
__device__ __forceinline__ bool invert_3x4(const float *m, float *inv)
{
    const double a = m[0], b = m[1], c = m[2], d = m[4], e = m[5], f = m[6], g = m[8], h = m[9], i = m[10];
    const double A = __dsub_rn(__dmul_rn(e, i), __dmul_rn(f, h));
    const double B = __dsub_rn(__dmul_rn(f, g), __dmul_rn(d, i));
    const double C = __dsub_rn(__dmul_rn(d, h), __dmul_rn(e, g));
    const double det = __dadd_rn(__dadd_rn(__dmul_rn(a, A), __dmul_rn(b, B)), __dmul_rn(c, C));
    if(!(fabs(det) > 1e-30) || !isfinite(det)) return false;
    const double r = 1.0 / det;
    const double M[9] = {A, __dsub_rn(__dmul_rn(c, h), __dmul_rn(b, i)), __dsub_rn(__dmul_rn(b, f), __dmul_rn(c, e)),
                         B, __dsub_rn(__dmul_rn(a, i), __dmul_rn(c, g)), __dsub_rn(__dmul_rn(c, d), __dmul_rn(a, f)),
                         C, __dsub_rn(__dmul_rn(b, g), __dmul_rn(a, h)), __dsub_rn(__dmul_rn(a, e), __dmul_rn(b, d))};
    const double t[3] = {m[3], m[7], m[11]};
    for(int row = 0; row < 3; ++row)
    {
        double acc = 0.0;
        for(int k = 0; k < 3; ++k)
        {
            const double v = __dmul_rn(M[3 * row + k], r);
            inv[4 * row + k] = __double2float_rn(v);
            acc = __dadd_rn(acc, __dmul_rn(v, t[k]));
        }
        inv[4 * row + 3] = __double2float_rn(-acc);
    }
    return true;
}

__global__ void k_instance_boxes(const vkg_instance *__restrict__ inst, uint32_t n, const blas_box *__restrict__ bb,
                                 uint32_t nblas, box6 *__restrict__ tbox, uint32_t *__restrict__ scene_enc,
                                 uint32_t *__restrict__ err)
{
    __shared__ uint32_t s_lo[3], s_hi[3];
    if(threadIdx.x < 3)
    {
        s_lo[threadIdx.x] = fenc(__int_as_float(0x7f800000));
        s_hi[threadIdx.x] = fenc(__int_as_float(0xff800000));
    }
    __syncthreads();
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i < n)
    {
        const vkg_instance I = inst[i];
        box6 b;
        uint32_t bl = I.blas;
        if(bl >= nblas)
        {
            atomicOr(err, BUILD_ERR_INDEX);
            bl = 0;
        }
        const blas_box B = bb[bl];
        float inv[12];
        if(!invert_3x4(I.transform, inv)) atomicOr(err, BUILD_ERR_SINGULAR);
        if(B.num_tris == 0)
        {
            // an empty mesh: a point box at the instance origin (the traversal skips it)
            for(int a = 0; a < 3; ++a) b.lo[a] = b.hi[a] = I.transform[4 * a + 3];
        }
        else
        {
            // the union of the transformed boxes two levels below the BLAS root (a rotated mesh's own
            // bounds would be loose: a sphere's rotated bounding cube holds up to 5x its volume)
            double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
            const node8 *root = B.nodes;
            const uint32_t *rw = reinterpret_cast<const uint32_t *>(root);
            const int nch = (int)(rw[3] >> 24);
            for(int k = 0; k < nch; ++k)
            {
                const uint32_t c = rw[16 + k];
                double clo[3], chi[3];
                if(c & LEAF_BIT)
                {
                    node_child_box(root, k, clo, chi);
                    grow_transformed(I.transform, clo, chi, lo, hi);
                    continue;
                }
                const node8 *ch = B.nodes + c;
                const int gch = (int)(reinterpret_cast<const uint32_t *>(ch)[3] >> 24);
                for(int g = 0; g < gch; ++g)
                {
                    node_child_box(ch, g, clo, chi);
                    grow_transformed(I.transform, clo, chi, lo, hi);
                }
            }
            // rounded outward; the collapse grows every box by its margin on top
            for(int a = 0; a < 3; ++a)
            {
                b.lo[a] = __double2float_rd(lo[a]);
                b.hi[a] = __double2float_ru(hi[a]);
            }
        }
        tbox[i] = b;
        for(int a = 0; a < 3; ++a)
        {
            atomicMin(&s_lo[a], fenc(b.lo[a]));
            atomicMax(&s_hi[a], fenc(b.hi[a]));
        }
    }
    __syncthreads();
    if(threadIdx.x < 3)
    {
        atomicMin(&scene_enc[threadIdx.x], s_lo[threadIdx.x]);
        atomicMax(&scene_enc[3 + threadIdx.x], s_hi[threadIdx.x]);
    }
}

// instance records in leaf (sorted) order and in input order
__global__ void k_instance_records(const vkg_instance *__restrict__ inst, const uint32_t *__restrict__ sorted,
                                   uint32_t n, uint32_t nblas, inst_rec *__restrict__ out, inst_rec *__restrict__ by_id)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= n) return;
    const uint32_t id = sorted[i];
    const vkg_instance I = inst[id];
    inst_rec r{};
    if(!invert_3x4(I.transform, r.w2o))
        for(int k = 0; k < 12; ++k) r.w2o[k] = 0.f;
    for(int k = 0; k < 12; ++k) r.o2w[k] = I.transform[k];
    r.blas = I.blas < nblas ? I.blas : 0u;
    r.instance = id;
    r.material = I.material;
    out[i] = r;
    by_id[id] = r;
}

// The primitive-independent part of a build: make_boxes(tbox, scene_enc, err) fills the n primitive
// boxes, the scene box (ordered uints) and error bits; Morton codes, the radix sort, the Karras tree,
// the refit and the 8-wide collapse follow; make_records(sorted) writes the leaf records in sorted
// order. On success bvh holds the nodes, Morton codes, sorted order, scene box, margin and depth, and
// err_bits the error bits that make_boxes raised. The caller frees bvh on failure.
template<class MakeBoxes, class MakeRecords>
vkg_status build_core(vkg_ctx *ctx, vkg_bvh *bvh, uint32_t n, uint32_t leaf_max, cudaStream_t st,
                      MakeBoxes make_boxes, MakeRecords make_records, uint32_t &err_bits)
{
    cudaEvent_t ev0, ev1;
    cudaEventCreate(&ev0);
    cudaEventCreate(&ev1);
    cudaEventRecord(ev0, st);

    // scratch
    box6 *tbox = nullptr, *lbox = nullptr, *ibox = nullptr;
    uint32_t *keys0 = nullptr, *keys1 = nullptr, *vals0 = nullptr, *vals1 = nullptr, *counts = nullptr;
    uint32_t *left = nullptr, *right = nullptr, *first = nullptr, *last = nullptr, *iparent = nullptr,
             *lparent = nullptr, *visits = nullptr, *node_ref = nullptr, *small = nullptr;
    node8 *nodes_tmp = nullptr;
    float *d_margin = nullptr;
    const uint32_t nblocks = (n + SORT_TILE - 1) / SORT_TILE;
    const uint32_t ni = n > 1 ? n - 1 : 1;
    const uint32_t capacity = n + 8;
    cudaError_t e = cudaSuccess;
    auto chk = [&](cudaError_t x) {
        if(e == cudaSuccess) e = x;
    };
    chk(dalloc(&tbox, n, st));
    chk(dalloc(&lbox, n, st));
    chk(dalloc(&ibox, ni, st));
    chk(dalloc(&keys0, n, st));
    chk(dalloc(&keys1, n, st));
    chk(dalloc(&vals0, n, st));
    chk(dalloc(&vals1, n, st));
    chk(dalloc(&counts, (size_t)256 * nblocks, st));
    chk(dalloc(&left, ni, st));
    chk(dalloc(&right, ni, st));
    chk(dalloc(&first, ni, st));
    chk(dalloc(&last, ni, st));
    chk(dalloc(&iparent, ni, st));
    chk(dalloc(&lparent, n, st));
    chk(dalloc(&visits, ni, st));
    chk(dalloc(&node_ref, capacity, st));
    chk(dalloc(&nodes_tmp, capacity, st));
    chk(dalloc(&small, 16, st));
    chk(dalloc(&d_margin, 1, st));
    chk(dalloc(&bvh->d_morton, n, st));
    chk(dalloc(&bvh->d_sorted, n, st));
    if(e != cudaSuccess)
        return set_error(ctx, VKG_ERR_OUT_OF_MEMORY, "BVH build: device allocation failed (%s)", cudaGetErrorString(e));
    // small[0..5] scene box (ordered uints), [6] error flags, [8..10] collapse info
    uint32_t init[16] = {0xFF800000u, 0xFF800000u, 0xFF800000u, 0x007FFFFFu, 0x007FFFFFu, 0x007FFFFFu, 0, 0,
                         0,           0,           0,           0,           0,           0,           0, 0};
    // +inf encodes as 0xFF800000, -inf as 0x007FFFFF
    chk(cudaMemcpyAsync(small, init, sizeof(init), cudaMemcpyHostToDevice, st));
    chk(cudaMemsetAsync(visits, 0, sizeof(uint32_t) * ni, st));

    const int T = 256;
    const uint32_t g = (n + T - 1) / T;
    make_boxes(tbox, small, small + 6);
    k_morton<<<g, T, 0, st>>>(tbox, n, small, keys0, vals0, bvh->d_morton);
    uint32_t *kin = keys0, *kout = keys1, *vin = vals0, *vout = vals1;
    for(int shift = 0; shift < 30; shift += 8)
    {
        k_radix_hist<<<nblocks, SORT_THREADS, 0, st>>>(kin, n, shift, counts, nblocks);
        k_scan_exclusive<<<1, 1024, 0, st>>>(counts, 256u * nblocks, nullptr);
        k_radix_scatter<<<nblocks, SORT_THREADS, 0, st>>>(kin, vin, n, shift, counts, nblocks, kout, vout);
        std::swap(kin, kout);
        std::swap(vin, vout);
    }
    chk(cudaMemcpyAsync(bvh->d_sorted, vin, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, st));
    k_gather_leaf_boxes<<<g, T, 0, st>>>(tbox, vin, n, lbox);
    if(n > 1)
    {
        k_karras<<<(ni + T - 1) / T, T, 0, st>>>(kin, n, left, right, first, last, iparent, lparent);
        k_refit<<<g, T, 0, st>>>(lparent, iparent, left, right, lbox, ibox, visits, n);
    }
    collapse_args A{left, right, first, last, ibox, lbox, n, leaf_max, capacity, small, node_ref, nodes_tmp,
                    small + 8, d_margin};
    k_collapse<<<1, COLLAPSE_THREADS, 0, st>>>(A);
    make_records(static_cast<const uint32_t *>(vin));
    chk(cudaGetLastError());

    uint32_t info[16];
    float margin = 0.f;
    chk(cudaMemcpyAsync(info, small, sizeof(info), cudaMemcpyDeviceToHost, st));
    chk(cudaMemcpyAsync(&margin, d_margin, sizeof(float), cudaMemcpyDeviceToHost, st));
    chk(cudaStreamSynchronize(st));
    if(e == cudaSuccess)
    {
        bvh->num_nodes = info[8];
        bvh->depth = info[9];
        bvh->margin = margin;
        for(int a = 0; a < 3; ++a)
        {
            uint32_t lo = info[a], hi = info[3 + a];
            uint32_t lb = (lo & 0x80000000u) ? (lo & 0x7FFFFFFFu) : ~lo;
            uint32_t hb = (hi & 0x80000000u) ? (hi & 0x7FFFFFFFu) : ~hi;
            std::memcpy(&bvh->scene_min[a], &lb, 4);
            std::memcpy(&bvh->scene_max[a], &hb, 4);
        }
        chk(dalloc(&bvh->d_nodes, bvh->num_nodes, st));
        if(e == cudaSuccess)
            chk(cudaMemcpyAsync(bvh->d_nodes, nodes_tmp, sizeof(node8) * bvh->num_nodes, cudaMemcpyDeviceToDevice,
                                st));
    }
    for(void *p: {(void *)tbox, (void *)lbox, (void *)ibox, (void *)keys0, (void *)keys1, (void *)vals0,
                  (void *)vals1, (void *)counts, (void *)left, (void *)right, (void *)first, (void *)last,
                  (void *)iparent, (void *)lparent, (void *)visits, (void *)node_ref, (void *)nodes_tmp,
                  (void *)small, (void *)d_margin})
        cudaFreeAsync(p, st);
    cudaEventRecord(ev1, st);
    chk(cudaEventSynchronize(ev1));
    cudaEventElapsedTime(&bvh->build_ms, ev0, ev1);
    cudaEventDestroy(ev0);
    cudaEventDestroy(ev1);
    if(e != cudaSuccess) return cuda_check(ctx, e, "BVH build");
    err_bits = info[6];
    if(info[10] & BUILD_ERR_CAPACITY) return set_error(ctx, VKG_ERR_CAPACITY, "BVH build: node capacity exceeded");
    const uint32_t max_depth = (TRAVERSAL_STACK - 1) / 7 + 1;
    if(bvh->depth > max_depth)
        return set_error(ctx, VKG_ERR_CAPACITY, "BVH build: depth %u exceeds the traversal limit %u", bvh->depth,
                         max_depth);
    return VKG_OK;
}

}// namespace
}// namespace vkg

using namespace vkg;

extern "C" vkg_status vkg_bvh_build(vkg_ctx *ctx, const float *d_xyz, uint32_t num_vertices,
                                    const uint32_t *d_indices, uint32_t num_tris, const vkg_bvh_build_options *opts,
                                    vkg_bvh **out, void *stream_)
{
    if(!ctx) return VKG_ERR_INVALID_ARGUMENT;
    if(!out) return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_bvh_build: out is NULL");
    *out = nullptr;
    if(num_tris > 0 && (!d_xyz || !d_indices || num_vertices == 0))
        return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_bvh_build: NULL geometry for %u triangles", num_tris);
    if(num_tris >= MAX_TRIS)
        return set_error(ctx, VKG_ERR_CAPACITY, "vkg_bvh_build: %u triangles exceed the maximum of %u", num_tris,
                         MAX_TRIS - 1);
    uint32_t leaf_max = (opts && opts->leaf_max) ? opts->leaf_max : 2u;
    if(leaf_max > LEAF_MAX_LIMIT)
        return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_bvh_build: leaf_max %u > %u", leaf_max, LEAF_MAX_LIMIT);
    if(vkg_status s = bind_device(ctx); s != VKG_OK) return s;

    cudaStream_t st = static_cast<cudaStream_t>(stream_);
    auto *bvh = new vkg_bvh();
    bvh->num_tris = num_tris;
    bvh->leaf_max = leaf_max;
    if(num_tris == 0)
    {
        *out = bvh;
        return VKG_OK;
    }
    const uint32_t n = num_tris;
    if(cudaMallocAsync(reinterpret_cast<void **>(&bvh->d_tris), n * sizeof(tri_rec) + 16, st) != cudaSuccess)
    {
        vkg_bvh_destroy(ctx, bvh);
        return set_error(ctx, VKG_ERR_OUT_OF_MEMORY, "vkg_bvh_build: device allocation failed");
    }
    const int T = 256;
    const uint32_t g = (n + T - 1) / T;
    uint32_t err_bits = 0;
    vkg_status s = build_core(
            ctx, bvh, n, leaf_max, st,
            [&](box6 *tbox, uint32_t *scene_enc, uint32_t *err) {
                k_tri_boxes<<<g, T, 0, st>>>(d_xyz, num_vertices, d_indices, n, tbox, scene_enc, err);
            },
            [&](const uint32_t *sorted) {
                k_tri_records<<<g, T, 0, st>>>(d_xyz, num_vertices, d_indices, sorted, n, bvh->d_tris);
            },
            err_bits);
    if(s == VKG_OK && (err_bits & BUILD_ERR_INDEX))
        s = set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_bvh_build: triangle index >= num_vertices (%u)", num_vertices);
    if(s != VKG_OK)
    {
        vkg_bvh_destroy(ctx, bvh);
        return s;
    }
    bvh->bytes = sizeof(node8) * bvh->num_nodes + sizeof(tri_rec) * n + 8 * (size_t)n;
    *out = bvh;
    return VKG_OK;
}

extern "C" vkg_status vkg_bvh_info_get(const vkg_bvh *bvh, vkg_bvh_info *out)
{
    if(!bvh || !out) return VKG_ERR_INVALID_ARGUMENT;
    std::memset(out, 0, sizeof(*out));
    out->num_tris = bvh->num_tris;
    out->num_nodes = bvh->num_nodes;
    out->depth = bvh->depth;
    out->leaf_max = bvh->leaf_max;
    for(int a = 0; a < 3; ++a)
    {
        out->scene_min[a] = bvh->scene_min[a];
        out->scene_max[a] = bvh->scene_max[a];
    }
    out->margin = bvh->margin;
    out->bytes = bvh->bytes;
    out->d_nodes = bvh->d_nodes;
    out->d_tris = bvh->d_tris;
    out->d_morton = bvh->d_morton;
    out->d_sorted = bvh->d_sorted;
    out->build_ms = bvh->build_ms;
    return VKG_OK;
}

extern "C" vkg_status vkg_bvh_destroy(vkg_ctx *ctx, vkg_bvh *bvh)
{
    if(!bvh) return VKG_OK;
    if(ctx) bind_device(ctx);
    cudaFree(bvh->d_nodes);
    cudaFree(bvh->d_tris);
    cudaFree(bvh->d_morton);
    cudaFree(bvh->d_sorted);
    delete bvh;
    return VKG_OK;
}

// ---- two-level BVH -----------------------------------------------------------------------------
// The top level is the same 8-wide quantised BVH, built by the same core over the instances' world
// boxes (the 8 transformed corners of the mesh's bounds, rounded outward); its leaves index
// 128-byte instance records (world <-> object transforms, BLAS, input index, material). Mirrors
// RayBuilder::create_toplevel (RayBuilder.cpp:386-760), which builds the driver TLAS over entries
// carrying a vk_transform_matrix (:518).
extern "C" vkg_status vkg_tlas_build(vkg_ctx *ctx, const vkg_bvh *const *blas, uint32_t num_blas,
                                     const vkg_instance *d_instances, uint32_t num_instances,
                                     const vkg_bvh_build_options *opts, vkg_tlas **out, void *stream_)
{
    if(!ctx) return VKG_ERR_INVALID_ARGUMENT;
    if(!out) return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_tlas_build: out is NULL");
    *out = nullptr;
    if(num_instances > 0 && (!d_instances || !blas || num_blas == 0))
        return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_tlas_build: NULL instances or BLAS array");
    for(uint32_t b = 0; b < num_blas; ++b)
        if(!blas[b]) return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_tlas_build: BLAS %u is NULL", b);
    if(num_instances >= MAX_TRIS)
        return set_error(ctx, VKG_ERR_CAPACITY, "vkg_tlas_build: %u instances exceed the maximum", num_instances);
    const uint32_t leaf_max = (opts && opts->leaf_max) ? opts->leaf_max : 2u;
    if(leaf_max > LEAF_MAX_LIMIT)
        return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_tlas_build: leaf_max %u > %u", leaf_max, LEAF_MAX_LIMIT);
    if(vkg_status s = bind_device(ctx); s != VKG_OK) return s;
    cudaStream_t st = static_cast<cudaStream_t>(stream_);
    auto *t = new vkg_tlas();
    t->num_instances = num_instances;
    t->num_blas = num_blas;
    t->top.leaf_max = leaf_max;
    std::vector<blas_ref> refs(num_blas);
    std::vector<blas_box> boxes(num_blas);
    for(uint32_t b = 0; b < num_blas; ++b)
    {
        refs[b] = blas_ref{blas[b]->d_nodes, blas[b]->d_tris, blas[b]->num_tris, 0u};
        for(int a = 0; a < 3; ++a)
        {
            boxes[b].lo[a] = blas[b]->scene_min[a];
            boxes[b].hi[a] = blas[b]->scene_max[a];
        }
        boxes[b].num_tris = blas[b]->num_tris;
        boxes[b].nodes = blas[b]->d_nodes;
    }
    blas_box *d_bb = nullptr;
    cudaError_t e = cudaSuccess;
    if(num_blas)
    {
        e = cudaMalloc(&t->d_blas, num_blas * sizeof(blas_ref));
        if(e == cudaSuccess) e = cudaMalloc(&d_bb, num_blas * sizeof(blas_box));
        if(e == cudaSuccess)
            e = cudaMemcpyAsync(t->d_blas, refs.data(), num_blas * sizeof(blas_ref), cudaMemcpyHostToDevice, st);
        if(e == cudaSuccess) e = cudaMemcpyAsync(d_bb, boxes.data(), num_blas * sizeof(blas_box), cudaMemcpyHostToDevice, st);
    }
    if(e == cudaSuccess && num_instances)
    {
        e = cudaMalloc(&t->d_inst, num_instances * sizeof(inst_rec));
        if(e == cudaSuccess) e = cudaMalloc(&t->d_inst_by_id, num_instances * sizeof(inst_rec));
    }
    if(e != cudaSuccess)
    {
        cudaFree(d_bb);
        vkg_tlas_destroy(ctx, t);
        return cuda_check(ctx, e, "vkg_tlas_build");
    }
    if(num_instances == 0)
    {
        cudaStreamSynchronize(st);
        cudaFree(d_bb);
        *out = t;
        return VKG_OK;
    }
    const uint32_t n = num_instances;
    const int T = 256;
    const uint32_t g = (n + T - 1) / T;
    uint32_t err_bits = 0;
    vkg_status s = build_core(
            ctx, &t->top, n, leaf_max, st,
            [&](box6 *tbox, uint32_t *scene_enc, uint32_t *err) {
                k_instance_boxes<<<g, T, 0, st>>>(d_instances, n, d_bb, num_blas, tbox, scene_enc, err);
            },
            [&](const uint32_t *sorted) {
                k_instance_records<<<g, T, 0, st>>>(d_instances, sorted, n, num_blas, t->d_inst, t->d_inst_by_id);
            },
            err_bits);
    cudaFree(d_bb);
    t->top.num_tris = n;
    if(s == VKG_OK && (err_bits & BUILD_ERR_INDEX))
        s = set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_tlas_build: an instance's BLAS index >= %u", num_blas);
    if(s == VKG_OK && (err_bits & BUILD_ERR_SINGULAR))
        s = set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_tlas_build: an instance transform is singular");
    if(s == VKG_OK && t->top.depth > TLAS_MAX_DEPTH)
        s = set_error(ctx, VKG_ERR_CAPACITY, "vkg_tlas_build: top-level depth %u exceeds %u", t->top.depth, TLAS_MAX_DEPTH);
    if(s != VKG_OK)
    {
        vkg_tlas_destroy(ctx, t);
        return s;
    }
    t->top.bytes = sizeof(node8) * t->top.num_nodes + 2 * sizeof(inst_rec) * (size_t)n;
    *out = t;
    return VKG_OK;
}

extern "C" vkg_status vkg_tlas_info_get(const vkg_tlas *t, vkg_tlas_info *out)
{
    if(!t || !out) return VKG_ERR_INVALID_ARGUMENT;
    std::memset(out, 0, sizeof(*out));
    out->num_instances = t->num_instances;
    out->num_blas = t->num_blas;
    out->num_nodes = t->top.num_nodes;
    out->depth = t->top.depth;
    for(int a = 0; a < 3; ++a)
    {
        out->scene_min[a] = t->top.scene_min[a];
        out->scene_max[a] = t->top.scene_max[a];
    }
    out->d_nodes = t->top.d_nodes;
    out->d_instances = t->d_inst;
    out->d_instances_by_id = t->d_inst_by_id;
    out->build_ms = t->top.build_ms;
    return VKG_OK;
}

extern "C" vkg_status vkg_tlas_destroy(vkg_ctx *ctx, vkg_tlas *t)
{
    if(!t) return VKG_OK;
    if(ctx) bind_device(ctx);
    cudaFree(t->top.d_nodes);
    cudaFree(t->top.d_morton);
    cudaFree(t->top.d_sorted);
    cudaFree(t->d_inst);
    cudaFree(t->d_inst_by_id);
    cudaFree(t->d_blas);
    delete t;
    return VKG_OK;
}

// ---- allocation-free build ----------------------------------------------------------------------
// For callers that cannot allocate device memory after start-up (for example an engine that
// sub-allocates everything from one arena it received at initialisation, or code recording work
// that must not synchronise): the build's temporaries live in one file-scope device array of fixed
// size, so the call itself performs no allocation. The caller passes the inputs and the output
// buffers (nodes, triangle records, info words).
namespace vkg
{
namespace
{

constexpr uint32_t NOALLOC_MAX_TRIS = 16384;
constexpr uint32_t NOALLOC_SORT_BLOCKS = (NOALLOC_MAX_TRIS + SORT_TILE - 1) / SORT_TILE;

struct noalloc_scratch
{
    box6 tbox[NOALLOC_MAX_TRIS], lbox[NOALLOC_MAX_TRIS], ibox[NOALLOC_MAX_TRIS];
    uint32_t keys0[NOALLOC_MAX_TRIS], keys1[NOALLOC_MAX_TRIS], vals0[NOALLOC_MAX_TRIS], vals1[NOALLOC_MAX_TRIS];
    uint32_t counts[256 * NOALLOC_SORT_BLOCKS];
    uint32_t left[NOALLOC_MAX_TRIS], right[NOALLOC_MAX_TRIS], first[NOALLOC_MAX_TRIS], last[NOALLOC_MAX_TRIS];
    uint32_t iparent[NOALLOC_MAX_TRIS], lparent[NOALLOC_MAX_TRIS], visits[NOALLOC_MAX_TRIS];
    uint32_t node_ref[NOALLOC_MAX_TRIS + 8];
    uint32_t morton[NOALLOC_MAX_TRIS];
    uint32_t small[16];
    float margin[4];
};

// ~2.2 MB, held by every GPU that loads libvkg until the process exits. Host code must not use the
// symbol's host-side name as a device address: the address comes from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_noalloc_scratch[sizeof(noalloc_scratch)];

std::mutex g_noalloc_mutex;
void *g_noalloc_ptr[128] = {};

// per device, on first use, with that device current
vkg_status noalloc_scratch_for_current_device(noalloc_scratch **out)
{
    int dev = -1;
    if(cudaGetDevice(&dev) != cudaSuccess) return VKG_ERR_CUDA;
    if(dev < 0 || dev >= 128) return VKG_ERR_NOT_SUPPORTED;
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if(!g_noalloc_ptr[dev])
    {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if(e != cudaSuccess || p == nullptr) return VKG_ERR_CUDA;
        g_noalloc_ptr[dev] = p;
    }
    *out = static_cast<noalloc_scratch *>(g_noalloc_ptr[dev]);
    return VKG_OK;
}

// the scratch keeps the previous call's contents: reset what the build expects to start at zero
__global__ void k_noalloc_reset(noalloc_scratch *s, uint32_t n)
{
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i < n) s->visits[i] = 0u;
    if(i < 16)
    {
        const uint32_t init = i < 3 ? 0xFF800000u : (i < 6 ? 0x007FFFFFu : 0u); // +inf / -inf encodings, flags
        s->small[i] = init;
    }
    if(i == 0) s->margin[0] = 0.f;
}

// info words: [0] nodes, [1] depth, [2] error flags (1 = index >= num_vertices, 2 = node capacity),
// [3] margin (float bits), [4..6] scene min, [7..9] scene max (float bits)
constexpr uint32_t NOALLOC_FLAG_DEPTH = 4u;

__global__ void k_noalloc_info(const noalloc_scratch *s, uint32_t n, uint32_t *info)
{
    if(threadIdx.x != 0 || blockIdx.x != 0) return;
    for(int k = 0; k < 16; ++k) info[k] = 0u;
    if(n == 0) return;
    info[0] = s->small[8];
    info[1] = s->small[9];
    info[2] = s->small[10] | s->small[6];
    // deeper than the traversal stack supports (the limit vkg_bvh_build enforces)
    if(s->small[9] > (TRAVERSAL_STACK - 1) / 7 + 1) info[2] |= NOALLOC_FLAG_DEPTH;
    info[3] = __float_as_uint(s->margin[0]);
    for(int a = 0; a < 3; ++a)
    {
        info[4 + a] = __float_as_uint(fdec(s->small[a]));
        info[7 + a] = __float_as_uint(fdec(s->small[3 + a]));
    }
}

}// namespace
}// namespace vkg

extern "C" vkg_status vkg_bvh_build_noalloc(const float *d_xyz, uint32_t num_vertices, const uint32_t *d_indices,
                                            uint32_t num_tris, uint32_t leaf_max, void *d_nodes,
                                            uint32_t node_capacity, void *d_tris, uint32_t *d_info, void *stream_)
{
    if(num_tris > NOALLOC_MAX_TRIS) return VKG_ERR_CAPACITY;
    if(!d_info) return VKG_ERR_INVALID_ARGUMENT;
    if(leaf_max == 0) leaf_max = 2u;
    if(leaf_max > LEAF_MAX_LIMIT) return VKG_ERR_INVALID_ARGUMENT;
    if(num_tris > 0 && (!d_xyz || !d_indices || num_vertices == 0 || !d_nodes || !d_tris)) return VKG_ERR_INVALID_ARGUMENT;
    if(num_tris > 0 && node_capacity < num_tris) return VKG_ERR_INVALID_ARGUMENT;
    if((reinterpret_cast<uintptr_t>(d_nodes) & 15u) || (reinterpret_cast<uintptr_t>(d_tris) & 15u))
        return VKG_ERR_INVALID_ARGUMENT;
    cudaStream_t st = static_cast<cudaStream_t>(stream_);
    noalloc_scratch *s = nullptr;
    if(vkg_status r = noalloc_scratch_for_current_device(&s); r != VKG_OK) return r;
    const uint32_t n = num_tris;
    if(n == 0)
    {
        k_noalloc_info<<<1, 1, 0, st>>>(s, 0, d_info);
        return cudaGetLastError() == cudaSuccess ? VKG_OK : VKG_ERR_CUDA;
    }
    const int T = 256;
    const uint32_t g = (n + T - 1) / T;
    const uint32_t nblocks = (n + SORT_TILE - 1) / SORT_TILE;
    k_noalloc_reset<<<(n + 15 + T - 1) / T, T, 0, st>>>(s, n);
    k_tri_boxes<<<g, T, 0, st>>>(d_xyz, num_vertices, d_indices, n, s->tbox, s->small, s->small + 6);
    k_morton<<<g, T, 0, st>>>(s->tbox, n, s->small, s->keys0, s->vals0, s->morton);
    uint32_t *kin = s->keys0, *kout = s->keys1, *vin = s->vals0, *vout = s->vals1;
    for(int shift = 0; shift < 30; shift += 8)
    {
        k_radix_hist<<<nblocks, SORT_THREADS, 0, st>>>(kin, n, shift, s->counts, nblocks);
        k_scan_exclusive<<<1, 1024, 0, st>>>(s->counts, 256u * nblocks, nullptr);
        k_radix_scatter<<<nblocks, SORT_THREADS, 0, st>>>(kin, vin, n, shift, s->counts, nblocks, kout, vout);
        std::swap(kin, kout);
        std::swap(vin, vout);
    }
    k_gather_leaf_boxes<<<g, T, 0, st>>>(s->tbox, vin, n, s->lbox);
    if(n > 1)
    {
        k_karras<<<(n - 1 + T - 1) / T, T, 0, st>>>(kin, n, s->left, s->right, s->first, s->last, s->iparent,
                                                      s->lparent);
        k_refit<<<g, T, 0, st>>>(s->lparent, s->iparent, s->left, s->right, s->lbox, s->ibox, s->visits, n);
    }
    const uint32_t capacity = std::min<uint32_t>(node_capacity, NOALLOC_MAX_TRIS + 8);
    collapse_args A{s->left, s->right, s->first, s->last, s->ibox, s->lbox, n, leaf_max, capacity, s->small,
                    s->node_ref, static_cast<node8 *>(d_nodes), s->small + 8, s->margin};
    k_collapse<<<1, COLLAPSE_THREADS, 0, st>>>(A);
    k_tri_records<<<g, T, 0, st>>>(d_xyz, num_vertices, d_indices, vin, n, static_cast<tri_rec *>(d_tris));
    k_noalloc_info<<<1, 1, 0, st>>>(s, n, d_info);
    return cudaGetLastError() == cudaSuccess ? VKG_OK : VKG_ERR_CUDA;
}
