// Environment map and its importance-sampling tables (not in the reference: vierkant only looks
// the environment up when a BSDF-sampled ray misses, shaders/slang/raypipeline.slang:747-781).
//
// Mapping: equirectangular, u = 0.5 + 0.5 * atan2(x, -z) / pi, v = acos(y) / pi
// (shaders/slang/unlit/panorama.slang:12-15); radiance is piecewise constant per texel.
//
// Sampling distribution: texel weight = luminance * sin(theta at the texel centre). The weights
// are summed with FP64 prefix sums on the GPU (the only FP64 arithmetic of the library) and turned
// into a Walker alias table whose buckets are all computed in parallel:
//   normalised weights w (mean 1) split into light (w < 1) and heavy (w >= 1) texels, in index
//   order; D = exclusive FP64 prefix sum of light deficits (1 - w), E = exclusive FP64 prefix sum
//   of heavy excesses (w - 1). A sequential sweep that fills each light bucket from the current
//   heavy texel and turns a heavy texel into a bucket of its own once its excess is used up yields:
//     light k:  prob = w, alias = heavy m with m = min{m : E[m+1] >= D[k]}
//     heavy m:  i = min{i : D[i+1] > E[m+1]}; prob = 1 + E[m+1] - D[i+1], alias = heavy m+1
//               (prob 1, alias itself when no such light exists or m is the last heavy)
//   which every thread evaluates with two binary searches. Every texel's total probability is
//   exactly its normalised weight (the excess of heavy m is consumed by the lights whose deficit
//   intervals start inside it plus the next heavy's overshoot).
// Solid-angle pdf of a direction in texel t: w_t / (2 pi^2 sin(theta)).
#include "internal.hpp"
#include "pathtrace.cuh"

#include <cstring>

namespace vkg
{
namespace
{

constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 8;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

template<typename T>
__device__ __forceinline__ T block_exclusive_scan(T v, T *smem, T &total)
{
    // smem: SCAN_THREADS entries; fixed summation tree -> deterministic
    const int tid = threadIdx.x;
    smem[tid] = v;
    __syncthreads();
    for(int o = 1; o < SCAN_THREADS; o <<= 1)
    {
        T add = tid >= o ? smem[tid - o] : T(0);
        __syncthreads();
        smem[tid] += add;
        __syncthreads();
    }
    total = smem[SCAN_THREADS - 1];
    T incl = smem[tid];
    __syncthreads();
    return incl - v;
}

// phase 1: per-tile sums
template<typename T>
__global__ void k_scan_tile_sums(const T *__restrict__ in, size_t n, T *__restrict__ sums)
{
    __shared__ T smem[SCAN_THREADS];
    size_t base = (size_t)blockIdx.x * SCAN_TILE + (size_t)threadIdx.x * SCAN_ITEMS;
    T s = T(0);
    for(int k = 0; k < SCAN_ITEMS; ++k)
        if(base + k < n) s += in[base + k];
    T total;
    block_exclusive_scan<T>(s, smem, total);
    if(threadIdx.x == 0) sums[blockIdx.x] = total;
}

// phase 2: exclusive scan of the tile sums (one CTA, sequential over chunks)
template<typename T>
__global__ void k_scan_sums(T *__restrict__ sums, size_t n, T *__restrict__ total_out)
{
    __shared__ T smem[SCAN_THREADS];
    __shared__ T carry;
    if(threadIdx.x == 0) carry = T(0);
    __syncthreads();
    for(size_t base = 0; base < n; base += SCAN_THREADS)
    {
        size_t i = base + threadIdx.x;
        T v = i < n ? sums[i] : T(0);
        T total;
        T ex = block_exclusive_scan<T>(v, smem, total);
        T c = carry;
        if(i < n) sums[i] = c + ex;
        __syncthreads();
        if(threadIdx.x == 0) carry = c + total;
        __syncthreads();
    }
    if(threadIdx.x == 0 && total_out) *total_out = carry;
}

// phase 3: tile-local exclusive scan + tile offset; out may alias in
template<typename T>
__global__ void k_scan_apply(const T *in, size_t n, const T *__restrict__ sums, T *out)
{
    __shared__ T smem[SCAN_THREADS];
    size_t base = (size_t)blockIdx.x * SCAN_TILE + (size_t)threadIdx.x * SCAN_ITEMS;
    T v[SCAN_ITEMS];
    T s = T(0);
    for(int k = 0; k < SCAN_ITEMS; ++k)
    {
        v[k] = base + k < n ? in[base + k] : T(0);
        s += v[k];
    }
    T total;
    T run = block_exclusive_scan<T>(s, smem, total) + sums[blockIdx.x];
    for(int k = 0; k < SCAN_ITEMS; ++k)
    {
        if(base + k < n) out[base + k] = run;
        run += v[k];
    }
}

template<typename T>
cudaError_t exclusive_scan(const T *in, T *out, size_t n, T *tile_sums, T *total, cudaStream_t st)
{
    size_t tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
    if(tiles == 0) tiles = 1;
    k_scan_tile_sums<T><<<(unsigned)tiles, SCAN_THREADS, 0, st>>>(in, n, tile_sums);
    k_scan_sums<T><<<1, SCAN_THREADS, 0, st>>>(tile_sums, tiles, total);
    k_scan_apply<T><<<(unsigned)tiles, SCAN_THREADS, 0, st>>>(in, n, tile_sums, out);
    return cudaGetLastError();
}

__global__ void k_env_procedural(uint32_t w, uint32_t h, float sx, float sy, float sz, float peak, float width,
                                 float *__restrict__ rgb)
{
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if(t >= w * h) return;
    uint32_t i = t % w, j = t / w;
    float3 d = env_texel_dir(i, j, w, h);
    float3 c = environment_white(d);
    // cos(g) - 1 = -|d - s|^2 / 2 for unit vectors: no cancellation near the lobe centre
    float ex = d.x - sx, ey = d.y - sy, ez = d.z - sz;
    float sun = peak * expf(-0.5f * (ex * ex + ey * ey + ez * ez) / width);
    rgb[3 * (size_t)t + 0] = c.x + sun;
    rgb[3 * (size_t)t + 1] = c.y + sun;
    rgb[3 * (size_t)t + 2] = c.z + sun;
}

__global__ void k_env_weights(const float *__restrict__ rgb, uint32_t w, uint32_t h, double *__restrict__ wt)
{
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if(t >= w * h) return;
    uint32_t j = t / w;
    double theta = ((double)j + 0.5) * 3.14159265358979323846 / (double)h;
    const float *c = rgb + 3 * (size_t)t;
    double lum = 0.2126 * (double)c[0] + 0.7152 * (double)c[1] + 0.0722 * (double)c[2];
    wt[t] = lum > 0.0 ? lum * sin(theta) : 0.0;
}

// normalised weights (mean 1), light/heavy flags
__global__ void k_env_normalise(const double *__restrict__ wt, uint32_t n, const double *__restrict__ total,
                                double *__restrict__ wn, float *__restrict__ pdf_w, uint32_t *__restrict__ light)
{
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if(t >= n) return;
    double s = *total;
    double v = s > 0.0 ? wt[t] * (double)n / s : 1.0;
    wn[t] = v;
    pdf_w[t] = (float)v;
    light[t] = v < 1.0 ? 1u : 0u;
}

__global__ void k_env_partition(const double *__restrict__ wn, const uint32_t *__restrict__ light,
                                const uint32_t *__restrict__ light_rank, uint32_t n, uint32_t *__restrict__ lights,
                                uint32_t *__restrict__ heavies, double *__restrict__ deficit,
                                double *__restrict__ excess)
{
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if(t >= n) return;
    uint32_t lr = light_rank[t];
    if(light[t])
    {
        lights[lr] = t;
        deficit[lr] = 1.0 - wn[t];
    }
    else
    {
        uint32_t hr = t - lr;
        heavies[hr] = t;
        excess[hr] = wn[t] - 1.0;
    }
}

__device__ __forceinline__ uint32_t lower_bound_d(const double *a, uint32_t n, double x)
{
    uint32_t lo = 0, hi = n;
    while(lo < hi)
    {
        uint32_t mid = (lo + hi) >> 1;
        if(a[mid] < x) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}
__device__ __forceinline__ uint32_t upper_bound_d(const double *a, uint32_t n, double x)
{
    uint32_t lo = 0, hi = n;
    while(lo < hi)
    {
        uint32_t mid = (lo + hi) >> 1;
        if(a[mid] <= x) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// D[0..nL] / E[0..nH]: exclusive prefix sums with the total appended
__global__ void k_alias_lights(const uint32_t *__restrict__ lights, const uint32_t *__restrict__ heavies,
                               const double *__restrict__ wn, const double *__restrict__ D,
                               const double *__restrict__ E, const uint32_t *__restrict__ counts,
                               env_alias *__restrict__ table)
{
    const uint32_t nL = counts[0], nH = counts[1];
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if(k >= nL || nH == 0) return;
    uint32_t t = lights[k];
    uint32_t m = lower_bound_d(E + 1, nH, D[k]);
    if(m >= nH) m = nH - 1;
    float p = (float)wn[t];
    table[t] = env_alias{fminf(fmaxf(p, 0.f), 1.f), heavies[m]};
}

__global__ void k_alias_heavies(const uint32_t *__restrict__ heavies, const double *__restrict__ D,
                                const double *__restrict__ E, const uint32_t *__restrict__ counts,
                                env_alias *__restrict__ table)
{
    const uint32_t nL = counts[0], nH = counts[1];
    uint32_t m = blockIdx.x * blockDim.x + threadIdx.x;
    if(m >= nH) return;
    uint32_t t = heavies[m];
    double e_incl = E[m + 1];
    uint32_t i = upper_bound_d(D + 1, nL, e_incl);
    env_alias a{1.f, t};
    if(i < nL && m + 1 < nH)
    {
        double p = 1.0 + e_incl - D[i + 1];
        a.prob = (float)fmin(fmax(p, 0.0), 1.0);
        a.alias = heavies[m + 1];
    }
    table[t] = a;
}

__global__ void k_counts_from_ranks(const uint32_t *__restrict__ light, const uint32_t *__restrict__ rank, uint32_t n,
                                    uint32_t *__restrict__ counts)
{
    uint32_t nl = rank[n - 1] + light[n - 1];
    counts[0] = nl;
    counts[1] = n - nl;
}

}// namespace

vkg_status env_build(vkg_ctx *ctx, const float *d_rgb_in, uint32_t w, uint32_t h, env_tables &out, cudaStream_t st)
{
    const size_t n = (size_t)w * h;
    out.w = w;
    out.h = h;
    cudaError_t e = cudaSuccess;
    auto chk = [&](cudaError_t x) {
        if(e == cudaSuccess) e = x;
    };
    chk(cudaMalloc(&out.rgb, n * 3 * sizeof(float)));
    chk(cudaMalloc(&out.pdf_w, n * sizeof(float)));
    chk(cudaMalloc(&out.alias, n * sizeof(env_alias)));
    double *wt = nullptr, *wn = nullptr, *dl = nullptr, *eh = nullptr, *dsums = nullptr, *dtot = nullptr;
    uint32_t *light = nullptr, *rank = nullptr, *lights = nullptr, *heavies = nullptr, *usums = nullptr,
             *counts = nullptr;
    const size_t tiles = (n + 1 + SCAN_TILE - 1) / SCAN_TILE + 1;
    chk(cudaMallocAsync(&wt, n * sizeof(double), st));
    chk(cudaMallocAsync(&wn, n * sizeof(double), st));
    chk(cudaMallocAsync(&dl, (n + 1) * sizeof(double), st));
    chk(cudaMallocAsync(&eh, (n + 1) * sizeof(double), st));
    chk(cudaMallocAsync(&dsums, tiles * sizeof(double), st));
    chk(cudaMallocAsync(&dtot, 4 * sizeof(double), st));
    chk(cudaMallocAsync(&light, n * sizeof(uint32_t), st));
    chk(cudaMallocAsync(&rank, n * sizeof(uint32_t), st));
    chk(cudaMallocAsync(&lights, n * sizeof(uint32_t), st));
    chk(cudaMallocAsync(&heavies, n * sizeof(uint32_t), st));
    chk(cudaMallocAsync(&usums, tiles * sizeof(uint32_t), st));
    chk(cudaMallocAsync(&counts, 4 * sizeof(uint32_t), st));
    if(e != cudaSuccess) return cuda_check(ctx, e, "env_build allocation");
    const int T = 256;
    const unsigned g = (unsigned)((n + T - 1) / T);
    chk(cudaMemcpyAsync(out.rgb, d_rgb_in, n * 3 * sizeof(float), cudaMemcpyDeviceToDevice, st));
    k_env_weights<<<g, T, 0, st>>>(out.rgb, w, h, wt);
    chk(exclusive_scan<double>(wt, dl, n, dsums, dtot, st)); // FP64 total of the texel weights
    k_env_normalise<<<g, T, 0, st>>>(wt, (uint32_t)n, dtot, wn, out.pdf_w, light);
    chk(exclusive_scan<uint32_t>(light, rank, n, usums, nullptr, st));
    k_counts_from_ranks<<<1, 1, 0, st>>>(light, rank, (uint32_t)n, counts);
    // compacted deficits / excesses, zero padded to n+1 entries, then FP64 exclusive prefix sums in
    // place: D[k] (k <= nL) and E[m] (m <= nH) include the totals at D[nL] / E[nH]
    chk(cudaMemsetAsync(dl, 0, (n + 1) * sizeof(double), st));
    chk(cudaMemsetAsync(eh, 0, (n + 1) * sizeof(double), st));
    k_env_partition<<<g, T, 0, st>>>(wn, light, rank, (uint32_t)n, lights, heavies, dl, eh);
    chk(exclusive_scan<double>(dl, dl, n + 1, dsums, nullptr, st));
    chk(exclusive_scan<double>(eh, eh, n + 1, dsums, nullptr, st));
    k_alias_lights<<<g, T, 0, st>>>(lights, heavies, wn, dl, eh, counts, out.alias);
    k_alias_heavies<<<g, T, 0, st>>>(heavies, dl, eh, counts, out.alias);
    chk(cudaGetLastError());
    for(void *p: {(void *)wt, (void *)wn, (void *)dl, (void *)eh, (void *)dsums, (void *)dtot, (void *)light,
                  (void *)rank, (void *)lights, (void *)heavies, (void *)usums, (void *)counts})
        cudaFreeAsync(p, st);
    return cuda_check(ctx, e, "env_build");
}

void env_free(env_tables &t)
{
    cudaFree(t.rgb);
    cudaFree(t.pdf_w);
    cudaFree(t.alias);
    t = env_tables{};
}

}// namespace vkg

using namespace vkg;

extern "C" vkg_status vkg_env_procedural_sky(vkg_ctx *ctx, uint32_t width, uint32_t height, const float sun_dir[3],
                                             float sun_peak, float sun_width, float *d_rgb, void *stream)
{
    if(!ctx) return VKG_ERR_INVALID_ARGUMENT;
    if(!sun_dir || !d_rgb || width == 0 || height == 0)
        return set_error(ctx, VKG_ERR_INVALID_ARGUMENT, "vkg_env_procedural_sky: invalid argument");
    if((uint64_t)width * height > (1ull << 28))
        return set_error(ctx, VKG_ERR_CAPACITY, "vkg_env_procedural_sky: map too large");
    if(vkg_status s = bind_device(ctx); s != VKG_OK) return s;
    const uint32_t n = width * height;
    k_env_procedural<<<(n + 255) / 256, 256, 0, static_cast<cudaStream_t>(stream)>>>(
            width, height, sun_dir[0], sun_dir[1], sun_dir[2], sun_peak, sun_width, d_rgb);
    return cuda_check(ctx, cudaGetLastError(), "k_env_procedural");
}
