// Generators of the stress workload (two-level scene): a cube-sphere mesh, a procedural terrain whose
// heights are fractional Brownian motion over 3-D simplex noise, and seeded instance transforms.
//
// The noise basis is the one vierkant's shaders use (shaders/slang/utils/simplex.slang:27-83, the
// Ashima Arts / McEwan-Gustavson 3-D simplex noise, MIT): skew the point onto the simplex lattice,
// order the corners by comparing the fractional coordinates, hash each corner through the
// permutation polynomial (34x + 1)x mod 289, pick its gradient from a 7 x 7 grid folded onto an
// octahedron, normalise with the Taylor inverse square root 1.79284291400159 - 0.85373472095314 r,
// and sum the radial kernels max(0.6 - r^2, 0)^4 scaled by 42. Restated here in plain C++.
#include "internal.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

namespace
{

inline float mod289(float x) { return x - std::floor(x * (1.0f / 289.0f)) * 289.0f; }
inline float perm(float x) { return mod289((x * 34.0f + 1.0f) * x); }

float simplex3(float vx, float vy, float vz)
{
    const float F = 1.0f / 3.0f, G = 1.0f / 6.0f;
    // cell of the skewed lattice and the offset from its origin corner
    const float s = (vx + vy + vz) * F;
    const float ix = std::floor(vx + s), iy = std::floor(vy + s), iz = std::floor(vz + s);
    const float t = (ix + iy + iz) * G;
    const float x0[3] = {vx - ix + t, vy - iy + t, vz - iz + t};
    // the simplex's second and third corners: the axes in decreasing order of x0
    const float gxy = x0[0] >= x0[1] ? 1.f : 0.f, gyz = x0[1] >= x0[2] ? 1.f : 0.f, gzx = x0[2] >= x0[0] ? 1.f : 0.f;
    const float g[3] = {gxy, gyz, gzx}, l[3] = {1.f - gxy, 1.f - gyz, 1.f - gzx};
    const float i1[3] = {std::min(g[0], l[2]), std::min(g[1], l[0]), std::min(g[2], l[1])};
    const float i2[3] = {std::max(g[0], l[2]), std::max(g[1], l[0]), std::max(g[2], l[1])};
    float x[4][3];
    for(int a = 0; a < 3; ++a)
    {
        x[0][a] = x0[a];
        x[1][a] = x0[a] - i1[a] + G;
        x[2][a] = x0[a] - i2[a] + 2.0f * G;
        x[3][a] = x0[a] - 0.5f;
    }
    const float cx[4] = {0.f, i1[0], i2[0], 1.f}, cy[4] = {0.f, i1[1], i2[1], 1.f}, cz[4] = {0.f, i1[2], i2[2], 1.f};
    const float mx = mod289(ix), my = mod289(iy), mz = mod289(iz);
    float sum = 0.f;
    for(int k = 0; k < 4; ++k)
    {
        const float p = perm(perm(perm(mz + cz[k]) + my + cy[k]) + mx + cx[k]);
        // gradient: the hash as a point of a 7 x 7 grid in [-1, 1]^2, folded onto the octahedron
        const float j = p - 49.0f * std::floor(p * (1.0f / 49.0f));
        const float gx_ = std::floor(j * (1.0f / 7.0f)), gy_ = std::floor(j - 7.0f * gx_);
        float gx = gx_ * (2.0f / 7.0f) - 1.0f + 1.0f / 7.0f, gy = gy_ * (2.0f / 7.0f) - 1.0f + 1.0f / 7.0f;
        const float gz = 1.0f - std::fabs(gx) - std::fabs(gy);
        if(gz < 0.f)
        {
            gx += (std::floor(gx) * 2.0f + 1.0f) * -1.0f;
            gy += (std::floor(gy) * 2.0f + 1.0f) * -1.0f;
        }
        const float r2g = gx * gx + gy * gy + gz * gz;
        const float norm = 1.79284291400159f - 0.85373472095314f * r2g;
        const float d = (gx * x[k][0] + gy * x[k][1] + gz * x[k][2]) * norm;
        const float r2 = x[k][0] * x[k][0] + x[k][1] * x[k][1] + x[k][2] * x[k][2];
        float m = std::max(0.6f - r2, 0.f);
        m = m * m;
        sum += m * m * d;
    }
    return 42.0f * sum;
}

void cubesphere_mesh(uint32_t n, float radius, float *xyz, uint32_t *idx)
{
    static const float N6[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
    static const float U6[6][3] = {{0, 0, -1}, {0, 0, 1}, {1, 0, 0}, {1, 0, 0}, {1, 0, 0}, {-1, 0, 0}};
    const uint32_t vpf = (n + 1) * (n + 1);
    for(uint32_t f = 0; f < 6; ++f)
    {
        const float *Nf = N6[f], *Uf = U6[f];
        const float V[3] = {Nf[1] * Uf[2] - Uf[1] * Nf[2], Nf[2] * Uf[0] - Uf[2] * Nf[0], Nf[0] * Uf[1] - Uf[0] * Nf[1]};
        for(uint32_t j = 0; j <= n; ++j)
            for(uint32_t i = 0; i <= n; ++i)
            {
                const float a = 2.0f * (float)i / (float)n - 1.0f, b = 2.0f * (float)j / (float)n - 1.0f;
                float q[3];
                for(int c = 0; c < 3; ++c) q[c] = (Nf[c] + a * Uf[c]) + b * V[c];
                const float inv = radius / std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2]);
                float *dst = xyz + 3 * (size_t)(f * vpf + j * (n + 1) + i);
                for(int c = 0; c < 3; ++c) dst[c] = q[c] * inv;
            }
        for(uint32_t j = 0; j < n; ++j)
            for(uint32_t i = 0; i < n; ++i)
            {
                const uint32_t v00 = f * vpf + j * (n + 1) + i, v10 = v00 + 1, v01 = v00 + (n + 1), v11 = v01 + 1;
                uint32_t *t = idx + 6 * (size_t)((f * n + j) * n + i);
                const uint32_t tt[6] = {v00, v10, v11, v00, v11, v01};
                std::memcpy(t, tt, sizeof(tt));
            }
    }
}

template<class F>
void parallel_rows(uint32_t rows, F f)
{
    const uint32_t nt = std::max(1u, std::min<uint32_t>(std::thread::hardware_concurrency(), 64u));
    std::vector<std::thread> th;
    for(uint32_t t = 0; t < nt; ++t)
        th.emplace_back([&, t]() {
            for(uint32_t r = t; r < rows; r += nt) f(r);
        });
    for(auto &x: th) x.join();
}

}// namespace

using namespace vkg;

extern "C" {

vkg_status vkg_geometry_cubesphere(uint32_t n, float radius, float *xyz, uint32_t *indices)
{
    if(n == 0 || !xyz || !indices) return VKG_ERR_INVALID_ARGUMENT;
    cubesphere_mesh(n, radius, xyz, indices);
    return VKG_OK;
}

vkg_status vkg_geometry_terrain(uint32_t n, float extent, float height, float frequency, uint32_t octaves,
                                uint32_t seed, float *xyz, uint32_t *indices)
{
    if(n < 2 || n > 16384 || !xyz || !indices || octaves == 0 || octaves > 16) return VKG_ERR_INVALID_ARGUMENT;
    const float step = extent / (float)(n - 1), x0 = -0.5f * extent;
    // the seed moves the noise along its third axis
    const float zoff = (float)(seed % 65536u) * 0.6180339887f;
    parallel_rows(n, [&](uint32_t j) {
        for(uint32_t i = 0; i < n; ++i)
        {
            const float x = x0 + step * (float)i, z = x0 + step * (float)j;
            float amp = 1.0f, f = frequency, h = 0.f;
            for(uint32_t o = 0; o < octaves; ++o)
            {
                h += amp * simplex3(x * f, z * f, zoff + (float)o * 17.0f);
                amp *= 0.5f;
                f *= 2.0f;
            }
            float *v = xyz + 3 * ((size_t)j * n + i);
            v[0] = x;
            v[1] = height * h;
            v[2] = z;
        }
    });
    // two triangles per quad, counter-clockwise seen from +y
    parallel_rows(n - 1, [&](uint32_t j) {
        for(uint32_t i = 0; i + 1 < n; ++i)
        {
            const uint32_t v00 = j * n + i, v10 = v00 + 1, v01 = v00 + n, v11 = v01 + 1;
            uint32_t *t = indices + 6 * ((size_t)j * (n - 1) + i);
            const uint32_t tt[6] = {v00, v01, v11, v00, v11, v10};
            std::memcpy(t, tt, sizeof(tt));
        }
    });
    return VKG_OK;
}

// n instances: translation uniform in [lo, hi], rotation uniform (Shoemake's unit quaternion from three
// uniforms), uniform scale U[smin, smax], mesh uniform in [0, num_meshes), material uniform in
// [mat_base, mat_base + num_mats); PCG32(seed, stream), 9 draws per instance in that order
vkg_status vkg_instances_random(uint64_t seed, uint64_t stream, uint32_t n, uint32_t num_meshes, uint32_t mat_base,
                                uint32_t num_mats, const float lo[3], const float hi[3], float smin, float smax,
                                vkg_instance *out)
{
    if(!out || !lo || !hi || num_meshes == 0 || num_mats == 0) return VKG_ERR_INVALID_ARGUMENT;
    pcg32 g = pcg32_seed(seed, stream);
    for(uint32_t k = 0; k < n; ++k)
    {
        float t[3];
        for(int a = 0; a < 3; ++a) t[a] = lo[a] + (hi[a] - lo[a]) * u01(pcg32_next(g));
        const double u1 = u01(pcg32_next(g)), u2 = u01(pcg32_next(g)), u3 = u01(pcg32_next(g));
        const double r1 = std::sqrt(1.0 - u1), r2 = std::sqrt(u1), tp = 6.283185307179586;
        const double qx = r1 * std::sin(tp * u2), qy = r1 * std::cos(tp * u2), qz = r2 * std::sin(tp * u3),
                     qw = r2 * std::cos(tp * u3);
        const float s = smin + (smax - smin) * u01(pcg32_next(g));
        const uint32_t mesh = std::min(num_meshes - 1, (uint32_t)(u01(pcg32_next(g)) * (float)num_meshes));
        const uint32_t mat = mat_base + std::min(num_mats - 1, (uint32_t)(u01(pcg32_next(g)) * (float)num_mats));
        const double R[9] = {1 - 2 * (qy * qy + qz * qz), 2 * (qx * qy - qz * qw),     2 * (qx * qz + qy * qw),
                             2 * (qx * qy + qz * qw),     1 - 2 * (qx * qx + qz * qz), 2 * (qy * qz - qx * qw),
                             2 * (qx * qz - qy * qw),     2 * (qy * qz + qx * qw),     1 - 2 * (qx * qx + qy * qy)};
        vkg_instance &I = out[k];
        std::memset(&I, 0, sizeof(I));
        for(int r = 0; r < 3; ++r)
        {
            for(int c = 0; c < 3; ++c) I.transform[4 * r + c] = (float)(R[3 * r + c] * s);
            I.transform[4 * r + 3] = t[r];
        }
        I.blas = mesh;
        I.material = mat;
    }
    return VKG_OK;
}

}// extern "C"
