/*
 * Pinhole camera rays. TEST INFRASTRUCTURE ONLY (CPU oracle).
 *
 * Convention of the reference's raygen (shaders/slang/raypipeline.slang:58-89 with the projection
 * of include/vierkant/projection.hpp:48-57, aperture 0): pixel (x + jx, y + jy) maps to
 * ndc = 2 * p / size - 1, the camera-space direction is (ndc.x * tan(fovy/2) * aspect,
 * -ndc.y * tan(fovy/2), -1) (image y grows downward), rotated by the camera-to-world basis and
 * normalised as v * (1 / sqrt(dot(v, v))). tan(fovy/2) is a caller-supplied float so host and
 * device never evaluate tan() themselves. tmin = 1e-4, tmax = 1e4 (ray_common.slang:12-15).
 *
 * Batch jitter (project-defined): ray r = s * W * H + y * W + x takes PCG32 draws 2r and 2r+1 of
 * the stream (seed, stream), i.e. two draws per pixel in row-major order.
 */
#include "oracle.h"

#include <math.h>

static void norm3(const float v[3], float out[3])
{
    float inv = 1.0f / sqrtf(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    for(int i = 0; i < 3; ++i) out[i] = v[i] * inv;
}

void orc_camera_lookat(const float eye[3], const float target[3], const float up[3], float tan_half_fovy,
                       uint32_t width, uint32_t height, orc_camera *cam)
{
    float f[3] = {target[0] - eye[0], target[1] - eye[1], target[2] - eye[2]}, fw[3], r[3], rr[3], u[3];
    norm3(f, fw);
    r[0] = fw[1] * up[2] - up[1] * fw[2];
    r[1] = fw[2] * up[0] - up[2] * fw[0];
    r[2] = fw[0] * up[1] - up[0] * fw[1];
    norm3(r, rr);
    u[0] = rr[1] * fw[2] - fw[1] * rr[2];
    u[1] = rr[2] * fw[0] - fw[2] * rr[0];
    u[2] = rr[0] * fw[1] - fw[0] * rr[1];
    for(int i = 0; i < 3; ++i)
    {
        cam->eye[i] = eye[i];
        cam->right[i] = rr[i];
        cam->up[i] = u[i];
        cam->back[i] = -fw[i];
    }
    cam->tan_half_fovy = tan_half_fovy;
    cam->aspect = (float)width / (float)height;
    cam->width = width;
    cam->height = height;
}

void orc_camera_ray(const orc_camera *cam, uint32_t x, uint32_t y, float jx, float jy, orc_ray *ray)
{
    float sx = ((float)x + jx) / (float)cam->width;
    float sy = ((float)y + jy) / (float)cam->height;
    float nx = 2.0f * sx - 1.0f, ny = 2.0f * sy - 1.0f;
    float cx = nx * (cam->tan_half_fovy * cam->aspect);
    float cy = -(ny * cam->tan_half_fovy);
    float cz = -1.0f;
    float d[3];
    for(int i = 0; i < 3; ++i) d[i] = (cam->right[i] * cx + cam->up[i] * cy) + cam->back[i] * cz;
    norm3(d, ray->d);
    for(int i = 0; i < 3; ++i) ray->o[i] = cam->eye[i];
    ray->tmin = 1e-4f;
    ray->tmax = 1e4f;
}

void orc_camera_rays_pcg(const orc_camera *cam, uint64_t seed, uint64_t stream, uint32_t spp, orc_ray *rays)
{
    orc_pcg32 g;
    orc_pcg32_seed(&g, seed, stream);
    for(uint32_t s = 0; s < spp; ++s)
        for(uint32_t y = 0; y < cam->height; ++y)
            for(uint32_t x = 0; x < cam->width; ++x)
            {
                float jx = orc_u01(orc_pcg32_next(&g));
                float jy = orc_u01(orc_pcg32_next(&g));
                size_t r = ((size_t)s * cam->height + y) * cam->width + x;
                orc_camera_ray(cam, x, y, jx, jy, &rays[r]);
            }
}
