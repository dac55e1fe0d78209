// The C++20 wrapper's owning classes on the GPU (TEST INFRASTRUCTURE, built by
// tests/test_gpu_cxx_wrapper.py): vierkant::gb::context / bvh trace the 20,480-triangle icosphere from
// a 256x256 camera, and vierkant::gb::PBRPathTracer renders two batches of a one-triangle-pair scene.
//   wrapper_gpu <out dir>   writes <out>/hits.bin (vkg_hit records) and <out>/image.bin (crop rgb),
//                           prints "batches N paths P" and "error caught: 1"
#include <vierkant_gb/PBRPathTracer.hpp>

#include <cuda_runtime.h>

#include <cstdio>
#include <fstream>
#include <string>
#include <vector>

namespace gb = vierkant::gb;

template<class T>
static T *upload(const std::vector<T> &v)
{
    T *d = nullptr;
    cudaMalloc(&d, v.size() * sizeof(T));
    cudaMemcpy(d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
    return d;
}

int main(int argc, char **argv)
{
    if(argc < 2) return 2;
    const std::string dir = argv[1];
    auto ctx = gb::context::create(0);
    uint32_t nv = 0, nt = 0;
    gb::check(vkg_geometry_icosphere_counts(5, &nv, &nt), "counts");
    std::vector<float> xyz(3 * nv);
    std::vector<uint32_t> idx(3 * nt);
    gb::check(vkg_geometry_icosphere(1.f, 5, xyz.data(), idx.data()), "icosphere");
    float *d_xyz = upload(xyz);
    uint32_t *d_idx = upload(idx);
    auto bvh = gb::bvh::build(ctx, d_xyz, nv, d_idx, nt);
    const uint32_t W = 256, H = 256;
    vkg_camera cam = gb::camera_lookat({0, 0, 3}, {0, 0, 0}, {0, 1, 0}, 60.f * 3.14159265358979f / 180.f, W, H);
    vkg_ray *d_rays = nullptr;
    vkg_hit *d_hits = nullptr;
    cudaMalloc(&d_rays, W * H * sizeof(vkg_ray));
    cudaMalloc(&d_hits, W * H * sizeof(vkg_hit));
    ctx->check(vkg_camera_rays(ctx->handle(), &cam, 0x5EED, 1, 1, d_rays, nullptr), "vkg_camera_rays");
    bvh->closest_hit(d_rays, W * H, d_hits);
    std::vector<vkg_hit> hits(W * H);
    cudaMemcpy(hits.data(), d_hits, hits.size() * sizeof(vkg_hit), cudaMemcpyDeviceToHost);
    std::ofstream(dir + "/hits.bin", std::ios::binary)
            .write(reinterpret_cast<const char *>(hits.data()), std::streamsize(hits.size() * sizeof(vkg_hit)));
    std::vector<vkg_ray> rays(W * H);
    cudaMemcpy(rays.data(), d_rays, rays.size() * sizeof(vkg_ray), cudaMemcpyDeviceToHost);
    std::ofstream(dir + "/rays.bin", std::ios::binary)
            .write(reinterpret_cast<const char *>(rays.data()), std::streamsize(rays.size() * sizeof(vkg_ray)));
    std::ofstream(dir + "/tan.bin", std::ios::binary).write(reinterpret_cast<const char *>(&cam.tan_half_fovy), 4);

    // a path-tracer scene: the icosphere, one material, a constant environment
    std::vector<uint32_t> tri_mat(nt, 0u);
    vkg_material mat{};
    gb::check(vkg_material_defaults(&mat), "vkg_material_defaults");
    std::vector<float> env(8 * 4 * 3, 0.5f);
    uint32_t *d_tm = upload(tri_mat);
    vkg_material *d_mat = upload(std::vector<vkg_material>{mat});
    float *d_env = upload(env);
    vkg_scene_desc desc{d_xyz, nv, d_idx, nt, d_tm, d_mat, 1u, d_env, 8u, 4u, 0u};
    auto scene = gb::scene::create(ctx, desc);
    gb::PBRPathTracer::create_info_t info;
    info.seed = 7;
    info.settings.resolution[0] = W;
    info.settings.resolution[1] = H;
    info.settings.num_samples = 4;
    for(int k = 0; k < 4; ++k) info.settings.crop[k] = std::vector<uint32_t>{96, 96, 64, 64}[k];
    auto pt = gb::PBRPathTracer::create(ctx, info);
    float *d_img = nullptr;
    cudaMalloc(&d_img, 64 * 64 * 3 * sizeof(float));
    vkg_camera pcam = gb::camera_lookat({0, 0, 3}, {0, 0, 0}, {0, 1, 0}, 0.8f, W, H);
    pt->render_scene(scene, pcam, d_img);
    auto res = pt->render_scene(scene, pcam, d_img);
    cudaDeviceSynchronize();
    auto st = pt->statistics();
    std::vector<float> img(64 * 64 * 3);
    cudaMemcpy(img.data(), d_img, img.size() * sizeof(float), cudaMemcpyDeviceToHost);
    std::ofstream(dir + "/image.bin", std::ios::binary)
            .write(reinterpret_cast<const char *>(img.data()), std::streamsize(img.size() * sizeof(float)));
    std::printf("batches %zu paths %llu samples %u\n", pt->current_batch(), (unsigned long long)st.paths,
                res.num_samples);
    // a failing call throws at the wrapper level with the context's message
    int caught = 0;
    try
    {
        pt->settings.mis_mode = 7;
        pt->render_scene(scene, pcam, d_img);
    } catch(const gb::error &e)
    {
        caught = e.status() == VKG_ERR_INVALID_ARGUMENT && std::string(e.what()).find("mis_mode") != std::string::npos;
    }
    std::printf("error caught: %d\n", caught);
    for(void *p: {(void *)d_xyz, (void *)d_idx, (void *)d_rays, (void *)d_hits, (void *)d_tm, (void *)d_mat,
                  (void *)d_env, (void *)d_img})
        cudaFree(p);
    return 0;
}
