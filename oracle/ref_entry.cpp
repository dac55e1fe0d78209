// C entry points around the reference's OWN intersection code (src/intersection.cpp and
// src/triangle_intersection.h, compiled unmodified from the reference checkout against the
// project-written shim in oracle/ref_shim/). TEST INFRASTRUCTURE ONLY: this file is the
// "reference" CPU arm and the pin for the C restatement in oracle/intersect.c. The product
// library never links it.
//
// Closest-hit harness: the reference has no bulk ray-cast loop (Scene::pick loops objects,
// Scene.cpp:222-242); this harness loops rays x triangles over host threads and calls
// vierkant::intersect(const Triangle&, const Ray&) (intersection.cpp:114-129), keeping the
// closest accepted hit: t in (tmin, tmax), ties to the smaller triangle id.
#include <vierkant/intersection.hpp>

#include <atomic>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

namespace
{
// record layout shared with the C oracle and the product: {o[3], tmin, d[3], tmax}
struct ray_rec
{
    float o[3];
    float tmin;
    float d[3];
    float tmax;
};
struct hit_rec
{
    uint32_t prim;
    float t, u, v;
};

inline vierkant::Ray make_ray(const ray_rec &r)
{
    // assign members directly: the stored direction is already normalised and the
    // Ray(origin, direction) constructor would normalise it a second time
    vierkant::Ray ray;
    ray.origin = glm::vec3(r.o[0], r.o[1], r.o[2]);
    ray.direction = glm::vec3(r.d[0], r.d[1], r.d[2]);
    return ray;
}
}// namespace

extern "C" {

int vkref_intersect_ray_triangle(const float ray_o[3], const float ray_d[3], const float tri[9], float out[3])
{
    vierkant::Ray ray;
    ray.origin = glm::vec3(ray_o[0], ray_o[1], ray_o[2]);
    ray.direction = glm::vec3(ray_d[0], ray_d[1], ray_d[2]);
    vierkant::Triangle t{glm::vec3(tri[0], tri[1], tri[2]), glm::vec3(tri[3], tri[4], tri[5]),
                         glm::vec3(tri[6], tri[7], tri[8])};
    auto res = vierkant::intersect(t, ray);
    out[0] = res.distance;
    out[1] = res.u;
    out[2] = res.v;
    return static_cast<int>(res.type);
}

int vkref_intersect_ray_aabb(const float ray_o[3], const float ray_d[3], const float bmin[3], const float bmax[3],
                             float *out_t)
{
    vierkant::Ray ray;
    ray.origin = glm::vec3(ray_o[0], ray_o[1], ray_o[2]);
    ray.direction = glm::vec3(ray_d[0], ray_d[1], ray_d[2]);
    vierkant::AABB box(glm::vec3(bmin[0], bmin[1], bmin[2]), glm::vec3(bmax[0], bmax[1], bmax[2]));
    auto res = box.intersect(ray);
    *out_t = res.distance;
    return static_cast<int>(res.type);
}

int vkref_intersect_ray_sphere(const float ray_o[3], const float ray_d[3], const float center[3], float radius,
                               float *out_t)
{
    vierkant::Ray ray;
    ray.origin = glm::vec3(ray_o[0], ray_o[1], ray_o[2]);
    ray.direction = glm::vec3(ray_d[0], ray_d[1], ray_d[2]);
    vierkant::Sphere s(glm::vec3(center[0], center[1], center[2]), radius);
    auto res = vierkant::intersect(s, ray);
    *out_t = res.distance;
    return static_cast<int>(res.type);
}

int vkref_intersect_ray_plane(const float ray_o[3], const float ray_d[3], const float coeffs[4], float *out_t)
{
    vierkant::Ray ray;
    ray.origin = glm::vec3(ray_o[0], ray_o[1], ray_o[2]);
    ray.direction = glm::vec3(ray_d[0], ray_d[1], ray_d[2]);
    vierkant::Plane p(coeffs[0], coeffs[1], coeffs[2], coeffs[3]);
    auto res = vierkant::intersect(p, ray);
    *out_t = res.distance;
    return static_cast<int>(res.type);
}

uint32_t vkref_triangle_aabb_overlap(const float tri[9], const float bmin[3], const float bmax[3])
{
    vierkant::Triangle t{glm::vec3(tri[0], tri[1], tri[2]), glm::vec3(tri[3], tri[4], tri[5]),
                         glm::vec3(tri[6], tri[7], tri[8])};
    vierkant::AABB box(glm::vec3(bmin[0], bmin[1], bmin[2]), glm::vec3(bmax[0], bmax[1], bmax[2]));
    return vierkant::intersect(t, box);
}

uint32_t vkref_triangle_triangle_overlap(const float a[9], const float b[9])
{
    vierkant::Triangle t1{glm::vec3(a[0], a[1], a[2]), glm::vec3(a[3], a[4], a[5]), glm::vec3(a[6], a[7], a[8])};
    vierkant::Triangle t2{glm::vec3(b[0], b[1], b[2]), glm::vec3(b[3], b[4], b[5]), glm::vec3(b[6], b[7], b[8])};
    return vierkant::intersect(t1, t2);
}

// Triangle soup for the CPU BVH traversal (oracle/lbvh.c, orc_bvh_closest_hit_fn): the oracle's BVH
// decides which triangles a ray meets, and every triangle test is the reference's
// vierkant::intersect(const Triangle&, const Ray&) (intersection.cpp:114-129) on the original vertices.
void *vkref_mesh_create(const float *xyz, const uint32_t *indices, uint32_t num_tris)
{
    auto *tris = new std::vector<vierkant::Triangle>(num_tris);
    for(uint32_t i = 0; i < num_tris; ++i)
    {
        for(int k = 0; k < 3; ++k)
        {
            const float *p = xyz + 3 * size_t(indices[3 * size_t(i) + k]);
            (*tris)[i][k] = glm::vec3(p[0], p[1], p[2]);
        }
    }
    return tris;
}

void vkref_mesh_destroy(void *mesh) { delete static_cast<std::vector<vierkant::Triangle> *>(mesh); }

// orc_tri_fn: 1 (INTERSECT) with {t, u, v}, else 0; the stored direction is used as given
int vkref_mesh_intersect(void *mesh, uint32_t prim, const float o[3], const float d[3], float tuv[3])
{
    const auto &tris = *static_cast<const std::vector<vierkant::Triangle> *>(mesh);
    vierkant::Ray ray;
    ray.origin = glm::vec3(o[0], o[1], o[2]);
    ray.direction = glm::vec3(d[0], d[1], d[2]);
    auto res = vierkant::intersect(tris[prim], ray);
    if(res.type != vierkant::INTERSECT) { return 0; }
    tuv[0] = res.distance;
    tuv[1] = res.u;
    tuv[2] = res.v;
    return 1;
}

// Brute-force closest hit over all host threads (num_threads <= 0: hardware_concurrency).
// Triangles are gathered from an indexed mesh (fp32 xyz, uint32 indices, Geometry.hpp:14).
int vkref_closest_hit_bruteforce(const float *xyz, const uint32_t *indices, uint32_t num_tris, const void *rays_v,
                                 uint32_t num_rays, void *hits_v, int num_threads, int cull_back_faces)
{
    const auto *rays = static_cast<const ray_rec *>(rays_v);
    auto *hits = static_cast<hit_rec *>(hits_v);
    std::vector<vierkant::Triangle> tris(num_tris);
    for(uint32_t i = 0; i < num_tris; ++i)
    {
        for(int k = 0; k < 3; ++k)
        {
            const float *p = xyz + 3 * size_t(indices[3 * size_t(i) + k]);
            tris[i][k] = glm::vec3(p[0], p[1], p[2]);
        }
    }
    if(num_threads <= 0) { num_threads = static_cast<int>(std::max(1u, std::thread::hardware_concurrency())); }
    std::atomic<uint32_t> next{0};
    constexpr uint32_t chunk = 16;
    auto worker = [&]() {
        for(;;)
        {
            uint32_t begin = next.fetch_add(chunk);
            if(begin >= num_rays) { break; }
            uint32_t end = std::min(num_rays, begin + chunk);
            for(uint32_t r = begin; r < end; ++r)
            {
                const ray_rec &rr = rays[r];
                vierkant::Ray ray = make_ray(rr);
                hit_rec best{0xFFFFFFFFu, rr.tmax, 0.f, 0.f};
                for(uint32_t i = 0; i < num_tris; ++i)
                {
                    auto res = vierkant::intersect(tris[i], ray);
                    if(res.type != vierkant::INTERSECT) { continue; }
                    if(cull_back_faces)
                    {
                        // front face <=> det = dot(e1, cross(d, e2)) > 0 (counter-clockwise seen from the origin)
                        glm::vec3 e1 = tris[i].v1 - tris[i].v0, e2 = tris[i].v2 - tris[i].v0;
                        if(glm::dot(e1, glm::cross(ray.direction, e2)) < 0.f) { continue; }
                    }
                    float t = res.distance;
                    if(!(t > rr.tmin && t < rr.tmax)) { continue; }
                    if(t < best.t || (t == best.t && i < best.prim)) { best = {i, t, res.u, res.v}; }
                }
                if(best.prim == 0xFFFFFFFFu) { best = {0xFFFFFFFFu, 0.f, 0.f, 0.f}; }
                hits[r] = best;
            }
        }
    };
    std::vector<std::thread> pool;
    for(int i = 0; i < num_threads; ++i) { pool.emplace_back(worker); }
    for(auto &t: pool) { t.join(); }
    return num_threads;
}

}// extern "C"
