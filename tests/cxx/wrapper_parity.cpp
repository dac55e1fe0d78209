// The C++20 wrapper (include/vierkant_gb/*.hpp) against the reference's own intersection code.
// TEST INFRASTRUCTURE: compiled by tests/test_cxx_wrapper.py together with the reference's unmodified
// src/intersection.cpp (oracle/ref_shim provides glm and crocore) and linked with libvkg.so.
//
//   wrapper_parity <dir>   reads <dir>/<kind>.in (float32 rows) for the six golden case kinds and writes
//                          <dir>/<kind>.gb (the wrapper's results) and <dir>/<kind>.ref (the reference's)
//                          as rows of {int32 type, float32 t, u, v}; then checks 200,000 seeded random
//                          ray-triangle and ray-box cases and prints "random mismatches: N"
#include <vierkant/intersection.hpp>

#include <vierkant_gb/PBRPathTracer.hpp>
#include <vierkant_gb/intersection.hpp>
#include <vierkant_gb/raytracing.hpp>

#include <cstdio>
#include <cstring>
#include <fstream>
#include <random>
#include <string>
#include <vector>

namespace gb = vierkant::gb;

struct row
{
    int32_t type;
    float t, u, v;
};

static std::vector<float> read_floats(const std::string &path)
{
    std::ifstream f(path, std::ios::binary | std::ios::ate);
    std::vector<float> out(size_t(f.tellg()) / 4);
    f.seekg(0);
    f.read(reinterpret_cast<char *>(out.data()), std::streamsize(out.size() * 4));
    return out;
}

static void write_rows(const std::string &path, const std::vector<row> &rows)
{
    std::ofstream f(path, std::ios::binary);
    f.write(reinterpret_cast<const char *>(rows.data()), std::streamsize(rows.size() * sizeof(row)));
}

static glm::vec3 g3(const float *p) { return glm::vec3(p[0], p[1], p[2]); }

static gb::vec3 w3(const float *p) { return gb::vec3(p[0], p[1], p[2]); }

// rays are built by member assignment on both sides (the directions are used as stored)
static vierkant::Ray ref_ray(const float *o, const float *d)
{
    vierkant::Ray r;
    r.origin = g3(o);
    r.direction = g3(d);
    return r;
}

static gb::Ray gb_ray(const float *o, const float *d)
{
    gb::Ray r;
    r.origin = w3(o);
    r.direction = w3(d);
    return r;
}

int main(int argc, char **argv)
{
    if(argc < 2) { return 2; }
    std::string dir = argv[1];
    // ray_triangle.in: o[3] d[3] tri[9]
    {
        auto x = read_floats(dir + "/ray_triangle.in");
        std::vector<row> a, b;
        for(size_t i = 0; i + 15 <= x.size(); i += 15)
        {
            const float *p = &x[i];
            vierkant::Triangle rt{g3(p + 6), g3(p + 9), g3(p + 12)};
            gb::Triangle wt{w3(p + 6), w3(p + 9), w3(p + 12)};
            auto r = vierkant::intersect(rt, ref_ray(p, p + 3));
            auto w = gb::intersect(gb_ray(p, p + 3), wt);
            a.push_back({int32_t(w.type), w.distance, w.u, w.v});
            b.push_back({int32_t(r.type), r.distance, r.u, r.v});
        }
        write_rows(dir + "/ray_triangle.gb", a);
        write_rows(dir + "/ray_triangle.ref", b);
    }
    // ray_aabb.in: o[3] d[3] lo[3] hi[3]; both as AABB::intersect and as the free function
    {
        auto x = read_floats(dir + "/ray_aabb.in");
        std::vector<row> a, b;
        for(size_t i = 0; i + 12 <= x.size(); i += 12)
        {
            const float *p = &x[i];
            vierkant::AABB rb(g3(p + 6), g3(p + 9));
            gb::AABB wb(w3(p + 6), w3(p + 9));
            auto r = rb.intersect(ref_ray(p, p + 3));
            auto w = wb.intersect(gb_ray(p, p + 3));
            auto w2 = gb::intersect(gb_ray(p, p + 3), wb);
            if(w2.type != w.type || std::memcmp(&w2.distance, &w.distance, 4) != 0) { w.type = gb::intersection_type(7); }
            a.push_back({int32_t(w.type), w.distance, 0.f, 0.f});
            b.push_back({int32_t(r.type), r.distance, 0.f, 0.f});
        }
        write_rows(dir + "/ray_aabb.gb", a);
        write_rows(dir + "/ray_aabb.ref", b);
    }
    // ray_sphere.in: o[3] d[3] c[3] r
    {
        auto x = read_floats(dir + "/ray_sphere.in");
        std::vector<row> a, b;
        for(size_t i = 0; i + 10 <= x.size(); i += 10)
        {
            const float *p = &x[i];
            auto r = vierkant::intersect(vierkant::Sphere(g3(p + 6), p[9]), ref_ray(p, p + 3));
            auto w = gb::intersect(gb::Sphere(w3(p + 6), p[9]), gb_ray(p, p + 3));
            a.push_back({int32_t(w.type), w.distance, 0.f, 0.f});
            b.push_back({int32_t(r.type), r.distance, 0.f, 0.f});
        }
        write_rows(dir + "/ray_sphere.gb", a);
        write_rows(dir + "/ray_sphere.ref", b);
    }
    // ray_plane.in: o[3] d[3] plane[4]
    {
        auto x = read_floats(dir + "/ray_plane.in");
        std::vector<row> a, b;
        for(size_t i = 0; i + 10 <= x.size(); i += 10)
        {
            const float *p = &x[i];
            auto r = vierkant::intersect(vierkant::Plane(p[6], p[7], p[8], p[9]), ref_ray(p, p + 3));
            auto w = gb::intersect(gb::Plane(p[6], p[7], p[8], p[9]), gb_ray(p, p + 3));
            a.push_back({int32_t(w.type), w.distance, 0.f, 0.f});
            b.push_back({int32_t(r.type), r.distance, 0.f, 0.f});
        }
        write_rows(dir + "/ray_plane.gb", a);
        write_rows(dir + "/ray_plane.ref", b);
    }
    // tri_box.in: tri[9] lo[3] hi[3]
    {
        auto x = read_floats(dir + "/tri_box.in");
        std::vector<row> a, b;
        for(size_t i = 0; i + 15 <= x.size(); i += 15)
        {
            const float *p = &x[i];
            vierkant::Triangle rt{g3(p), g3(p + 3), g3(p + 6)};
            gb::Triangle wt{w3(p), w3(p + 3), w3(p + 6)};
            uint32_t r = vierkant::intersect(rt, vierkant::AABB(g3(p + 9), g3(p + 12)));
            uint32_t w = gb::intersect(gb::AABB(w3(p + 9), w3(p + 12)), wt);
            a.push_back({int32_t(w), 0.f, 0.f, 0.f});
            b.push_back({int32_t(r), 0.f, 0.f, 0.f});
        }
        write_rows(dir + "/tri_box.gb", a);
        write_rows(dir + "/tri_box.ref", b);
    }
    // tri_tri.in: a[9] b[9]
    {
        auto x = read_floats(dir + "/tri_tri.in");
        std::vector<row> a, b;
        for(size_t i = 0; i + 18 <= x.size(); i += 18)
        {
            const float *p = &x[i];
            vierkant::Triangle r1{g3(p), g3(p + 3), g3(p + 6)}, r2{g3(p + 9), g3(p + 12), g3(p + 15)};
            gb::Triangle w1{w3(p), w3(p + 3), w3(p + 6)}, w2{w3(p + 9), w3(p + 12), w3(p + 15)};
            a.push_back({int32_t(gb::intersect(w1, w2)), 0.f, 0.f, 0.f});
            b.push_back({int32_t(vierkant::intersect(r1, r2)), 0.f, 0.f, 0.f});
        }
        write_rows(dir + "/tri_tri.gb", a);
        write_rows(dir + "/tri_tri.ref", b);
    }
    // seeded random cases: the Ray(origin, direction) constructor normalises on both sides
    std::mt19937 rng(0x5EED);
    std::uniform_real_distribution<float> U(-2.f, 2.f);
    size_t mismatches = 0;
    for(int i = 0; i < 100000; ++i)
    {
        float v[15];
        for(float &f: v) { f = U(rng); }
        vierkant::Ray rr(g3(v), g3(v + 3));
        gb::Ray wr(w3(v), w3(v + 3));
        if(std::memcmp(&rr.direction, &wr.direction, 12) != 0) { ++mismatches; }
        auto r = vierkant::intersect(vierkant::Triangle{g3(v + 6), g3(v + 9), g3(v + 12)}, rr);
        auto w = gb::intersect(gb::Triangle{w3(v + 6), w3(v + 9), w3(v + 12)}, wr);
        if(r.type != int(w.type) || (r.type && (std::memcmp(&r.distance, &w.distance, 4) || std::memcmp(&r.u, &w.u, 4) ||
                                                std::memcmp(&r.v, &w.v, 4))))
        {
            ++mismatches;
        }
        glm::vec3 lo = glm::min(g3(v + 6), g3(v + 9)), hi = glm::max(g3(v + 6), g3(v + 9));
        auto rb = vierkant::AABB(lo, hi).intersect(rr);
        auto wb = gb::AABB(gb::vec3(lo), gb::vec3(hi)).intersect(wr);
        if(rb.type != int(wb.type) || (rb.type && std::memcmp(&rb.distance, &wb.distance, 4))) { ++mismatches; }
    }
    // exceptions at the wrapper level: a null output is the one invalid argument the C ABI can see
    bool threw = false;
    try
    {
        gb::check(vkg_intersect_ray_triangle(nullptr, nullptr, nullptr, nullptr), "vkg_intersect_ray_triangle");
    } catch(const gb::error &e)
    {
        threw = e.status() == VKG_ERR_INVALID_ARGUMENT;
    }
    std::printf("random mismatches: %zu\nthrows: %d\n", mismatches, int(threw));
    return 0;
}
