// RayBuilder's wire records (material_struct_t, entry_t) read into the library's scene records.
//
// Layouts restated from the reference's struct definitions (RayBuilder.hpp:24-116 with glm's default
// packing: vec4 16 B, vec3 12 B, vec2 8 B, quat 16 B stored x y z w, all 4-byte aligned; the structs
// are alignas(16)) and checked against the shader twins' std430 layouts (ray/types.slang:17-32, :64-110).
#include "internal.hpp"

#include <cmath>
#include <cstring>

namespace
{

// byte offsets in RayBuilder::material_struct_t
namespace mat_off
{
constexpr size_t color = 0, emission = 16, metalness = 32, roughness = 36, transmission = 40, null_surface = 44;
constexpr size_t attenuation_color = 48, attenuation_distance = 60, ior = 64, clearcoat = 68,
                 clearcoat_roughness = 72, sheen_roughness = 76, sheen_color = 80;
constexpr size_t iridescence_strength = 96, iridescence_ior = 100, iridescence_thickness_range = 104;
constexpr size_t albedo_index = 112, normalmap_index = 116, emission_index = 120, ao_rough_metal_index = 124,
                 transmission_index = 128, texture_type_flags = 132, blend_mode = 136, alpha_cutoff = 140,
                 two_sided = 144,
                 phase_g = 148, scatter_factor = 152, dispersion = 156, scatter_color = 160,
                 diffuse_transmission = 172, diffuse_transmission_color = 176, diffuse_transmission_index = 188,
                 diffuse_transmission_color_index = 192;
}// namespace mat_off

// TextureTypeBits (shaders/slang/ray/types.slang:35-51) of the textures the tracer samples
namespace tex_bit
{
constexpr uint32_t color = 0x001, normal = 0x002, ao_rough_metal = 0x004, emission = 0x008, transmission = 0x040,
                   diffuse_transmission = 0x8000, diffuse_transmission_color = 0x10000;
constexpr uint32_t sampled = color | normal | ao_rough_metal | emission | transmission | diffuse_transmission |
                             diffuse_transmission_color;
}// namespace tex_bit

// byte offsets in RayBuilder::entry_t
namespace entry_off
{
constexpr size_t texture_matrix = 0, transform = 64, inv_transform = 104, aabb = 144, material_index = 168,
                 vertex_offset = 172, base_index = 176, buffer_index = 180;
}// namespace entry_off

template<class T>
T rd(const unsigned char *p, size_t off)
{
    T v;
    std::memcpy(&v, p + off, sizeof(T));
    return v;
}

void rd3(const unsigned char *p, size_t off, float *dst)
{
    std::memcpy(dst, p + off, 3 * sizeof(float));
}

}// namespace

extern "C" {

vkg_status vkg_materials_from_wire(const void *records, uint32_t n, vkg_material *out, uint32_t *dropped)
{
    if(n && (!records || !out)) return VKG_ERR_INVALID_ARGUMENT;
    uint32_t nd = 0;
    const auto *base = static_cast<const unsigned char *>(records);
    for(uint32_t i = 0; i < n; ++i)
    {
        const unsigned char *r = base + (size_t)i * VKG_WIRE_MATERIAL_BYTES;
        vkg_material m;
        vkg_material_defaults(&m);
        rd3(r, mat_off::color, m.base_color);
        m.alpha = rd<float>(r, mat_off::color + 12);
        m.alpha_cutoff = rd<float>(r, mat_off::alpha_cutoff);
        float em[4];
        std::memcpy(em, r + mat_off::emission, sizeof(em));
        for(int c = 0; c < 3; ++c) m.emission[c] = em[c] * em[3];
        m.metalness = rd<float>(r, mat_off::metalness);
        m.roughness = rd<float>(r, mat_off::roughness);
        m.transmission = rd<float>(r, mat_off::transmission);
        m.null_surface = rd<uint32_t>(r, mat_off::null_surface) ? 1u : 0u;
        rd3(r, mat_off::attenuation_color, m.attenuation_color);
        m.attenuation_distance = rd<float>(r, mat_off::attenuation_distance);
        m.ior = rd<float>(r, mat_off::ior);
        m.clearcoat = rd<float>(r, mat_off::clearcoat);
        m.clearcoat_roughness = rd<float>(r, mat_off::clearcoat_roughness);
        m.sheen_roughness = rd<float>(r, mat_off::sheen_roughness);
        rd3(r, mat_off::sheen_color, m.sheen_color);
        m.iridescence = rd<float>(r, mat_off::iridescence_strength);
        m.iridescence_ior = rd<float>(r, mat_off::iridescence_ior);
        m.iridescence_thickness = rd<float>(r, mat_off::iridescence_thickness_range + 4); // range.y
        m.twosided = rd<uint32_t>(r, mat_off::two_sided) ? 1u : 0u;
        m.phase_g = rd<float>(r, mat_off::phase_g);
        m.scatter_factor = rd<float>(r, mat_off::scatter_factor);
        rd3(r, mat_off::scatter_color, m.scatter_color);
        m.diffuse_transmission = rd<float>(r, mat_off::diffuse_transmission);
        rd3(r, mat_off::diffuse_transmission_color, m.diffuse_transmission_color);
        m.dispersion = rd<float>(r, mat_off::dispersion);
        // texture slots: the index where its TextureTypeBits flag is set (an index into the scene's
        // textures, vkg_scene_set_textures, as into the reference's u_textures)
        const uint32_t flags = rd<uint32_t>(r, mat_off::texture_type_flags);
        auto slot = [&](uint32_t bit, size_t off) { return (flags & bit) ? rd<uint32_t>(r, off) : VKG_NO_TEXTURE; };
        m.tex_color = slot(tex_bit::color, mat_off::albedo_index);
        m.tex_normal = slot(tex_bit::normal, mat_off::normalmap_index);
        m.tex_emission = slot(tex_bit::emission, mat_off::emission_index);
        m.tex_ao_rough_metal = slot(tex_bit::ao_rough_metal, mat_off::ao_rough_metal_index);
        m.tex_transmission = slot(tex_bit::transmission, mat_off::transmission_index);
        m.tex_diffuse_transmission = slot(tex_bit::diffuse_transmission, mat_off::diffuse_transmission_index);
        m.tex_diffuse_transmission_color =
                slot(tex_bit::diffuse_transmission_color, mat_off::diffuse_transmission_color_index);
        // BlendMode (Material.hpp:32-37): Opaque 0, Blend 1, Mask 2; another value reads as opaque and
        // counts as dropped
        const uint32_t blend = rd<uint32_t>(r, mat_off::blend_mode);
        m.blend_mode = blend <= VKG_BLEND_MASK ? blend : VKG_BLEND_OPAQUE;
        // left out: textures the tracer does not sample (displacement, thickness, clearcoat, sheen,
        // iridescence)
        bool unused = (flags & ~tex_bit::sampled) != 0 || blend > VKG_BLEND_MASK;
        nd += unused ? 1u : 0u;
        out[i] = m;
    }
    if(dropped) *dropped = nd;
    return VKG_OK;
}

vkg_status vkg_instances_from_wire(const void *records, uint32_t n, vkg_instance *out, vkg_wire_entry_info *info)
{
    if(n && (!records || !out)) return VKG_ERR_INVALID_ARGUMENT;
    const auto *base = static_cast<const unsigned char *>(records);
    for(uint32_t i = 0; i < n; ++i)
    {
        const unsigned char *r = base + (size_t)i * VKG_WIRE_ENTRY_BYTES;
        float t[3], q[4], s[3];
        rd3(r, entry_off::transform, t);
        std::memcpy(q, r + entry_off::transform + 12, sizeof(q)); // x y z w
        rd3(r, entry_off::transform + 28, s);
        // rotation matrix of the unit quaternion (x, y, z, w), in double, columns scaled by s
        const double x = q[0], y = q[1], z = q[2], w = q[3];
        const double R[3][3] = {{1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)},
                                {2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)},
                                {2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)}};
        vkg_instance in{};
        for(int row = 0; row < 3; ++row)
        {
            for(int c = 0; c < 3; ++c) in.transform[4 * row + c] = (float)(R[row][c] * (double)s[c]);
            in.transform[4 * row + 3] = t[row];
        }
        in.blas = rd<uint32_t>(r, entry_off::buffer_index);
        in.material = rd<uint32_t>(r, entry_off::material_index);
        out[i] = in;
        if(info)
        {
            vkg_wire_entry_info &e = info[i];
            e.buffer_index = in.blas;
            e.base_index = rd<uint32_t>(r, entry_off::base_index);
            e.vertex_offset = rd<int32_t>(r, entry_off::vertex_offset);
            rd3(r, entry_off::aabb, e.aabb_min);
            rd3(r, entry_off::aabb + 12, e.aabb_max);
            // texture_matrix: a glm::mat4 (column-major, element (row, column) at 4 column + row)
            // applied to (u, v, 0, 1): u' = M00 u + M01 v + M03, v' = M10 u + M11 v + M13
            float m[16];
            std::memcpy(m, r + entry_off::texture_matrix, sizeof(m));
            const float t6[6] = {m[0], m[4], m[12], m[1], m[5], m[13]};
            const float id6[6] = {1.f, 0.f, 0.f, 0.f, 1.f, 0.f};
            e.has_uv_transform = std::memcmp(t6, id6, sizeof(t6)) != 0 ? 1u : 0u;
            std::memcpy(e.uv_transform, t6, sizeof(t6));
        }
    }
    return VKG_OK;
}

}// extern "C"
