/*
 * vkg.h -- C ABI of the GB300 path-tracing hot path (library: vierkant_gb300/libvkg.so).
 *
 * Drop-in scope: the closest-hit ray-triangle / ray-AABB queries over a BVH and the multi-bounce
 * radiance estimator of vierkant's PBRPathTracer. Every entry point below names the reference
 * interface it replaces (paths relative to the vierkant source tree).
 *
 * Conventions
 *   - every call returns vkg_status (0 = VKG_OK); nothing throws across the ABI;
 *     vkg_last_error(ctx) returns a human-readable message for the last failure on that context.
 *   - device pointers (prefix d_) are caller-owned CUDA device memory; handles (vkg_bvh,
 *     vkg_scene, vkg_tracer) are library-owned and released by their *_destroy call.
 *   - `stream` is a cudaStream_t passed as void* (NULL = legacy default stream); GPU work is
 *     asynchronous on that stream unless the function says it synchronises.
 *   - one vkg_ctx per host thread (contexts are not internally locked).
 *   - plain C types only: no CUDA or C++ types appear in this header.
 */
#ifndef VKG_H
#define VKG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status ---------------------------------------------------------------------------------- */
typedef int vkg_status;
enum
{
    VKG_OK = 0,
    VKG_ERR_INVALID_ARGUMENT = 1,
    VKG_ERR_CUDA = 2,
    VKG_ERR_OUT_OF_MEMORY = 3,
    VKG_ERR_NOT_SUPPORTED = 4,
    VKG_ERR_TIMEOUT = 5,        /* a bounded device loop gave up (device work stopped cleanly) */
    VKG_ERR_STACK_OVERFLOW = 6, /* a traversal exceeded its stack; results of that launch are invalid */
    VKG_ERR_CAPACITY = 7        /* an input exceeds a documented maximum */
};

/* ---- value types ------------------------------------------------------------------------------ */
/* intersection.hpp:18-23 */
enum
{
    VKG_REJECT = 0,
    VKG_INTERSECT = 1,
    VKG_INSIDE = 2
};

/* ray record, 32 B: mirrors ray::Ray (shaders/slang/ray/ray_common.slang:23-29) */
typedef struct vkg_ray
{
    float origin[3];
    float tmin;
    float direction[3];
    float tmax;
} vkg_ray;

/* closest-hit record, 16 B: prim = triangle id (0xFFFFFFFF on miss), t, barycentrics u, v */
typedef struct vkg_hit
{
    uint32_t prim;
    float t, u, v;
} vkg_hit;

#define VKG_MISS 0xFFFFFFFFu

/* intersection.hpp:28-51 (ray_intersection / ray_triangle_intersection) */
typedef struct vkg_ray_intersection
{
    int type; /* VKG_REJECT / VKG_INTERSECT / VKG_INSIDE */
    float distance;
} vkg_ray_intersection;

typedef struct vkg_ray_triangle_intersection
{
    int type;
    float distance, u, v;
} vkg_ray_triangle_intersection;

/* ---- host scalar intersection API (pure, thread-safe, no allocation) ------------------------
 * Bit-identical to vierkant::intersect() in src/intersection.cpp. The ray direction is used as
 * given (vierkant::Ray's constructor normalises; callers that need that pass a unit vector).   */

/* replaces intersect(const Triangle&, const Ray&), intersection.hpp:79 / intersection.cpp:114-129 */
vkg_status vkg_intersect_ray_triangle(const float origin[3], const float direction[3], const float tri[9],
                                      vkg_ray_triangle_intersection *out);
/* replaces AABB::intersect(const Ray&) / intersect(const AABB&, const Ray&), intersection.hpp:90,349,
   intersection.cpp:308-312 */
vkg_status vkg_intersect_ray_aabb(const float origin[3], const float direction[3], const float bmin[3],
                                  const float bmax[3], vkg_ray_intersection *out);
/* replaces intersect(const OBB&, const Ray&), intersection.hpp:95 / intersection.cpp:152-184;
   axes = 3 unit column vectors (9 floats), half_lengths = 3 floats */
vkg_status vkg_intersect_ray_obb(const float origin[3], const float direction[3], const float center[3],
                                 const float axes[9], const float half_lengths[3], vkg_ray_intersection *out);
/* replaces intersect(const Sphere&, const Ray&), intersection.hpp:85 / intersection.cpp:133-148 */
vkg_status vkg_intersect_ray_sphere(const float origin[3], const float direction[3], const float center[3],
                                    float radius, vkg_ray_intersection *out);
/* replaces intersect(const Plane&, const Ray&), intersection.hpp:74 / intersection.cpp:10-21;
   plane = (a, b, c, d) as in Plane(float a, float b, float c, float d) (normalised internally) */
vkg_status vkg_intersect_ray_plane(const float origin[3], const float direction[3], const float plane[4],
                                   vkg_ray_intersection *out);
/* replaces intersect(const Triangle&, const AABB&), intersection.hpp:101 / intersection.cpp:364-370
   (triangle-box overlap, Akenine-Moeller separating axes); returns 0/1 in *out */
vkg_status vkg_intersect_triangle_aabb(const float tri[9], const float bmin[3], const float bmax[3],
                                       uint32_t *out);
/* replaces intersect(const Triangle&, const Triangle&), intersection.hpp:105 / intersection.cpp:374-378
   (triangle-triangle overlap, Guigue-Devillers orientation predicates); returns 0/1 in *out */
vkg_status vkg_intersect_triangle_triangle(const float a[9], const float b[9], uint32_t *out);

/* ---- context ---------------------------------------------------------------------------------- */
typedef struct vkg_ctx vkg_ctx;

/* library version string, e.g. "vkg 0.1 sm_103a" */
const char *vkg_version(void);
/* create a context bound to CUDA device `device` */
vkg_status vkg_ctx_create(int device, vkg_ctx **out);
vkg_status vkg_ctx_destroy(vkg_ctx *ctx);
/* last error message of this context ("" if none); valid until the next call on ctx */
const char *vkg_last_error(const vkg_ctx *ctx);

/* ---- geometry generators (host, deterministic) ----------------------------------------------
 * replaces Geometry::IcoSphere(radius, tessellation), Geometry.hpp:149 / Geometry.cpp:566-613:
 * 12 + 3 * sum(20 * 4^i, i < tess) unshared vertices, 20 * 4^tess triangles */
vkg_status vkg_geometry_icosphere_counts(uint32_t tess, uint32_t *num_vertices, uint32_t *num_tris);
vkg_status vkg_geometry_icosphere(float radius, uint32_t tess, float *xyz, uint32_t *indices);

/* Cornell box (5 quads over [-1,1]^3, open toward +z) + `num_spheres` cube-spheres of
 * 12 * n^2 triangles each with PCG32-drawn radius / centre / GGX material. Counts first, then
 * fill. per-triangle material id -> tri_material; materials: see vkg_material. */
/* Disney material record (the reference's material_struct_t, RayBuilder.hpp:40-116). A triangle whose material has transmission > 0 or diffuse_transmission > 0
   is never culled: rays leave such objects through their back faces. Texture slots index the scene's
   textures (vkg_scene_set_textures) or hold VKG_NO_TEXTURE; they take effect on meshes with texture
   coordinates (vkg_scene_set_texcoords) as the reference's closest-hit shader applies them
   (raypipeline.slang:526-606): colour multiplies base_color (rgb), emission multiplies a non-zero
   emission or replaces a zero one (rgb), ao_rough_metal multiplies roughness (g) and metalness (b),
   transmission multiplies transmission (r), diffuse_transmission multiplies diffuse_transmission (a),
   diffuse_transmission_color multiplies diffuse_transmission_color (rgb); normal: a tangent-space
   normal map (rg, needs tangents: vkg_scene_set_tangents). */
#define VKG_NO_TEXTURE 0xFFFFFFFFu
typedef struct vkg_material
{
    float base_color[3];
    float roughness;            /* perceptual roughness; the BSDF's alpha is max(0.001, roughness^2) */
    float metalness;
    float emission[3];
    uint32_t twosided;          /* 1: back faces are not culled (RayBuilder.cpp:521-522) */
    float transmission;         /* weight of the dielectric (refracting) lobe, [0, 1] */
    float ior;                  /* index of refraction of the interior; > 0 when transmission > 0 */
    float clearcoat;            /* clearcoat factor, >= 0 */
    float clearcoat_roughness;  /* alpha of the clearcoat's GTR2 term */
    float sheen_color[3];
    float sheen_roughness;
    float diffuse_transmission; /* share of the diffuse lobe sent through the surface, [0, 1] */
    float diffuse_transmission_color[3];
    float iridescence;          /* iridescence_strength: weight of the thin-film specular lobes, [0, 1] */
    float iridescence_ior;      /* the thin film's index of refraction (1.3) */
    float iridescence_thickness; /* film thickness in nm (the reference's thickness_range.y, 400) */
    /* homogeneous interior medium (Material.hpp:101-120): sigma_t = -log(attenuation_color) /
       attenuation_distance, single-scattering albedo from scatter_factor * scatter_color; a finite
       attenuation_distance or null_surface makes the material a medium boundary */
    float attenuation_color[3];  /* (0, 1], 1: no extinction */
    float attenuation_distance;  /* > 0, +inf: no medium */
    float scatter_color[3];      /* multi-scatter albedo tint, [0, 1] */
    float scatter_factor;        /* [0, 1] */
    float phase_g;               /* Henyey-Greenstein asymmetry, (-1, 1) */
    uint32_t null_surface;       /* 1: no surface interaction; emission becomes the medium's */
    /* chromatic dispersion (KHR_materials_dispersion, the reference's material_struct_t::dispersion,
       RayBuilder.hpp:99-100): 20 / Abbe number, >= 0; with transmission > 0 a path samples one
       wavelength in [400, 700] nm at such a surface and refracts with the Cauchy ior of that
       wavelength (ior at the d-line); the first transmission locks the wavelength for the rest of the
       path and tints its throughput by the wavelength's colour (raypipeline.slang:481-491, :651-659) */
    float dispersion;
    uint32_t tex_color, tex_normal, tex_emission, tex_ao_rough_metal, tex_transmission;
    uint32_t tex_diffuse_transmission, tex_diffuse_transmission_color;
    /* alpha masking / blending (material_struct_t color.a, blend_mode, alpha_cutoff,
       RayBuilder.hpp:42, :87-89; the any-hit stages, raypipeline.slang:686-720 and
       visibility_test.slang:45-87). A material with blend_mode VKG_BLEND_MASK or VKG_BLEND_BLEND that
       is not a null surface is tested at every candidate hit: alpha times the colour texture's alpha
       (level 0, at the hit's texture coordinates) is the coverage a. MASK: a < alpha_cutoff is no hit.
       BLEND: a < xi is no hit, xi uniform in [0, 1): for a path's extension ray the first uniform of
       the segment that shades the hit, the same for every candidate of the ray (the reference's
       any_hit draws from a copy of the payload's stream); for shadow rays an independent uniform per
       (ray, instance, triangle). Opaque materials ignore alpha. */
    float alpha;        /* base colour alpha, [0, 1] (1) */
    uint32_t blend_mode; /* VKG_BLEND_OPAQUE (0), VKG_BLEND_BLEND (1), VKG_BLEND_MASK (2): Material.hpp:32-37 */
    float alpha_cutoff; /* MASK threshold (0.5) */
    /* texture-coordinate transform: the entry's texture_matrix (raypipeline.slang:350), which the
       reference fills from the colour texture's KHR_texture_transform (gltf.cpp:162-194,
       RayBuilder.cpp:596-597, :633). With has_uv_transform != 0 every texture the closest-hit stage
       samples is read at (u', v') = (t0 u + t1 v + t2, t3 u + t4 v + t5); the coverage test and the
       texture LOD use the untransformed coordinates, as the reference's any_hit and lod_constant do. */
    uint32_t has_uv_transform; /* 0: identity (default) */
    float uv_transform[6];     /* row-major 2 x 3 */
} vkg_material; /* 208 B */
enum
{
    VKG_BLEND_OPAQUE = 0,
    VKG_BLEND_BLEND = 1,
    VKG_BLEND_MASK = 2
};
/* ---- analytic lights ----------------------------------------------------------------------
 * The reference's LightType (punctual_light.hpp:20-34); AREA is reserved for emissive triangles and
 * rejected here, as the reference leaves it out of the light list (PBRPathTracer.cpp:633-634). */
enum
{
    VKG_LIGHT_OMNI = 0,
    VKG_LIGHT_SPOT = 1,
    VKG_LIGHT_DIRECTIONAL = 2,
    VKG_LIGHT_AREA = 3,
    VKG_LIGHT_RECT = 4,
    VKG_LIGHT_SPHERE = 5,
    VKG_LIGHT_TUBE = 6,
    VKG_LIGHT_DISK = 7
};
/* the shader-side light record, same 80-byte layout as the reference's light_t
   (punctual_light.hpp:67-90, ray_common.slang:109-131) */
typedef struct vkg_light
{
    float position[3];
    uint32_t type;
    float color[3];
    float intensity;
    float direction[3];       /* propagation direction (unit); rect / disk emit along it, tube axis */
    float range;              /* omni / spot range window, +inf: pure inverse square */
    float spot_angle_scale;
    float spot_angle_offset;
    float angular_size;       /* directional: > 0 makes a sun disc of this cone half-angle (radians) */
    float size_y;             /* rect half-height, tube half-length */
    float tangent[3];         /* rect in-plane x axis (unit, orthogonal to direction) */
    float size_x;             /* sphere / disk / tube radius, rect half-width */
} vkg_light;                  /* 80 B */
/* a light-source asset (lightsource_t, punctual_light.hpp:43-57) */
typedef struct vkg_light_source
{
    uint32_t type;
    float color[3];
    float intensity;
    float range;              /* <= 0: +inf */
    float inner_cone_angle, outer_cone_angle;
    float size[2];            /* x: radius or rect half-width, y: rect half-height or tube half-length */
} vkg_light_source;
/* convert_light (punctual_light.hpp:92-111): place an asset with an object transform (row-major
   3x3 rotation, translation) */
vkg_status vkg_light_convert(const vkg_light_source *src, const float rotation[9], const float translation[3],
                             vkg_light *out);

/* fills *m with the reference's defaults: base colour 1, roughness 1, ior 1.5, diffuse-transmission colour 1,
   iridescence ior 1.3 and thickness 400 nm, attenuation colour 1 at +inf distance, scatter colour 1,
   alpha 1, alpha cutoff 0.5, no textures, everything else 0 */
vkg_status vkg_material_defaults(vkg_material *m);
vkg_status vkg_scene_cornell_counts(uint32_t num_spheres, uint32_t n, uint32_t *num_vertices, uint32_t *num_tris,
                                    uint32_t *num_materials);
vkg_status vkg_scene_cornell(uint64_t seed, uint64_t stream, uint32_t num_spheres, uint32_t n, float *xyz,
                             uint32_t *indices, uint32_t *tri_material, vkg_material *materials);

/* ---- camera rays ---------------------------------------------------------------------------- */
/* pinhole camera (raypipeline.slang:58-89 with projection.hpp:48-57, aperture 0) */
typedef struct vkg_camera
{
    float eye[3];
    float right[3], up[3], back[3]; /* camera-to-world rotation columns */
    float tan_half_fovy;            /* tan(fovy / 2), evaluated by the caller */
    float aspect;                   /* width / height */
    uint32_t width, height;
} vkg_camera;
/* look-at helper (host): forward = normalize(target - eye), right = normalize(forward x up) */
vkg_status vkg_camera_lookat(const float eye[3], const float target[3], const float up[3], float tan_half_fovy,
                             uint32_t width, uint32_t height, vkg_camera *out);
/* one jittered ray per pixel and sample: ray r = s*W*H + y*W + x uses PCG32(seed, stream) draws
 * 2r and 2r+1 as the sub-pixel offset. d_rays holds spp*W*H records. */
vkg_status vkg_camera_rays(vkg_ctx *ctx, const vkg_camera *cam, uint64_t seed, uint64_t stream, uint32_t spp,
                           vkg_ray *d_rays, void *stream_);

/* ---- BVH ------------------------------------------------------------------------------------- *
 * replaces RayBuilder::create_mesh_structures (BLAS build, RayBuilder.cpp:98-300,
 * vkCmdBuildAccelerationStructuresKHR :274) and compaction (:305-356): LBVH (30-bit Morton codes,
 * radix sort, Karras hierarchy, refit) collapsed to an 8-wide BVH with 8-bit quantised child
 * boxes, built entirely on the GPU. */
typedef struct vkg_bvh vkg_bvh;

typedef struct vkg_bvh_build_options
{
    uint32_t leaf_max; /* max triangles per leaf range, 1..16 (0 -> default 2) */
} vkg_bvh_build_options;

typedef struct vkg_bvh_info
{
    uint32_t num_tris, num_nodes, depth, leaf_max;
    float scene_min[3], scene_max[3], margin;
    size_t bytes;              /* device bytes held by the BVH */
    const void *d_nodes;       /* num_nodes x 96 B nodes */
    const void *d_tris;        /* num_tris x 48 B triangle records (sorted order) */
    const uint32_t *d_morton;  /* num_tris Morton codes, input order */
    const uint32_t *d_sorted;  /* num_tris triangle ids, sorted order */
    float build_ms;            /* GPU time of the last build */
} vkg_bvh_info;

/* builds from device vertex (fp32 xyz) and index (uint32, 3 per triangle) buffers. Synchronises
 * `stream` before returning (the node count is needed on the host). */
vkg_status vkg_bvh_build(vkg_ctx *ctx, const float *d_xyz, uint32_t num_vertices, const uint32_t *d_indices,
                         uint32_t num_tris, const vkg_bvh_build_options *opts, vkg_bvh **out, void *stream);
vkg_status vkg_bvh_info_get(const vkg_bvh *bvh, vkg_bvh_info *out);

/* Allocation-free BVH build. No counterpart in the reference: it exists for callers that cannot
 * allocate device memory once they are running -- for example an engine that carves all of its
 * device memory out of one arena at start-up, or code that records work where an allocation would
 * synchronise the device. It produces the same nodes and triangle records as vkg_bvh_build, but
 * keeps every temporary in one fixed device array inside libvkg (about 2.2 MB, held by each GPU
 * that loads the library until the process exits) and calls no allocator.
 *   - at most VKG_NOALLOC_MAX_TRIS triangles; larger inputs return VKG_ERR_CAPACITY
 *   - the caller provides d_nodes (node_capacity >= num_tris nodes of 96 B, 16-byte aligned),
 *     d_tris (num_tris records of 48 B, 16-byte aligned) and d_info (16 uint32 words, device):
 *     [0] node count, [1] depth, [2] error flags (1: an index >= num_vertices, 2: node capacity,
 *     4: the tree is deeper than the library's traversal supports -- vkg_bvh_build refuses such a
 *     tree with VKG_ERR_CAPACITY), [3] box margin (float bits), [4..6] scene min, [7..9] scene max
 *   - works on the current CUDA device; its first call on a device looks up the array's device
 *     address (cudaGetSymbolAddress), so make that first call before any stream capture; the
 *     address is kept per device for the life of the process and assumes the device's primary
 *     context (after cudaDeviceReset, or under another context made current through the driver
 *     API, it is stale)
 *   - all calls share the one array: calls that overlap on the GPU (other streams, other threads)
 *     race and must be serialised by the caller
 *   - asynchronous on `stream`; no vkg_ctx (no error message: the status code says what failed) */
#define VKG_NOALLOC_MAX_TRIS 16384u
vkg_status vkg_bvh_build_noalloc(const float *d_xyz, uint32_t num_vertices, const uint32_t *d_indices,
                                 uint32_t num_tris, uint32_t leaf_max, void *d_nodes, uint32_t node_capacity,
                                 void *d_tris, uint32_t *d_info, void *stream);
vkg_status vkg_bvh_destroy(vkg_ctx *ctx, vkg_bvh *bvh);

/* ---- bulk ray queries (replaces TraceRay / RayQuery, raypipeline.slang:182, visibility_test.slang:45-87)
 * closest hit: accepts Moeller-Trumbore INTERSECT results with tmin < t < tmax, keeps the smallest t,
 * ties -> smaller triangle id; hit ids are bit-identical to a brute-force loop over
 * intersect(Triangle, Ray). any hit: d_occluded[i] = 1 if any such hit exists. */
enum
{
    VKG_RAY_CULL_BACK_FACES = 1u, /* RAY_FLAG_CULL_BACK_FACING_TRIANGLES: reject det < 0 (clockwise seen from origin) */
    VKG_RAY_COUNT_STATS = 2u,     /* also count node visits / triangle tests (slower; see vkg_ray_stats_get) */
    VKG_RAY_KEEP_ORDER = 4u       /* trace in the given order: no binning of large batches (below) */
};
/* Batches of 2^19 rays or more are traced in bins: rays are grouped by the cell of the scene box
 * (8 x 8 x 8) that holds their origin and by their direction (64 octahedral bins), and each group is
 * traced together; tiles of rays that are coherent already (most runs of 32 consecutive rays in one
 * bin, as camera rays are) keep their order. Results, counters and error flags are those of tracing
 * in the given order; only the speed differs. The context keeps the scratch (8 B per ray plus 128 KB
 * per SM-sized tile, grown on demand; calls on different streams are ordered by an event). Calls made
 * while the stream is being captured into a CUDA graph, calls with VKG_RAY_KEEP_ORDER, calls whose
 * scratch cannot be allocated, and the host variant's 2^20-ray chunks trace in the given order. */
vkg_status vkg_closest_hit(vkg_ctx *ctx, const vkg_bvh *bvh, const vkg_ray *d_rays, uint32_t num_rays,
                           vkg_hit *d_hits, uint32_t flags, void *stream);
vkg_status vkg_any_hit(vkg_ctx *ctx, const vkg_bvh *bvh, const vkg_ray *d_rays, uint32_t num_rays,
                       uint32_t *d_occluded, uint32_t flags, void *stream);
/* host-buffer variant: copies rays host->device, traces, copies hits device->host, synchronises.
 * h_rays / h_hits may be pinned or pageable host memory. */
vkg_status vkg_closest_hit_host(vkg_ctx *ctx, const vkg_bvh *bvh, const vkg_ray *h_rays, uint32_t num_rays,
                                vkg_hit *h_hits, uint32_t flags, void *stream);
/* node visits / triangle tests accumulated by launches with VKG_RAY_COUNT_STATS since the last reset */
vkg_status vkg_ray_stats_get(vkg_ctx *ctx, uint64_t *node_visits, uint64_t *tri_tests, int reset);


/* ---- two-level BVH (instances over bottom-level BVHs) ------------------------------------------- *
 * RayBuilder::create_toplevel (RayBuilder.cpp:386-760) builds the driver TLAS over mesh entries that
 * carry a vk_transform_matrix (:518). Here the top level is the same 8-wide quantised BVH over the
 * instances' world boxes; a ray reaching an instance leaf is moved to object space (separately
 * rounded float operations) and traced through that instance's BLAS. Transforms with a negative
 * determinant mirror the geometry and therefore flip the back-face rule. */
typedef struct vkg_instance
{
    float transform[12]; /* object -> world, row-major 3x4 (VkTransformMatrixKHR layout) */
    uint32_t blas;       /* index into the BLAS array given to vkg_tlas_build */
    uint32_t material;   /* material index for the path tracer */
    uint32_t pad[2];
} vkg_instance;          /* 64 B */
/* closest hit of a two-level query; a miss has prim = instance = 0xFFFFFFFF. Closest-hit ties
 * (equal t) go to the smaller instance, then the smaller triangle. */
typedef struct vkg_inst_hit
{
    uint32_t prim;       /* triangle id within the instance's mesh */
    uint32_t instance;   /* input index of the instance */
    float t, u, v;
    uint32_t pad[3];
} vkg_inst_hit;          /* 32 B */
typedef struct vkg_tlas vkg_tlas;
typedef struct vkg_tlas_info
{
    uint32_t num_instances, num_blas, num_nodes, depth;
    float scene_min[3], scene_max[3];
    const void *d_nodes;           /* 96 B nodes */
    const void *d_instances;       /* 128 B records {w2o[12], o2w[12], blas, instance, material, pad[5]}, leaf order */
    const void *d_instances_by_id; /* the same records in input order */
    float build_ms;
} vkg_tlas_info;
/* d_instances: device array; the BLASes must outlive the TLAS. Synchronises like vkg_bvh_build. */
vkg_status vkg_tlas_build(vkg_ctx *ctx, const vkg_bvh *const *blas, uint32_t num_blas, const vkg_instance *d_instances,
                          uint32_t num_instances, const vkg_bvh_build_options *opts, vkg_tlas **out, void *stream);
vkg_status vkg_tlas_info_get(const vkg_tlas *tlas, vkg_tlas_info *out);
vkg_status vkg_tlas_destroy(vkg_ctx *ctx, vkg_tlas *tlas);
/* flags: VKG_RAY_CULL_BACK_FACES (object-space facing) */
vkg_status vkg_tlas_closest_hit(vkg_ctx *ctx, const vkg_tlas *tlas, const vkg_ray *d_rays, uint32_t n,
                                vkg_inst_hit *d_hits, uint32_t flags, void *stream);
vkg_status vkg_tlas_any_hit(vkg_ctx *ctx, const vkg_tlas *tlas, const vkg_ray *d_rays, uint32_t n, uint32_t *d_occluded,
                            uint32_t flags, void *stream);
/* stress workload generators (two-level scenes) */
/* cube-sphere of n x n quads per face: 6 (n+1)^2 vertices, 12 n^2 outward triangles */
vkg_status vkg_geometry_cubesphere(uint32_t n, float radius, float *xyz, uint32_t *indices);
/* terrain: n x n vertex grid over [-extent/2, extent/2]^2 (x, z), y = height * fBm, with `octaves`
 * octaves (lacunarity 2, gain 0.5) of 3-D simplex noise (the basis of shaders/slang/utils/simplex.slang)
 * at (x f, z f, seed offset); 2 (n-1)^2 triangles counter-clockwise seen from +y */
vkg_status vkg_geometry_terrain(uint32_t n, float extent, float height, float frequency, uint32_t octaves,
                                uint32_t seed, float *xyz, uint32_t *indices);
/* n random instances from PCG32(seed, stream): translation U[lo, hi], uniform rotation, scale
 * U[smin, smax], mesh U{0..num_meshes-1}, material mat_base + U{0..num_mats-1} */
vkg_status vkg_instances_random(uint64_t seed, uint64_t stream, uint32_t n, uint32_t num_meshes, uint32_t mat_base,
                                uint32_t num_mats, const float lo[3], const float hi[3], float smin, float smax,
                                vkg_instance *out);

/* ---- environment map ------------------------------------------------------------------------ *
 * Equirectangular fp32 RGB, u = 0.5 + 0.5 * atan2(x, -z) / pi, v = acos(y) / pi
 * (shaders/slang/unlit/panorama.slang:12-15), texel (i, j) at d_rgb[3 * (j * width + i)].
 * Procedural sky: procedural_environment.slang:7-11 (environment_white) plus a sun lobe
 * sun_peak * exp((dot(d, sun_dir) - 1) / sun_width) evaluated at each texel centre. */
vkg_status vkg_env_procedural_sky(vkg_ctx *ctx, uint32_t width, uint32_t height, const float sun_dir[3],
                                  float sun_peak, float sun_width, float *d_rgb, void *stream);

/* ---- scene (replaces RayBuilder::build_scene_acceleration + the trace_data buffers,
 *      src/RayBuilder.cpp:784, PBRPathTracer.cpp:529-653) ----------------------------------------
 * One triangle mesh with per-triangle material ids, a material table and an environment map. The
 * scene copies what it needs (the caller's buffers may be freed afterwards), builds the BVH, marks
 * two-sided triangles and builds the environment's importance-sampling tables (FP64 prefix sums
 * + alias table). Synchronises `stream`. */
typedef struct vkg_scene vkg_scene;
typedef struct vkg_scene_desc
{
    const float *d_xyz;
    uint32_t num_vertices;
    const uint32_t *d_indices;
    uint32_t num_tris;
    const uint32_t *d_tri_material; /* per triangle, index into d_materials */
    const vkg_material *d_materials;
    uint32_t num_materials;
    const float *d_env_rgb; /* equirect map, env_width x env_height x 3 fp32 */
    uint32_t env_width, env_height;
    uint32_t leaf_max; /* BVH leaf size (0 -> 2) */
} vkg_scene_desc;
vkg_status vkg_scene_create(vkg_ctx *ctx, const vkg_scene_desc *desc, vkg_scene **out, void *stream);
/* instanced scenes (RayBuilder's BLAS-per-mesh + TLAS-over-entries layout, RayBuilder.cpp:98-300,
 * :386-760): meshes are copied and get one BVH each, the instances (device array; material indexes
 * d_materials) a two-level BVH. Mesh triangles are one-sided unless the mesh is flagged two-sided. */
typedef struct vkg_mesh_desc
{
    const float *d_xyz;     /* position of vertex k at byte offset k * vertex_stride */
    uint32_t num_vertices;
    const uint32_t *d_indices;
    uint32_t num_tris;
    uint32_t twosided;
    uint32_t vertex_stride; /* bytes between positions, a multiple of 4 (0: 12, packed xyz; 24: the
                               reference's packed_vertex_t, packed_vertex.slang:17-23) */
} vkg_mesh_desc;
typedef struct vkg_instanced_scene_desc
{
    const vkg_mesh_desc *meshes; /* host array */
    uint32_t num_meshes;
    const vkg_instance *d_instances;
    uint32_t num_instances;
    const vkg_material *d_materials;
    uint32_t num_materials;
    const float *d_env_rgb;
    uint32_t env_width, env_height;
    uint32_t leaf_max; /* BVH leaf size of the meshes (0 -> 2) */
} vkg_instanced_scene_desc;
vkg_status vkg_scene_create_instanced(vkg_ctx *ctx, const vkg_instanced_scene_desc *desc, vkg_scene **out,
                                      void *stream);
/* the two-level BVH of an instanced scene (NULL for a single-level scene) */
vkg_status vkg_scene_tlas(const vkg_scene *scene, const vkg_tlas **out);
vkg_status vkg_scene_destroy(vkg_ctx *ctx, vkg_scene *scene);
/* Vertex normals for smooth shading (interpolate_vertex, raypipeline.slang:336-360): the shading
 * normal of a hit is the vertex normals interpolated with the barycentric weights (1 - u - v, u, v),
 * normalised and turned to the side the ray hit; without them (the default) it is the face normal.
 * mesh: 0 for a single-level scene, the mesh index of an instanced scene. d_src: device records at
 * `stride` bytes (0: packed) of `format` -- VKG_NORMALS_FLOAT3 (3 floats, normalised on upload) or
 * VKG_NORMALS_OCT_SNORM16 (the octahedral snorm16 pair of packed_vertex_t, packed_vertex.slang:17-23:
 * pass the vertex buffer + 12 and stride 24); one record per vertex of the mesh; NULL removes them.
 * Copied; waits for the device, then synchronises `stream`. */
enum
{
    VKG_NORMALS_FLOAT3 = 0u,
    VKG_NORMALS_OCT_SNORM16 = 1u
};
vkg_status vkg_scene_set_normals(vkg_ctx *ctx, vkg_scene *scene, uint32_t mesh, const void *d_src, uint32_t stride,
                                 uint32_t format, void *stream);
/* Vertex tangents for normal maps (utils::Vertex::tangent): the same formats and rules as the normals;
 * the bitangent is normalize(cross(normal, tangent)), negated for back faces (raypipeline.slang:545-549). */
vkg_status vkg_scene_set_tangents(vkg_ctx *ctx, vkg_scene *scene, uint32_t mesh, const void *d_src, uint32_t stride,
                                  uint32_t format, void *stream);
/* Texture coordinates (utils::Vertex::tex_coord), interpolated with the barycentric weights:
 * VKG_TEXCOORD_FLOAT2 (two floats) or VKG_TEXCOORD_HALF2 (two fp16, packed_vertex_t: vertex buffer + 20,
 * stride 24) at `stride` bytes (0: packed); NULL removes them (textures are then not sampled). */
enum
{
    VKG_TEXCOORD_FLOAT2 = 0u,
    VKG_TEXCOORD_HALF2 = 1u
};
vkg_status vkg_scene_set_texcoords(vkg_ctx *ctx, vkg_scene *scene, uint32_t mesh, const void *d_src, uint32_t stride,
                                   uint32_t format, void *stream);
/* The scene's textures (replacing any before): RGBA8 texels read as UNORM (the reference's textures
 * are R8G8B8A8_UNORM, model_loading.cpp:12-24), row-major from the host, copied. Each gets a full mip
 * chain (level k + 1 = the rounded mean of 2 x 2 texels of level k, the last row / column repeated for
 * odd sizes) and is sampled trilinearly at level lambda = lod_constant + log2(cone width) +
 * 0.5 log2(width * height) - log2(|N.V|) (sample_texture_lod, lod_constant, raypipeline.slang:
 * 299-320; the ray cone starts at width 0 with the camera's pixel spread angle and grows by spread x t
 * after each surface, :113-114, :280-286, :608), lambda clamped to the chain; texel centres at
 * (i + 0.5) / width; wrap per axis. */
enum
{
    VKG_WRAP_REPEAT = 0u,
    VKG_WRAP_CLAMP_TO_EDGE = 1u,
    VKG_WRAP_MIRRORED_REPEAT = 2u
};
typedef struct vkg_texture_desc
{
    const uint8_t *h_rgba8; /* width * height * 4 bytes */
    uint32_t width, height;
    uint32_t wrap_s, wrap_t;
} vkg_texture_desc;
vkg_status vkg_scene_set_textures(vkg_ctx *ctx, vkg_scene *scene, const vkg_texture_desc *textures, uint32_t n,
                                  void *stream);
/* the scene's analytic lights (host array, copied; n = 0 removes them). Directions and tangents are
   normalised; the sun of the tracer settings comes first in the light list of a render. */
vkg_status vkg_scene_set_lights(vkg_ctx *ctx, vkg_scene *scene, const vkg_light *lights, uint32_t n);
/* the scene's BVH (owned by the scene) for direct ray queries */
vkg_status vkg_scene_bvh(const vkg_scene *scene, const vkg_bvh **out);
/* device views of the environment sampling tables: per texel normalised weight (mean 1, fp32) and
 * alias buckets {fp32 probability, uint32 alias} (8 B each) */
vkg_status vkg_scene_env_tables(const vkg_scene *scene, const float **d_weights, const void **d_alias,
                                uint32_t *width, uint32_t *height);

/* ---- path tracer (replaces PBRPathTracer, include/vierkant/PBRPathTracer.hpp:37-386) ---------- */
/* a homogeneous medium given directly (the reference's medium_params_t, include/vierkant/media.hpp:26-49,
   converted as to_media does, src/media.cpp:6-23): sigma_t = -log(attenuation_color) /
   attenuation_distance, single-scattering albedo from scatter_factor x scatter_color (Kulla-Conty),
   emitted radiance emission_color x emission_intensity */
typedef struct vkg_medium_params
{
    float attenuation_color[3]; /* (0.7, 0.7, 0.7), each in (0, 1] */
    float attenuation_distance; /* 1, finite and > 0 */
    float scatter_factor;       /* 0, in [0, 1] */
    float scatter_color[3];     /* (1, 1, 1), each in [0, 1] */
    float phase_g;              /* 0, in (-1, 1) */
    float ior;                  /* 1 */
    float emission_color[3];    /* (1, 1, 1) */
    float emission_intensity;   /* 0 */
} vkg_medium_params;            /* 56 B */
vkg_status vkg_medium_params_default(vkg_medium_params *out);
enum
{
    VKG_CAMERA_MEDIUM_DETECT = 0, /* the reference's default (PBRPathTracer.cpp:471-525, :598-605): in an
                                     instanced scene, the material of the smallest instance whose world
                                     box (its mesh's box under the instance transform) contains the eye
                                     and whose material has a finite attenuation distance; else vacuum */
    VKG_CAMERA_MEDIUM_GIVEN = 1,  /* settings.camera_medium (settings_t::camera_medium set) */
};
/* PBRPathTracer::settings_t (PBRPathTracer.hpp:42-110): the fields of the traced path */
typedef struct vkg_settings
{
    uint32_t resolution[2];           /* {1280, 720} */
    uint32_t max_num_batches;         /* 0 = no limit */
    uint32_t num_samples;             /* samples per pixel per batch (one render call = one batch) */
    uint32_t max_trace_depth;         /* path segments including the camera ray (6) */
    float max_path_beta;              /* clamp of indirect throughput, 0 = off */
    uint32_t suspend_trace_when_done; /* render is a no-op once max_num_batches batches are done */
    uint32_t disable_material;        /* override base colours with 0.8 */
    uint32_t mis_mode;                /* 0 = MIS, 1 = NEE only, 2 = BSDF only */
    uint32_t draw_skybox;             /* camera rays that miss show the environment */
    float environment;                /* environment radiance factor (Scene::environment_factor) */
    uint32_t rr_start_depth;          /* Russian roulette from this surface interaction on
                                         (q = 1 - max(beta)); 0 = the reference's rule
                                         max(beta) <= 0.05 * depth (raypipeline.slang:668-677) */
    uint32_t crop[4];                 /* x0, y0, width, height of the traced window (0 size: full) */
    uint32_t samples_per_wave;        /* paths in flight = pixels x this (0 = automatic) */
    uint32_t suppress_refractive_caustics; /* drop light-body / sun hits on refractive-caustic paths */
    /* sunlight_params_t (PBRPathTracer.hpp:23-33): a directional light folded in as light 0 when
       sun_intensity > 0; direction from (elevation, azimuth) as the reference's quaternion does */
    float sun_color[3];
    float sun_intensity;
    float sun_spherical_coords[2];    /* elevation, azimuth (radians) */
    float sun_angular_size;           /* cone half-angle of the disc (radians); 0: a delta light */
    uint32_t denoising;               /* settings_t::denoising: the output is the a-trous filtered image */
    float clip_near;                  /* the camera's near clipping distance, for the pixel depth
                                         near / view-space distance (camera_params.hpp:37); 0: 0.1 */
    /* the medium the camera sits in (paths start with it on their media stack,
       raypipeline.slang:128-135): VKG_CAMERA_MEDIUM_DETECT or VKG_CAMERA_MEDIUM_GIVEN */
    uint32_t camera_medium_mode;
    vkg_medium_params camera_medium;  /* used when camera_medium_mode = VKG_CAMERA_MEDIUM_GIVEN */
    /* random streams: VKG_RNG_PCG32 (0, default): PCG32 per path, initstate = the create-info seed,
       initseq = (batch << 40) ^ (sample * pixels + pixel); VKG_RNG_REFERENCE (1): the reference
       shaders' streams. In the latter, render call k takes the k-th output of the create-info
       seed's std::minstd_rand0 (std::default_random_engine of libstdc++ and libc++,
       PBRPathTracer.cpp:32, :588) as the batch seed; a pixel (x, y) of the full resolution starts
       the chain xxhash32(batch seed, width * y + x) (raypipeline.slang:95), draws its sub-pixel
       offset 2 rnd() - 1 (:100); each sample s of N draws the lens sample (2 rnd(), unused by a
       pinhole) and jitters by frac(Hammersley(s, N) + offset) (:102-108, sampling.slang:9-13); segment
       i hashes the chain with i (:150) and takes its uniforms from the LCG rnd() started at the
       chain (random.slang:27-36). The samples of a pixel continue one chain, so one sample per pixel
       is traced per wave (samples_per_wave is ignored). Not with a radiance cache. The estimator's
       use of the uniforms (8 per segment, one per decision) is the library's either way. */
    uint32_t rng_mode;
} vkg_settings;
enum
{
    VKG_RNG_PCG32 = 0,
    VKG_RNG_REFERENCE = 1
};
/* the camera medium a render of `scene` seen from `eye` would detect: the material index, or
   0xFFFFFFFF for vacuum (always vacuum for single-level scenes, which have no objects) */
vkg_status vkg_scene_camera_medium(const vkg_scene *scene, const float eye[3], uint32_t *material);

/* ---- glTF 2.0 ingestion (host only; the reference's model/gltf.cpp path) --------------------
 * vkg_gltf_load reads a .gltf (base64 or file buffers) or .glb file into meshes (one per triangle
 * primitive; float positions, uint32 indices, optional normals / texture coordinates / tangents),
 * instances (node placements, object -> world 3x4, mesh index in `blas`, material), materials
 * (vkg_material, texture slots indexing the asset's textures; alphaMode / alphaCutoff / the base
 * colour's alpha into blend_mode / alpha_cutoff / alpha; the colour texture's KHR_texture_transform
 * into uv_transform), textures (PNG and JPEG images decoded to RGBA8)
 * and KHR_lights_punctual lights (vkg_light); those feed vkg_scene_create_instanced,
 * vkg_scene_set_normals / _texcoords / _tangents / _textures and vkg_scene_set_lights. Errors: a status and
 * the message in err (may be NULL). The mesh pointers stay valid until vkg_gltf_destroy. */
typedef struct vkg_gltf vkg_gltf;
typedef struct vkg_gltf_counts
{
    uint32_t num_meshes, num_instances, num_materials, num_lights;
    uint32_t skipped_primitives; /* non-triangle primitives left out */
    uint32_t num_textures;       /* glTF textures (vkg_gltf_textures) */
    uint32_t skipped_textures;   /* textures whose image is neither a PNG nor a JPEG this loader decodes
                                    (their material slots are empty) */
} vkg_gltf_counts;
vkg_status vkg_gltf_load(const char *path, vkg_gltf **out, char *err, size_t err_len);
vkg_status vkg_gltf_counts_get(const vkg_gltf *g, vkg_gltf_counts *out);
vkg_status vkg_gltf_mesh(const vkg_gltf *g, uint32_t index, const float **xyz, uint32_t *num_vertices,
                         const uint32_t **indices, uint32_t *num_tris);
/* the mesh's vertex normals (3 floats per vertex, the primitive's NORMAL attribute) or NULL when the
   primitive has none; for vkg_scene_set_normals */
vkg_status vkg_gltf_mesh_normals(const vkg_gltf *g, uint32_t index, const float **normals);
/* the mesh's TEXCOORD_0 (2 floats per vertex) / tangents (3 floats per vertex: TANGENT xyz, or computed
   from NORMAL and TEXCOORD_0 as Geometry::compute_tangents does) or NULL; for vkg_scene_set_texcoords /
   vkg_scene_set_tangents */
vkg_status vkg_gltf_mesh_texcoords(const vkg_gltf *g, uint32_t index, const float **uv);
vkg_status vkg_gltf_mesh_tangents(const vkg_gltf *g, uint32_t index, const float **tangents);
/* the asset's textures (num_textures records; texel pointers valid until vkg_gltf_destroy), in glTF
   texture order, which the materials' texture slots index: for vkg_scene_set_textures */
vkg_status vkg_gltf_textures(const vkg_gltf *g, vkg_texture_desc *out);
vkg_status vkg_gltf_instances(const vkg_gltf *g, vkg_instance *out);
vkg_status vkg_gltf_materials(const vkg_gltf *g, vkg_material *out);
vkg_status vkg_gltf_lights(const vkg_gltf *g, vkg_light *out);
vkg_status vkg_gltf_destroy(vkg_gltf *g);

/* ---- RayBuilder wire records (host only) ----------------------------------------------------
 * The byte images RayBuilder uploads for its ray pipeline, read as they are: the C++ layouts of
 * RayBuilder::material_struct_t (RayBuilder.hpp:40-116) and RayBuilder::entry_t (RayBuilder.hpp:24-37)
 * with glm's default packing, which equal their shader twins' std430 layouts (ray/types.slang:17-32,
 * :64-110; the shader pads both to a multiple of 16 bytes). */
#define VKG_WIRE_MATERIAL_BYTES 208u
#define VKG_WIRE_ENTRY_BYTES 192u
/* material_struct_t -> vkg_material: colour rgb, emission rgb x emission.a (the emissive strength, as
   the closest-hit shader multiplies them), the scalar lobes, sheen colour rgb, iridescence strength /
   ior and the thickness range's maximum (what the shader reads), the media fields and two_sided.
   The texture slots take the index of each texture whose TextureTypeBits flag is set (colour, normal,
   ao_rough_metal, emission, transmission, diffuse transmission and its colour; types.slang:35-51),
   VKG_NO_TEXTURE otherwise. Colour alpha, blend mode and alpha cutoff are read into alpha,
   blend_mode and alpha_cutoff (a blend mode other than 0-2 reads as opaque). The textures the tracer
   does not sample (displacement, thickness, clearcoat, sheen, iridescence) are dropped; *dropped (may
   be NULL) counts the records that use any of them or an unknown blend mode. Dispersion is read into
   vkg_material::dispersion. */
vkg_status vkg_materials_from_wire(const void *records, uint32_t n, vkg_material *out, uint32_t *dropped);
/* per entry: where its triangles are in the mesh buffers */
typedef struct vkg_wire_entry_info
{
    uint32_t buffer_index;  /* the mesh (vertex / index buffer pair) */
    uint32_t base_index;    /* first index of the entry in the index buffer */
    int32_t vertex_offset;  /* added to every index */
    float aabb_min[3], aabb_max[3]; /* object-space box */
    /* the entry's texture_matrix (RayBuilder.hpp:26, applied to (u, v, 0, 1)) as vkg_material's
       uv_transform: a caller copies it into the entry's material (has_uv_transform = 0 when identity) */
    uint32_t has_uv_transform;
    float uv_transform[6];
} vkg_wire_entry_info;
/* entry_t -> vkg_instance: object -> world = T R S of the entry's transform_t (translation, rotation
   quaternion stored x y z w, scale; the shader's apply_transform, utils/transform.slang:19-24) as a
   row-major 3x4, blas = buffer_index, material = material_index. info (may be NULL): n records. */
vkg_status vkg_instances_from_wire(const void *records, uint32_t n, vkg_instance *out, vkg_wire_entry_info *info);

/* per-pixel output record, the layout of the reference's pixel_data_t (pixel_data.slang:9-21):
   accumulated radiance, coverage of the last batch, reversed-z depth, primary-hit normal
   (octahedral, two snorm16), object id (0xFFFF on a miss), primary-hit albedo (RGBA8) — the
   G-buffer fields come from each pixel's last sample, as the reference's raygen loop leaves them */
typedef struct vkg_pixel_data
{
    float radiance[3];
    float alpha;
    float depth;
    uint32_t normal;
    uint32_t object_id;
    uint32_t albedo;
} vkg_pixel_data; /* 32 B */

typedef struct vkg_tracer_create_info
{
    uint32_t seed; /* create_info_t::seed (PBRPathTracer.hpp:138) */
    vkg_settings settings;
} vkg_tracer_create_info;

/* statistics_t / timings_t (PBRPathTracer.hpp:112-127) of the last render */
typedef struct vkg_tracer_stats
{
    double raytrace_ms;
    double total_ms;
    uint64_t paths;
    uint64_t extension_rays;
    uint64_t shadow_rays;
    uint32_t batch;
    uint32_t pad;
    double train_ms;         /* radiance-cache training inside total_ms (0 without a cache) */
    uint64_t cache_queries;  /* rendering paths that ended in the radiance cache */
    uint64_t train_records;  /* training records (path vertices with targets) of the last render */
} vkg_tracer_stats;

typedef struct vkg_tracer vkg_tracer;
vkg_status vkg_settings_default(vkg_settings *out);
/* the pixel records of the traced window (crop) after the last render: d_out holds width x height */
vkg_status vkg_tracer_pixel_data(vkg_tracer *tracer, vkg_pixel_data *d_out, void *stream);
/* bloom + tonemap composition of an HDR rgba image (PBRPathTracer.cpp:405-465): bloom of the
   half-resolution luma-thresholded image blurred by `blur_iterations` separable 9-tap Gaussian passes
   (RGBA16F intermediates), then 1 - exp(-(hdr + bloom) * exposure) and pow(., 1 / gamma); tonemap = 0
   copies the HDR image */
typedef struct vkg_post_fx_settings
{
    uint32_t tonemap, bloom;   /* settings_t::tonemap / bloom */
    float exposure, gamma;     /* settings_t::exposure (2) / gamma (1) */
    float brightness_thresh[2]; /* Bloom::create_info_t::brightness_thresh (0.95, 1.1) */
    uint32_t blur_iterations;  /* 3 (PBRPathTracer.cpp:799) */
} vkg_post_fx_settings;
vkg_status vkg_post_fx_default(vkg_post_fx_settings *s);
vkg_status vkg_post_fx(vkg_ctx *ctx, const float *d_hdr_rgba, uint32_t width, uint32_t height,
                       const vkg_post_fx_settings *s, float *d_out_rgba, void *stream);

/* the reference's denoise pass (PBRPathTracer.cpp:346-403, denoise.slang): five edge-avoiding
   a-trous passes (steps 1, 2, 4, 8, 16) over albedo-demodulated radiance with luminance, normal and
   depth weights; d_out_rgba: width x height x 4 floats (alpha 0, as the shader writes), d_out_depth
   (may be NULL): the pixels' depth */
vkg_status vkg_denoise(vkg_ctx *ctx, const vkg_pixel_data *d_pixels, uint32_t width, uint32_t height,
                       float *d_out_rgba, float *d_out_depth, void *stream);
/* PBRPathTracer::create (PBRPathTracer.hpp:144) */
vkg_status vkg_tracer_create(vkg_ctx *ctx, const vkg_tracer_create_info *info, vkg_tracer **out);
vkg_status vkg_tracer_set_settings(vkg_tracer *tracer, const vkg_settings *settings);
vkg_status vkg_tracer_get_settings(const vkg_tracer *tracer, vkg_settings *out);
/* PBRPathTracer::render_scene (PBRPathTracer.hpp:161): traces one batch of num_samples paths per
 * pixel of the crop window and blends it into the running mean (new + b * old) / (b + 1)
 * (raypipeline.slang:258-266). d_rgb_out (crop width x height x 3 fp32, may be NULL) receives the
 * accumulated image. Asynchronous on `stream`. */
vkg_status vkg_tracer_render(vkg_tracer *tracer, const vkg_scene *scene, const vkg_camera *camera, float *d_rgb_out,
                             void *stream);
/* PBRPathTracer::reset_accumulator / current_batch (PBRPathTracer.hpp:169-174) */
vkg_status vkg_tracer_reset_accumulator(vkg_tracer *tracer);
vkg_status vkg_tracer_current_batch(const vkg_tracer *tracer, uint32_t *out);
/* PBRPathTracer::statistics (PBRPathTracer.hpp:179); waits for the last render */
vkg_status vkg_tracer_statistics(vkg_tracer *tracer, vkg_tracer_stats *out);
vkg_status vkg_tracer_destroy(vkg_tracer *tracer);


/* ---- batched uneven rendering (not in the reference) ------------------------------------------ *
 * Many (scene, camera, settings) jobs of uneven size rendered together: the paths of all jobs share
 * one set of wavefront queues (every path carries its job index), waves are packed from whole
 * samples of the jobs, and a render is one CUDA-graph launch. Each job's image equals what
 * vkg_tracer_render would produce for it alone with the same seed and settings (same PCG32 streams,
 * same per-pixel summation order; textures and alpha-tested materials included). No radiance cache
 * and no media in batch mode. */
typedef struct vkg_batch vkg_batch;
typedef struct vkg_batch_job
{
    const vkg_scene *scene;
    vkg_camera camera;        /* camera->width / height must equal settings.resolution */
    vkg_settings settings;    /* resolution, crop, num_samples, max_trace_depth, rr_start_depth, ... */
    uint32_t seed;            /* PBRPathTracer create-info seed of this job */
    uint32_t pad;
    float *d_rgb_out;         /* crop width x height x 3 fp32 running mean (device; may be NULL) */
} vkg_batch_job;
typedef struct vkg_batch_tuning
{
    uint32_t extend_kernel;   /* 1: grid-stride queue kernels, 2: persistent work-stealing tracers */
    uint32_t ctas_per_sm;     /* grid of the grid-stride queue kernels = SMs x this */
    uint32_t wave_paths;      /* paths in flight per wave */
    uint32_t use_graph;       /* 1: capture a render as a CUDA graph and replay it */
    uint32_t block_size;      /* threads per block of the queue kernels: 64 or 128 */
    uint32_t stack_depth;     /* traversal stack entries: 64 (used when every BVH is at most 10 deep) or 128 */
} vkg_batch_tuning;
typedef struct vkg_batch_stats
{
    double render_ms;         /* GPU time of the last render */
    uint64_t paths;
    uint64_t extension_rays;
    uint64_t shadow_rays;
    uint32_t waves;           /* waves per render */
    uint32_t batch;           /* renders accumulated */
} vkg_batch_stats;
vkg_status vkg_batch_tuning_default(vkg_batch_tuning *out);
/* jobs are copied; the scenes and output buffers must outlive the batch */
vkg_status vkg_batch_create(vkg_ctx *ctx, const vkg_batch_job *jobs, uint32_t njobs, const vkg_batch_tuning *tuning,
                            vkg_batch **out);
/* times every candidate tuning on a one-sample-per-job render and keeps the fastest (*chosen, optional,
 * receives it); the accumulation is reset. Synchronises. */
vkg_status vkg_batch_autotune(vkg_batch *batch, void *stream, vkg_batch_tuning *chosen);
vkg_status vkg_batch_set_tuning(vkg_batch *batch, const vkg_batch_tuning *tuning);
/* one batch of num_samples paths per pixel for every job, blended into each job's running mean */
vkg_status vkg_batch_render(vkg_batch *batch, void *stream);
vkg_status vkg_batch_reset_accumulator(vkg_batch *batch);
vkg_status vkg_batch_statistics(vkg_batch *batch, vkg_batch_stats *out);
vkg_status vkg_batch_destroy(vkg_batch *batch);

/* ---- neural radiance cache (not in the reference) -------------------------------------------- *
 * A small MLP (80 inputs -> 5 hidden layers of 64, ReLU -> RGB; BF16 weights and activations, FP32
 * accumulation) over a multiresolution hash grid (position) and degree-4 spherical harmonics
 * (outgoing direction, normal) plus roughness and albedo, trained online with a relative-L2 loss
 * and Adam. Feature records are 13 floats: position xyz, outgoing direction xyz, normal xyz,
 * roughness, albedo rgb. */
typedef struct vkg_nrc vkg_nrc;
typedef struct vkg_nrc_config
{
    uint32_t levels;          /* hash-grid levels (16) */
    uint32_t log2_table_size; /* entries per level = 2^this (19) */
    uint32_t base_resolution; /* coarsest grid resolution (16) */
    uint32_t max_resolution;  /* finest grid resolution (2048) */
    float learning_rate;      /* Adam (1e-2) */
    float beta1, beta2, epsilon;
    uint32_t seed;
    float scene_min[3], scene_max[3]; /* positions are normalised to this box */
    uint32_t batch_size;      /* training samples per optimiser step (65536) */
    uint32_t train_paths;     /* training paths traced per frame (65536) */
    uint32_t terminate_depth; /* rendering paths end in the cache at this surface interaction (2) */
    uint32_t train_depth;     /* training targets are recorded at the first this-many interactions (4) */
    uint32_t train_steps;     /* optimiser steps per frame; 0: ceil(train_paths * train_depth / batch_size) */
    uint32_t infer_kernel;    /* 0: default (2), 1: mma.sync MLP, 2: tcgen05 MLP, 3: tcgen05 MLP with the encoding fused */
    uint32_t train_kernel;    /* 0: default (3), 1: mma.sync forward / backward + FP32 CUDA-core weight
                                 gradients, 2: mma.sync forward / backward + tcgen05 weight gradients,
                                 3: everything on tcgen05 (forward, backward through the layers, weight
                                 gradients) */
} vkg_nrc_config;
typedef struct vkg_nrc_info_t
{
    uint32_t levels, table_size;
    float growth;
    uint32_t level_resolution[16];
    uint32_t num_mlp_params;
    uint64_t num_grid_params;
    float *d_mlp_params;  /* FP32 master weights, layer l is [in][out] row-major */
    float *d_grid_params; /* FP32 master hash-grid features [level][entry][2] */
    float *d_mlp_grads;   /* gradients of the last vkg_nrc_backward (zeroed by vkg_nrc_adam_step) */
    float *d_grid_grads;
    uint32_t step;            /* optimiser steps taken */
    uint32_t kernel_error;    /* nonzero: a tensor-core kernel gave up waiting (its results are void) */
    uint32_t infer_kernel;    /* the inference kernel in use (1..3, see vkg_nrc_config) */
    uint32_t train_kernel;    /* the training kernels in use (1..3) */
} vkg_nrc_info_t;
vkg_status vkg_nrc_config_default(vkg_nrc_config *out);
vkg_status vkg_nrc_create(vkg_ctx *ctx, const vkg_nrc_config *cfg, vkg_nrc **out);
vkg_status vkg_nrc_destroy(vkg_nrc *nrc);
vkg_status vkg_nrc_info(const vkg_nrc *nrc, vkg_nrc_info_t *out);
/* prediction for n feature records -> n x 3 fp32 */
vkg_status vkg_nrc_infer(vkg_nrc *nrc, const float *d_features, uint32_t n, float *d_rgb, void *stream);
/* accumulate the gradients of the relative-L2 loss against n x 3 targets (no parameter update) */
vkg_status vkg_nrc_backward(vkg_nrc *nrc, const float *d_features, const float *d_targets, uint32_t n, void *stream);
/* one Adam update from the accumulated gradients (consumes them) */
vkg_status vkg_nrc_adam_step(vkg_nrc *nrc, void *stream);
/* backward + Adam; *h_loss (optional) receives the mean loss of the batch (synchronises) */
vkg_status vkg_nrc_train_step(vkg_nrc *nrc, const float *d_features, const float *d_targets, uint32_t n,
                              float *h_loss, void *stream);
/* overwrite the FP32 master parameters (either may be NULL) */
vkg_status vkg_nrc_load_params(vkg_nrc *nrc, const float *d_mlp, const float *d_grid, void *stream);
/* checkpoints (not in the reference): vkg_nrc_save writes the cache's training state -- FP32 MLP
 * weights and hash-grid features with both Adam moments and the step count -- to one file: a
 * 128-byte little-endian header (magic "VKGNRC01", version 1, the grid layout: levels,
 * log2_table_size, base and max resolution, the scene box, the parameter counts, the step, the
 * optimiser constants, the payload size and an FNV-1a 64 checksum of the payload), then the
 * payload: MLP weights, first and second moments (num_mlp_params floats each), grid features,
 * first and second moments (num_grid_params floats each). vkg_nrc_load reads such a file into a
 * cache created with the same grid layout (else VKG_ERR_INVALID_ARGUMENT), checks the checksum and
 * restores the BF16 / FP16 operand copies. Both synchronise `stream`. */
vkg_status vkg_nrc_save(vkg_nrc *nrc, const char *path, void *stream);
vkg_status vkg_nrc_load(vkg_nrc *nrc, const char *path, void *stream);
/* Attach a radiance cache to a path tracer (NULL detaches; the cache must outlive its use). With a
 * cache attached, vkg_tracer_render ends every rendering path at its terminate_depth-th surface
 * interaction in the cache: the path adds throughput x (emission + predicted outgoing radiance)
 * and stops. After the frame it traces train_paths training paths through random pixels of the
 * crop window with the plain estimator (up to max_trace_depth, Russian roulette as configured),
 * records their first train_depth interactions together with the radiance that followed each,
 * and runs train_steps optimiser steps on batches of batch_size records, all on `stream`. */
vkg_status vkg_tracer_attach_cache(vkg_tracer *tracer, vkg_nrc *cache);
#ifdef __cplusplus
}
#endif
#endif /* VKG_H */
