/*
 * CPU oracle for the path-tracing hot path. TEST INFRASTRUCTURE ONLY.
 *
 * This is a plain-C restatement of the reference's algorithms (vierkant: src/intersection.cpp,
 * src/Geometry.cpp, shaders/slang/...) plus the project-defined parts the reference does not have
 * (PCG32 streams, LBVH -> 8-wide BVH build, camera-ray batches). It exists only to check the CUDA
 * product path: tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it; the
 * product library (vierkant_gb300/libvkg.so) never does.
 *
 * Pinning: the ray-triangle / ray-box restatements are checked bit-for-bit against the
 * reference's own src/intersection.cpp compiled unmodified into oracle/_ref/libvkref.so
 * (see oracle/Makefile) and against the committed fixtures in tests/golden/.
 *
 * Compiled with -ffp-contract=off: every float operation rounds separately, like the
 * reference's x86-64 build (no FMA without -march). Where the GPU kernels use a fused
 * multiply-add on purpose (box slab tests), the oracle calls fmaf() explicitly.
 */
#ifndef VKG_ORACLE_H
#define VKG_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- records (identical layouts to include/vkg.h) ---------------------------------------- */
typedef struct { float o[3]; float tmin; float d[3]; float tmax; } orc_ray; /* 32 B */
typedef struct { uint32_t prim; float t, u, v; } orc_hit;                   /* 16 B */

#define ORC_MISS 0xFFFFFFFFu

/* ---- RNG -------------------------------------------------------------------------------- */
typedef struct { uint64_t state, inc; } orc_pcg32;
void orc_pcg32_seed(orc_pcg32 *g, uint64_t initstate, uint64_t initseq);
uint32_t orc_pcg32_next(orc_pcg32 *g);
void orc_pcg32_advance(orc_pcg32 *g, uint64_t delta);
float orc_u01(uint32_t x);
void orc_pcg32_fill(uint64_t initstate, uint64_t initseq, uint64_t skip, uint32_t n, uint32_t *out);
uint32_t orc_xxhash32(uint32_t lhs, uint32_t rhs);
uint32_t orc_lcg(uint32_t *prev);
float orc_rnd(uint32_t *prev);

/* ---- intersection (intersection.cpp) --------------------------------------------------- */
int orc_intersect_ray_triangle(const float o[3], const float d[3], const float tri[9], float out_tuv[3]);
int orc_intersect_ray_triangle_cull(const float o[3], const float d[3], const float tri[9], int cull_back,
                                    float out_tuv[3]);
int orc_intersect_ray_aabb(const float o[3], const float d[3], const float bmin[3], const float bmax[3], float *t);
int orc_closest_hit_bruteforce(const float *xyz, const uint32_t *idx, uint32_t ntri, const orc_ray *rays,
                               uint32_t nray, orc_hit *hits, int nthreads, int cull_back);
int orc_any_hit_bruteforce(const float *xyz, const uint32_t *idx, uint32_t ntri, const orc_ray *rays,
                           uint32_t nray, uint32_t *occluded, int nthreads, int cull_back);

/* ---- geometry (Geometry.cpp) and scenes ------------------------------------------------ */
uint32_t orc_icosphere_counts(uint32_t tess, uint32_t *num_tris);
void orc_icosphere(float radius, uint32_t tess, float *xyz, uint32_t *idx);
void orc_cubesphere(float radius, const float center[3], uint32_t n, float *xyz, uint32_t *idx, uint32_t vbase);
typedef struct {
    float radius, center[3];
    float roughness, metalness, base[3];
} orc_sphere_params;
void orc_cornell_sphere_params(uint64_t seed, uint64_t stream, uint32_t nspheres, orc_sphere_params *out);
void orc_cornell_scene(uint64_t seed, uint64_t stream, uint32_t nspheres, uint32_t n, float *xyz, uint32_t *idx,
                       uint32_t *tri_material);

/* ---- camera rays ----------------------------------------------------------------------- */
typedef struct {
    float eye[3];
    float right[3], up[3], back[3]; /* camera-to-world rotation columns */
    float tan_half_fovy, aspect;
    uint32_t width, height;
} orc_camera;
void orc_camera_lookat(const float eye[3], const float target[3], const float up[3], float tan_half_fovy,
                       uint32_t width, uint32_t height, orc_camera *cam);
void orc_camera_ray(const orc_camera *cam, uint32_t x, uint32_t y, float jx, float jy, orc_ray *ray);
void orc_camera_rays_pcg(const orc_camera *cam, uint64_t seed, uint64_t stream, uint32_t spp, orc_ray *rays);

/* ---- LBVH -> 8-wide BVH ---------------------------------------------------------------- */
typedef struct {
    float origin[3];
    uint8_t exps[3];
    uint8_t nchild;
    uint8_t qlo[3][8];
    uint8_t qhi[3][8];
    uint32_t child[8];
} orc_node8; /* 96 B */

typedef struct {
    float v[12]; /* v0.xyz, e1.xyz, e2.xyz, prim_id bits, pad, pad */
} orc_tri;   /* 48 B */

typedef struct {
    uint32_t num_tris, num_nodes, depth, leaf_max;
    float scene_min[3], scene_max[3], margin;
    uint32_t *morton;      /* [num_tris] in triangle (input) order */
    uint32_t *sorted_prim; /* [num_tris] */
    uint32_t *bvh2_left, *bvh2_right; /* [num_tris-1], child encoding: bit31 leaf */
    orc_node8 *nodes;      /* [num_nodes] */
    orc_tri *tris;         /* [num_tris] in sorted order */
} orc_bvh;

int orc_bvh_build(const float *xyz, const uint32_t *idx, uint32_t ntri, uint32_t leaf_max, orc_bvh *out);
void orc_bvh_free(orc_bvh *b);
int orc_bvh_closest_hit(const orc_bvh *b, const orc_ray *rays, uint32_t nray, orc_hit *hits, int nthreads,
                        int cull_back, uint64_t *stats /* [2]: node visits, tri tests; may be NULL */);
int orc_bvh_any_hit(const orc_bvh *b, const orc_ray *rays, uint32_t nray, uint32_t *occluded, int nthreads,
                    int cull_back);
/* closest hit over the same BVH with the triangle test supplied by the caller: fn(ctx, prim, o, d, tuv)
   returns 1 (INTERSECT) with tuv = {t, u, v} for the triangle with original index prim. No culling. */
typedef int (*orc_tri_fn)(void *ctx, uint32_t prim, const float o[3], const float d[3], float tuv[3]);
int orc_bvh_closest_hit_fn(const orc_bvh *b, const orc_ray *rays, uint32_t nray, orc_hit *hits, int nthreads,
                           orc_tri_fn fn, void *fn_ctx, uint64_t *stats);
/* single ray; cull_mode 0 none, 1 all back faces, 2 back faces of triangles with twosided[prim] == 0 */
void orc_bvh_trace1(const orc_bvh *b, const orc_ray *ray, int cull_mode, const uint8_t *twosided, int any,
                    orc_hit *hit, uint32_t *occ);
/* the same with a candidate filter (the any-hit stage): a candidate that would count (the nearest so
   far, or any for any = 1) counts only if accept(ctx, prim, u, v) returns nonzero */
typedef int (*orc_accept_fn)(const void *ctx, uint32_t prim, float u, float v);
void orc_bvh_trace1_filter(const orc_bvh *b, const orc_ray *ray, int cull_mode, const uint8_t *twosided, int any,
                           orc_accept_fn accept, const void *ctx, orc_hit *hit, uint32_t *occ);
/* two-level queries: instances in input order, w2o [ninst][12], hits are 32-byte {prim, inst, t, u, v, pad} */
int orc_tlas_closest_hit(const orc_bvh *const *blas, const float *w2o, const uint32_t *inst_blas, uint32_t ninst,
                         const orc_ray *rays, uint32_t nray, int cull, void *hits, int nthreads);
int orc_tlas_any_hit(const orc_bvh *const *blas, const float *w2o, const uint32_t *inst_blas, uint32_t ninst,
                     const orc_ray *rays, uint32_t nray, int cull, uint32_t *occluded, int nthreads);

/* ---- path tracer (FP32 twin of the GPU kernels / FP64 radiance oracle) ------------------ */
typedef struct {
    float base[3];
    float roughness, metalness;
    float emission[3];
    uint32_t twosided;
    float transmission, ior, clearcoat, clearcoat_roughness;
    float sheen_color[3], sheen_roughness;
    float diffuse_transmission, diffuse_transmission_color[3];
    float iridescence, iridescence_ior, iridescence_thickness;
    float attenuation_color[3], attenuation_distance, scatter_color[3], scatter_factor, phase_g;
    uint32_t null_surface;
    float dispersion; /* KHR_materials_dispersion: 20 / Abbe number (with transmission > 0) */
    uint32_t tex_color, tex_normal, tex_emission, tex_ao_rough_metal, tex_transmission;
    uint32_t tex_diffuse_transmission, tex_diffuse_transmission_color; /* 0xFFFFFFFF: none */
    /* coverage (material_struct_t color.a, blend_mode, alpha_cutoff, RayBuilder.hpp:42, :87-89):
       blend_mode 0 opaque, 1 blend, 2 mask (Material.hpp:32-37) */
    float alpha;
    uint32_t blend_mode;
    float alpha_cutoff;
    /* texture-coordinate transform of the closest-hit stage (raypipeline.slang:350): with
       has_uv_transform, (u, v) -> (t0 u + t1 v + t2, t3 u + t4 v + t5) */
    uint32_t has_uv_transform;
    float uv_transform[6];
} orc_pt_material; /* same 208-byte layout as vkg_material */
uint32_t orc_pt_material_size(void);

/* a texture: size, level count, wrap modes (s: bits 0-7, t: bits 8-15; 0 repeat, 1 clamp to edge,
   2 mirrored repeat) and the first texel of each level in the scene's RGBA8 texel array; the same
   80-byte layout as the library's records */
typedef struct {
    uint32_t width, height, levels, wrap;
    uint32_t offset[16];
} orc_tex_rec;

typedef struct {
    const float *xyz;
    const uint32_t *idx;
    const uint32_t *tri_mat;
    const orc_pt_material *mats;
    uint32_t ntri, nmat;
    const float *nrm; /* unit vertex normals (3 per vertex) for smooth shading, or NULL: face normals */
    const float *uv;  /* texture coordinates (2 per vertex) or NULL */
    const float *tng; /* unit vertex tangents (3 per vertex) or NULL */
    const orc_tex_rec *tex; /* ntex textures over the RGBA8 texels (0: textures are not sampled) */
    const uint32_t *texels;
    uint32_t ntex;
} orc_pt_scene;
/* one trilinear texture sample (FP64), as the tracer samples textures */
void orc_tex_sample(const orc_tex_rec *rec, const uint32_t *texels, double u, double v, double lambda, double out[4]);

typedef struct {
    const float *rgb;        /* w*h*3 */
    const float *weight;     /* w*h normalised weights (mean 1) */
    const float *alias_prob; /* w*h, FP32 twin only (NULL: CDF sampling) */
    const uint32_t *alias;   /* w*h, FP32 twin only */
    const double *cdf;       /* w*h+1, FP64 oracle only */
    uint32_t w, h;
} orc_pt_env;

/* an analytic light, same 80-byte layout as vkg_light (the reference's light_t) */
typedef struct {
    float position[3];
    uint32_t type; /* 0 omni, 1 spot, 2 directional, 4 rect, 5 sphere, 6 tube, 7 disk */
    float color[3], intensity;
    float direction[3], range;
    float spot_angle_scale, spot_angle_offset, angular_size, size_y;
    float tangent[3], size_x;
} orc_pt_light;

/* the per-pixel record, same 32-byte layout as vkg_pixel_data (the reference's pixel_data_t) */
typedef struct {
    float radiance[3], alpha, depth;
    uint32_t normal, object_id, albedo;
} orc_pixel;

typedef struct {
    uint32_t seed;
    uint32_t batch;
    uint32_t spp;
    uint32_t max_depth, rr_depth, mis_mode, disable_material, draw_skybox;
    float max_path_beta, environment;
    uint32_t crop[4]; /* x0, y0, w, h (pixels of the full resolution camera) */
    uint32_t num_lights, suppress_caustics;
    const orc_pt_light *lights; /* the sun (if any) first */
    orc_pixel *pixels;          /* optional: the crop's pixel records (radiance left 0), as the tracer writes them */
    float clip_near;            /* near clipping distance for the records' depth */
    /* the camera's medium (raypipeline.slang:128-135): camera_medium = 14 floats in the order of the
       reference's medium_params_t (attenuation colour, distance, scatter factor, scatter colour, g,
       ior, emission colour, intensity), or camera_material = a material whose medium it is (its own
       ior also for a null surface); NULL / 0xFFFFFFFF: vacuum */
    const float *camera_medium;
    uint32_t camera_material;
} orc_pt_settings;

/* the sun of the tracer settings as a directional light (PBRPathTracer.cpp:610-624): propagation
   direction = +z rotated by the quaternion of the Euler angles (elevation, azimuth, 0) */
void orc_sun_light(const float color[3], float intensity, const float spherical_coords[2], float angular_size,
                   orc_pt_light *out);

/* an instanced scene for the FP64 oracle: meshes (each with the oracle's BVH) and instances with an
   object -> world 3x4 transform, a mesh and a material index into the scene's materials */
typedef struct {
    const orc_bvh *const *mesh_bvh;
    const float *const *mesh_xyz;
    const uint32_t *const *mesh_idx;
    const uint32_t *mesh_nvert;
    const uint8_t *mesh_twosided;
    uint32_t num_meshes;
    const float *o2w;        /* [num_instances][12] */
    const uint32_t *inst_mesh, *inst_mat;
    uint32_t num_instances;
    const float *const *mesh_nrm; /* per mesh: unit vertex normals or NULL (the array itself may be NULL) */
    const float *const *mesh_uv;  /* per mesh: texture coordinates or NULL (the array may be NULL) */
    const float *const *mesh_tng; /* per mesh: unit tangents or NULL (the array may be NULL) */
} orc_pt_instances;

/* mean radiance per crop pixel over spp paths (out: crop_w*crop_h*3 doubles); stats[0] extension
   rays, stats[1] shadow rays (may be NULL); sq: per-pixel mean of the squared luminance (may be NULL) */
int orc_pt_render(int fp64, const orc_pt_scene *scene, const orc_bvh *bvh, const orc_pt_env *env,
                  const orc_camera *cam, const orc_pt_settings *set, double *out, double *sq, uint64_t *stats,
                  int nthreads);
/* the same for an instanced scene (FP64 oracle only; scene supplies the materials) */
/* variance split of the FP64 estimator at the surface reached by segment fork_depth (a radiance cache
   ending paths there): split[pixel] = {mean luminance, per-sample variance, tail variance an exact cache
   would remove, fraction of samples reaching the fork}; stats: extension / shadow rays of the first
   trace of each sample */
int orc_pt_variance_split(const orc_pt_scene *scene, const orc_bvh *bvh, const orc_pt_env *env, const orc_camera *cam,
                          const orc_pt_settings *set, uint32_t fork_depth, double *split, uint64_t *stats,
                          int nthreads);
int orc_pt_render_instanced(const orc_pt_scene *scene, const orc_pt_instances *inst, const orc_pt_env *env,
                            const orc_camera *cam, const orc_pt_settings *set, double *out, double *sq,
                            uint64_t *stats, int nthreads);
/* pixel-record packing and the a-trous denoise pass (denoise.c) */
void orc_oct_encode(const float n[3], float p[2]);
void orc_oct_decode(const float p[2], float n[3]);
uint32_t orc_pack_snorm_2x16(float x, float y);
void orc_unpack_snorm_2x16(uint32_t p, float out[2]);
uint32_t orc_pack_rgba8(float r, float g, float b, float a);
void orc_unpack_rgb8(uint32_t c, float out[3]);
void orc_denoise(const orc_pixel *px, uint32_t w, uint32_t h, float *out_rgba);
/* bloom + tonemap composition of an HDR rgba image (postfx.c) */
void orc_post_fx(const float *hdr, uint32_t w, uint32_t h, int tonemap, int bloom, float exposure, float gamma,
                 float lo, float hi, uint32_t iterations, float *out);

/* one BSDF sample / evaluation in FP64 (sample_disney / eval_disney): u = (lobe, x, y); the return
   value of orc_bsdf_eval is the mixture pdf */
void orc_bsdf_sample(const orc_pt_material *m, const double n[3], const double v[3], double eta, const double u[3],
                     double dir[3], double *pdf, double f[3], int *transmission);
void orc_phase_hg_sample(double x, double y, double g, double dir[3], double *pdf);
double orc_phase_hg(double cos_theta, double g);
double orc_cauchy_ior(double ior, double dispersion, double lambda);
void orc_lambda_rgb(double lambda, double out[3]);
void orc_iridescent_fresnel(double outside, double film, const double f0[3], double thickness, double cos1,
                            double out[3]);
double orc_bsdf_eval(const orc_pt_material *m, const double l[3], const double n[3], const double v[3], double eta,
                     double f[3]);
/* FP64 env tables from an rgb map: weights (mean 1, as float) and the CDF (w*h+1 doubles) */
void orc_pt_env_tables(const float *rgb, uint32_t w, uint32_t h, float *weight, double *cdf);
/* procedural sky in double precision (environment_white + sun lobe), rounded to float */
void orc_pt_env_procedural(uint32_t w, uint32_t h, const float sun_dir[3], double peak, double width, float *rgb);

#ifdef __cplusplus
}
#endif
#endif
