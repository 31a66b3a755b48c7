/*
 * kf_oracle.h — CPU oracle for the GB300 path tracer.
 *
 * TEST INFRASTRUCTURE ONLY. The oracle is the checker: a scalar C++
 * restatement of kuafu's ray-tracing shaders (resources/shaders/PathTrace.*,
 * resources/shaders/base/ *.glsl) and of the host code that feeds them
 * (src/core/camera.cpp, src/core/scene.cpp). Only tests, the smoke check and
 * the CPU-baseline leg of the benchmark may load it; the product (libkf) never
 * links or calls it.
 *
 * It consumes the same flattened scene layouts (include/kf_types.h) that the
 * CUDA kernels consume, so both sides render from identical bytes.
 */
#ifndef KF_ORACLE_H
#define KF_ORACLE_H

#include "../include/kf_types.h"

#ifdef __cplusplus
extern "C" {
#endif

enum { KF_ORACLE_RNG_PHILOX = 0, KF_ORACLE_RNG_TEA_LCG = 1 };
enum { KF_ORACLE_FP32 = 0, KF_ORACLE_FP64 = 1 };

typedef struct kf_oracle_view {
    const kf_camera_ubo* camera;
    uint32_t width, height;     /* full image size (gl_LaunchSizeEXT) */
    uint32_t x0, y0;            /* crop origin */
    uint32_t crop_w, crop_h;    /* crop size (0 = full image) */
    kf_push_constants pc;
    uint32_t seed;
    uint32_t frame;
    uint32_t camera_index;
    uint32_t rng_mode;          /* KF_ORACLE_RNG_* */
    uint32_t tea_clock;         /* stand-in for clockARB() in TEA/LCG mode */
    uint32_t precision;         /* KF_ORACLE_FP32 / KF_ORACLE_FP64 */
    uint32_t threads;           /* 0 = all hardware threads */
    uint32_t use_bvh;           /* 0 = brute force over all triangles, 1 = per-geometry CPU BVH */
} kf_oracle_view;

typedef struct kf_oracle_out {
    float* path_radiance;       /* [spp][crop pixels][3]  per-sample `color` (PathTrace.rgen:140), or NULL */
    float* pixel_color;         /* [crop pixels][3]  finalColor = colors / spp (rgen:144), or NULL */
    double* pixel_color64;      /* [crop pixels][3]  same, accumulated in FP64, or NULL */
    float* albedo;              /* [crop pixels][3]  AOV (rgen:114-117), or NULL */
    float* normal;              /* [crop pixels][3]  AOV, or NULL */
    kf_hit* primary_hits;       /* [spp][crop pixels]  first closest hit of each sample, or NULL */
    uint32_t* path_depths;      /* [spp][crop pixels]  number of closest-hit traces per path, or NULL */
    uint64_t rays_primary;
    uint64_t rays_extension;
    uint64_t rays_shadow;
} kf_oracle_out;

/* Render one frame's samples for a crop (PathTrace.rgen main). Returns 0 on success, 3 when
 * a vertex, material or geometry index of the scene is out of range. */
int kf_oracle_render(const kf_flat_scene* scene, const kf_oracle_view* view, kf_oracle_out* out);

/* Closest hit of arbitrary world-space rays against the scene (traceRayEXT, rgen:97-107).
 * rays: [n][8] = {ox, oy, oz, tmin, dx, dy, dz, tmax}. */
int kf_oracle_trace(const kf_flat_scene* scene, const float* rays, uint32_t n, uint32_t use_bvh, kf_hit* out);

/* ---- unit-level exports for known-answer and table tests ---- */
void kf_oracle_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
uint32_t kf_oracle_tea(uint32_t v0, uint32_t v1);                 /* Random.glsl:7-21 */
float kf_oracle_rnd_lcg(uint32_t* state);                          /* Random.glsl:26-39 */
float kf_oracle_uniform(uint32_t seed, uint32_t pixel, uint32_t camera, uint32_t sample,
                        uint32_t frame, uint32_t depth, uint32_t purpose, uint32_t draw);
float kf_oracle_sin(float x);
float kf_oracle_cos(float x);
float kf_oracle_exp2(float x);
/* watertight ray/triangle test (Woop, Benthin, Wald, JCGT 2013). Returns 1 on hit. */
int kf_oracle_intersect(const float org[3], const float dir[3], const float v0[3], const float v1[3],
                        const float v2[3], float tmin, float tmax, float* t, float* u, float* v);
/* sampling / BRDF helpers, evaluated on fixed inputs (Random.glsl, Sampling.glsl). */
void kf_oracle_sample_ggx(float u0, float u1, float a2, const float n[3], float out[3]);
void kf_oracle_cosine_hemisphere(float u0, float u1, const float n[3], float out[3]);
float kf_oracle_schlick(float cosine, float ior);
float kf_oracle_ggx_d(float ndoth, float a2);
float kf_oracle_g1(float d, float a2);
void kf_oracle_schlick_fresnel(const float f0[3], float ldoth, float out[3]);
void kf_oracle_perpendicular(const float u[3], float out[3]);          /* Random.glsl:58-65 */
/* rejection samplers drawing from kuafu's lcg stream `*state` (advanced in place) */
void kf_oracle_uniform_sphere_lcg(uint32_t* state, float out[3]);      /* Sampling.glsl:72-83 */
void kf_oracle_disk_lcg(uint32_t* state, float out[2]);                /* Sampling.glsl:124-134 */

/* Host-side camera math (src/core/camera.cpp:92-124, scene.cpp:236-250), FP64 inverses. */
void kf_oracle_camera_ubo(const float position[3], const float front[3], const float up[3],
                          float width, float height, float fx, float fy, float cx, float cy,
                          float skew, kf_camera_ubo* out);

/* sRGB encode of a linear value into an 8-bit code (the B8G8R8A8_SRGB frame, config.hpp:144). */
uint8_t kf_oracle_srgb8(float linear);

/* ---- scene construction, so a CPU render needs nothing of the product ---- */
/* Unit icosphere of `level` subdivisions with smooth normals (Geometry::recalculateNormals,
 * geometry.cpp:268-295) and spherical uv. Writes up to vcap vertices / icap indices; returns
 * the counts in *nv / *ni (call with caps 0 to size the buffers). Returns 0 on success. */
int kf_oracle_icosphere(int level, kf_vertex* v, uint32_t vcap, uint32_t* idx, uint32_t icap, uint32_t* nv,
                        uint32_t* ni);
/* gl_WorldToObjectEXT rows of a column-major object->world matrix (rt.cpp:127-137): the
 * inverse affine map in FP64, rounded to float. Returns 0, or 1 for a singular matrix. */
int kf_oracle_instance_rows(const float transform[16], float rows[12]);
/* Scene::uploadLightBuffers (scene.cpp:252-292). dir: {direction xyz, color rgb, strength,
 * softness} or NULL for no directional light; points: n x {position xyz, color rgb, radius,
 * strength}; actives: n x {view (column-major 16), color rgb, fov, strength, softness,
 * texID, pad}. texID outside [0, num_textures) reads as -1. */
void kf_oracle_light_ubos(const float* dir, const float* points, uint32_t num_points, const float* actives,
                          uint32_t num_actives, uint32_t num_textures, kf_dir_light_ubo* d, kf_point_lights_ubo* p,
                          kf_active_lights_ubo* a);

#ifdef __cplusplus
}
#endif

#endif /* KF_ORACLE_H */
