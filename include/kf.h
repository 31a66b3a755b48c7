/*
 * kf.h — C-ABI of libkf, the GB300-native replacement for kuafu's render path.
 *
 * kuafu exposes a C++ class API (include/kuafu.hpp, include/core/{scene,camera,
 * geometry,light,config}.hpp); SAPIEN links it as libkuafu.so. This header is
 * the flat, exception-free boundary underneath an equivalent C++ facade
 * (include/kuafu_gb300/kuafu.hpp): plain pointers and sizes, opaque handles,
 * int status codes and a thread-local error string. Every entry point names the
 * kuafu function it replaces.
 *
 * Threading: like kuafu (single-threaded, mutable globals) a renderer and the
 * objects created from it must be used from one thread at a time.
 */
#ifndef KF_H
#define KF_H

#include <stddef.h>
#include <stdint.h>

#include "kf_types.h"

#ifdef __cplusplus
extern "C" {
#endif

#if defined(_WIN32)
#define KF_API __declspec(dllexport)
#else
#define KF_API __attribute__((visibility("default")))
#endif

/* ---- status codes (kuafu throws std::runtime_error: stdafx.hpp:61-67) ---- */
#define KF_OK 0
#define KF_ERR_INVALID_ARGUMENT 1 /* KF_ASSERT failures on bad handles / values */
#define KF_ERR_OUT_OF_RANGE 2     /* scene.cpp:54 "Geometry Instances out of bound." */
#define KF_ERR_LIMIT 3            /* scene.cpp:61,116 buffer size exceeded */
#define KF_ERR_CUDA 4             /* device / driver failure */
#define KF_ERR_NOT_IMPLEMENTED 5  /* scene.cpp:153,157 "Not implemented!" */
#define KF_ERR_STATE 6            /* call order violated (e.g. render without camera) */
#define KF_ERR_NO_DEVICE 7        /* no CUDA device: there is no CPU fallback */
#define KF_ERR_OUT_OF_MEMORY 8
#define KF_ERR_INTERNAL 9
#define KF_ERR_TIMEOUT 10         /* a bounded device-side wait gave up */

/* Thread-local message of the last failing call on this thread. */
KF_API const char* kf_last_error(void);
KF_API int kf_version(void);

typedef struct kf_renderer_s* kf_renderer; /* kuafu::Kuafu */
typedef struct kf_scene_s* kf_scene;       /* kuafu::Scene */
typedef struct kf_camera_s* kf_camera;     /* kuafu::Camera */
typedef struct kf_geometry_s* kf_geometry; /* std::shared_ptr<kuafu::Geometry> */
typedef struct kf_instance_s* kf_instance; /* std::shared_ptr<kuafu::GeometryInstance> */
typedef struct kf_light_s* kf_light;       /* std::shared_ptr<PointLight / ActiveLight> */

/* ---- kuafu::Config (include/core/config.hpp:35-177) ---- */
typedef struct kf_config {
    int32_t initial_width;         /* setInitialWidth  (default 800) */
    int32_t initial_height;        /* setInitialHeight (default 600) */
    uint32_t spp;                  /* setPerPixelSampleRate (default 32) */
    uint32_t path_depth;           /* setPathDepth (default 8) */
    uint32_t max_path_depth;       /* getMaxPathDepth (12) */
    uint32_t russian_roulette;     /* setRussianRoulette (default 1) */
    uint32_t rr_min_bounces;       /* setRussianRouletteMinBounces (default 4) */
    uint32_t nee;                  /* setNextEventEstimation (default 1, unused as in kuafu) */
    uint32_t nee_min_bounces;      /* setNextEventEstimationMinBounces (default 0, unused) */
    uint32_t accumulate_frames;    /* setAccumulatingFrames (default 1) */
    uint32_t use_denoiser;         /* setUseDenoiser (default 0) */
    uint32_t present;              /* setPresent: accepted, rendering is always headless */
    uint32_t max_geometries;       /* setGeometryLimit (default 128) */
    uint32_t max_instances;        /* setGeometryInstanceLimit (default 256) */
    uint32_t max_textures;         /* setTextureLimit (default 128) */
    uint32_t max_materials;        /* setMaterialLimit (default 256) */
    /* GB300 additions */
    uint32_t seed;                 /* Philox seed (key word 0 is seed ^ pixel_index) */
    uint32_t blas_leaf_size;       /* max triangles per BVH leaf (default 1) */
    uint32_t tlas_leaf_size;       /* max instances per TLAS leaf (default 1) */
    uint64_t max_paths_in_flight;  /* wavefront chunk size (default 1<<24) */
    uint32_t debug_outputs;        /* 1: keep per-path radiance and primary hits for download */
    uint32_t profile;              /* 1: time kernels with CUDA events (kf_stats.*_ms) */
    uint32_t use_graph;            /* 1: replay the per-frame launch sequence as a CUDA graph (default 1) */
    uint32_t device;               /* CUDA device ordinal (default 0) */
    uint32_t host_only;            /* 1: scene management and export only, no device is touched;
                                      rendering calls then fail with KF_ERR_NO_DEVICE */
    uint32_t traversal;            /* 0: one thread per ray; 1: persistent warps with dynamic
                                      ray fetch (default). Both give identical results. */
    uint32_t bvh_builder;          /* 0: GPU LBVH (Morton order); 1: host SAH (default: full
                                      sweep up to 4096 primitives, binned above, SAH-optimal
                                      4-wide collapse; fewer node visits per ray); 2: GPU PLOC
                                      (locally-ordered clustering). Same hits. */
    uint32_t dyn_refill_below;     /* persistent traversal: a warp fetches new rays when fewer
                                      lanes than this are busy (1..32, default 16) */
    uint32_t dyn_steps;            /* ... and runs this many traversal steps between fetches
                                      (1..64, default 32) */
    uint32_t blas_share;           /* 1 (default): geometries with identical positions and
                                      indices (materials may differ) share one BLAS in the
                                      node and triangle pools, built once; 0: one copy per
                                      geometry. Same hits either way. */
} kf_config;

/* Fills kuafu's defaults (config.hpp:140-176). */
KF_API void kf_config_init(kf_config* cfg);

/* ---- kuafu::Kuafu (include/kuafu.hpp:31-93, src/kuafu.cpp) ---- */
KF_API int kf_renderer_create(const kf_config* cfg, kf_renderer* out);          /* Kuafu(config), kuafu.cpp:27-63 */
KF_API int kf_renderer_destroy(kf_renderer r);
KF_API int kf_renderer_get_config(kf_renderer r, kf_config* out);               /* Kuafu::getConfig */
KF_API int kf_renderer_set_config(kf_renderer r, const kf_config* cfg);         /* Config setters */
KF_API int kf_renderer_get_scene(kf_renderer r, kf_scene* out);                 /* Kuafu::getScene */
KF_API int kf_renderer_create_scene(kf_renderer r, kf_scene* out);              /* Kuafu::createScene */
KF_API int kf_renderer_set_scene(kf_renderer r, kf_scene s);                    /* Kuafu::setScene */
KF_API int kf_renderer_remove_scene(kf_renderer r, kf_scene s);                 /* Kuafu::removeScene */
KF_API int kf_renderer_is_running(kf_renderer r, int* out);                     /* Kuafu::isRunning */
/* Renders one frame of the current scene through its current camera: spp samples
 * per pixel, accumulated into the camera's running mean (Kuafu::run, kuafu.cpp:72-85;
 * Context::render, context.cpp:522-540). Work is queued on the renderer's stream. */
KF_API int kf_renderer_run(kf_renderer r);
KF_API int kf_renderer_synchronize(kf_renderer r);
/* The cudaStream_t every kernel of this renderer is launched on (for CUDA-event timing). */
KF_API int kf_renderer_get_stream(kf_renderer r, void** out_stream);
/* Latest frame as sRGB-encoded BGRA8, w*h*4 bytes (Kuafu::downloadLatestFrame,
 * kuafu.cpp:87-95; Camera::downloadLatestFrame, camera.cpp:188-207). */
KF_API int kf_renderer_download_latest_frame(kf_renderer r, kf_camera cam, uint8_t* out_bgra, size_t bytes);

/* Extra render targets of a camera (rt.cpp:497-512 + depth). */
enum {
    KF_AOV_RADIANCE_F32 = 0,  /* float4 per pixel: the accumulated "rgba" target */
    KF_AOV_ALBEDO_F32 = 1,    /* float4 per pixel: "albedo" target */
    KF_AOV_NORMAL_F32 = 2,    /* float4 per pixel: "normal" target */
    KF_AOV_DEPTH_F32 = 3,     /* float per pixel: primary-hit distance (0 on miss), sample 0 */
    KF_AOV_SUM_F64 = 4,       /* double4 per pixel: FP64 sum of every frame's finalColor */
    KF_AOV_PATH_RADIANCE = 5, /* float4 per path [spp][h][w] of the last frame (debug_outputs) */
    KF_AOV_PRIMARY_HITS = 6,  /* kf_hit per path [spp][h][w] of the last frame (debug_outputs) */
    KF_AOV_DENOISED_F32 = 7,  /* float4 per pixel: output of the learned denoiser */
    KF_AOV_SEGMENTATION = 8   /* uint32 x 4 per pixel: instance, geometry, material, primitive of
                                 the first hit of sample 0 (0xFFFFFFFF x 3, 0 on a miss); the
                                 segmentation SAPIEN asks of kuafu (README.md:66-67) */
};
KF_API int kf_renderer_download_aov(kf_renderer r, kf_camera cam, int kind, void* out, size_t bytes);

typedef struct kf_stats {
    uint64_t frames;
    uint64_t rays_primary;
    uint64_t rays_extension;
    uint64_t rays_shadow;
    uint64_t node_visits;     /* closest-hit traversal; counted only with kf_renderer_count_traversal */
    uint64_t tri_tests;
    uint64_t inst_visits;
    uint64_t shadow_node_visits; /* any-hit (shadow) traversal; counted only with kf_renderer_count_traversal */
    uint64_t shadow_tri_tests;
    uint64_t shadow_inst_visits;
    double extend_ms;         /* summed CUDA-event durations (profile = 1) */
    double shadow_ms;
    double shade_ms;
    double frame_ms;
    double bvh_build_ms;
    int32_t frame_count;      /* kuafu's global::frameCount */
    uint32_t last_spp;
    uint32_t blas_nodes;
    uint32_t tlas_nodes;
    uint64_t tlas_refits;     /* TLAS refits (transform-only updates) of the current scene */
} kf_stats;
KF_API int kf_renderer_get_stats(kf_renderer r, kf_stats* out);
KF_API int kf_renderer_reset_stats(kf_renderer r);
/* Restart accumulation: the next run() stores its frame instead of blending it
 * (kuafu sets global::frameCount = -1 only when the camera moves, camera.cpp:41-51,
 * or the scene changes; this exposes the same reset directly). */
KF_API int kf_renderer_reset_frame(kf_renderer r);
/* Re-trace the last frame's traversal with per-ray counters (node / triangle /
 * instance visits) to give algorithmic bytes per ray. */
KF_API int kf_renderer_count_traversal(kf_renderer r, int enable);

/* ---- process-global material table (global.hpp:33-35, geometry.cpp:241-249) ---- */
typedef struct kf_material {       /* kuafu::NiceMaterial (geometry.hpp:11-30) */
    float diffuse_color[3];
    float alpha;
    float metallic;
    float specular;
    float roughness;
    float ior;
    float transmission;
    float emission[3];
    float emission_strength;
    int32_t diffuse_tex;            /* texture ids from kf_texture_create, -1 = none */
    int32_t metallic_tex;
    int32_t roughness_tex;
    int32_t transmission_tex;
} kf_material;
KF_API void kf_material_init(kf_material* m);             /* NiceMaterial defaults */
KF_API int kf_material_add(const kf_material* m, uint32_t* out_index);
KF_API uint32_t kf_material_count(void);
KF_API int kf_material_get(uint32_t index, kf_material* out);
KF_API int kf_material_clear(void);

/* ---- textures (vkCore::Texture: RGBA8, sRGB, linear/repeat sampler) ---- */
KF_API int kf_texture_create(const uint8_t* rgba8, uint32_t width, uint32_t height, int srgb, int32_t* out_id);
KF_API uint32_t kf_texture_count(void);

/* ---- kuafu::Geometry (geometry.hpp:32-46) ---- */
KF_API int kf_geometry_create(const kf_vertex* vertices, uint32_t num_vertices, const uint32_t* indices,
                              uint32_t num_indices, const uint32_t* mat_index, uint32_t num_mat_index,
                              kf_geometry* out);
KF_API int kf_geometry_set_material(kf_geometry g, const kf_material* m);   /* Geometry::setMaterial */
KF_API int kf_geometry_set_flags(kf_geometry g, int opaque, int hide_render, int dynamic_);
KF_API int kf_geometry_recalculate_normals(kf_geometry g);                  /* Geometry::recalculateNormals */
KF_API int kf_geometry_get_info(kf_geometry g, uint32_t* num_vertices, uint32_t* num_indices);
KF_API int kf_geometry_get_data(kf_geometry g, kf_vertex* vertices, uint32_t* indices, uint32_t* mat_index);
KF_API int kf_geometry_release(kf_geometry g);
/* Procedural meshes (geometry.cpp:297-537) plus the level-n icosphere. */
enum { KF_MESH_YZ_PLANE = 0, KF_MESH_CUBE = 1, KF_MESH_SPHERE = 2, KF_MESH_CAPSULE = 3, KF_MESH_ICOSPHERE = 4 };
KF_API int kf_geometry_create_builtin(int kind, float param0, float param1, const kf_material* m, kf_geometry* out);
/* loadScene / loadObj (geometry.hpp:56-57, geometry.cpp:46-265) for Wavefront OBJ + MTL:
 * one geometry per material used (faces merged per material), per-corner vertices, fan
 * triangulation, flat normals where the file has none, V flipped, materials mapped as
 * kuafu maps assimp's keys (roughness from Ns) and deduplicated in the global table.
 * Call with out = NULL to get the count; then with capacity >= count. Texture maps are
 * not decoded. */
KF_API int kf_load_scene(const char* path, int dynamic, kf_geometry* out, uint32_t capacity, uint32_t* count);

/* ---- kuafu::Scene (include/core/scene.hpp:40-295, src/core/scene.cpp) ---- */
KF_API int kf_scene_submit_geometry(kf_scene s, kf_geometry g);             /* submitGeometry */
KF_API int kf_scene_clear_geometries(kf_scene s);                          /* clearGeometries */
KF_API int kf_scene_remove_geometry(kf_scene s, kf_geometry g);            /* removeGeometry: not implemented in kuafu */
KF_API int kf_scene_submit_instance(kf_scene s, kf_geometry g, const float transform[16], kf_instance* out);
KF_API int kf_instance_set_transform(kf_instance i, const float transform[16]);  /* GeometryInstance::setTransform */
KF_API int kf_scene_remove_instance(kf_scene s, kf_instance i);            /* removeGeometryInstance */
KF_API int kf_scene_clear_instances(kf_scene s);                           /* clearGeometryInstances */
KF_API int kf_scene_instance_count(kf_scene s, uint32_t* out);
KF_API int kf_scene_get_instance(kf_scene s, uint32_t index, kf_instance* out);  /* getGeometryInstance */
KF_API int kf_instance_release(kf_instance i);
KF_API int kf_scene_set_clear_color(kf_scene s, const float rgba[4]);      /* setClearColor */
KF_API int kf_scene_get_clear_color(kf_scene s, float rgba[4]);
/* Scene::setEnvironmentMap / removeEnvironmentMap (scene.cpp:182-188; uploaded by
 * uploadEnvironmentMap, scene.cpp:294-310; sampled on every miss by PathTrace.rmiss:14-29
 * as texture(environmentMap, vec3(-d.y, d.z, -d.x)) instead of the clear colour).
 * Faces +X, -X, +Y, -Y, +Z, -Z, each size x size texels, rows top to bottom; lookup:
 * cube-face selection and face coordinates of the Vulkan / GL cube-map rules, bilinear
 * within the face with clamp-to-edge (no filtering across face seams). */
KF_API int kf_scene_set_environment_map(kf_scene s, const float* rgba32f, uint32_t size);
/* The same from RGBA8 texels (srgb != 0: decoded with the sRGB transfer function). */
KF_API int kf_scene_set_environment_map_rgba8(kf_scene s, const uint8_t* rgba8, uint32_t size, int srgb);
/* The same from an uncompressed KTX 1.1 cube map file (the format kuafu loads): RGB or
 * RGBA, 8-bit (UNORM or sRGB), 16-bit float or 32-bit float texels; mip level 0 is used. */
KF_API int kf_scene_set_environment_map_file(kf_scene s, const char* path);
KF_API int kf_scene_remove_environment_map(kf_scene s);
KF_API int kf_scene_mark_geometries_changed(kf_scene s);
KF_API int kf_scene_mark_instances_changed(kf_scene s);

typedef struct kf_directional_light { float direction[3]; float color[3]; float strength; float softness; } kf_directional_light; /* light.hpp:9-14 */
typedef struct kf_point_light { float position[3]; float color[3]; float radius; float strength; } kf_point_light;             /* light.hpp:16-21 */
typedef struct kf_active_light { float view[16]; float color[3]; float fov; float strength; float softness; int32_t tex_id; } kf_active_light; /* light.hpp:31-39 */

KF_API int kf_scene_set_directional_light(kf_scene s, const kf_directional_light* l);  /* setDirectionalLight */
KF_API int kf_scene_remove_directional_light(kf_scene s);                              /* removeDirectionalLight */
KF_API int kf_scene_add_point_light(kf_scene s, const kf_point_light* l, kf_light* out);   /* addPointLight */
KF_API int kf_scene_add_active_light(kf_scene s, const kf_active_light* l, kf_light* out); /* addActiveLight */
KF_API int kf_light_update_point(kf_light l, const kf_point_light* p);
KF_API int kf_light_update_active(kf_light l, const kf_active_light* a);
KF_API int kf_scene_remove_light(kf_scene s, kf_light l);                  /* removePointLight / removeActiveLight */

KF_API int kf_scene_create_camera(kf_scene s, int width, int height, kf_camera* out);  /* createCamera */
KF_API int kf_scene_remove_camera(kf_scene s, kf_camera c);                /* removeCamera */
KF_API int kf_scene_set_camera(kf_scene s, kf_camera c);                   /* setCamera */
KF_API int kf_scene_get_camera(kf_scene s, kf_camera* out);                /* getCamera */

/* Flattened scene as the kernels consume it (scene.cpp:231-467). Pointers stay
 * valid until the scene changes. Used by tests to feed the oracle. */
KF_API int kf_scene_export(kf_scene s, kf_flat_scene* out);

/* ---- kuafu::Camera (include/core/camera.hpp:40-174, src/core/camera.cpp) ---- */
KF_API int kf_camera_set_position(kf_camera c, const float p[3]);          /* setPosition */
KF_API int kf_camera_set_front(kf_camera c, const float f[3]);             /* setFront */
KF_API int kf_camera_set_up(kf_camera c, const float u[3]);                /* setUp */
KF_API int kf_camera_set_pose(kf_camera c, const float pose[16]);          /* setPose */
KF_API int kf_camera_get_pose(kf_camera c, float pose[16]);                /* getPose */
KF_API int kf_camera_set_full_perspective(kf_camera c, float width, float height, float fx, float fy, float cx,
                                          float cy, float skew);          /* setFullPerspective */
KF_API int kf_camera_set_size(kf_camera c, int width, int height);         /* setSize */
KF_API int kf_camera_reset_view(kf_camera c);                              /* resetView */
KF_API int kf_camera_get_size(kf_camera c, int* width, int* height);
KF_API int kf_camera_get_ubo(kf_camera c, kf_camera_ubo* out);             /* uploadCameraBuffer, scene.cpp:236-250 */

/* ---- batched offscreen rendering: many cameras / scenes in one wavefront ----
 * kuafu renders one camera of the current scene per run(); SAPIEN renders many views
 * by calling it in turn. Here the views of any scenes of this renderer are traced
 * together: their paths form one path space, each bounce is one launch of each kernel
 * over all views, and the whole sequence is captured in one CUDA graph (replayed while
 * the batch's layout is unchanged). Each view is an independent single frame
 * (frameCount -1, no blending), written to its camera's targets exactly as
 * kf_renderer_run would write it for the same frame word; all views of a batch share
 * one frame word. spp 0 = the config's spp. A camera may appear once per batch. */
typedef struct kf_batch_item {
    kf_scene scene;
    kf_camera camera;
    uint32_t spp;
    uint32_t pad;
} kf_batch_item;
KF_API int kf_renderer_run_batch(kf_renderer r, const kf_batch_item* items, uint32_t count);

/* Autotuner of batched rendering (no counterpart in kuafu, whose launch shapes are the
 * ray-tracing pipeline's): measures the batch with one knob changed at a time —
 * traversal kernel, paths in flight, launch grids, the persistent traversal's refill
 * threshold and steps between refills, BLAS leaf size — each over `reps`
 * timed batches after a warm-up, and leaves the renderer configured with the fastest
 * (kf_renderer_get_config shows it). Results stay identical: every knob only changes
 * how the same per-path arithmetic is scheduled, or the BVH that finds the same hits. */
typedef struct kf_autotune_result {
    uint32_t traversal;
    uint32_t blas_leaf_size;
    uint64_t max_paths_in_flight;
    uint32_t grid_extend;      /* blocks of the thread-per-ray traversal kernels */
    uint32_t grid_shade;       /* blocks of the shading / gather kernels */
    uint32_t candidates;       /* configurations measured */
    float best_ms;             /* median batch time of the chosen configuration */
    float start_ms;            /* ... of the configuration the renderer had before */
    uint32_t start_traversal;
    uint32_t start_blas_leaf_size;
    uint64_t start_max_paths_in_flight;
    uint32_t dyn_refill_below;   /* persistent traversal scheduling chosen */
    uint32_t dyn_steps;
} kf_autotune_result;
KF_API int kf_renderer_autotune(kf_renderer r, const kf_batch_item* items, uint32_t count, uint32_t reps,
                                kf_autotune_result* out);

/* Achievable L2 read bandwidth of the renderer's GPU in GB/s: a `bytes` buffer (1 MiB ..
 * 1 GiB; one that fits in L2, e.g. 32 MiB) read `passes` times through L2 by a
 * full-occupancy grid, best of `reps` CUDA-event-timed launches on the renderer's stream.
 * The denominator of the traversal kernels' L2 roofline. No counterpart in kuafu. */
KF_API int kf_renderer_measure_l2_read(kf_renderer r, uint64_t bytes, uint32_t passes, uint32_t reps,
                                       double* gbs);

/* ---- tensor-core building blocks of the learned denoiser (device pointers; no
 * counterpart in kuafu, whose OptiX denoiser is closed code, denoiser.cpp:257-316) ---- */
/* y[n,y,x,y_coff+co] = act(bias[co] + sum x[n,y+dy,x+dx,ci] * w[tap][co][ci]), NHWC BF16,
 * zero padding, FP32 accumulation; w: [9][w_rows][cin], w_rows % 16 == 0, cin a multiple of
 * 32 (or 16 for images at least 96 wide); x, weight and y 16-byte aligned. */
KF_API int kf_conv3x3_bf16(const void* x, int n, int h, int w, int cin, const void* weight, int w_rows,
                           const float* bias, int cout, int relu, void* y, int y_cstride, int y_coff, void* stream);
/* d[m][n] += sum_k a[m][k] * b[n][k], BF16 K-major operands (16-byte aligned, k % 8 == 0),
 * FP32 accumulation into d (row stride ldd >= n) by split-K atomics: d is added to, not
 * overwritten. */
KF_API int kf_gemm_bf16_tn(const void* a, int m, const void* b, int n, int k, float* d, int ldd, int splits,
                           void* stream);
/* Error word of the tensor-core kernels (0 = none; set when a bounded wait expired); cleared on read. */
KF_API int kf_tc_error(uint32_t* out);
/* Self-test of the bounded waits: one kernel waits on an mbarrier that nothing arrives on,
 * gives up after budget_cycles SM cycles (1 .. 2e9) and sets the error word to 99, which
 * kf_tc_error then reports; no fault, the context stays usable. */
KF_API int kf_tc_wait_probe(uint64_t budget_cycles, void* stream);

/* ---- learned denoiser: replaces kuafu's OptiX pass (Config::setUseDenoiser,
 * config.cpp:142; context.cpp:651-670 feeds rgba + albedo + normal to OptiX and
 * writes the result back over the presented image). Here a U-Net (3x3 convs,
 * 32/64/96/128/160 channels) over log radiance, albedo, normal and depth,
 * trained on this renderer's own low-spp / high-spp pairs. ---- */
typedef struct kf_denoiser_s* kf_denoiser;
/* A denoiser with He-initialised weights (seeded), owned by renderer r:
 * kf_renderer_destroy frees the denoisers still alive, after which their handles are
 * invalid (kf_denoiser_destroy must not be called on them any more). */
KF_API int kf_denoiser_create(kf_renderer r, uint32_t seed, kf_denoiser* out);
KF_API int kf_denoiser_destroy(kf_denoiser d);
KF_API int kf_denoiser_num_params(kf_denoiser d, uint64_t* out);
/* FP32 master parameters (per conv: weights [9][cout][cin] then bias [cout]), host memory. */
KF_API int kf_denoiser_get_params(kf_denoiser d, float* out, uint64_t count);
KF_API int kf_denoiser_set_params(kf_denoiser d, const float* in, uint64_t count); /* resets Adam state */
KF_API int kf_denoiser_save(kf_denoiser d, const char* path);
KF_API int kf_denoiser_load(kf_denoiser d, const char* path);
/* Renders one training pair with camera c of scene s: one frame of low_spp samples
 * (the input) and the mean of high_frames frames of high_spp from the FP64
 * accumulation (the target). Width and height divisible by 16; all views of a
 * denoiser share one size. No kuafu counterpart (OptiX ships a trained network). */
KF_API int kf_denoiser_add_view(kf_denoiser d, kf_scene s, kf_camera c, uint32_t low_spp, uint32_t high_spp,
                                uint32_t high_frames);
/* As kf_denoiser_add_view with num_inputs inputs (one frame of low_spp[i] samples each,
 * independent random streams) paired with one shared target: num_inputs training pairs
 * for the cost of one target render. 1 <= num_inputs <= 64. No kuafu counterpart. */
KF_API int kf_denoiser_add_view_inputs(kf_denoiser d, kf_scene s, kf_camera c, const uint32_t* low_spp,
                                       uint32_t num_inputs, uint32_t high_spp, uint32_t high_frames);
/* Number of training pairs (inputs) added so far. */
KF_API int kf_denoiser_num_views(kf_denoiser d, uint32_t* out);
/* iters Adam steps over batch random crops (crop x crop, crop % 16 == 0); *mean_loss may be NULL. */
KF_API int kf_denoiser_train(kf_denoiser d, uint32_t iters, uint32_t batch, uint32_t crop, float lr,
                             float* mean_loss);
/* Denoises camera c's accumulated radiance into its KF_AOV_DENOISED_F32 target. */
KF_API int kf_denoiser_apply(kf_denoiser d, kf_camera c);
/* Attach (or detach with NULL) the denoiser that kf_renderer_run uses when the config's
 * use_denoiser is set: the presented frame (kf_renderer_download_latest_frame) is then
 * the denoised radiance; the accumulation target itself is left untouched. */
KF_API int kf_renderer_set_denoiser(kf_renderer r, kf_denoiser d);
/* Tensor-level entry points (device pointers, stream = the renderer's). The network
 * works on g(x) = asinh(x / 0.1) of linear radiance x.
 * feat [n][h][w][32] BF16 network input (channels 0..2 g(noisy radiance), 3..5 albedo,
 * 6..8 normal, 9 t / (1 + t), 10 log2(samples) / 8, rest 0); base [n][h][w] float4 FP32
 * residual added to the network output (NULL = none; the renderer passes g(noisy));
 * out [n][h][w][4] FP32 prediction in g space (channel 3 = 0); target [n][h][w] float4
 * linear radiance; h, w % 16 == 0; base, target and the buffers kf_denoiser_camera_features
 * fills 16-byte aligned. train_step computes the L1 + gradient loss in g space
 * and its gradients (copied to grads_dev, may be NULL, FP32, num_params) and, if apply,
 * one Adam step with learning rate lr. */
KF_API int kf_denoiser_forward(kf_denoiser d, const void* feat, const float* base, int n, int h, int w, float* out);
/* The network input of camera c's current frame, as kf_denoiser_apply builds it: BF16
 * features [hp][wp][32] (g(radiance), albedo, normal, t / (1 + t), log2(samples) / 8, then
 * zeros) and the FP32 residual base [hp][wp] float4 (g(radiance)), with hp, wp the frame
 * size rounded up to 16 (padding pixels zero). *hp, *wp are set first; feat_dev and
 * base_dev (device memory of hp * wp pixels) may be NULL to query the size only. */
KF_API int kf_denoiser_camera_features(kf_denoiser d, kf_camera c, void* feat_dev, float* base_dev, int* hp,
                                       int* wp);
KF_API int kf_denoiser_train_step(kf_denoiser d, const void* feat, const float* base, const float* target, int n,
                                  int h, int w, float lr, float* grads_dev, int apply, float* loss);

/* ---- FP64 relative-MSE reduction: mean over pixels and channels of
 * (x - ref)^2 / (ref^2 + eps), rgb of float4 pixels (16-byte aligned images), reduced in
 * FP64; num_pixels > 0 ---- */
KF_API int kf_relmse(kf_renderer r, const float* x_dev, const float* ref_dev, uint64_t num_pixels, double eps,
                     double* out);

/* The same reduction for callers that cannot call cudaMalloc: an application
 * whose device memory is owned by its own pool allocator, or a frame loop that
 * must not take the device-wide synchronisation cudaMalloc / cudaFree imply.
 * It allocates nothing: its per-block partials live in a static device array of
 * 4096 + 1 doubles (32 KiB) that every GPU loading libkf keeps until exit.
 * Limit: 0 < num_pixels <= 268435456 (2^28), else KF_ERR_INVALID_ARGUMENT /
 * KF_ERR_LIMIT. Runs on `stream` (a cudaStream_t, NULL = default stream) of the
 * current device. Every call looks up the array's device address on the current
 * device; the first call on a device also loads the module there, so make that
 * first call before any stream capture. Calls share the array: calls that overlap
 * on the GPU (other streams, other threads) race and must be serialised by the
 * caller. Blocks until *out is written. No counterpart in the reference. */
KF_API int kf_relmse_noalloc(const float* x_dev, const float* ref_dev, uint64_t num_pixels, double eps,
                             void* stream, double* out);

#ifdef __cplusplus
}
#endif

#endif /* KF_H */
