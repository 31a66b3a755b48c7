/*
 * kf_types.h — plain-C data layouts shared by the GB300 path tracer (libkf),
 * its C-ABI callers and the CPU oracle.
 *
 * Every struct here reproduces a buffer / uniform layout that kuafu's shaders
 * consume, byte for byte, so that a scene flattened by the host code can be
 * handed to the CUDA kernels and to the oracle unchanged:
 *
 *   kf_vertex            48 B  include/core/context/vertex.hpp:28-34, unpacked at
 *                              resources/shaders/PathTrace.rchit:52-64
 *   kf_material_gpu      80 B  include/core/geometry.hpp:70-87 (NiceMaterialSSBO),
 *                              resources/shaders/base/Geometry.glsl:1-19
 *   kf_dir_light_ubo     32 B  include/core/light.hpp:41-44, base/Light.glsl:4-9
 *   kf_point_lights_ubo 1 KB   include/core/light.hpp:46-49, base/Light.glsl:12-16
 *   kf_active_lights_ubo       include/core/light.hpp:51-58, base/Light.glsl:20-33
 *   kf_camera_ubo       320 B  include/core/camera.hpp:181-192, base/Camera.glsl:1-13
 *   kf_push_constants    48 B  include/core/rt/rt.hpp:31-42, base/PushConstants.glsl:1-16
 *
 * Matrices are glm-style column-major float[16]: m[col*4 + row].
 * No code lives here; only layouts and limits.
 */
#ifndef KF_TYPES_H
#define KF_TYPES_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* include/core/context/global.hpp:37-39 (specialization constants in base/Light.glsl:1-2) */
#define KF_MAX_POINT_LIGHTS 32
#define KF_MAX_ACTIVE_LIGHTS 8

/* Ray interval used by every traversal in kuafu (PathTrace.rgen:72-73, PathTrace.rchit:180). */
#define KF_T_MIN 0.001f
#define KF_T_MAX 10000.0f
/* Directional-light shadow ray length (PathTrace.rchit:220). */
#define KF_DIR_LIGHT_TMAX 1e6f

/* kuafu's M_PI (resources/shaders/base/Random.glsl:1) — deliberately not pi. */
#define KF_REF_PI 3.141592f

typedef struct kf_vertex {
    float pos[3];
    float normal[3];
    float color[3];
    float uv[2];
    float pad;
} kf_vertex;

typedef struct kf_material_gpu {
    float diffuse[4];  /* rgb + pad */
    float emission[4]; /* rgb + strength */
    float alpha;
    float metallic;
    float specular;
    float roughness;
    float ior;
    float transmission;
    int32_t diffuse_tex;
    int32_t metallic_tex;
    int32_t roughness_tex;
    int32_t transmission_tex;
    int32_t pad0;
    int32_t pad1;
} kf_material_gpu;

typedef struct kf_dir_light_ubo {
    float direction[4]; /* normalized direction + softness */
    float rgbs[4];      /* rgb + strength (0 = off) */
} kf_dir_light_ubo;

typedef struct kf_point_lights_ubo {
    float posr[KF_MAX_POINT_LIGHTS][4]; /* position + radius */
    float rgbs[KF_MAX_POINT_LIGHTS][4]; /* rgb + strength (<=0 = slot off) */
} kf_point_lights_ubo;

typedef struct kf_active_lights_ubo {
    float view[KF_MAX_ACTIVE_LIGHTS][16];
    float proj[KF_MAX_ACTIVE_LIGHTS][16];
    float front[KF_MAX_ACTIVE_LIGHTS][4];    /* front + in-use flag (w>0) */
    float rgbs[KF_MAX_ACTIVE_LIGHTS][4];     /* rgb + strength */
    float position[KF_MAX_ACTIVE_LIGHTS][4];
    float sftp[KF_MAX_ACTIVE_LIGHTS][4];     /* softness, fov, texID, pad */
} kf_active_lights_ubo;

typedef struct kf_camera_ubo {
    float view[16];
    float proj[16];
    float view_inv[16];
    float proj_inv[16];
    float position[4]; /* xyz + aperture */
    float front[4];    /* xyz + focal distance */
    float pad1[4];
    float pad2[4];
} kf_camera_ubo;

typedef struct kf_push_constants {
    float clear_color[4];
    int32_t frame_count;
    uint32_t spp;
    uint32_t max_path_depth;
    uint32_t use_env_map;
    uint32_t russian_roulette;
    uint32_t rr_min_bounces;
    uint32_t nee;     /* carried but unused, as in kuafu (config.hpp:167-168) */
    uint32_t nee_min; /* carried but unused */
} kf_push_constants;

/* An RGBA8 texture as kuafu's vkCore uploads it (R8G8B8A8_SRGB, vkCore.hpp:585),
 * sampled with linear filtering and repeat addressing (vkCore.hpp:619-637). */
typedef struct kf_texture_desc {
    const uint8_t* rgba8;
    uint32_t width;
    uint32_t height;
    uint32_t srgb; /* 1: decode sRGB -> linear before filtering */
    uint32_t pad;
} kf_texture_desc;

/* One geometry (a BLAS in kuafu): per-geometry vertex / index / matIndex buffers
 * (PathTrace.rchit:26-42). */
typedef struct kf_flat_geometry {
    const kf_vertex* vertices;
    uint32_t num_vertices;
    uint32_t num_triangles;
    const uint32_t* indices;   /* 3 * num_triangles */
    const uint32_t* mat_index; /* num_triangles entries are read (matIndices[gl_PrimitiveID]) */
    uint32_t opaque;           /* 0 -> any-hit alpha test (rt.cpp:101-102) */
    uint32_t hide_render;      /* 1 -> dummy BLAS, never hit (rt.cpp:156) */
} kf_flat_geometry;

/* One TLAS instance: object->world = transform (column-major mat4, rt.cpp:127-137);
 * world->object is the host-computed inverse 3x4 (row-major rows of the affine map),
 * i.e. what gl_WorldToObjectEXT holds. */
typedef struct kf_flat_instance {
    float transform[16];
    float world_to_object[12];
    uint32_t geometry_index;
    uint32_t pad[3];
} kf_flat_instance;

/* A whole flattened scene, as kuafu's Scene::upload* functions lay it out
 * (src/core/scene.cpp:231-467). */
typedef struct kf_flat_scene {
    const kf_flat_geometry* geometries;
    uint32_t num_geometries;
    uint32_t num_instances;
    const kf_flat_instance* instances;
    const kf_material_gpu* materials;
    uint32_t num_materials;
    uint32_t num_textures;
    const kf_texture_desc* textures;
    kf_dir_light_ubo dlight;
    kf_point_lights_ubo plights;
    kf_active_lights_ubo alights;
    /* environment cube map (NULL = none): faces +X, -X, +Y, -Y, +Z, -Z, each
     * env_size x env_size linear RGBA32F texels, rows top to bottom */
    const float* env_rgba32f;
    uint32_t env_size;
    uint32_t env_pad;
} kf_flat_scene;

/* Closest-hit record (what traceRayEXT hands to the hit shaders). */
typedef struct kf_hit {
    float t;
    float u; /* attribs.x: barycentric weight of vertex 1 */
    float v; /* attribs.y: barycentric weight of vertex 2 */
    uint32_t instance; /* gl_InstanceID, 0xFFFFFFFF on miss */
    uint32_t prim;     /* gl_PrimitiveID */
    uint32_t pad[3];
} kf_hit;

/* Random-stream purposes. The product replaces kuafu's per-path TEA/LCG stream
 * (base/Random.glsl:7-39) by counter-based Philox4x32-10 sub-streams, one per
 * (bounce, purpose), so that every draw the shaders make has a fixed address:
 *   ctr = {sample, frame, (depth << 8) | purpose, draw >> 2}
 *   key = {seed ^ pixel_index, camera_index}
 *   u   = (philox(ctr, key)[draw & 3] >> 8) * 2^-24   (24-bit uniform, like rnd())
 */
enum {
    KF_RNG_JITTER = 0,  /* PathTrace.rgen:35 */
    KF_RNG_LENS = 1,    /* PathTrace.rgen:42 (only drawn when aperture > 0) */
    KF_RNG_BSDF = 2,    /* PathTrace.rchit:403-446 */
    KF_RNG_RR = 3,      /* PathTrace.rgen:128 */
    KF_RNG_ANYHIT = 4,  /* PathTrace.rahit:44 */
    KF_RNG_DIRLIGHT = 8,        /* PathTrace.rchit:215-218 + calcDirectContribution */
    KF_RNG_POINT0 = 16,         /* + i, PathTrace.rchit:243-254 */
    KF_RNG_ACTIVE0 = 48         /* + i, PathTrace.rchit:280-311 */
};

#ifdef __cplusplus
}
#endif

#endif /* KF_TYPES_H */
