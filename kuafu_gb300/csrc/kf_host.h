// kf_host.h — host-side object model behind the C-ABI (mirrors kuafu's Kuafu,
// Scene, Camera, Geometry, GeometryInstance and light objects).
#pragma once

#include <cuda_runtime.h>

#include <array>
#include <atomic>
#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "../../include/kf.h"
#include "kf_util.h"
#include "kf_wavefront.h"

struct kf_scene_s;
struct kf_renderer_s;

struct kf_geometry_s {
    std::atomic<int> refs{1};
    std::vector<kf_vertex> vertices;
    std::vector<uint32_t> indices;
    std::vector<uint32_t> mat_index;
    bool opaque = true;
    bool hide_render = false;
    bool dynamic_ = false;
    uint64_t version = 1;       // material and flags (opaque, hideRender): instance records and TLAS
    uint64_t vert_version = 1;  // vertex data (recalculated normals): geometry upload and BLAS
};

struct kf_instance_s {
    std::atomic<int> refs{1};
    kf_geometry_s* geometry = nullptr;
    kf_scene_s* scene = nullptr;
    float transform[16];
};

struct kf_light_s {
    int kind = 0; // 1 point, 2 active
    kf_point_light point{};
    kf_active_light active{};
    kf_scene_s* scene = nullptr;
};

struct kf_camera_s {
    kf_scene_s* scene = nullptr;
    int width = 1, height = 1;
    float position[3] = {0, 0, 0};
    float front[3] = {1, 0, 0};
    float up[3] = {0, 0, 1};
    float right[3] = {0, -1, 0};
    float fx = 0.5f, fy = 0.5f, cx = 0.5f, cy = 0.5f, skew = 0.0f;
    float aperture = 0.0f, focal_length = 5.0f;
    float view[16];
    float proj[16];
    // render targets (allocated on first render at the camera size)
    kf::DeviceBuffer<float4> accum, albedo, normal, denoised;
    kf::DeviceBuffer<kf::dbl4> sum64;
    kf::DeviceBuffer<float> depth;
    kf::DeviceBuffer<uchar4> bgra;
    kf::DeviceBuffer<uint4> seg;
    bool has_frame = false;
    int target_w = 0, target_h = 0;
    // where this camera's paths of its last frame sit in the renderer's per-path buffers
    uint64_t last_path_start = 0;
    uint32_t last_spp = 0;
};

// Device copy of a scene, rebuilt when its geometry / instances change.
struct SceneGpu {
    kf::DeviceBuffer<float4> verts;
    kf::DeviceBuffer<uint32_t> indices, matidx;
    kf::DeviceBuffer<uint4> geom;
    kf::DeviceBuffer<kf_material_gpu> materials;
    kf::DeviceBuffer<kf::InstanceRec> inst;
    kf::DeviceBuffer<kf::Node4> blas_nodes, tlas_nodes;
    kf::DeviceBuffer<kf::Tri> tris;
    kf::DeviceBuffer<uint32_t> tlas_inst;
    kf::DeviceBuffer<kf_dir_light_ubo> dlight;
    kf::DeviceBuffer<kf_point_lights_ubo> plights;
    kf::DeviceBuffer<kf_active_lights_ubo> alights;
    kf::DeviceBuffer<uint4> tex_info;
    kf::DeviceBuffer<uchar4> texels;
    kf::DeviceBuffer<float> srgb_decode;
    kf::DeviceBuffer<float4> env;
    uint64_t built_env_version = 0;
    std::vector<uint32_t> blas_root;                 // per geometry
    std::vector<std::array<float, 6>> blas_box;      // per geometry object-space box
    std::vector<std::array<double, 10>> blas_bound; // per geometry: vertex box and bounding sphere
    std::vector<uint32_t> tri_offset, vert_offset;   // per geometry
    uint64_t built_geom_stamp = 0;
    uint32_t built_bvh_key = 0;  // builder, leaf size and sharing the BLAS were built with
    uint64_t built_inst_stamp = 0;
    uint64_t built_xform_stamp = 0;
    uint64_t built_vert_sum = 0;   // sum of the geometries' vert_version the buffers were built from
    uint64_t built_flag_sum = 0;   // sum of the geometries' version the instance records hold
    std::vector<kf::Node4> tlas_host_nodes; // TLAS topology kept for refits
    std::vector<uint32_t> tlas_host_inst;
    uint64_t tlas_refits = 0;
    uint64_t built_material_version = 0;
    uint64_t built_texture_version = 0;
    uint32_t blas_node_count = 0, tlas_node_count = 0;
    uint64_t generation = 0;      // bumped whenever a device buffer may have moved
    uint64_t content_version = 0; // bumped whenever any device content changed
    kf::SceneDev view{};
};

struct kf_scene_s {
    kf_renderer_s* renderer = nullptr;
    std::vector<kf_geometry_s*> geometries;
    std::vector<kf_instance_s*> instances;
    float clear_color[4] = {0, 0, 0, 1};
    // environment cube map: 6 faces of env_size^2 linear RGBA texels (empty = none)
    std::vector<float> env_texels;
    uint32_t env_size = 0;
    uint64_t env_version = 0;
    bool has_dir_light = false;
    kf_directional_light dir_light{};
    std::vector<kf_light_s*> point_lights;
    std::vector<kf_light_s*> active_lights;
    std::vector<std::unique_ptr<kf_camera_s>> cameras;
    kf_camera_s* current_camera = nullptr;
    uint64_t geom_stamp = 1;  // bumped on geometry set changes
    uint64_t inst_stamp = 1;  // bumped on instance set changes (TLAS rebuild)
    uint64_t xform_stamp = 1; // bumped on instance transform changes (TLAS refit)
    SceneGpu gpu;
    // export cache (kf_scene_export)
    std::vector<kf_flat_geometry> x_geoms;
    std::vector<kf_flat_instance> x_insts;
    std::vector<kf_material_gpu> x_mats;
    std::vector<kf_texture_desc> x_texs;
    ~kf_scene_s();
};

// A batched launch: the scenes of the batch concatenated into one set of geometry / BVH
// pools (indices rebased), so that one wavefront serves every view; each view keeps its
// own TLAS root, lights, environment and render targets in its ItemDev.
struct BatchState {
    std::vector<kf_scene_s*> scenes;   // distinct scenes, in order of first use
    std::vector<uint64_t> generations; // their SceneGpu generations when the pools were built
    kf::DeviceBuffer<float4> verts;
    kf::DeviceBuffer<uint32_t> indices, matidx, tlas_inst;
    kf::DeviceBuffer<uint4> geom;
    kf::DeviceBuffer<kf::InstanceRec> inst;
    kf::DeviceBuffer<kf::Node4> blas_nodes, tlas_nodes;
    kf::DeviceBuffer<kf::Tri> tris;
    std::vector<uint32_t> roots;       // per scene: TLAS root in tlas_nodes (kNoRoot: empty)
    kf::SceneDev view{};
    uint64_t generation = 0;           // bumped whenever a pool may have moved
    kf::DeviceBuffer<kf::ItemDev> items;
    cudaGraphExec_t graph_exec = nullptr;
    std::string graph_key;
    ~BatchState() {
        if (graph_exec) cudaGraphExecDestroy(graph_exec);
    }
};

// Wavefront buffers sized for one chunk of paths.
struct WaveBuffers {
    kf::DeviceBuffer<float4> q_o0, q_o1, q_d0, q_d1, hit, weight, nee_w, nee_in, contrib, sq_o, sq_d;
    kf::DeviceBuffer<uint32_t> counters, hit_prim, sel, scount;
    kf::DeviceBuffer<uint64_t> req;
    kf::DeviceBuffer<uint8_t> vis;
    kf::DeviceBuffer<float4> radiance;      // per path of the frame
    kf::DeviceBuffer<kf_hit> primary;       // per path of the frame (debug)
    kf::DeviceBuffer<unsigned long long> stats;
    kf::DeviceBuffer<uint16_t> path_item;   // batched launches: item of each path of a chunk
    uint32_t chunk_cap = 0, slot_cap = 0;
    uint64_t radiance_cap = 0;
};

struct kf_renderer_s {
    kf_config cfg{};
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    std::vector<std::unique_ptr<kf_scene_s>> scenes;
    kf_scene_s* current = nullptr;
    int32_t frame_count = -1;   // kuafu's global::frameCount
    uint32_t frame_index = 0;   // Philox frame word, advances every rendered frame
    bool running = true;
    const kf_camera_s* last_camera = nullptr;
    float last_position[3] = {0, 0, 0};
    WaveBuffers wave;
    kf::DeviceBuffer<kf::FrameDev> frame_dev;
    kf::DeviceBuffer<double> scratch64;
    kf_stats stats{};
    bool count_traversal = false;
    uint32_t grid_extend = 0, grid_shade = 0;
    uint32_t grid_dyn = 0, grid_dyn_shadow = 0; // persistent traversal: one resident wave each
    // CUDA graph of one frame's launch sequence
    cudaGraphExec_t graph_exec = nullptr;
    std::string graph_key;
    // events for profiling
    cudaEvent_t ev[8] = {};
    // second stream of the bounce loop: each bounce's shadow traversal and NEE gather run on
    // it, beside the next bounce's closest-hit traversal (fork / join events, no timing)
    cudaStream_t stream2 = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    // learned denoiser used by run() when cfg.use_denoiser is set
    kf_denoiser_s* denoiser = nullptr;
    // every denoiser created on this renderer (owned: freed by the renderer's destructor)
    std::vector<kf_denoiser_s*> denoisers;
    // batched launches (kf_renderer_run_batch)
    std::unique_ptr<BatchState> batch;
    ~kf_renderer_s();
};

namespace kf {

// A texture of the process-global table (kuafu's global::textureIndex space).
struct HostTexture {
    uint32_t w, h, srgb;
    std::vector<uint8_t> rgba;
};

// host math (glm conventions: column-major mat4)
void look_at(const float eye[3], const float front[3], const float up[3], float out[16]);
void projection_from_intrinsics(int w, int h, float fx, float fy, float cx, float cy, float skew, float out[16]);
void inverse4_d(const float in[16], float out[16]);
void affine_inverse_rows(const float m[16], float out_rows[12]);
void perspective(float fovy, float aspect, float znear, float zfar, float out[16]);

void camera_update_view(kf_camera_s* c);
void camera_update_proj(kf_camera_s* c);
void camera_ubo(const kf_camera_s* c, kf_camera_ubo* out);

void scene_light_ubos(const kf_scene_s* s, kf_dir_light_ubo* d, kf_point_lights_ubo* p, kf_active_lights_ubo* a);
void scene_sync_gpu(kf_renderer_s* r, kf_scene_s* s);
void render_frame(kf_renderer_s* r, kf_scene_s* s, kf_camera_s* c, uint32_t spp);
// Brings every scene up to date and (re)builds the batch's concatenated pools if any changed.
void batch_sync(kf_renderer_s* r, const std::vector<kf_scene_s*>& scenes);
// One frame of every (scene, camera, spp) item in one wavefront (kf_renderer_run_batch).
void render_batch(kf_renderer_s* r, const kf_batch_item* items, uint32_t count);
// kf_renderer_autotune (kf_autotune.cu)
void autotune_batch(kf_renderer_s* r, const kf_batch_item* items, uint32_t count, uint32_t reps,
                    kf_autotune_result* out);
// Achievable L2 read bandwidth in GB/s (kf_autotune.cu).
double measure_l2_read(kf_renderer_s* r, uint64_t bytes, uint32_t passes, uint32_t reps);

// global tables
std::vector<kf_material_gpu> flatten_materials();
const std::vector<float>& srgb_decode_table();
const std::vector<float>& srgb_threshold_table();

// procedural meshes
void mesh_yz_plane(std::vector<kf_vertex>& v, std::vector<uint32_t>& i);
void mesh_cube(std::vector<kf_vertex>& v, std::vector<uint32_t>& i);
void mesh_sphere(std::vector<kf_vertex>& v, std::vector<uint32_t>& i);
void mesh_capsule(float half_length, float radius, std::vector<kf_vertex>& v, std::vector<uint32_t>& i);
void mesh_icosphere(int level, std::vector<kf_vertex>& v, std::vector<uint32_t>& i);
void recalculate_normals(std::vector<kf_vertex>& v, const std::vector<uint32_t>& i);

} // namespace kf
