// kf_wavefront.h — device data views and kernel launchers of the wavefront path tracer.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "kf_device.cuh"

namespace kf {

constexpr int kMaxLightSlots = 1 + KF_MAX_POINT_LIGHTS + KF_MAX_ACTIVE_LIGHTS; // 41

// Everything a kernel needs to read about one scene (device pointers).
struct SceneDev {
    const float4* verts;             // 3 float4 per vertex (kf_vertex, 48 B)
    const uint32_t* indices;         // 3 per triangle, geometry-local vertex indices
    const uint32_t* matidx;          // material index per triangle
    const uint4* geom;               // per geometry {vertex_offset, tri_offset, num_tris, flags}
    const kf_material_gpu* materials;
    const InstanceRec* inst;
    const Node4* blas_nodes;
    const Tri* tris;
    const Node4* tlas_nodes;
    const uint32_t* tlas_inst;
    const kf_dir_light_ubo* dlight;
    const kf_point_lights_ubo* plights;
    const kf_active_lights_ubo* alights;
    const uint4* tex_info;           // per texture {texel offset, width, height, srgb}
    const uchar4* texels;
    const float* srgb_decode;        // 256 entries
    const float4* env;               // environment cube map: 6 faces of env_size^2 texels (null = none)
    uint32_t env_size;
    uint32_t num_instances;
    uint32_t has_tlas;
    uint32_t num_textures;
    uint32_t num_slots;              // shadow-ray light slots in use
    uint8_t slot_group[kMaxLightSlots]; // 0 directional, 1 point, 2 active
    uint8_t slot_index[kMaxLightSlots];
};

// Per-frame constants, resident in device memory so a captured graph can replay them.
struct FrameDev {
    kf_camera_ubo cam;
    kf_push_constants pc;
    uint32_t width, height, npix, seed;
    uint32_t frame, camera_index, pad0, pad1;
};

constexpr uint32_t kNoRoot = 0xFFFFFFFFu;

// One view of a batched launch: its frame constants, where its paths start in the
// batch's path space, and what of its scene the kernels need beyond the shared
// (concatenated) geometry / BVH pools: TLAS root, light slots, environment, AOVs.
struct ItemDev {
    FrameDev f;
    uint64_t path_start;
    uint32_t root;            // TLAS root node in the batch's node pool (kNoRoot: nothing to hit)
    uint32_t num_slots;
    uint8_t slot_group[kMaxLightSlots];
    uint8_t slot_index[kMaxLightSlots];
    uint16_t pad;
    const kf_dir_light_ubo* dlight;
    const kf_point_lights_ubo* plights;
    const kf_active_lights_ubo* alights;
    const float4* env;
    uint32_t env_size;
    uint32_t inst_base;       // first instance of the item's scene in the batch's instance pool
    uint32_t geom_base;       // first geometry of the item's scene in the batch's geometry pool
    uint32_t pad3;
    float4* albedo;
    float4* normal;
    float* depth;
    uint4* seg;
};

// Batch description handed to the kernels (items == nullptr: a single-view frame).
struct BatchDev {
    const ItemDev* items;
    uint32_t num_items;
    uint32_t pad;
};

// Per-chunk wavefront state.
struct WaveDev {
    float4* q_o[2];       // ray queue: origin.xyz + path id bits
    float4* q_d[2];       // ray queue: direction.xyz
    uint32_t* counters;   // [0],[1] ray queue counts, [2] shadow count, [3],[4] fetch cursors,
                          // [5] rays of the bounce that hit
    float4* hit;          // t, u, v, instance bits
    uint32_t* hit_prim;
    uint32_t* sel;        // queue positions of this bounce's rays that hit ([5] of them)
    uint32_t* scount;     // per light slot j: shadow rays queued, at sq_o/sq_d[j * chunk_cap + k]
    uint32_t nslot;       // light slots with a shadow queue (scount entries)
    float4* weight;       // throughput carried to the next bounce
    float4* nee_w;        // throughput that scales this bounce's NEE
    float4* nee_in;       // per hit (hit-list order), 6 float4: what k_nee needs of k_shade's shading
    uint64_t* req;        // shadow slots requested this bounce (bit j = slot j)
    float4* contrib;      // [slot][chunk] light contribution
    uint8_t* vis;         // [slot][chunk] 1 = unoccluded
    float4* sq_o;         // shadow queue: origin.xyz + tmax
    float4* sq_d;         // shadow queue: direction.xyz + (slot << 26 | path) bits
    float4* radiance;     // per global path (frame): accumulated `color`
    kf_hit* primary;      // per global path, debug (may be null)
    float4* albedo;       // per pixel AOVs
    float4* normal;
    float* depth;
    uint4* seg;           // per pixel {instance, geometry, material, primitive} of sample 0's first hit
    unsigned long long* stats; // [0] primary, [1] extension, [2] shadow, [3] nodes, [4] tris, [5] inst
    uint16_t* path_item;       // batched launch: item of each path of the chunk
    uint32_t chunk_cap;
};

// Every launcher takes the batch description b: b.items == nullptr renders the single
// view of f with the scene's own TLAS and lights; otherwise f is unused and each path
// takes its frame constants, TLAS root, lights and AOV targets from its item.
void launch_raygen(const FrameDev* f, const BatchDev& b, const WaveDev& w, uint64_t chunk_start, uint32_t chunk_n,
                   cudaStream_t st);
void launch_extend(const SceneDev& s, const FrameDev* f, const BatchDev& b, const WaveDev& w, int cur,
                   uint32_t depth, uint64_t chunk_start, uint32_t grid, bool count_mode, cudaStream_t st);
// k_miss ends the paths whose ray missed and lists the others in w.sel; k_shade shades those.
void launch_shade(const SceneDev& s, const FrameDev* f, const BatchDev& b, const WaveDev& w, int cur,
                  uint32_t depth, uint64_t chunk_start, uint32_t grid, cudaStream_t st);
void launch_miss(const SceneDev& s, const FrameDev* f, const BatchDev& b, const WaveDev& w, int cur,
                 uint32_t depth, uint64_t chunk_start, uint32_t grid, cudaStream_t st);
// Light samples (shadow queues, contributions, NEE requests) of the hits k_shade shaded.
void launch_nee(const SceneDev& s, const FrameDev* f, const BatchDev& b, const WaveDev& w, uint32_t depth,
                uint64_t chunk_start, uint32_t grid, cudaStream_t st);
void launch_shadow(const SceneDev& s, const BatchDev& b, const WaveDev& w, uint32_t grid, bool count_mode,
                   cudaStream_t st);
// Persistent traversal with dynamic ray fetch (closest hit, or shadow rays when `shadow`).
// Needs w.counters[3] (closest) / w.counters[4] (shadow) zeroed before the launch.
// refill_below (1..32) and steps (1..64): the warp scheduling of the persistent kernel.
void launch_trace_dyn(const SceneDev& s, const FrameDev* f, const BatchDev& b, const WaveDev& w, int cur,
                      uint32_t depth, uint64_t chunk_start, bool shadow, uint32_t grid, bool count_mode,
                      uint32_t refill_below, uint32_t steps, cudaStream_t st);
// resident blocks per SM of the persistent traversal kernel (closest-hit or shadow variant)
uint32_t trace_dyn_blocks_per_sm(bool shadow);
void launch_gather(const SceneDev& s, const BatchDev& b, const WaveDev& w, int cur, uint64_t chunk_start,
                   uint32_t grid, cudaStream_t st);
void launch_resolve(const FrameDev* f, const float4* radiance, uint32_t npix, uint32_t spp, float4* accum,
                    dbl4* sum64, cudaStream_t st);
void launch_srgb(const float4* img, uint32_t npix, uchar4* out, cudaStream_t st);
void upload_srgb_thresholds(const float* thresh256);
void launch_relmse(const float4* x, const float4* ref, uint64_t n, double eps, double* partial, uint32_t blocks,
                   double* out, cudaStream_t st);

} // namespace kf
