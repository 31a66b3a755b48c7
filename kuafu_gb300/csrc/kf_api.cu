// kf_api.cu — the C-ABI (include/kf.h): exception-free entry points over the
// host object model. Each function mirrors the kuafu method named in kf.h.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <string>

#include "kf_denoise.h"
#include "kf_host.h"
#include "kf_obj.h"

namespace kf {
std::mutex& global_mutex() {
    static std::mutex m;
    return m;
}
std::vector<kf_material> g_materials;
std::vector<HostTexture> g_textures;
uint64_t g_material_version = 1, g_texture_version = 1;

// sRGB transfer tables computed in FP64 (IEC 61966-2-1 piecewise curve).
const std::vector<float>& srgb_decode_table() {
    static const std::vector<float> t = [] {
        std::vector<float> v(256);
        for (int i = 0; i < 256; ++i) {
            const double c = i / 255.0;
            v[i] = (float)(c <= 0.04045 ? c / 12.92 : std::pow((c + 0.055) / 1.055, 2.4));
        }
        return v;
    }();
    return t;
}
// thresh[k] = linear value at which the 8-bit sRGB code reaches k (k - 0.5 on the code axis).
const std::vector<float>& srgb_threshold_table() {
    static const std::vector<float> t = [] {
        std::vector<float> v(256);
        v[0] = -INFINITY;
        for (int k = 1; k < 256; ++k) {
            const double c = (k - 0.5) / 255.0;
            v[k] = (float)(c <= 0.04045 ? c / 12.92 : std::pow((c + 0.055) / 1.055, 2.4));
        }
        return v;
    }();
    return t;
}
} // namespace kf

using namespace kf;

namespace {
thread_local std::string t_error;
}

namespace kf {
void set_last_error(const std::string& msg) { t_error = msg; }
}

namespace {
int fail(int code, const std::string& msg) {
    t_error = msg;
    return code;
}

template <class F> int guarded(F&& f) {
    try {
        f();
        return KF_OK;
    } catch (const KfError& e) {
        return fail(e.code, e.what());
    } catch (const std::bad_alloc&) {
        return fail(KF_ERR_OUT_OF_MEMORY, "host allocation failed");
    } catch (const std::exception& e) {
        return fail(KF_ERR_INTERNAL, e.what());
    }
}

#define REQ(cond, msg) KF_REQUIRE(cond, KF_ERR_INVALID_ARGUMENT, msg)

void camera_init(kf_camera_s* c, int w, int h) {
    // Camera::Camera (camera.cpp:8-18) + resetView (camera.cpp:20-30)
    c->width = w;
    c->height = h;
    c->cx = (float)w * 0.5f;
    c->cy = (float)h * 0.5f;
    c->fx = c->fy = (float)w * 0.5f;
    camera_update_proj(c);
    c->position[0] = c->position[1] = c->position[2] = 0.0f;
    const float up[3] = {0, 0, 1}, right[3] = {0, -1, 0}, front[3] = {1, 0, 0};
    std::memcpy(c->up, up, sizeof(up));
    std::memcpy(c->right, right, sizeof(right));
    std::memcpy(c->front, front, sizeof(front));
    camera_update_view(c);
}

kf_camera_s* scene_new_camera(kf_scene_s* s, int w, int h) {
    auto cam = std::make_unique<kf_camera_s>();
    cam->scene = s;
    camera_init(cam.get(), w, h);
    s->cameras.push_back(std::move(cam));
    return s->cameras.back().get();
}

kf_scene_s* new_scene(kf_renderer_s* r) {
    auto s = std::make_unique<kf_scene_s>();
    s->renderer = r;
    s->current_camera = scene_new_camera(s.get(), 1, 1); // Scene::Scene (scene.hpp:215-217)
    r->scenes.push_back(std::move(s));
    return r->scenes.back().get();
}

void geometry_retain(kf_geometry_s* g) { g->refs.fetch_add(1); }
void geometry_release(kf_geometry_s* g) {
    if (g && g->refs.fetch_sub(1) == 1) delete g;
}
void instance_release(kf_instance_s* i) {
    if (i && i->refs.fetch_sub(1) == 1) {
        geometry_release(i->geometry);
        delete i;
    }
}

kf_scene_s* check_scene(kf_scene s) {
    REQ(s != nullptr, "invalid scene handle");
    return s;
}
kf_camera_s* check_camera(kf_camera c) {
    REQ(c != nullptr, "invalid camera handle");
    return c;
}

void material_to_table(const kf_material* m, uint32_t* idx) {
    std::lock_guard<std::mutex> lk(global_mutex());
    g_materials.push_back(*m);
    ++g_material_version;
    if (idx) *idx = (uint32_t)(g_materials.size() - 1);
}

void frame_reset(kf_renderer_s* r) { r->frame_count = -1; }

void sync_stream(kf_renderer_s* r) {
    if (!r->cfg.host_only) KF_CUDA_CHECK(cudaStreamSynchronize(r->stream));
}

} // namespace

kf_scene_s::~kf_scene_s() {
    for (kf_instance_s* i : instances) {
        i->scene = nullptr;
        instance_release(i);
    }
    for (kf_geometry_s* g : geometries) geometry_release(g);
    for (kf_light_s* l : point_lights) delete l;
    for (kf_light_s* l : active_lights) delete l;
}

kf_renderer_s::~kf_renderer_s() {
    if (stream) cudaStreamSynchronize(stream);
    for (kf_denoiser_s* d : denoisers) kf::denoiser_destroy(d);
    denoisers.clear();
    denoiser = nullptr;
    if (graph_exec) cudaGraphExecDestroy(graph_exec);
    for (cudaEvent_t e : ev)
        if (e) cudaEventDestroy(e);
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (ev_join) cudaEventDestroy(ev_join);
    scenes.clear();
    if (stream2) {
        cudaStreamSynchronize(stream2);
        cudaStreamDestroy(stream2);
    }
    if (stream) cudaStreamDestroy(stream);
}

extern "C" {

KF_API const char* kf_last_error(void) { return t_error.c_str(); }
KF_API int kf_version(void) { return 10000; }

KF_API void kf_config_init(kf_config* c) {
    if (!c) return;
    std::memset(c, 0, sizeof(*c));
    c->initial_width = 800;
    c->initial_height = 600;
    c->spp = 32;
    c->path_depth = 8;
    c->max_path_depth = 12;
    c->russian_roulette = 1;
    c->rr_min_bounces = 4;
    c->nee = 1;
    c->nee_min_bounces = 0;
    c->accumulate_frames = 1;
    c->use_denoiser = 0;
    c->present = 1;
    c->max_geometries = 128;
    c->max_instances = 256;
    c->max_textures = 128;
    c->max_materials = 256;
    c->seed = 0;
    c->blas_leaf_size = 1;
    c->tlas_leaf_size = 1;
    c->max_paths_in_flight = 1ull << 24;
    c->debug_outputs = 0;
    c->profile = 0;
    c->use_graph = 1;
    c->device = 0;
    c->host_only = 0;
    c->traversal = 1;
    c->bvh_builder = 1;
    c->dyn_refill_below = 16;
    c->dyn_steps = 32;
    c->blas_share = 1;
}

KF_API int kf_renderer_create(const kf_config* cfg, kf_renderer* out) {
    return guarded([&] {
        REQ(out != nullptr, "out is null");
        *out = nullptr;
        auto r = std::make_unique<kf_renderer_s>();
        if (cfg)
            r->cfg = *cfg;
        else
            kf_config_init(&r->cfg);
        if (!r->cfg.host_only) {
            int ndev = 0;
            cudaError_t e = cudaGetDeviceCount(&ndev);
            KF_REQUIRE(e == cudaSuccess && ndev > 0, KF_ERR_NO_DEVICE,
                       "no CUDA device available: the path tracer has no CPU fallback");
            KF_REQUIRE((int)r->cfg.device < ndev, KF_ERR_NO_DEVICE, "requested CUDA device does not exist");
            r->device = (int)r->cfg.device;
            KF_CUDA_CHECK(cudaSetDevice(r->device));
            KF_CUDA_CHECK(cudaDeviceGetAttribute(&r->num_sms, cudaDevAttrMultiProcessorCount, r->device));
            KF_CUDA_CHECK(cudaStreamCreateWithFlags(&r->stream, cudaStreamNonBlocking));
            KF_CUDA_CHECK(cudaStreamCreateWithFlags(&r->stream2, cudaStreamNonBlocking));
            for (cudaEvent_t& ev : r->ev) KF_CUDA_CHECK(cudaEventCreate(&ev));
            KF_CUDA_CHECK(cudaEventCreateWithFlags(&r->ev_fork, cudaEventDisableTiming));
            KF_CUDA_CHECK(cudaEventCreateWithFlags(&r->ev_join, cudaEventDisableTiming));
            upload_srgb_thresholds(srgb_threshold_table().data());
        }
        // persistent grids: enough resident warps to hide traversal latency
        r->grid_extend = (uint32_t)r->num_sms * 16;
        r->grid_shade = (uint32_t)r->num_sms * 16; // 16 blocks per SM measured fastest (4, 8, 16)
        if (!r->cfg.host_only) {
            r->grid_dyn = (uint32_t)r->num_sms * trace_dyn_blocks_per_sm(false);
            r->grid_dyn_shadow = (uint32_t)r->num_sms * trace_dyn_blocks_per_sm(true);
        }
        // Kuafu::Kuafu (kuafu.cpp:27-63): a scene with a 1x1 camera; present mode adds
        // a camera of the initial size and makes it current.
        kf_scene_s* s = new_scene(r.get());
        r->current = s;
        if (r->cfg.present) {
            s->current_camera = scene_new_camera(s, r->cfg.initial_width, r->cfg.initial_height);
        }
        *out = r.release();
    });
}

KF_API int kf_renderer_destroy(kf_renderer r) {
    return guarded([&] {
        if (!r) return;
        if (!r->cfg.host_only) {
            cudaSetDevice(r->device);
            if (r->stream) cudaStreamSynchronize(r->stream);
        }
        delete r;
    });
}

static void require_device(kf_renderer_s* r) {
    KF_REQUIRE(!r->cfg.host_only, KF_ERR_NO_DEVICE,
               "renderer was created host-only: rendering needs a CUDA device (there is no CPU fallback)");
}

KF_API int kf_renderer_get_config(kf_renderer r, kf_config* out) {
    return guarded([&] {
        REQ(r && out, "null argument");
        *out = r->cfg;
    });
}
KF_API int kf_renderer_set_config(kf_renderer r, const kf_config* cfg) {
    return guarded([&] {
        REQ(r && cfg, "null argument");
        const uint32_t dev = r->cfg.device;
        r->cfg = *cfg;
        r->cfg.device = dev;
        // Config::setPathDepth clamps to the maximum (config.cpp:29-40, with the clamp
        // immediately overwritten in kuafu; the value given is used as is).
    });
}
KF_API int kf_renderer_get_scene(kf_renderer r, kf_scene* out) {
    return guarded([&] {
        REQ(r && out, "null argument");
        *out = r->current;
    });
}
KF_API int kf_renderer_create_scene(kf_renderer r, kf_scene* out) {
    return guarded([&] {
        REQ(r && out, "null argument");
        *out = new_scene(r);
    });
}
KF_API int kf_renderer_set_scene(kf_renderer r, kf_scene s) {
    return guarded([&] {
        REQ(r && s, "Trying to set an invalid scene!");
        auto it = std::find_if(r->scenes.begin(), r->scenes.end(), [&](auto& p) { return p.get() == s; });
        REQ(it != r->scenes.end(), "scene does not belong to this renderer");
        if (r->current == s) return;
        r->current = s;
        frame_reset(r);
    });
}
KF_API int kf_renderer_remove_scene(kf_renderer r, kf_scene s) {
    return guarded([&] {
        REQ(r && s, "Trying to remove an invalid scene!");
        auto it = std::find_if(r->scenes.begin(), r->scenes.end(), [&](auto& p) { return p.get() == s; });
        REQ(it != r->scenes.end(), "scene does not belong to this renderer");
        sync_stream(r);
        if (r->graph_exec) {
            cudaGraphExecDestroy(r->graph_exec);
            r->graph_exec = nullptr;
            r->graph_key.clear();
        }
        if (r->current == s) r->current = nullptr;
        r->scenes.erase(it);
    });
}
KF_API int kf_renderer_is_running(kf_renderer r, int* out) {
    return guarded([&] {
        REQ(r && out, "null argument");
        *out = r->running ? 1 : 0;
    });
}

KF_API int kf_renderer_run(kf_renderer r) {
    return guarded([&] {
        REQ(r, "invalid renderer");
        KF_REQUIRE(r->current, KF_ERR_STATE, "no current scene");
        kf_scene_s* s = r->current;
        kf_camera_s* c = s->current_camera;
        KF_REQUIRE(c, KF_ERR_STATE, "Trying to render with an invalid camera!");
        require_device(r);
        KF_CUDA_CHECK(cudaSetDevice(r->device));
        // Camera::update (camera.cpp:41-51): a moved camera restarts accumulation
        if (r->last_camera != c || std::memcmp(r->last_position, c->position, sizeof(r->last_position)) != 0) {
            frame_reset(r);
            r->last_camera = c;
            std::memcpy(r->last_position, c->position, sizeof(r->last_position));
        }
        camera_update_view(c);
        KF_REQUIRE(!r->cfg.use_denoiser || r->denoiser, KF_ERR_STATE,
                   "use_denoiser is set but no denoiser is attached (kf_renderer_set_denoiser)");
        render_frame(r, s, c, r->cfg.spp);
        if (r->cfg.use_denoiser) present_denoised(r, c);
    });
}

// Validated copy of a batch: scenes of this renderer, cameras of their scene, each once.
static std::vector<kf_batch_item> checked_batch(kf_renderer r, const kf_batch_item* items, uint32_t count) {
    REQ(r && (items || count == 0), "null argument");
    require_device(r);
    KF_CUDA_CHECK(cudaSetDevice(r->device));
    std::vector<kf_batch_item> v(items, items + count);
    for (uint32_t i = 0; i < count; ++i) {
        kf_scene_s* s = check_scene(v[i].scene);
        kf_camera_s* c = check_camera(v[i].camera);
        REQ(c->scene == s, "batch camera does not belong to its scene");
        REQ(std::find_if(r->scenes.begin(), r->scenes.end(), [&](auto& p) { return p.get() == s; }) !=
                r->scenes.end(),
            "batch scene does not belong to this renderer");
        for (uint32_t j = 0; j < i; ++j) REQ(v[j].camera != c, "a camera appears twice in one batch");
        camera_update_view(c);
        if (!v[i].spp) v[i].spp = r->cfg.spp;
    }
    return v;
}

KF_API int kf_renderer_run_batch(kf_renderer r, const kf_batch_item* items, uint32_t count) {
    return guarded([&] {
        std::vector<kf_batch_item> v = checked_batch(r, items, count);
        if (count) render_batch(r, v.data(), count);
    });
}

KF_API int kf_renderer_autotune(kf_renderer r, const kf_batch_item* items, uint32_t count, uint32_t reps,
                                kf_autotune_result* out) {
    return guarded([&] {
        std::vector<kf_batch_item> v = checked_batch(r, items, count);
        REQ(count > 0, "empty batch");
        REQ(!r->cfg.profile && !r->count_traversal, "autotune measures the production path: profile and "
                                                    "traversal counting must be off");
        autotune_batch(r, v.data(), count, reps, out);
    });
}

KF_API int kf_renderer_measure_l2_read(kf_renderer r, uint64_t bytes, uint32_t passes, uint32_t reps,
                                       double* gbs) {
    return guarded([&] {
        REQ(r && gbs, "null argument");
        REQ(bytes >= (1u << 20) && bytes <= (1ull << 30), "probe size must be in [1 MiB, 1 GiB]");
        require_device(r);
        *gbs = measure_l2_read(r, bytes, passes, reps);
    });
}

KF_API int kf_renderer_synchronize(kf_renderer r) {
    return guarded([&] {
        REQ(r, "invalid renderer");
        sync_stream(r);
    });
}

KF_API int kf_renderer_get_stream(kf_renderer r, void** out) {
    return guarded([&] {
        REQ(r && out, "null argument");
        require_device(r);
        *out = (void*)r->stream;
    });
}

KF_API int kf_renderer_download_latest_frame(kf_renderer r, kf_camera cam, uint8_t* out, size_t bytes) {
    return guarded([&] {
        REQ(r && out, "null argument");
        require_device(r);
        kf_camera_s* c = check_camera(cam);
        KF_REQUIRE(c->has_frame, KF_ERR_STATE, "Invalid call to Camera::downloadLatestFrame");
        const size_t need = (size_t)c->target_w * c->target_h * 4;
        KF_REQUIRE(bytes >= need, KF_ERR_OUT_OF_RANGE, "output buffer too small for the frame");
        KF_CUDA_CHECK(cudaMemcpyAsync(out, c->bgra.ptr, need, cudaMemcpyDeviceToHost, r->stream));
        sync_stream(r);
    });
}

KF_API int kf_renderer_download_aov(kf_renderer r, kf_camera cam, int kind, void* out, size_t bytes) {
    return guarded([&] {
        REQ(r && out, "null argument");
        require_device(r);
        kf_camera_s* c = check_camera(cam);
        KF_REQUIRE(c->has_frame, KF_ERR_STATE, "no frame rendered for this camera");
        const size_t npix = (size_t)c->target_w * c->target_h;
        const void* src = nullptr;
        size_t need = 0;
        switch (kind) {
            case KF_AOV_RADIANCE_F32: src = c->accum.ptr; need = npix * 16; break;
            case KF_AOV_ALBEDO_F32: src = c->albedo.ptr; need = npix * 16; break;
            case KF_AOV_NORMAL_F32: src = c->normal.ptr; need = npix * 16; break;
            case KF_AOV_DEPTH_F32: src = c->depth.ptr; need = npix * 4; break;
            case KF_AOV_SUM_F64: src = c->sum64.ptr; need = npix * 32; break;
            case KF_AOV_PATH_RADIANCE:
                src = r->wave.radiance.ptr + c->last_path_start;
                need = (size_t)c->last_spp * npix * 16;
                break;
            case KF_AOV_PRIMARY_HITS:
                KF_REQUIRE(r->cfg.debug_outputs, KF_ERR_STATE, "primary hits need debug_outputs = 1");
                src = r->wave.primary.ptr + c->last_path_start;
                need = (size_t)c->last_spp * npix * sizeof(kf_hit);
                break;
            case KF_AOV_SEGMENTATION: src = c->seg.ptr; need = npix * 16; break;
            case KF_AOV_DENOISED_F32:
                KF_REQUIRE(c->denoised.count == npix, KF_ERR_STATE, "no denoised frame for this camera");
                src = c->denoised.ptr;
                need = npix * 16;
                break;
            default: throw KfError(KF_ERR_INVALID_ARGUMENT, "unknown AOV kind");
        }
        KF_REQUIRE(bytes >= need, KF_ERR_OUT_OF_RANGE, "output buffer too small for the AOV");
        KF_CUDA_CHECK(cudaMemcpyAsync(out, src, need, cudaMemcpyDeviceToHost, r->stream));
        sync_stream(r);
    });
}

KF_API int kf_renderer_get_stats(kf_renderer r, kf_stats* out) {
    return guarded([&] {
        REQ(r && out, "null argument");
        sync_stream(r);
        if (r->wave.stats.count) {
            unsigned long long h[16] = {};
            KF_CUDA_CHECK(cudaMemcpy(h, r->wave.stats.ptr, sizeof(h), cudaMemcpyDeviceToHost));
            r->stats.rays_primary = h[0];
            r->stats.rays_extension = h[1];
            r->stats.rays_shadow = h[2];
            r->stats.node_visits = h[3];
            r->stats.tri_tests = h[4];
            r->stats.inst_visits = h[5];
            r->stats.shadow_node_visits = h[6];
            r->stats.shadow_tri_tests = h[7];
            r->stats.shadow_inst_visits = h[8];
        }
        *out = r->stats;
    });
}
KF_API int kf_renderer_reset_frame(kf_renderer r) {
    return guarded([&] {
        REQ(r, "invalid renderer");
        frame_reset(r);
    });
}
KF_API int kf_renderer_reset_stats(kf_renderer r) {
    return guarded([&] {
        REQ(r, "invalid renderer");
        sync_stream(r);
        if (r->wave.stats.count && !r->cfg.host_only)
            KF_CUDA_CHECK(cudaMemset(r->wave.stats.ptr, 0, r->wave.stats.bytes()));
        const int32_t fc = r->stats.frame_count;
        const uint32_t bn = r->stats.blas_nodes, tn = r->stats.tlas_nodes, ls = r->stats.last_spp;
        std::memset(&r->stats, 0, sizeof(r->stats));
        r->stats.frame_count = fc;
        r->stats.blas_nodes = bn;
        r->stats.tlas_nodes = tn;
        r->stats.last_spp = ls;
    });
}
KF_API int kf_renderer_count_traversal(kf_renderer r, int enable) {
    return guarded([&] {
        REQ(r, "invalid renderer");
        r->count_traversal = enable != 0;
    });
}

// ---- materials ----
KF_API void kf_material_init(kf_material* m) {
    if (!m) return;
    std::memset(m, 0, sizeof(*m));
    m->diffuse_color[0] = m->diffuse_color[1] = m->diffuse_color[2] = 1.0f;
    m->alpha = 1.0f;
    m->metallic = 0.0f;
    m->specular = 0.5f;
    m->roughness = 0.5f;
    m->ior = 1.4f;
    m->transmission = 0.0f;
    m->emission[0] = m->emission[1] = m->emission[2] = 1.0f;
    m->emission_strength = 0.0f;
    m->diffuse_tex = m->metallic_tex = m->roughness_tex = m->transmission_tex = -1;
}
KF_API int kf_material_add(const kf_material* m, uint32_t* out_index) {
    return guarded([&] {
        REQ(m, "null material");
        material_to_table(m, out_index);
    });
}
KF_API uint32_t kf_material_count(void) {
    std::lock_guard<std::mutex> lk(global_mutex());
    return (uint32_t)g_materials.size();
}
KF_API int kf_material_get(uint32_t index, kf_material* out) {
    return guarded([&] {
        REQ(out, "null argument");
        std::lock_guard<std::mutex> lk(global_mutex());
        KF_REQUIRE(index < g_materials.size(), KF_ERR_OUT_OF_RANGE, "material index out of range");
        *out = g_materials[index];
    });
}
KF_API int kf_material_clear(void) {
    std::lock_guard<std::mutex> lk(global_mutex());
    g_materials.clear();
    ++g_material_version;
    return KF_OK;
}

KF_API int kf_texture_create(const uint8_t* rgba8, uint32_t width, uint32_t height, int srgb, int32_t* out_id) {
    return guarded([&] {
        REQ(rgba8 && width && height && out_id, "invalid texture arguments");
        std::lock_guard<std::mutex> lk(global_mutex());
        HostTexture t;
        t.w = width;
        t.h = height;
        t.srgb = srgb ? 1u : 0u;
        t.rgba.assign(rgba8, rgba8 + (size_t)width * height * 4);
        g_textures.push_back(std::move(t));
        ++g_texture_version;
        *out_id = (int32_t)(g_textures.size() - 1);
    });
}
KF_API uint32_t kf_texture_count(void) {
    std::lock_guard<std::mutex> lk(global_mutex());
    return (uint32_t)g_textures.size();
}

// ---- geometry ----
KF_API int kf_geometry_create(const kf_vertex* v, uint32_t nv, const uint32_t* idx, uint32_t nidx,
                              const uint32_t* mat_index, uint32_t n_mat, kf_geometry* out) {
    return guarded([&] {
        REQ(out, "null argument");
        REQ(nidx % 3 == 0, "index count must be a multiple of 3");
        REQ((v || nv == 0) && (idx || nidx == 0), "null vertex or index data");
        REQ(n_mat >= nidx / 3, "matIndex must hold one entry per triangle");
        for (uint32_t i = 0; i < nidx; ++i)
            KF_REQUIRE(idx[i] < nv, KF_ERR_OUT_OF_RANGE, "vertex index out of range");
        for (uint32_t i = 0; i < nv; ++i)
            for (int k = 0; k < 3; ++k)
                REQ(std::isfinite(v[i].pos[k]), "vertex position is not finite");
        auto g = new kf_geometry_s();
        g->vertices.assign(v, v + nv);
        g->indices.assign(idx, idx + nidx);
        g->mat_index.assign(mat_index, mat_index + n_mat);
        *out = g;
    });
}
KF_API int kf_geometry_set_material(kf_geometry g, const kf_material* m) {
    return guarded([&] {
        REQ(g && m, "null argument");
        // Geometry::setMaterial (geometry.cpp:241-249)
        g->opaque = m->alpha >= 1.0f;
        uint32_t idx = 0;
        material_to_table(m, &idx);
        for (auto& x : g->mat_index) x = idx;
        ++g->version;
    });
}
KF_API int kf_geometry_set_flags(kf_geometry g, int opaque, int hide_render, int dynamic_) {
    return guarded([&] {
        REQ(g, "null geometry");
        g->opaque = opaque != 0;
        g->hide_render = hide_render != 0;
        g->dynamic_ = dynamic_ != 0;
        ++g->version;
    });
}
KF_API int kf_geometry_recalculate_normals(kf_geometry g) {
    return guarded([&] {
        REQ(g, "null geometry");
        recalculate_normals(g->vertices, g->indices);
        ++g->vert_version;
    });
}
KF_API int kf_geometry_get_info(kf_geometry g, uint32_t* nv, uint32_t* ni) {
    return guarded([&] {
        REQ(g, "null geometry");
        if (nv) *nv = (uint32_t)g->vertices.size();
        if (ni) *ni = (uint32_t)g->indices.size();
    });
}
KF_API int kf_geometry_get_data(kf_geometry g, kf_vertex* v, uint32_t* idx, uint32_t* mat) {
    return guarded([&] {
        REQ(g, "null geometry");
        if (v) std::memcpy(v, g->vertices.data(), sizeof(kf_vertex) * g->vertices.size());
        if (idx) std::memcpy(idx, g->indices.data(), sizeof(uint32_t) * g->indices.size());
        if (mat) std::memcpy(mat, g->mat_index.data(), sizeof(uint32_t) * (g->indices.size() / 3));
    });
}
KF_API int kf_geometry_release(kf_geometry g) {
    return guarded([&] { geometry_release(g); });
}
KF_API int kf_load_scene(const char* path, int dynamic, kf_geometry* out, uint32_t capacity, uint32_t* count) {
    return guarded([&] {
        REQ(path && count, "null argument");
        std::vector<ObjMesh> meshes;
        load_obj(path, meshes);
        *count = (uint32_t)meshes.size();
        if (!out) return;
        KF_REQUIRE(capacity >= meshes.size(), KF_ERR_OUT_OF_RANGE, "output array too small for the scene's geometries");
        // materials: reuse an identical entry of the global table (geometry.cpp:154-173)
        std::vector<uint32_t> mat_idx(meshes.size());
        {
            std::lock_guard<std::mutex> lk(global_mutex());
            for (size_t k = 0; k < meshes.size(); ++k) {
                const kf_material& m = meshes[k].material;
                size_t j = 0;
                for (; j < g_materials.size(); ++j)
                    if (std::memcmp(&g_materials[j], &m, sizeof(m)) == 0) break;
                if (j == g_materials.size()) {
                    g_materials.push_back(m);
                    ++g_material_version;
                }
                mat_idx[k] = (uint32_t)j;
            }
        }
        for (size_t k = 0; k < meshes.size(); ++k) {
            auto g = new kf_geometry_s();
            g->vertices = std::move(meshes[k].vertices);
            g->indices = std::move(meshes[k].indices);
            g->mat_index.assign(g->indices.size() / 3, mat_idx[k]);
            g->opaque = meshes[k].material.alpha >= 1.0f; // geometry.cpp:226
            g->dynamic_ = dynamic != 0;
            out[k] = g;
        }
    });
}
KF_API int kf_geometry_create_builtin(int kind, float p0, float p1, const kf_material* m, kf_geometry* out) {
    return guarded([&] {
        REQ(out, "null argument");
        kf_material def;
        kf_material_init(&def);
        const kf_material* mm = m ? m : &def;
        auto g = new kf_geometry_s();
        try {
            switch (kind) {
                case KF_MESH_YZ_PLANE: mesh_yz_plane(g->vertices, g->indices); break;
                case KF_MESH_CUBE: mesh_cube(g->vertices, g->indices); break;
                case KF_MESH_SPHERE: mesh_sphere(g->vertices, g->indices); break;
                case KF_MESH_CAPSULE: mesh_capsule(p0, p1, g->vertices, g->indices); break;
                case KF_MESH_ICOSPHERE: mesh_icosphere((int)p0, g->vertices, g->indices); break;
                default: throw KfError(KF_ERR_INVALID_ARGUMENT, "unknown builtin mesh kind");
            }
            // createX: isOpaque = alpha >= 1; matIndex = one fresh material for every index slot
            g->opaque = mm->alpha >= 1.0f;
            uint32_t idx = 0;
            material_to_table(mm, &idx);
            g->mat_index.assign(g->indices.size(), idx);
            g->dynamic_ = true;
        } catch (...) {
            delete g;
            throw;
        }
        *out = g;
    });
}

// ---- scene ----
KF_API int kf_scene_submit_geometry(kf_scene s, kf_geometry g) {
    return guarded([&] {
        check_scene(s);
        REQ(g, "null geometry");
        KF_REQUIRE(s->geometries.size() < s->renderer->cfg.max_geometries, KF_ERR_LIMIT,
                   "Failed to submit geometry because geometries buffer size has been exceeded.");
        geometry_retain(g);
        s->geometries.push_back(g);
        ++s->geom_stamp;
    });
}
KF_API int kf_scene_clear_geometries(kf_scene s) {
    return guarded([&] {
        check_scene(s);
        for (kf_instance_s* i : s->instances) {
            i->scene = nullptr;
            instance_release(i);
        }
        s->instances.clear();
        for (kf_geometry_s* g : s->geometries) geometry_release(g);
        s->geometries.clear();
        ++s->geom_stamp;
        ++s->inst_stamp;
    });
}
KF_API int kf_scene_remove_geometry(kf_scene s, kf_geometry g) {
    (void)s;
    (void)g;
    return fail(KF_ERR_NOT_IMPLEMENTED, "Not implemented!");
}
KF_API int kf_scene_submit_instance(kf_scene s, kf_geometry g, const float transform[16], kf_instance* out) {
    return guarded([&] {
        check_scene(s);
        REQ(g && transform, "null argument");
        // Scene::submitGeometryInstance (scene.cpp:58-77)
        KF_REQUIRE(s->instances.size() <= s->renderer->cfg.max_instances, KF_ERR_LIMIT,
                   "Failed to submit geometry instance because instance buffer size has been exceeded.");
        const bool known = std::find(s->geometries.begin(), s->geometries.end(), g) != s->geometries.end();
        REQ(known, "Geometry not submitted!");
        float rows[12];
        affine_inverse_rows(transform, rows); // rejects singular transforms
        auto in = new kf_instance_s();
        in->geometry = g;
        geometry_retain(g);
        in->scene = s;
        std::memcpy(in->transform, transform, sizeof(in->transform));
        in->refs.store(out ? 2 : 1); // the scene's reference + the caller's handle
        s->instances.push_back(in);
        ++s->inst_stamp;
        if (out) *out = in;
    });
}
KF_API int kf_instance_set_transform(kf_instance i, const float transform[16]) {
    return guarded([&] {
        REQ(i && transform, "null argument");
        float rows[12];
        affine_inverse_rows(transform, rows);
        std::memcpy(i->transform, transform, sizeof(i->transform));
        if (i->scene) ++i->scene->xform_stamp; // TLAS refit before the next frame
    });
}
KF_API int kf_scene_remove_instance(kf_scene s, kf_instance i) {
    return guarded([&] {
        check_scene(s);
        REQ(i, "Deleting an invalid geometry instance!");
        auto it = std::find(s->instances.begin(), s->instances.end(), i);
        if (it == s->instances.end()) return;
        s->instances.erase(it);
        i->scene = nullptr;
        instance_release(i);
        ++s->inst_stamp;
    });
}
KF_API int kf_scene_clear_instances(kf_scene s) {
    return guarded([&] {
        check_scene(s);
        for (kf_instance_s* i : s->instances) {
            i->scene = nullptr;
            instance_release(i);
        }
        s->instances.clear();
        ++s->inst_stamp;
    });
}
KF_API int kf_scene_instance_count(kf_scene s, uint32_t* out) {
    return guarded([&] {
        check_scene(s);
        REQ(out, "null argument");
        *out = (uint32_t)s->instances.size();
    });
}
KF_API int kf_scene_get_instance(kf_scene s, uint32_t index, kf_instance* out) {
    return guarded([&] {
        check_scene(s);
        REQ(out, "null argument");
        KF_REQUIRE(index < s->instances.size(), KF_ERR_OUT_OF_RANGE, "Geometry Instances out of bound.");
        *out = s->instances[index];
    });
}
KF_API int kf_instance_release(kf_instance i) {
    return guarded([&] { instance_release(i); });
}
KF_API int kf_scene_set_clear_color(kf_scene s, const float rgba[4]) {
    return guarded([&] {
        check_scene(s);
        REQ(rgba, "null argument");
        std::memcpy(s->clear_color, rgba, sizeof(s->clear_color));
        frame_reset(s->renderer); // Scene::setClearColor resets frameCount (scene.hpp:101-105)
    });
}
namespace {
void set_env(kf_scene_s* s, std::vector<float>&& texels, uint32_t size) {
    s->env_texels = std::move(texels);
    s->env_size = size;
    ++s->env_version;
}

float half_to_float(uint16_t h) {
    const uint32_t sign = (uint32_t)(h >> 15) << 31, exp = (h >> 10) & 0x1Fu, man = h & 0x3FFu;
    uint32_t bits;
    if (exp == 0) {
        if (man == 0) {
            bits = sign;
        } else { // subnormal: renormalise
            int e = -1;
            uint32_t m = man;
            do {
                ++e;
                m <<= 1;
            } while ((m & 0x400u) == 0);
            bits = sign | ((uint32_t)(127 - 15 - e) << 23) | ((m & 0x3FFu) << 13);
        }
    } else if (exp == 31) {
        bits = sign | 0x7F800000u | (man << 13);
    } else {
        bits = sign | ((exp + 127 - 15) << 23) | (man << 13);
    }
    float f;
    std::memcpy(&f, &bits, 4);
    return f;
}

// Minimal KTX 1.1 reader (Khronos KTX file format 1.1): uncompressed cube maps, level 0.
void load_ktx_cube(const char* path, std::vector<float>& out, uint32_t& size) {
    FILE* f = std::fopen(path, "rb");
    KF_REQUIRE(f, KF_ERR_INVALID_ARGUMENT, std::string("cannot open ") + path);
    std::vector<uint8_t> b;
    {
        uint8_t buf[65536];
        size_t n;
        while ((n = std::fread(buf, 1, sizeof(buf), f)) > 0) b.insert(b.end(), buf, buf + n);
        std::fclose(f);
    }
    static const uint8_t kId[12] = {0xAB, 'K', 'T', 'X', ' ', '1', '1', 0xBB, '\r', '\n', 0x1A, '\n'};
    KF_REQUIRE(b.size() >= 64 && std::memcmp(b.data(), kId, 12) == 0, KF_ERR_INVALID_ARGUMENT,
               std::string("not a KTX 1.1 file: ") + path);
    uint32_t hv[13];
    std::memcpy(hv, b.data() + 12, sizeof(hv));
    const bool swap = hv[0] == 0x01020304u;
    KF_REQUIRE(swap || hv[0] == 0x04030201u, KF_ERR_INVALID_ARGUMENT, "KTX: bad endianness word");
    auto rd = [&](uint32_t v) {
        return swap ? ((v >> 24) | ((v >> 8) & 0xFF00u) | ((v << 8) & 0xFF0000u) | (v << 24)) : v;
    };
    const uint32_t gl_type = rd(hv[1]), gl_format = rd(hv[3]), gl_internal = rd(hv[4]);
    const uint32_t w = rd(hv[6]), h = rd(hv[7]), faces = rd(hv[10]), kv = rd(hv[12]);
    KF_REQUIRE(faces == 6 && w == h && w > 0, KF_ERR_INVALID_ARGUMENT, "KTX: not a square cube map");
    const int comps = gl_format == 0x1908u ? 4 : (gl_format == 0x1907u ? 3 : 0); // GL_RGBA, GL_RGB
    const int tsize = gl_type == 0x1401u ? 1 : (gl_type == 0x140Bu ? 2 : (gl_type == 0x1406u ? 4 : 0));
    KF_REQUIRE(comps && tsize, KF_ERR_INVALID_ARGUMENT,
               "KTX: only uncompressed RGB / RGBA with 8-bit, half or float texels are supported");
    const bool srgb = gl_internal == 0x8C43u || gl_internal == 0x8C41u; // GL_SRGB8_ALPHA8, GL_SRGB8
    const std::vector<float>& dec = srgb_decode_table();
    size_t off = 64 + (size_t)kv;
    KF_REQUIRE(off + 4 <= b.size(), KF_ERR_INVALID_ARGUMENT, "KTX: truncated");
    uint32_t image_size;
    std::memcpy(&image_size, b.data() + off, 4);
    image_size = rd(image_size);
    off += 4;
    const size_t row = ((size_t)w * comps * tsize + 3) / 4 * 4; // rows are 4-byte aligned
    KF_REQUIRE(image_size >= row * h, KF_ERR_INVALID_ARGUMENT, "KTX: face size does not match the header");
    const size_t face_bytes = ((size_t)image_size + 3) / 4 * 4;
    KF_REQUIRE(off + 6 * face_bytes <= b.size() + 3, KF_ERR_INVALID_ARGUMENT, "KTX: truncated face data");
    out.assign((size_t)6 * w * h * 4, 0.0f);
    for (uint32_t fc = 0; fc < 6; ++fc) {
        const uint8_t* fb = b.data() + off + fc * face_bytes;
        for (uint32_t y = 0; y < h; ++y)
            for (uint32_t x = 0; x < w; ++x) {
                float* o = out.data() + (((size_t)fc * h + y) * w + x) * 4;
                o[3] = 1.0f;
                for (int c = 0; c < comps; ++c) {
                    const uint8_t* p = fb + y * row + ((size_t)x * comps + c) * tsize;
                    float v;
                    if (tsize == 1) {
                        v = (srgb && c < 3) ? dec[*p] : (float)*p / 255.0f;
                    } else if (tsize == 2) {
                        uint16_t hb;
                        std::memcpy(&hb, p, 2);
                        if (swap) hb = (uint16_t)((hb >> 8) | (hb << 8));
                        v = half_to_float(hb);
                    } else {
                        uint32_t fb32;
                        std::memcpy(&fb32, p, 4);
                        fb32 = rd(fb32);
                        std::memcpy(&v, &fb32, 4);
                    }
                    o[c] = v;
                }
            }
    }
    size = w;
}
} // namespace

KF_API int kf_scene_set_environment_map(kf_scene s, const float* rgba32f, uint32_t size) {
    return guarded([&] {
        check_scene(s);
        REQ(rgba32f && size > 0, "null or empty environment map");
        REQ(size <= 16384, "environment map faces larger than 16384^2");
        set_env(s, std::vector<float>(rgba32f, rgba32f + (size_t)6 * size * size * 4), size);
    });
}
KF_API int kf_scene_set_environment_map_rgba8(kf_scene s, const uint8_t* rgba8, uint32_t size, int srgb) {
    return guarded([&] {
        check_scene(s);
        REQ(rgba8 && size > 0, "null or empty environment map");
        REQ(size <= 16384, "environment map faces larger than 16384^2");
        const std::vector<float>& dec = srgb_decode_table();
        std::vector<float> t((size_t)6 * size * size * 4);
        for (size_t i = 0; i < t.size(); ++i)
            t[i] = (srgb && (i & 3) != 3) ? dec[rgba8[i]] : (float)rgba8[i] / 255.0f;
        set_env(s, std::move(t), size);
    });
}
KF_API int kf_scene_set_environment_map_file(kf_scene s, const char* path) {
    return guarded([&] {
        check_scene(s);
        REQ(path, "null path");
        std::vector<float> t;
        uint32_t size = 0;
        load_ktx_cube(path, t, size);
        set_env(s, std::move(t), size);
    });
}
KF_API int kf_scene_remove_environment_map(kf_scene s) {
    return guarded([&] {
        check_scene(s);
        set_env(s, std::vector<float>(), 0);
    });
}
KF_API int kf_scene_get_clear_color(kf_scene s, float rgba[4]) {
    return guarded([&] {
        check_scene(s);
        REQ(rgba, "null argument");
        std::memcpy(rgba, s->clear_color, sizeof(s->clear_color));
    });
}
KF_API int kf_scene_mark_geometries_changed(kf_scene s) {
    return guarded([&] {
        check_scene(s);
        ++s->geom_stamp;
    });
}
KF_API int kf_scene_mark_instances_changed(kf_scene s) {
    return guarded([&] {
        check_scene(s);
        ++s->inst_stamp;
    });
}

KF_API int kf_scene_set_directional_light(kf_scene s, const kf_directional_light* l) {
    return guarded([&] {
        check_scene(s);
        REQ(l, "null light");
        s->dir_light = *l;
        s->has_dir_light = true;
    });
}
KF_API int kf_scene_remove_directional_light(kf_scene s) {
    return guarded([&] {
        check_scene(s);
        s->has_dir_light = false;
    });
}
KF_API int kf_scene_add_point_light(kf_scene s, const kf_point_light* l, kf_light* out) {
    return guarded([&] {
        check_scene(s);
        REQ(l, "null light");
        if (out) *out = nullptr;
        // Scene::addPointLight warns and drops lights past the limit (scene.hpp:159-164)
        KF_REQUIRE(s->point_lights.size() < KF_MAX_POINT_LIGHTS, KF_ERR_LIMIT,
                   "Reached max point light number. The light will not be added!");
        auto L = new kf_light_s();
        L->kind = 1;
        L->point = *l;
        L->scene = s;
        s->point_lights.push_back(L);
        if (out) *out = L;
    });
}
KF_API int kf_scene_add_active_light(kf_scene s, const kf_active_light* l, kf_light* out) {
    return guarded([&] {
        check_scene(s);
        REQ(l, "null light");
        if (out) *out = nullptr;
        KF_REQUIRE(s->active_lights.size() < KF_MAX_ACTIVE_LIGHTS, KF_ERR_LIMIT,
                   "Reached max active light number. The light will not be added!");
        auto L = new kf_light_s();
        L->kind = 2;
        L->active = *l;
        L->scene = s;
        s->active_lights.push_back(L);
        if (out) *out = L;
    });
}
KF_API int kf_light_update_point(kf_light l, const kf_point_light* p) {
    return guarded([&] {
        REQ(l && p && l->kind == 1, "not a point light");
        l->point = *p;
    });
}
KF_API int kf_light_update_active(kf_light l, const kf_active_light* a) {
    return guarded([&] {
        REQ(l && a && l->kind == 2, "not an active light");
        l->active = *a;
    });
}
KF_API int kf_scene_remove_light(kf_scene s, kf_light l) {
    return guarded([&] {
        check_scene(s);
        REQ(l, "Deleting an invalid light!");
        auto& v = l->kind == 1 ? s->point_lights : s->active_lights;
        auto it = std::find(v.begin(), v.end(), l);
        REQ(it != v.end(), "light does not belong to this scene");
        v.erase(it);
        delete l;
    });
}

KF_API int kf_scene_create_camera(kf_scene s, int w, int h, kf_camera* out) {
    return guarded([&] {
        check_scene(s);
        REQ(out && w > 0 && h > 0, "invalid camera size");
        *out = scene_new_camera(s, w, h);
    });
}
KF_API int kf_scene_remove_camera(kf_scene s, kf_camera c) {
    return guarded([&] {
        check_scene(s);
        REQ(c, "Trying to remove an invalid camera!");
        auto it = std::find_if(s->cameras.begin(), s->cameras.end(), [&](auto& p) { return p.get() == c; });
        REQ(it != s->cameras.end(), "Trying to remove an camera which does not belong to the scene!");
        kf_renderer_s* r = s->renderer;
        sync_stream(r);
        if (r->graph_exec) {
            cudaGraphExecDestroy(r->graph_exec);
            r->graph_exec = nullptr;
            r->graph_key.clear();
        }
        if (s->current_camera == c) s->current_camera = nullptr;
        if (r->last_camera == c) r->last_camera = nullptr;
        s->cameras.erase(it);
    });
}
KF_API int kf_scene_set_camera(kf_scene s, kf_camera c) {
    return guarded([&] {
        check_scene(s);
        REQ(c, "Trying to set an invalid camera!");
        auto it = std::find_if(s->cameras.begin(), s->cameras.end(), [&](auto& p) { return p.get() == c; });
        REQ(it != s->cameras.end(), "Trying to set a camera that does not belong to the scene!");
        s->current_camera = c;
    });
}
KF_API int kf_scene_get_camera(kf_scene s, kf_camera* out) {
    return guarded([&] {
        check_scene(s);
        REQ(out, "null argument");
        *out = s->current_camera;
    });
}

KF_API int kf_scene_export(kf_scene s, kf_flat_scene* out) {
    return guarded([&] {
        check_scene(s);
        REQ(out, "null argument");
        std::memset(out, 0, sizeof(*out));
        s->x_geoms.clear();
        for (kf_geometry_s* g : s->geometries) {
            kf_flat_geometry fg{};
            fg.vertices = g->vertices.data();
            fg.num_vertices = (uint32_t)g->vertices.size();
            fg.num_triangles = (uint32_t)(g->indices.size() / 3);
            fg.indices = g->indices.data();
            fg.mat_index = g->mat_index.data();
            fg.opaque = g->opaque ? 1u : 0u;
            fg.hide_render = g->hide_render ? 1u : 0u;
            s->x_geoms.push_back(fg);
        }
        s->x_insts.clear();
        for (kf_instance_s* in : s->instances) {
            kf_flat_instance fi{};
            std::memcpy(fi.transform, in->transform, sizeof(fi.transform));
            affine_inverse_rows(in->transform, fi.world_to_object);
            size_t gi = 0;
            for (; gi < s->geometries.size(); ++gi)
                if (s->geometries[gi] == in->geometry) break;
            fi.geometry_index = (uint32_t)gi;
            s->x_insts.push_back(fi);
        }
        {
            std::lock_guard<std::mutex> lk(global_mutex());
            s->x_mats = flatten_materials();
            s->x_texs.clear();
            for (const HostTexture& t : g_textures) {
                kf_texture_desc d{};
                d.rgba8 = t.rgba.data();
                d.width = t.w;
                d.height = t.h;
                d.srgb = t.srgb;
                s->x_texs.push_back(d);
            }
        }
        out->geometries = s->x_geoms.data();
        out->num_geometries = (uint32_t)s->x_geoms.size();
        out->instances = s->x_insts.data();
        out->num_instances = (uint32_t)s->x_insts.size();
        out->materials = s->x_mats.data();
        out->num_materials = (uint32_t)s->x_mats.size();
        out->textures = s->x_texs.data();
        out->num_textures = (uint32_t)s->x_texs.size();
        scene_light_ubos(s, &out->dlight, &out->plights, &out->alights);
        out->env_rgba32f = s->env_size ? s->env_texels.data() : nullptr;
        out->env_size = s->env_size;
    });
}

// ---- camera ----
KF_API int kf_camera_set_position(kf_camera c, const float p[3]) {
    return guarded([&] {
        check_camera(c);
        REQ(p, "null argument");
        std::memcpy(c->position, p, sizeof(c->position));
        camera_update_view(c);
    });
}
KF_API int kf_camera_set_front(kf_camera c, const float f[3]) {
    return guarded([&] {
        check_camera(c);
        REQ(f, "null argument");
        std::memcpy(c->front, f, sizeof(c->front));
        camera_update_view(c);
    });
}
KF_API int kf_camera_set_up(kf_camera c, const float u[3]) {
    return guarded([&] {
        check_camera(c);
        REQ(u, "null argument");
        std::memcpy(c->up, u, sizeof(c->up));
        camera_update_view(c);
    });
}
KF_API int kf_camera_set_pose(kf_camera c, const float pose[16]) {
    return guarded([&] {
        check_camera(c);
        REQ(pose, "null argument");
        // Camera::setPose (camera.cpp:131-139)
        c->position[0] = pose[12]; c->position[1] = pose[13]; c->position[2] = pose[14];
        c->front[0] = -pose[8]; c->front[1] = -pose[9]; c->front[2] = -pose[10];
        c->up[0] = pose[4]; c->up[1] = pose[5]; c->up[2] = pose[6];
        if (c->scene && c->scene->renderer) frame_reset(c->scene->renderer);
    });
}
KF_API int kf_camera_get_pose(kf_camera c, float pose[16]) {
    return guarded([&] {
        check_camera(c);
        REQ(pose, "null argument");
        // Camera::getPose (camera.cpp:32-39): columns front, -right, up, position
        const float m[16] = {c->front[0],  c->front[1],  c->front[2],  0.0f, -c->right[0], -c->right[1],
                             -c->right[2], 0.0f,         c->up[0],     c->up[1], c->up[2],  0.0f,
                             c->position[0], c->position[1], c->position[2], 1.0f};
        std::memcpy(pose, m, sizeof(m));
    });
}
KF_API int kf_camera_set_full_perspective(kf_camera c, float w, float h, float fx, float fy, float cx, float cy,
                                          float skew) {
    return guarded([&] {
        check_camera(c);
        REQ(w >= 1.0f && h >= 1.0f, "invalid image size");
        c->width = (int)w;
        c->height = (int)h;
        c->fx = fx; c->fy = fy; c->cx = cx; c->cy = cy; c->skew = skew;
        camera_update_proj(c);
    });
}
KF_API int kf_camera_set_size(kf_camera c, int w, int h) {
    return guarded([&] {
        check_camera(c);
        REQ(w > 0 && h > 0, "invalid image size");
        c->width = w;
        c->height = h;
        c->cx = (float)w / 2.0f;
        c->cy = (float)h / 2.0f;
        camera_update_proj(c);
    });
}
KF_API int kf_camera_reset_view(kf_camera c) {
    return guarded([&] {
        check_camera(c);
        c->position[0] = c->position[1] = c->position[2] = 0.0f;
        const float up[3] = {0, 0, 1}, right[3] = {0, -1, 0}, front[3] = {1, 0, 0};
        std::memcpy(c->up, up, sizeof(up));
        std::memcpy(c->right, right, sizeof(right));
        std::memcpy(c->front, front, sizeof(front));
        camera_update_view(c);
        if (c->scene && c->scene->renderer) frame_reset(c->scene->renderer);
    });
}
KF_API int kf_camera_get_size(kf_camera c, int* w, int* h) {
    return guarded([&] {
        check_camera(c);
        if (w) *w = c->width;
        if (h) *h = c->height;
    });
}
KF_API int kf_camera_get_ubo(kf_camera c, kf_camera_ubo* out) {
    return guarded([&] {
        check_camera(c);
        REQ(out, "null argument");
        camera_update_view(c);
        camera_ubo(c, out);
    });
}

KF_API int kf_relmse(kf_renderer r, const float* x, const float* ref, uint64_t n, double eps, double* out) {
    return guarded([&] {
        REQ(r && x && ref && out, "null argument");
        REQ(n > 0, "relMSE over zero pixels");
        REQ(((uintptr_t)x & 15) == 0 && ((uintptr_t)ref & 15) == 0, "images must be 16-byte aligned (float4 pixels)");
        require_device(r);
        const uint32_t blocks = (uint32_t)std::max(1, std::min(r->num_sms * 4, (int)((n + 255) / 256)));
        if (r->scratch64.count < (size_t)blocks + 1) r->scratch64.resize(blocks + 1, r->stream);
        launch_relmse(reinterpret_cast<const float4*>(x), reinterpret_cast<const float4*>(ref), n, eps,
                      r->scratch64.ptr, blocks, r->scratch64.ptr + blocks, r->stream);
        KF_CUDA_CHECK(cudaMemcpyAsync(out, r->scratch64.ptr + blocks, sizeof(double), cudaMemcpyDeviceToHost, r->stream));
        sync_stream(r);
    });
}

} // extern "C"

// ---- tensor-core building blocks (kf_conv.cu) ----
#include "kf_conv.h"

extern "C" {
KF_API int kf_conv3x3_bf16(const void* x, int n, int h, int w, int cin, const void* weight, int w_rows,
                           const float* bias, int cout, int relu, void* y, int y_cstride, int y_coff, void* stream) {
    return guarded([&] {
        REQ(x && weight && y, "null tensor");
        conv3x3_bf16(static_cast<const __nv_bfloat16*>(x), n, h, w, cin, static_cast<const __nv_bfloat16*>(weight),
                     w_rows, bias, cout, relu != 0, static_cast<__nv_bfloat16*>(y), y_cstride, y_coff,
                     static_cast<cudaStream_t>(stream));
    });
}
KF_API int kf_gemm_bf16_tn(const void* a, int m, const void* b, int n, int k, float* d, int ldd, int splits,
                           void* stream) {
    return guarded([&] {
        REQ(a && b && d, "null tensor");
        gemm_bf16_tn(static_cast<const __nv_bfloat16*>(a), m, static_cast<const __nv_bfloat16*>(b), n, k, d, ldd,
                     splits, static_cast<cudaStream_t>(stream));
    });
}
KF_API int kf_tc_wait_probe(uint64_t budget_cycles, void* stream) {
    return guarded([&] {
        REQ(budget_cycles <= (uint64_t)INT64_MAX, "budget out of range");
        tc_wait_probe((long long)budget_cycles, static_cast<cudaStream_t>(stream));
    });
}
KF_API int kf_tc_error(uint32_t* out) {
    return guarded([&] {
        REQ(out, "null argument");
        *out = tc_take_error();
    });
}
}

// ---- learned denoiser (kf_denoise.cu) ----
#include <cstdio>

namespace {
constexpr uint32_t kDenoiserMagic = 0x4E44464Bu; // "KFDN"
constexpr uint32_t kDenoiserVersion = 1;

kf_denoiser_s* check_denoiser(kf_denoiser d) {
    REQ(d, "invalid denoiser");
    return d;
}
} // namespace

extern "C" {
KF_API int kf_denoiser_create(kf_renderer r, uint32_t seed, kf_denoiser* out) {
    return guarded([&] {
        REQ(r && out, "null argument");
        require_device(r);
        KF_CUDA_CHECK(cudaSetDevice(r->device));
        kf_denoiser_s* d = denoiser_create(r, seed);
        r->denoisers.push_back(d);
        *out = d;
    });
}
KF_API int kf_denoiser_destroy(kf_denoiser d) {
    return guarded([&] {
        if (!d) return;
        kf_renderer_s* r = denoiser_renderer(d);
        auto it = std::find(r->denoisers.begin(), r->denoisers.end(), d);
        REQ(it != r->denoisers.end(), "unknown denoiser");
        r->denoisers.erase(it);
        if (r->denoiser == d) r->denoiser = nullptr;
        cudaStreamSynchronize(r->stream);
        denoiser_destroy(d);
    });
}
KF_API int kf_denoiser_num_params(kf_denoiser d, uint64_t* out) {
    return guarded([&] {
        REQ(out, "null argument");
        *out = denoiser_num_params(check_denoiser(d));
    });
}
KF_API int kf_denoiser_get_params(kf_denoiser d, float* out, uint64_t count) {
    return guarded([&] {
        REQ(out, "null argument");
        denoiser_get_params(check_denoiser(d), out, count);
    });
}
KF_API int kf_denoiser_set_params(kf_denoiser d, const float* in, uint64_t count) {
    return guarded([&] {
        REQ(in, "null argument");
        denoiser_set_params(check_denoiser(d), in, count);
    });
}
KF_API int kf_denoiser_save(kf_denoiser d, const char* path) {
    return guarded([&] {
        REQ(path, "null path");
        const size_t n = denoiser_num_params(check_denoiser(d));
        std::vector<float> p(n);
        denoiser_get_params(d, p.data(), n);
        FILE* f = std::fopen(path, "wb");
        KF_REQUIRE(f, KF_ERR_INVALID_ARGUMENT, std::string("cannot open ") + path);
        const uint32_t hdr[3] = {kDenoiserMagic, kDenoiserVersion, (uint32_t)n};
        const bool ok = std::fwrite(hdr, sizeof(hdr), 1, f) == 1 && std::fwrite(p.data(), 4, n, f) == n;
        std::fclose(f);
        KF_REQUIRE(ok, KF_ERR_INTERNAL, std::string("short write to ") + path);
    });
}
KF_API int kf_denoiser_load(kf_denoiser d, const char* path) {
    return guarded([&] {
        REQ(path, "null path");
        const size_t n = denoiser_num_params(check_denoiser(d));
        FILE* f = std::fopen(path, "rb");
        KF_REQUIRE(f, KF_ERR_INVALID_ARGUMENT, std::string("cannot open ") + path);
        uint32_t hdr[3] = {0, 0, 0};
        std::vector<float> p(n);
        const bool ok = std::fread(hdr, sizeof(hdr), 1, f) == 1 && hdr[0] == kDenoiserMagic &&
                        hdr[1] == kDenoiserVersion && hdr[2] == n && std::fread(p.data(), 4, n, f) == n;
        std::fclose(f);
        KF_REQUIRE(ok, KF_ERR_INVALID_ARGUMENT, std::string("not a denoiser parameter file of this network: ") + path);
        denoiser_set_params(d, p.data(), n);
    });
}
KF_API int kf_denoiser_add_view_inputs(kf_denoiser d, kf_scene s, kf_camera c, const uint32_t* low_spp,
                                       uint32_t num_inputs, uint32_t high_spp, uint32_t high_frames) {
    return guarded([&] {
        check_denoiser(d);
        kf_scene_s* sc = check_scene(s);
        kf_camera_s* cam = check_camera(c);
        REQ(cam->scene == sc, "the camera does not belong to the scene");
        REQ(sc->renderer == denoiser_renderer(d), "the scene belongs to another renderer");
        REQ(low_spp && num_inputs >= 1 && num_inputs <= 64, "between 1 and 64 inputs per view");
        for (uint32_t i = 0; i < num_inputs; ++i) REQ(low_spp[i] > 0, "sample counts must be positive");
        REQ(high_spp > 0 && high_frames > 0, "sample counts must be positive");
        kf_renderer_s* r = denoiser_renderer(d);
        KF_CUDA_CHECK(cudaSetDevice(r->device));
        camera_update_view(cam);
        denoiser_add_view(d, sc, cam, low_spp, num_inputs, high_spp, high_frames);
        r->last_camera = nullptr; // the next run() restarts accumulation
    });
}
KF_API int kf_denoiser_add_view(kf_denoiser d, kf_scene s, kf_camera c, uint32_t low_spp, uint32_t high_spp,
                                uint32_t high_frames) {
    return kf_denoiser_add_view_inputs(d, s, c, &low_spp, 1, high_spp, high_frames);
}
KF_API int kf_denoiser_num_views(kf_denoiser d, uint32_t* out) {
    return guarded([&] {
        REQ(out, "null argument");
        *out = denoiser_num_views(check_denoiser(d));
    });
}
KF_API int kf_denoiser_train(kf_denoiser d, uint32_t iters, uint32_t batch, uint32_t crop, float lr,
                             float* mean_loss) {
    return guarded([&] {
        check_denoiser(d);
        KF_CUDA_CHECK(cudaSetDevice(denoiser_renderer(d)->device));
        const float l = denoiser_train(d, iters, batch, crop, lr);
        if (mean_loss) *mean_loss = l;
    });
}
KF_API int kf_denoiser_apply(kf_denoiser d, kf_camera c) {
    return guarded([&] {
        check_denoiser(d);
        kf_camera_s* cam = check_camera(c);
        kf_renderer_s* r = denoiser_renderer(d);
        REQ(cam->scene && cam->scene->renderer == r, "the camera belongs to another renderer");
        KF_CUDA_CHECK(cudaSetDevice(r->device));
        denoiser_apply(d, cam);
        sync_stream(r);
    });
}
KF_API int kf_renderer_set_denoiser(kf_renderer r, kf_denoiser d) {
    return guarded([&] {
        REQ(r, "invalid renderer");
        REQ(!d || denoiser_renderer(d) == r, "the denoiser belongs to another renderer");
        r->denoiser = d;
    });
}
// float4 and 16-byte BF16 accesses: base, target and feature buffers are 16-byte aligned
static bool aligned16(const void* p) { return ((uintptr_t)p & 15) == 0; }

KF_API int kf_denoiser_forward(kf_denoiser d, const void* feat, const float* base, int n, int h, int w, float* out) {
    return guarded([&] {
        REQ(feat && out && n > 0 && h > 0 && w > 0, "invalid tensor");
        REQ(aligned16(base), "base must be 16-byte aligned");
        check_denoiser(d);
        denoiser_forward(d, feat, base, n, h, w, out);
        sync_stream(denoiser_renderer(d));
    });
}
KF_API int kf_denoiser_camera_features(kf_denoiser d, kf_camera c, void* feat_dev, float* base_dev, int* hp,
                                       int* wp) {
    return guarded([&] {
        REQ(hp && wp, "null argument");
        check_denoiser(d);
        kf_camera_s* cam = check_camera(c);
        REQ(cam->scene && cam->scene->renderer == denoiser_renderer(d), "the camera belongs to another renderer");
        KF_REQUIRE(cam->has_frame, KF_ERR_STATE, "the camera has no frame");
        *hp = (cam->target_h + 15) / 16 * 16;
        *wp = (cam->target_w + 15) / 16 * 16;
        if (!feat_dev && !base_dev) return;
        REQ(feat_dev && base_dev, "both feature and base buffers are needed");
        REQ(aligned16(feat_dev) && aligned16(base_dev), "feature and base buffers must be 16-byte aligned");
        kf_renderer_s* r = denoiser_renderer(d);
        KF_CUDA_CHECK(cudaSetDevice(r->device));
        denoiser_camera_features(d, cam, feat_dev, base_dev);
        sync_stream(r);
    });
}
KF_API int kf_denoiser_train_step(kf_denoiser d, const void* feat, const float* base, const float* target, int n,
                                  int h, int w, float lr, float* grads_dev, int apply, float* loss) {
    return guarded([&] {
        REQ(feat && target && n > 0 && h > 0 && w > 0, "invalid tensor");
        REQ(aligned16(base) && aligned16(target), "base and target must be 16-byte aligned");
        check_denoiser(d);
        const float l = denoiser_train_step(d, feat, base, target, n, h, w, lr, grads_dev, apply != 0);
        if (loss) *loss = l;
    });
}
}
