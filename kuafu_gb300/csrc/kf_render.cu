// kf_render.cu — one frame: the wavefront schedule that replaces
// Context::render / recordSwapchainCommandBuffers (src/core/context/context.cpp:298-350,
// 522-540, 602-684), plus the host-side camera math of src/core/camera.cpp.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>

#include "kf_host.h"

namespace kf {

// ---------------------------------------------------------------------------
// Host math (glm conventions, column-major).
// ---------------------------------------------------------------------------
namespace {
inline void nrm3(const float v[3], float o[3]) {
    const float inv = 1.0f / std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    o[0] = v[0] * inv;
    o[1] = v[1] * inv;
    o[2] = v[2] * inv;
}
inline void cross3(const float a[3], const float b[3], float o[3]) {
    o[0] = a[1] * b[2] - b[1] * a[2];
    o[1] = a[2] * b[0] - b[2] * a[0];
    o[2] = a[0] * b[1] - b[0] * a[1];
}
inline float dot3(const float a[3], const float b[3]) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

void inverse4_dd(const double* a, double* inv) {
    double r[16];
    r[0] = a[5] * a[10] * a[15] - a[5] * a[11] * a[14] - a[9] * a[6] * a[15] + a[9] * a[7] * a[14] + a[13] * a[6] * a[11] - a[13] * a[7] * a[10];
    r[4] = -a[4] * a[10] * a[15] + a[4] * a[11] * a[14] + a[8] * a[6] * a[15] - a[8] * a[7] * a[14] - a[12] * a[6] * a[11] + a[12] * a[7] * a[10];
    r[8] = a[4] * a[9] * a[15] - a[4] * a[11] * a[13] - a[8] * a[5] * a[15] + a[8] * a[7] * a[13] + a[12] * a[5] * a[11] - a[12] * a[7] * a[9];
    r[12] = -a[4] * a[9] * a[14] + a[4] * a[10] * a[13] + a[8] * a[5] * a[14] - a[8] * a[6] * a[13] - a[12] * a[5] * a[10] + a[12] * a[6] * a[9];
    r[1] = -a[1] * a[10] * a[15] + a[1] * a[11] * a[14] + a[9] * a[2] * a[15] - a[9] * a[3] * a[14] - a[13] * a[2] * a[11] + a[13] * a[3] * a[10];
    r[5] = a[0] * a[10] * a[15] - a[0] * a[11] * a[14] - a[8] * a[2] * a[15] + a[8] * a[3] * a[14] + a[12] * a[2] * a[11] - a[12] * a[3] * a[10];
    r[9] = -a[0] * a[9] * a[15] + a[0] * a[11] * a[13] + a[8] * a[1] * a[15] - a[8] * a[3] * a[13] - a[12] * a[1] * a[11] + a[12] * a[3] * a[9];
    r[13] = a[0] * a[9] * a[14] - a[0] * a[10] * a[13] - a[8] * a[1] * a[14] + a[8] * a[2] * a[13] + a[12] * a[1] * a[10] - a[12] * a[2] * a[9];
    r[2] = a[1] * a[6] * a[15] - a[1] * a[7] * a[14] - a[5] * a[2] * a[15] + a[5] * a[3] * a[14] + a[13] * a[2] * a[7] - a[13] * a[3] * a[6];
    r[6] = -a[0] * a[6] * a[15] + a[0] * a[7] * a[14] + a[4] * a[2] * a[15] - a[4] * a[3] * a[14] - a[12] * a[2] * a[7] + a[12] * a[3] * a[6];
    r[10] = a[0] * a[5] * a[15] - a[0] * a[7] * a[13] - a[4] * a[1] * a[15] + a[4] * a[3] * a[13] + a[12] * a[1] * a[7] - a[12] * a[3] * a[5];
    r[14] = -a[0] * a[5] * a[14] + a[0] * a[6] * a[13] + a[4] * a[1] * a[14] - a[4] * a[2] * a[13] - a[12] * a[1] * a[6] + a[12] * a[2] * a[5];
    r[3] = -a[1] * a[6] * a[11] + a[1] * a[7] * a[10] + a[5] * a[2] * a[11] - a[5] * a[3] * a[10] - a[9] * a[2] * a[7] + a[9] * a[3] * a[6];
    r[7] = a[0] * a[6] * a[11] - a[0] * a[7] * a[10] - a[4] * a[2] * a[11] + a[4] * a[3] * a[10] + a[8] * a[2] * a[7] - a[8] * a[3] * a[6];
    r[11] = -a[0] * a[5] * a[11] + a[0] * a[7] * a[9] + a[4] * a[1] * a[11] - a[4] * a[3] * a[9] - a[8] * a[1] * a[7] + a[8] * a[3] * a[5];
    r[15] = a[0] * a[5] * a[10] - a[0] * a[6] * a[9] - a[4] * a[1] * a[10] + a[4] * a[2] * a[9] + a[8] * a[1] * a[6] - a[8] * a[2] * a[5];
    const double det = a[0] * r[0] + a[1] * r[4] + a[2] * r[8] + a[3] * r[12];
    for (int i = 0; i < 16; ++i) inv[i] = r[i] / det;
}
} // namespace

// glm::lookAt (right-handed), called by Camera::updateViewMatrix (camera.cpp:92-94).
void look_at(const float eye[3], const float front[3], const float up[3], float out[16]) {
    const float center[3] = {eye[0] + front[0], eye[1] + front[1], eye[2] + front[2]};
    const float fd[3] = {center[0] - eye[0], center[1] - eye[1], center[2] - eye[2]};
    float f[3], s[3], u[3], c[3];
    nrm3(fd, f);
    cross3(f, up, c);
    nrm3(c, s);
    cross3(s, f, u);
    for (int i = 0; i < 16; ++i) out[i] = (i % 5 == 0) ? 1.0f : 0.0f;
    out[0] = s[0]; out[4] = s[1]; out[8] = s[2];
    out[1] = u[0]; out[5] = u[1]; out[9] = u[2];
    out[2] = -f[0]; out[6] = -f[1]; out[10] = -f[2];
    out[12] = -dot3(s, eye);
    out[13] = -dot3(u, eye);
    out[14] = dot3(f, eye);
}

// Camera::updateProjectionMatrix (camera.cpp:111-124), near 0.1, far 100.
void projection_from_intrinsics(int w, int h, float fx, float fy, float cx, float cy, float skew, float out[16]) {
    const float nearp = 0.1f, farp = 100.0f;
    const float W = (float)w, H = (float)h;
    for (int i = 0; i < 16; ++i) out[i] = 0.0f;
    out[0] = (2.0f * fx) / W;
    out[4] = -2.0f * skew / W;
    out[5] = -(2.0f * fy) / H;
    out[8] = -2.0f * cx / W + 1.0f;
    out[9] = -2.0f * cy / H + 1.0f;
    out[10] = -farp / (farp - nearp);
    out[11] = -1.0f;
    out[14] = -farp * nearp / (farp - nearp);
    out[15] = 0.0f;
}

// glm::perspective (right-handed, depth [-1, 1]) used for active lights (scene.cpp:277-278).
void perspective(float fovy, float aspect, float znear, float zfar, float out[16]) {
    const float t = std::tan(fovy / 2.0f);
    for (int i = 0; i < 16; ++i) out[i] = 0.0f;
    out[0] = 1.0f / (aspect * t);
    out[5] = 1.0f / t;
    out[10] = -(zfar + znear) / (zfar - znear);
    out[11] = -1.0f;
    out[14] = -(2.0f * zfar * znear) / (zfar - znear);
}

// 4x4 inverse in FP64, rounded to float (replaces glm::inverse).
void inverse4_d(const float in[16], float out[16]) {
    double a[16], o[16];
    for (int i = 0; i < 16; ++i) a[i] = in[i];
    inverse4_dd(a, o);
    for (int i = 0; i < 16; ++i) out[i] = (float)o[i];
}

// Rows of the world->object affine map of a column-major object->world matrix
// (what gl_WorldToObjectEXT holds for an instance, rt.cpp:127-137), in FP64.
void affine_inverse_rows(const float m[16], float out_rows[12]) {
    double A[3][3], t[3];
    for (int r = 0; r < 3; ++r) {
        for (int c = 0; c < 3; ++c) A[r][c] = m[c * 4 + r];
        t[r] = m[3 * 4 + r];
    }
    const double det = A[0][0] * (A[1][1] * A[2][2] - A[1][2] * A[2][1]) -
                       A[0][1] * (A[1][0] * A[2][2] - A[1][2] * A[2][0]) +
                       A[0][2] * (A[1][0] * A[2][1] - A[1][1] * A[2][0]);
    KF_REQUIRE(det != 0.0 && std::isfinite(det), KF_ERR_INVALID_ARGUMENT, "instance transform is not invertible");
    double I[3][3];
    I[0][0] = (A[1][1] * A[2][2] - A[1][2] * A[2][1]) / det;
    I[0][1] = (A[0][2] * A[2][1] - A[0][1] * A[2][2]) / det;
    I[0][2] = (A[0][1] * A[1][2] - A[0][2] * A[1][1]) / det;
    I[1][0] = (A[1][2] * A[2][0] - A[1][0] * A[2][2]) / det;
    I[1][1] = (A[0][0] * A[2][2] - A[0][2] * A[2][0]) / det;
    I[1][2] = (A[0][2] * A[1][0] - A[0][0] * A[1][2]) / det;
    I[2][0] = (A[1][0] * A[2][1] - A[1][1] * A[2][0]) / det;
    I[2][1] = (A[0][1] * A[2][0] - A[0][0] * A[2][1]) / det;
    I[2][2] = (A[0][0] * A[1][1] - A[0][1] * A[1][0]) / det;
    for (int r = 0; r < 3; ++r) {
        const double tr = -(I[r][0] * t[0] + I[r][1] * t[1] + I[r][2] * t[2]);
        out_rows[r * 4 + 0] = (float)I[r][0];
        out_rows[r * 4 + 1] = (float)I[r][1];
        out_rows[r * 4 + 2] = (float)I[r][2];
        out_rows[r * 4 + 3] = (float)tr;
    }
}

void camera_update_view(kf_camera_s* c) { look_at(c->position, c->front, c->up, c->view); }
void camera_update_proj(kf_camera_s* c) {
    projection_from_intrinsics(c->width, c->height, c->fx, c->fy, c->cx, c->cy, c->skew, c->proj);
}

// Scene::uploadCameraBuffer (scene.cpp:236-250).
void camera_ubo(const kf_camera_s* c, kf_camera_ubo* o) {
    std::memset(o, 0, sizeof(*o));
    std::memcpy(o->view, c->view, sizeof(o->view));
    std::memcpy(o->proj, c->proj, sizeof(o->proj));
    inverse4_d(c->view, o->view_inv);
    inverse4_d(c->proj, o->proj_inv);
    o->position[0] = c->position[0]; o->position[1] = c->position[1]; o->position[2] = c->position[2];
    o->position[3] = c->aperture;
    o->front[0] = c->front[0]; o->front[1] = c->front[1]; o->front[2] = c->front[2];
    o->front[3] = c->focal_length;
    for (int i = 0; i < 4; ++i) o->pad1[i] = o->pad2[i] = 1.0f;
}

// ---------------------------------------------------------------------------
// Frame schedule.
// ---------------------------------------------------------------------------
namespace {

void ensure_targets(kf_renderer_s* r, kf_camera_s* c) {
    const size_t npix = (size_t)c->width * c->height;
    if (c->target_w != c->width || c->target_h != c->height || c->accum.count != npix) {
        c->accum.resize(npix, r->stream);
        c->sum64.resize(npix, r->stream);
        c->albedo.resize(npix, r->stream);
        c->normal.resize(npix, r->stream);
        c->depth.resize(npix, r->stream);
        c->seg.resize(npix, r->stream);
        c->bgra.resize(npix, r->stream);
        c->target_w = c->width;
        c->target_h = c->height;
        c->has_frame = false;
        KF_CUDA_CHECK(cudaMemsetAsync(c->accum.ptr, 0, c->accum.bytes(), r->stream));
        KF_CUDA_CHECK(cudaMemsetAsync(c->sum64.ptr, 0, c->sum64.bytes(), r->stream));
    }
}

void ensure_wave(kf_renderer_s* r, uint32_t chunk, uint32_t slots, uint64_t npaths) {
    WaveBuffers& W = r->wave;
    cudaStream_t st = r->stream;
    if (W.chunk_cap < chunk) {
        W.q_o0.resize(chunk, st); W.q_o1.resize(chunk, st);
        W.q_d0.resize(chunk, st); W.q_d1.resize(chunk, st);
        W.hit.resize(chunk, st); W.hit_prim.resize(chunk, st); W.sel.resize(chunk, st);
        W.weight.resize(chunk, st); W.nee_w.resize(chunk, st); W.nee_in.resize((size_t)6 * chunk, st);
        W.req.resize(chunk, st);
        W.chunk_cap = chunk;
        W.slot_cap = 0;
    }
    const uint32_t sl = std::max(slots, 1u);
    if (W.slot_cap < sl) {
        W.contrib.resize((size_t)sl * W.chunk_cap, st);
        W.vis.resize((size_t)sl * W.chunk_cap, st);
        W.sq_o.resize((size_t)sl * W.chunk_cap, st);
        W.sq_d.resize((size_t)sl * W.chunk_cap, st);
        W.slot_cap = sl;
    }
    if (W.radiance_cap < npaths) {
        W.radiance.resize(npaths, st);
        W.radiance_cap = npaths;
    }
    if (r->cfg.debug_outputs && W.primary.count < npaths) W.primary.resize(npaths, st);
    if (W.counters.count == 0) W.counters.resize(8, st);
    if (W.scount.count == 0) W.scount.resize(64, st);
    if (W.stats.count == 0) {
        W.stats.resize(16, st);
        KF_CUDA_CHECK(cudaMemsetAsync(W.stats.ptr, 0, W.stats.bytes(), st));
    }
}

WaveDev wave_view(kf_renderer_s* r, kf_camera_s* c) {
    WaveBuffers& W = r->wave;
    WaveDev w{};
    w.q_o[0] = W.q_o0.ptr; w.q_o[1] = W.q_o1.ptr;
    w.q_d[0] = W.q_d0.ptr; w.q_d[1] = W.q_d1.ptr;
    w.counters = W.counters.ptr;
    w.hit = W.hit.ptr;
    w.hit_prim = W.hit_prim.ptr;
    w.sel = W.sel.ptr;
    w.scount = W.scount.ptr;
    w.nslot = W.slot_cap;
    w.weight = W.weight.ptr;
    w.nee_w = W.nee_w.ptr;
    w.nee_in = W.nee_in.ptr;
    w.req = W.req.ptr;
    w.contrib = W.contrib.ptr;
    w.vis = W.vis.ptr;
    w.sq_o = W.sq_o.ptr;
    w.sq_d = W.sq_d.ptr;
    w.radiance = W.radiance.ptr;
    w.primary = r->cfg.debug_outputs ? W.primary.ptr : nullptr;
    w.albedo = c->albedo.ptr;
    w.normal = c->normal.ptr;
    w.depth = c->depth.ptr;
    w.seg = c->seg.ptr;
    w.stats = W.stats.ptr;
    w.chunk_cap = W.chunk_cap;
    return w;
}

} // namespace

// The bounce loop on two streams. Bounce d's shadow traversal and NEE gather (stream2)
// overlap bounce d+1's closest-hit traversal (stream): they share no buffer — the closest-hit
// kernel reads the next ray queue and writes hit records, the shadow kernel reads the shadow
// queue and writes visibility, the gather reads bounce d's queue and adds to the radiance.
// Everything bounce d+1 writes that bounce d's gather reads (its queue count, the NEE
// requests, contributions, visibility and radiance of the paths) is written by k_miss /
// k_shade, which wait for the gather (the join). Counters: [3] / [4] fetch cursors, [2]
// shadow count, [5] hit count, each zeroed on the stream that uses it next.
static void enqueue_paths_overlapped(kf_renderer_s* r, const SceneDev& sv, const FrameDev* fd, const BatchDev& b,
                                     const WaveDev& w, uint32_t max_depth, uint64_t npaths, uint32_t chunk) {
    cudaStream_t st = r->stream, st2 = r->stream2;
    const bool dyn = r->cfg.traversal == 1;
    for (uint64_t start = 0; start < npaths; start += chunk) {
        const uint32_t n = (uint32_t)std::min<uint64_t>(chunk, npaths - start);
        launch_raygen(fd, b, w, start, n, st);
        int cur = 0;
        for (uint32_t depth = 0; depth <= max_depth; ++depth) {
            KF_CUDA_CHECK(cudaMemsetAsync(w.counters + 3, 0, sizeof(uint32_t), st));
            if (dyn)
                launch_trace_dyn(sv, fd, b, w, cur, depth, start, false, r->grid_dyn, r->count_traversal,
                                 r->cfg.dyn_refill_below, r->cfg.dyn_steps, st);
            else
                launch_extend(sv, fd, b, w, cur, depth, start, r->grid_extend, r->count_traversal, st);
            if (depth > 0) KF_CUDA_CHECK(cudaStreamWaitEvent(st, r->ev_join, 0)); // previous gather done
            KF_CUDA_CHECK(cudaMemsetAsync(w.counters + (cur ^ 1), 0, sizeof(uint32_t), st));
            KF_CUDA_CHECK(cudaMemsetAsync(w.scount, 0, w.nslot * sizeof(uint32_t), st));
            KF_CUDA_CHECK(cudaMemsetAsync(w.counters + 5, 0, sizeof(uint32_t), st));
            launch_miss(sv, fd, b, w, cur, depth, start, r->grid_shade, st);
            launch_shade(sv, fd, b, w, cur, depth, start, r->grid_shade, st);
            launch_nee(sv, fd, b, w, depth, start, r->grid_shade, st);
            KF_CUDA_CHECK(cudaEventRecord(r->ev_fork, st));
            KF_CUDA_CHECK(cudaStreamWaitEvent(st2, r->ev_fork, 0));
            KF_CUDA_CHECK(cudaMemsetAsync(w.counters + 4, 0, sizeof(uint32_t), st2));
            if (dyn)
                launch_trace_dyn(sv, fd, b, w, cur, depth, start, true, r->grid_dyn_shadow, r->count_traversal,
                                 r->cfg.dyn_refill_below, r->cfg.dyn_steps, st2);
            else
                launch_shadow(sv, b, w, r->grid_extend, r->count_traversal, st2);
            launch_gather(sv, b, w, cur, start, r->grid_shade, st2);
            KF_CUDA_CHECK(cudaEventRecord(r->ev_join, st2));
            cur ^= 1;
        }
        KF_CUDA_CHECK(cudaStreamWaitEvent(st, r->ev_join, 0)); // last gather done
    }
}

// Records the bounce loop over npaths paths (chunks of `chunk`) into the renderer stream.
static void enqueue_paths(kf_renderer_s* r, const SceneDev& sv, const FrameDev* fd, const BatchDev& b,
                          const WaveDev& w, uint32_t max_depth, uint64_t npaths, uint32_t chunk, bool profile) {
    cudaStream_t st = r->stream;
    if (!profile) {
        enqueue_paths_overlapped(r, sv, fd, b, w, max_depth, npaths, chunk);
        return;
    }
    for (uint64_t start = 0; start < npaths; start += chunk) {
        const uint32_t n = (uint32_t)std::min<uint64_t>(chunk, npaths - start);
        launch_raygen(fd, b, w, start, n, st);
        int cur = 0;
        for (uint32_t depth = 0; depth <= max_depth; ++depth) {
            const bool dyn = r->cfg.traversal == 1;
            KF_CUDA_CHECK(cudaMemsetAsync(w.counters + (cur ^ 1), 0, sizeof(uint32_t), st));
            // [2] shadow queue count, [3] / [4] dynamic-fetch cursors, [5] rays that hit
            KF_CUDA_CHECK(cudaMemsetAsync(w.counters + 2, 0, 4 * sizeof(uint32_t), st));
            KF_CUDA_CHECK(cudaMemsetAsync(w.scount, 0, w.nslot * sizeof(uint32_t), st));
            if (profile) KF_CUDA_CHECK(cudaEventRecord(r->ev[0], st));
            if (dyn)
                launch_trace_dyn(sv, fd, b, w, cur, depth, start, false, r->grid_dyn, r->count_traversal,
                                 r->cfg.dyn_refill_below, r->cfg.dyn_steps, st);
            else
                launch_extend(sv, fd, b, w, cur, depth, start, r->grid_extend, r->count_traversal, st);
            if (profile) KF_CUDA_CHECK(cudaEventRecord(r->ev[1], st));
            launch_miss(sv, fd, b, w, cur, depth, start, r->grid_shade, st);
            launch_shade(sv, fd, b, w, cur, depth, start, r->grid_shade, st);
            launch_nee(sv, fd, b, w, depth, start, r->grid_shade, st);
            if (profile) KF_CUDA_CHECK(cudaEventRecord(r->ev[2], st));
            if (dyn)
                launch_trace_dyn(sv, fd, b, w, cur, depth, start, true, r->grid_dyn_shadow, r->count_traversal,
                                 r->cfg.dyn_refill_below, r->cfg.dyn_steps, st);
            else
                launch_shadow(sv, b, w, r->grid_extend, r->count_traversal, st);
            if (profile) KF_CUDA_CHECK(cudaEventRecord(r->ev[3], st));
            launch_gather(sv, b, w, cur, start, r->grid_shade, st);
            if (profile) {
                KF_CUDA_CHECK(cudaEventSynchronize(r->ev[3]));
                float a = 0, bb = 0, d = 0;
                KF_CUDA_CHECK(cudaEventElapsedTime(&a, r->ev[0], r->ev[1]));
                KF_CUDA_CHECK(cudaEventElapsedTime(&bb, r->ev[1], r->ev[2]));
                KF_CUDA_CHECK(cudaEventElapsedTime(&d, r->ev[2], r->ev[3]));
                r->stats.extend_ms += a;
                r->stats.shade_ms += bb;
                r->stats.shadow_ms += d;
            }
            cur ^= 1;
        }
    }
}

// Records the launch sequence of one frame into the renderer stream.
static void enqueue_frame(kf_renderer_s* r, const SceneDev& sv, const WaveDev& w, uint32_t npix, uint32_t spp,
                          uint32_t max_depth, uint64_t npaths, uint32_t chunk, kf_camera_s* c, bool profile) {
    const FrameDev* fd = r->frame_dev.ptr;
    enqueue_paths(r, sv, fd, BatchDev{nullptr, 0, 0}, w, max_depth, npaths, chunk, profile);
    launch_resolve(fd, w.radiance, npix, spp, c->accum.ptr, c->sum64.ptr, r->stream);
    launch_srgb(c->accum.ptr, npix, c->bgra.ptr, r->stream);
}

// Frame constants of camera c of scene s (push constants: PushConstants.glsl:1-16, filled
// as Context::update does, context.cpp:345-360).
static FrameDev make_frame(const kf_renderer_s* r, const kf_scene_s* s, const kf_camera_s* c, uint32_t spp,
                           int32_t frame_count) {
    FrameDev f{};
    camera_ubo(c, &f.cam);
    f.pc.clear_color[0] = s->clear_color[0];
    f.pc.clear_color[1] = s->clear_color[1];
    f.pc.clear_color[2] = s->clear_color[2];
    f.pc.clear_color[3] = s->clear_color[3];
    f.pc.frame_count = frame_count;
    f.pc.spp = spp;
    f.pc.max_path_depth = r->cfg.path_depth;
    f.pc.use_env_map = s->env_size ? 1u : 0u;
    f.pc.russian_roulette = r->cfg.russian_roulette;
    f.pc.rr_min_bounces = r->cfg.rr_min_bounces;
    f.pc.nee = r->cfg.nee;
    f.pc.nee_min = r->cfg.nee_min_bounces;
    f.width = (uint32_t)c->width;
    f.height = (uint32_t)c->height;
    f.npix = (uint32_t)c->width * (uint32_t)c->height;
    f.seed = r->cfg.seed;
    f.frame = r->frame_index;
    f.camera_index = 0;
    for (size_t i = 0; i < s->cameras.size(); ++i)
        if (s->cameras[i].get() == c) f.camera_index = (uint32_t)i;
    return f;
}

// Launch-shape parameters baked into a captured graph (grids, persistent-kernel scheduling).
static std::string launch_shape_key(const kf_renderer_s* r) {
    char b[96];
    std::snprintf(b, sizeof(b), "%u,%u,%u,%u,%u,%u", r->grid_extend, r->grid_shade, r->grid_dyn,
                  r->grid_dyn_shadow, r->cfg.dyn_refill_below, r->cfg.dyn_steps);
    return b;
}

// Everything of a scene's device view that a captured graph bakes into its kernel
// parameters (SceneDev is passed by value): buffer addresses, counts and the light-slot
// map. The slot map is rebuilt every frame from the light UBOs without moving a buffer,
// so switching which lights are on at an unchanged count must still recapture.
static std::string scene_view_key(const SceneDev& v) {
    std::string k;
    char b[64];
    const void* ptrs[] = {v.verts, v.indices, v.matidx, v.geom, v.materials, v.inst, v.blas_nodes, v.tris,
                          v.tlas_nodes, v.tlas_inst, v.dlight, v.plights, v.alights, v.tex_info, v.texels,
                          v.srgb_decode, v.env};
    for (const void* p : ptrs) {
        std::snprintf(b, sizeof(b), "%p,", p);
        k += b;
    }
    std::snprintf(b, sizeof(b), "%u,%u,%u,%u,%u:", v.env_size, v.num_instances, v.has_tlas, v.num_textures,
                  v.num_slots);
    k += b;
    for (uint32_t j = 0; j < v.num_slots && j < (uint32_t)kMaxLightSlots; ++j) {
        std::snprintf(b, sizeof(b), "%u.%u,", (unsigned)v.slot_group[j], (unsigned)v.slot_index[j]);
        k += b;
    }
    return k;
}

static uint32_t chunk_for(const kf_renderer_s* r, uint64_t npaths) {
    uint64_t cap = r->cfg.max_paths_in_flight ? r->cfg.max_paths_in_flight : (1ull << 24);
    cap = std::min<uint64_t>(cap, (1ull << 26) - 1);
    return (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(npaths, cap));
}

void render_frame(kf_renderer_s* r, kf_scene_s* s, kf_camera_s* c, uint32_t spp) {
    cudaStream_t st = r->stream;
    KF_REQUIRE(spp > 0, KF_ERR_INVALID_ARGUMENT, "samples per pixel must be positive");
    scene_sync_gpu(r, s);
    ensure_targets(r, c);
    const uint32_t npix = (uint32_t)c->width * (uint32_t)c->height;
    const uint64_t npaths = (uint64_t)npix * spp;
    const uint32_t chunk = chunk_for(r, npaths);
    const SceneDev& sv = s->gpu.view;
    ensure_wave(r, chunk, sv.num_slots, npaths);

    // Context::update (context.cpp:345-349): frame counter for the running mean
    if (r->cfg.accumulate_frames)
        ++r->frame_count;
    else
        r->frame_count = -1;

    const FrameDev f = make_frame(r, s, c, spp, r->frame_count);
    if (r->frame_dev.count == 0) r->frame_dev.resize(1, st);
    KF_CUDA_CHECK(cudaMemcpyAsync(r->frame_dev.ptr, &f, sizeof(f), cudaMemcpyHostToDevice, st));
    KF_CUDA_CHECK(cudaMemsetAsync(c->albedo.ptr, 0, c->albedo.bytes(), st));
    KF_CUDA_CHECK(cudaMemsetAsync(c->normal.ptr, 0, c->normal.bytes(), st));

    const WaveDev w = wave_view(r, c);
    const bool profile = r->cfg.profile != 0;
    cudaEvent_t f0 = r->ev[4], f1 = r->ev[5];
    if (profile) KF_CUDA_CHECK(cudaEventRecord(f0, st));
    const bool use_graph = r->cfg.use_graph && !profile && !r->count_traversal;
    if (use_graph) {
        // The launch sequence depends only on buffer addresses and sizes; the
        // per-frame values live in frame_dev, so a captured graph replays as is.
        char head[512];
        std::snprintf(head, sizeof(head), "%p|%p|%llu|%u|%u|%u|%llu|%u|%p|%p|%p|%p|%p|%u|%s|", (void*)s, (void*)c,
                      (unsigned long long)s->gpu.generation, npix, spp, r->cfg.path_depth,
                      (unsigned long long)npaths, chunk, (void*)w.q_o[0], (void*)w.radiance, (void*)w.contrib,
                      (void*)c->accum.ptr, (void*)w.primary, r->cfg.russian_roulette | (r->cfg.traversal << 1),
                      launch_shape_key(r).c_str());
        const std::string key = std::string(head) + scene_view_key(sv);
        if (!r->graph_exec || r->graph_key != key) {
            if (r->graph_exec) {
                cudaGraphExecDestroy(r->graph_exec);
                r->graph_exec = nullptr;
            }
            cudaGraph_t g = nullptr;
            KF_CUDA_CHECK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
            try {
                enqueue_frame(r, sv, w, npix, spp, r->cfg.path_depth, npaths, chunk, c, false);
            } catch (...) {
                cudaStreamEndCapture(st, &g);
                if (g) cudaGraphDestroy(g);
                throw;
            }
            KF_CUDA_CHECK(cudaStreamEndCapture(st, &g));
            KF_CUDA_CHECK(cudaGraphInstantiate(&r->graph_exec, g, 0));
            cudaGraphDestroy(g);
            r->graph_key = key;
        }
        KF_CUDA_CHECK(cudaGraphLaunch(r->graph_exec, st));
    } else {
        enqueue_frame(r, sv, w, npix, spp, r->cfg.path_depth, npaths, chunk, c, profile);
    }
    if (profile) {
        KF_CUDA_CHECK(cudaEventRecord(f1, st));
        KF_CUDA_CHECK(cudaEventSynchronize(f1));
        float ms = 0;
        KF_CUDA_CHECK(cudaEventElapsedTime(&ms, f0, f1));
        r->stats.frame_ms += ms;
    }
    c->has_frame = true;
    c->last_path_start = 0;
    c->last_spp = spp;
    r->stats.frames++;
    r->stats.last_spp = spp;
    r->stats.frame_count = r->frame_count;
    ++r->frame_index;
}

// One frame of every item in one wavefront: the items' paths are laid end to end in one
// path space, the bounce loop runs once over all of them (one launch per kernel per
// bounce and chunk), then each view is resolved into its own targets. Every view is an
// independent single frame (frameCount -1, no blending), all with the same frame word.
void render_batch(kf_renderer_s* r, const kf_batch_item* items, uint32_t count) {
    cudaStream_t st = r->stream;
    KF_REQUIRE(count > 0, KF_ERR_INVALID_ARGUMENT, "empty batch");
    KF_REQUIRE(count <= 65535, KF_ERR_LIMIT, "a batch holds at most 65535 views");
    std::vector<kf_scene_s*> scenes;
    std::vector<uint32_t> scene_of(count);
    for (uint32_t i = 0; i < count; ++i) {
        KF_REQUIRE(items[i].spp > 0, KF_ERR_INVALID_ARGUMENT, "samples per pixel must be positive");
        auto it = std::find(scenes.begin(), scenes.end(), items[i].scene);
        if (it == scenes.end()) {
            scenes.push_back(items[i].scene);
            it = scenes.end() - 1;
        }
        scene_of[i] = (uint32_t)(it - scenes.begin());
    }
    batch_sync(r, scenes);
    BatchState& B = *r->batch;
    std::vector<ItemDev> hv(count);
    uint64_t total = 0;
    uint32_t max_slots = 1;
    std::vector<uint32_t> inst_base(scenes.size(), 0), geom_base(scenes.size(), 0);
    for (size_t k = 1; k < scenes.size(); ++k) {
        inst_base[k] = inst_base[k - 1] + (uint32_t)scenes[k - 1]->instances.size();
        geom_base[k] = geom_base[k - 1] + (uint32_t)scenes[k - 1]->geometries.size();
    }
    for (uint32_t i = 0; i < count; ++i) {
        kf_scene_s* s = items[i].scene;
        kf_camera_s* c = items[i].camera;
        ensure_targets(r, c);
        ItemDev& it = hv[i];
        std::memset(&it, 0, sizeof(it));
        it.f = make_frame(r, s, c, items[i].spp, -1);
        it.path_start = total;
        total += (uint64_t)it.f.npix * items[i].spp;
        const uint32_t k = scene_of[i];
        it.root = B.roots[k];
        const SceneDev& sv = s->gpu.view;
        it.num_slots = sv.num_slots;
        std::memcpy(it.slot_group, sv.slot_group, sizeof(it.slot_group));
        std::memcpy(it.slot_index, sv.slot_index, sizeof(it.slot_index));
        it.dlight = sv.dlight;
        it.plights = sv.plights;
        it.alights = sv.alights;
        it.env = sv.env;
        it.env_size = sv.env_size;
        it.inst_base = inst_base[k];
        it.albedo = c->albedo.ptr;
        it.normal = c->normal.ptr;
        it.depth = c->depth.ptr;
        it.seg = c->seg.ptr;
        it.geom_base = geom_base[k];
        max_slots = std::max(max_slots, sv.num_slots);
    }
    const uint32_t chunk = chunk_for(r, total);
    ensure_wave(r, chunk, max_slots, total);
    if (r->wave.path_item.count < chunk) r->wave.path_item.resize(chunk, st);
    B.items.resize(count, st);
    KF_CUDA_CHECK(cudaMemcpyAsync(B.items.ptr, hv.data(), sizeof(ItemDev) * count, cudaMemcpyHostToDevice, st));
    for (uint32_t i = 0; i < count; ++i) {
        KF_CUDA_CHECK(cudaMemsetAsync(items[i].camera->albedo.ptr, 0, items[i].camera->albedo.bytes(), st));
        KF_CUDA_CHECK(cudaMemsetAsync(items[i].camera->normal.ptr, 0, items[i].camera->normal.bytes(), st));
    }
    WaveDev w = wave_view(r, items[0].camera);
    w.path_item = r->wave.path_item.ptr;
    const BatchDev bd{B.items.ptr, count, 0};
    auto enqueue = [&](bool profile) {
        enqueue_paths(r, B.view, nullptr, bd, w, r->cfg.path_depth, total, chunk, profile);
        for (uint32_t i = 0; i < count; ++i) {
            kf_camera_s* c = items[i].camera;
            launch_resolve(&B.items.ptr[i].f, w.radiance + hv[i].path_start, hv[i].f.npix, items[i].spp,
                           c->accum.ptr, c->sum64.ptr, st);
            launch_srgb(c->accum.ptr, hv[i].f.npix, c->bgra.ptr, st);
        }
    };
    const bool profile = r->cfg.profile != 0;
    cudaEvent_t f0 = r->ev[4], f1 = r->ev[5];
    if (profile) KF_CUDA_CHECK(cudaEventRecord(f0, st));
    if (r->cfg.use_graph && !profile && !r->count_traversal) {
        std::string key;
        char buf[160];
        std::snprintf(buf, sizeof(buf), "%llu|%u|%llu|%u|%p|%p|%p|%u|%u|", (unsigned long long)B.generation, count,
                      (unsigned long long)total, chunk, (void*)w.q_o[0], (void*)w.radiance, (void*)B.items.ptr,
                      r->cfg.path_depth, r->cfg.russian_roulette | (r->cfg.traversal << 1));
        key = buf + launch_shape_key(r) + "|" + scene_view_key(B.view) + "|";
        for (uint32_t i = 0; i < count; ++i) {
            std::snprintf(buf, sizeof(buf), "%p,%u,%u;", (void*)items[i].camera->accum.ptr, hv[i].f.npix,
                          items[i].spp);
            key += buf;
        }
        if (!B.graph_exec || B.graph_key != key) {
            if (B.graph_exec) {
                cudaGraphExecDestroy(B.graph_exec);
                B.graph_exec = nullptr;
            }
            cudaGraph_t g = nullptr;
            KF_CUDA_CHECK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
            try {
                enqueue(false);
            } catch (...) {
                cudaStreamEndCapture(st, &g);
                if (g) cudaGraphDestroy(g);
                throw;
            }
            KF_CUDA_CHECK(cudaStreamEndCapture(st, &g));
            KF_CUDA_CHECK(cudaGraphInstantiate(&B.graph_exec, g, 0));
            cudaGraphDestroy(g);
            B.graph_key = key;
        }
        KF_CUDA_CHECK(cudaGraphLaunch(B.graph_exec, st));
    } else {
        enqueue(profile);
    }
    if (profile) {
        KF_CUDA_CHECK(cudaEventRecord(f1, st));
        KF_CUDA_CHECK(cudaEventSynchronize(f1));
        float ms = 0;
        KF_CUDA_CHECK(cudaEventElapsedTime(&ms, f0, f1));
        r->stats.frame_ms += ms;
    }
    for (uint32_t i = 0; i < count; ++i) {
        kf_camera_s* c = items[i].camera;
        c->has_frame = true;
        c->last_path_start = hv[i].path_start;
        c->last_spp = items[i].spp;
    }
    r->stats.frames += count;
    r->stats.last_spp = items[count - 1].spp;
    ++r->frame_index;
}

} // namespace kf
