// kf_autotune.cu — picks the launch configuration of batched rendering by measurement:
// traversal kernel (thread per ray / persistent dynamic fetch), wavefront chunk size
// (paths in flight), launch grids of the per-ray kernels, the persistent kernel's warp
// scheduling (refill threshold, steps between refills) and the BLAS leaf size (the BVH
// shape), one knob at a time (coordinate descent), each candidate timed with CUDA events
// on the renderer's stream over `reps` batches after one warm-up batch (which also
// captures the batch graph and, for a new leaf size, rebuilds every BLAS).
//
// It also holds the L2 read-bandwidth probe that the traversal's roofline is stated
// against: the achievable rate at which this GPU's SMs read data that sits in L2.
#include <algorithm>
#include <vector>

#include "kf_host.h"

namespace kf {
namespace {

struct Knobs {
    uint32_t traversal;
    uint64_t chunk;
    uint32_t grid_extend, grid_shade;
    uint32_t leaf;
    uint32_t refill_below, steps; // persistent traversal's warp scheduling
};

void apply(kf_renderer_s* r, const std::vector<kf_scene_s*>& scenes, const Knobs& k) {
    r->cfg.traversal = k.traversal;
    r->cfg.max_paths_in_flight = k.chunk;
    r->grid_extend = k.grid_extend;
    r->grid_shade = k.grid_shade;
    r->cfg.dyn_refill_below = k.refill_below;
    r->cfg.dyn_steps = k.steps;
    if (r->cfg.blas_leaf_size != k.leaf) {
        r->cfg.blas_leaf_size = k.leaf;
        for (kf_scene_s* s : scenes) ++s->geom_stamp; // rebuild every BLAS with the new leaf size
    }
}

float time_batch(kf_renderer_s* r, const kf_batch_item* items, uint32_t count, uint32_t reps) {
    render_batch(r, items, count); // warm-up: rebuilds, graph capture
    KF_CUDA_CHECK(cudaStreamSynchronize(r->stream));
    cudaEvent_t e0 = r->ev[6], e1 = r->ev[7];
    std::vector<float> t;
    for (uint32_t i = 0; i < reps; ++i) {
        KF_CUDA_CHECK(cudaEventRecord(e0, r->stream));
        render_batch(r, items, count);
        KF_CUDA_CHECK(cudaEventRecord(e1, r->stream));
        KF_CUDA_CHECK(cudaEventSynchronize(e1));
        float ms = 0.0f;
        KF_CUDA_CHECK(cudaEventElapsedTime(&ms, e0, e1));
        t.push_back(ms);
    }
    std::sort(t.begin(), t.end());
    return t[t.size() / 2];
}

} // namespace

void autotune_batch(kf_renderer_s* r, const kf_batch_item* items, uint32_t count, uint32_t reps,
                    kf_autotune_result* out) {
    KF_REQUIRE(count > 0, KF_ERR_INVALID_ARGUMENT, "empty batch");
    reps = std::max(1u, reps);
    std::vector<kf_scene_s*> scenes;
    uint64_t total = 0;
    for (uint32_t i = 0; i < count; ++i) {
        if (std::find(scenes.begin(), scenes.end(), items[i].scene) == scenes.end()) scenes.push_back(items[i].scene);
        total += (uint64_t)items[i].camera->width * items[i].camera->height * items[i].spp;
    }
    const uint32_t sms = (uint32_t)std::max(1, r->num_sms);
    Knobs best{r->cfg.traversal, r->cfg.max_paths_in_flight ? r->cfg.max_paths_in_flight : (1ull << 24),
               r->grid_extend, r->grid_shade, std::max(1u, r->cfg.blas_leaf_size), r->cfg.dyn_refill_below,
               r->cfg.dyn_steps};
    const Knobs start = best;
    apply(r, scenes, best);
    float best_ms = time_batch(r, items, count, reps);
    const float start_ms = best_ms;
    uint32_t tried = 1;
    auto consider = [&](Knobs k) {
        apply(r, scenes, k);
        const float ms = time_batch(r, items, count, reps);
        ++tried;
        if (ms < best_ms) {
            best_ms = ms;
            best = k;
        }
    };
    // 1. traversal kernel
    {
        Knobs k = best;
        k.traversal = best.traversal ? 0u : 1u;
        consider(k);
    }
    // 2. paths in flight (larger chunks: fewer launches; smaller: less memory traffic per bounce)
    for (uint64_t c : {1ull << 22, 1ull << 23, 1ull << 24, 1ull << 25}) {
        if (c == best.chunk || (c >> 1) >= total) continue;
        Knobs k = best;
        k.chunk = c;
        consider(k);
    }
    // 3. launch grids (blocks per SM) of the shading / gather kernels and the thread-per-ray traversal
    for (uint32_t m : {4u, 8u, 16u}) {
        if (m * sms == best.grid_shade) continue;
        Knobs k = best;
        k.grid_shade = m * sms;
        consider(k);
    }
    if (best.traversal == 0)
        for (uint32_t m : {8u, 16u, 32u}) {
            if (m * sms == best.grid_extend) continue;
            Knobs k = best;
            k.grid_extend = m * sms;
            consider(k);
        }
    // 3b. persistent traversal: refill threshold and steps between refills
    if (best.traversal == 1) {
        for (uint32_t rb : {12u, 16u, 24u, 28u}) {
            if (rb == best.refill_below) continue;
            Knobs k = best;
            k.refill_below = rb;
            consider(k);
        }
        for (uint32_t ns : {8u, 16u, 32u}) {
            if (ns == best.steps) continue;
            Knobs k = best;
            k.steps = ns;
            consider(k);
        }
    }
    // 4. BVH shape: triangles per BLAS leaf
    for (uint32_t leaf : {1u, 2u, 4u, 8u}) {
        if (leaf == best.leaf) continue;
        Knobs k = best;
        k.leaf = leaf;
        consider(k);
    }
    apply(r, scenes, best);
    render_batch(r, items, count); // leaves the pools and graph of the winner in place
    KF_CUDA_CHECK(cudaStreamSynchronize(r->stream));
    if (out) {
        out->traversal = best.traversal;
        out->blas_leaf_size = best.leaf;
        out->max_paths_in_flight = best.chunk;
        out->grid_extend = best.grid_extend;
        out->grid_shade = best.grid_shade;
        out->dyn_refill_below = best.refill_below;
        out->dyn_steps = best.steps;
        out->candidates = tried;
        out->best_ms = best_ms;
        out->start_ms = start_ms;
        out->start_traversal = start.traversal;
        out->start_blas_leaf_size = start.leaf;
        out->start_max_paths_in_flight = start.chunk;
    }
}

// ---------------------------------------------------------------------------
// L2 read bandwidth. A buffer that fits in L2 (the caller's size, 32 MiB by default
// against the 126 MB L2) is read `passes` times by a full-occupancy grid with
// ld.global.cg (cached in L2 only, so L1 does not serve repeats); every thread keeps
// four independent 16-byte loads in flight per iteration. One untimed pass brings the
// buffer into L2; the timed launch is bracketed by CUDA events on the renderer's
// stream. Rate = passes x bytes / time, the best of `reps` launches.
// ---------------------------------------------------------------------------
namespace {
constexpr int kL2Threads = 512;

__global__ void __launch_bounds__(kL2Threads) k_l2_read(const float4* __restrict__ buf, uint64_t n4, uint32_t passes,
                                                         uint32_t* sink) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    uint32_t acc = 0;
    for (uint32_t p = 0; p < passes; ++p) {
        for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i + 3 * stride < n4; i += 4 * stride) {
            const float4 a = __ldcg(buf + i);
            const float4 b = __ldcg(buf + i + stride);
            const float4 c = __ldcg(buf + i + 2 * stride);
            const float4 d = __ldcg(buf + i + 3 * stride);
            acc ^= __float_as_uint(a.x) ^ __float_as_uint(a.y) ^ __float_as_uint(a.z) ^ __float_as_uint(a.w);
            acc ^= __float_as_uint(b.x) ^ __float_as_uint(b.y) ^ __float_as_uint(b.z) ^ __float_as_uint(b.w);
            acc ^= __float_as_uint(c.x) ^ __float_as_uint(c.y) ^ __float_as_uint(c.z) ^ __float_as_uint(c.w);
            acc ^= __float_as_uint(d.x) ^ __float_as_uint(d.y) ^ __float_as_uint(d.z) ^ __float_as_uint(d.w);
        }
    }
    if (acc == 0x9E3779B9u) sink[0] = acc; // keeps the loads; practically never taken
}
} // namespace

double measure_l2_read(kf_renderer_s* r, uint64_t bytes, uint32_t passes, uint32_t reps) {
    int dev = 0;
    KF_CUDA_CHECK(cudaGetDevice(&dev));
    int per_sm = 0;
    KF_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_l2_read, kL2Threads, 0));
    const uint32_t grid = (uint32_t)std::max(1, r->num_sms) * (uint32_t)std::max(1, per_sm);
    const uint64_t chunk = 4ull * grid * kL2Threads; // float4 per iteration of the whole grid
    const uint64_t n4 = std::max<uint64_t>(1, bytes / 16 / chunk) * chunk;
    passes = std::max(1u, passes);
    reps = std::max(1u, reps);
    cudaStream_t st = r->stream;
    TempAlloc tmp(st);
    float4* buf = tmp.alloc<float4>(n4);
    uint32_t* sink = tmp.alloc<uint32_t>(1);
    KF_CUDA_CHECK(cudaMemsetAsync(buf, 0x3C, n4 * sizeof(float4), st));
    k_l2_read<<<grid, kL2Threads, 0, st>>>(buf, n4, 1, sink); // into L2
    KF_CUDA_CHECK(cudaGetLastError());
    cudaEvent_t e0 = r->ev[6], e1 = r->ev[7];
    float best = 0.0f;
    for (uint32_t i = 0; i < reps; ++i) {
        KF_CUDA_CHECK(cudaEventRecord(e0, st));
        k_l2_read<<<grid, kL2Threads, 0, st>>>(buf, n4, passes, sink);
        KF_CUDA_CHECK(cudaEventRecord(e1, st));
        KF_CUDA_CHECK(cudaEventSynchronize(e1));
        float ms = 0.0f;
        KF_CUDA_CHECK(cudaEventElapsedTime(&ms, e0, e1));
        if (i == 0 || ms < best) best = ms;
    }
    KF_CUDA_CHECK(cudaGetLastError());
    return (double)n4 * 16.0 * passes / (best * 1e-3) / 1e9;
}

} // namespace kf
