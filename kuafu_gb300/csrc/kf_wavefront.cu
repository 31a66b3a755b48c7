// kf_wavefront.cu — the wavefront path tracer that replaces kuafu's single
// ray-tracing pipeline launch (src/core/rt/rt.cpp:637-666) and its shaders
// (resources/shaders/PathTrace.{rgen,rchit,rahit,rmiss}, PathTraceShadow.rmiss).
//
// One frame = every (pixel, sample) path of a camera, processed bounce by bounce:
//   raygen   camera rays, queued in pixel tiles            (PathTrace.rgen:30-75)
//   extend   closest hit, two-level BVH4 traversal         (traceRayEXT, rgen:97-107)
//   miss     environment / clear colour; lists the hits    (PathTrace.rmiss)
//   shade    emission / PrincipledBSDF sampling, RR,       (rchit:322-468, rgen:109-138)
//            next ray, NEE record
//   nee      light samples -> one shadow queue per light   (rchit:204-316)
//   shadow   any-hit occlusion of the shadow queues        (rchit:175-200)
//   gather   ordered NEE sum into the path radiance        (rchit:457-460, rgen:111)
// then a per-pixel resolve (rgen:140-166) and the sRGB frame (PostProcessing.frag).
// Queues are compacted in order: a block scan per tile with one atomic per tile (warp
// ballots + one atomic per warp where the warps of a block differ).
//
// This file is compiled with -fmad=false: float expressions round exactly as
// written, matching the CPU oracle operation for operation.
#include "kf_wavefront.h"

#include <string>

#include "kf_util.h"

namespace kf {

namespace {

constexpr uint32_t kMiss = 0xFFFFFFFFu;
constexpr int kStack = 96;
constexpr uint32_t kInstTag = 0x80000000u;
constexpr uint32_t kPopTag = 0xC0000000u;
constexpr uint32_t kLeafTag = 0x40000000u;
static_assert(kLeafTag == kLeafChildTag, "leaf child links are pushed as stack entries");
static_assert(kInstTag == kInstChildTag, "instance links of the TLAS are pushed as stack entries");
constexpr uint32_t kFull = 0xFFFFFFFFu;

struct HitOut {
    float t, u, v;
    uint32_t inst, prim;
};

struct TraceCounters {
    uint32_t nodes, tris, insts;
};

// Two-level traversal. SHADOW: any hit in [tmin, tmax] terminates (gl_RayFlags
// TerminateOnFirstHit | Opaque | SkipClosestHitShader, rchit:182-184).
// Stochastic alpha of non-opaque geometry (PathTrace.rahit:30-48): a candidate is
// ignored when alpha == 0 or when a uniform draw exceeds alpha. The draws come from
// the path's any-hit stream; their order follows the traversal order.
// The path's Philox key is derived only when a draw is needed (non-opaque geometry is
// rare): fetching a ray then costs no 64-bit division.
struct AnyHitCtx {
    const FrameDev* f; // the path's view
    uint64_t g;        // the path's index in its view
    Stream st;
};

// Sample and pixel of path g of a view (sample-major): a 32-bit division whenever g fits
// in 32 bits (a view below 2^32 paths), the 64-bit one otherwise.
__device__ __forceinline__ void split_path(uint64_t g, uint32_t npix, uint32_t& sample, uint32_t& pix) {
    if ((g >> 32) == 0) {
        const uint32_t g32 = (uint32_t)g;
        sample = g32 / npix;
        pix = g32 - sample * npix;
    } else {
        sample = (uint32_t)(g / npix);
        pix = (uint32_t)(g % npix);
    }
}

__device__ __forceinline__ PathKey path_key(const FrameDev& f, uint64_t g) {
    uint32_t sample, pix;
    split_path(g, f.npix, sample, pix);
    return PathKey{make_uint2(f.seed ^ pix, f.camera_index), sample, f.frame};
}

__device__ __forceinline__ bool anyhit_accept(const SceneDev& s, uint32_t geometry, uint32_t prim, AnyHitCtx& ah) {
    const uint4 gi = __ldg(s.geom + geometry);
    const float alpha = s.materials[__ldg(s.matidx + gi.y + prim)].alpha;
    if (alpha == 0.0f) return false;
    if (ah.st.next(path_key(*ah.f, ah.g)) > alpha) return false;
    return true;
}

// Traversal stack of one thread: the first kSmemStack entries live in shared
// memory laid out entry-major (entry * blockDim + thread, so a warp's accesses hit
// 32 different banks whatever each lane's depth), deeper entries in local memory.
constexpr int kSmemStack = 40;
constexpr int kThreadsTrace = 128;
struct TStack {
    uint32_t* sm; // &shared[threadIdx.x]
    uint32_t deep[kStack - kSmemStack];
    __device__ __forceinline__ void put(int i, uint32_t v) {
        if (i < kSmemStack)
            sm[i * kThreadsTrace] = v;
        else
            deep[i - kSmemStack] = v;
    }
    __device__ __forceinline__ uint32_t get(int i) const {
        return i < kSmemStack ? sm[i * kThreadsTrace] : deep[i - kSmemStack];
    }
};

// Resumable two-level traversal state: init() then step() until it returns true.
// One step processes one stack entry (a node with its leaf children, an instance
// entry or the return to the TLAS), so a warp can interleave rays step by step.
// The slab test of box4 on a node read in place: the near and far planes of each axis are
// loaded by the ray's direction signs (no selects), with the child links.
__device__ __forceinline__ int box4_dir(const PRay& r, const float4* p, float tmin, float tmax, float tn_out[4],
                                        int4& child, int4& cnt) {
    const int sx = r.ix >= 0.0f ? 0 : 1, sy = r.iy >= 0.0f ? 0 : 1, sz = r.iz >= 0.0f ? 0 : 1;
    const float4 nx = __ldg(p + sx), fx = __ldg(p + (1 - sx));
    const float4 ny = __ldg(p + 2 + sy), fy = __ldg(p + (3 - sy));
    const float4 nz = __ldg(p + 4 + sz), fz = __ldg(p + (5 - sz));
    child = __ldg(reinterpret_cast<const int4*>(p + 6));
    cnt = __ldg(reinterpret_cast<const int4*>(p + 7));
    int mask = 0;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        float t1x, t1y, t1z;
        const float t0x = slab1(lane(nx, c), lane(fx, c), r.ox, r.ix, t1x);
        const float t0y = slab1(lane(ny, c), lane(fy, c), r.oy, r.iy, t1y);
        const float t0z = slab1(lane(nz, c), lane(fz, c), r.oz, r.iz, t1z);
        float tn = fmaxf(tmin, t0x);
        float tf = fminf(__int_as_float(0x7f800000), t1x);
        tn = fmaxf(tn, t0y);
        tf = fminf(tf, t1y);
        tn = fmaxf(tn, t0z);
        tf = fminf(tf, t1z);
        tn_out[c] = tn;
        if (tn <= fminf(tf * KF_BOX_WIDEN, tmax * KF_TMAX_WIDEN)) mask |= 1 << c;
    }
    return mask;
}

template <bool SHADOW, bool COUNT> struct Tracer {
    PRay wr, r;
    TStack stack;
    int sp;
    bool in_blas, cur_opaque;
    uint32_t cur_inst, cur_geom;
    float tmin, best;
    HitOut h;
    TraceCounters cnt;

    // root: the TLAS root node of the ray's scene (kNoRoot: the ray hits nothing)
    __device__ __forceinline__ void init(uint32_t root, float ox, float oy, float oz, float dx, float dy, float dz,
                                         float tmin_, float tmax_) {
        h.inst = kMiss;
        h.t = h.u = h.v = 0.0f;
        h.prim = 0;
        wr.ox = ox; wr.oy = oy; wr.oz = oz;
        wr.dx = dx; wr.dy = dy; wr.dz = dz;
        prep_ray(wr);
        r = wr;
        sp = 0;
        if (root != kNoRoot) stack.put(sp++, root);
        in_blas = false;
        cur_inst = cur_geom = 0;
        cur_opaque = true;
        tmin = tmin_;
        best = tmax_;
    }

    // Returns true when the traversal is over (stack empty, or the first hit of a shadow ray).
    // Stack entries: kPopTag (back to the TLAS), kInstTag | instance, kLeafTag | (n-1) << 26 |
    // first (a BLAS leaf of n triangles, or a TLAS leaf of n instances in the leaf list), or a
    // node index. Node child links are entries of these kinds as they are.
    // The rare, cheap entries do not take a step of their own: a return to the TLAS goes on
    // to the next entry (a TLAS node or instance), and an instance entry goes on to the root
    // node of its BLAS, so the lanes of a warp mostly run the node or the leaf code together.
    __device__ __forceinline__ bool step(const SceneDev& s, AnyHitCtx* ah) {
        if (sp <= 0) return true;
        uint32_t e = stack.get(--sp);
        if (e == kPopTag) {
            in_blas = false;
            // back in the TLAS only boxes are tested: origin and reciprocal direction
            // (copying the shear terms too would keep them live in registers)
            r.ox = wr.ox; r.oy = wr.oy; r.oz = wr.oz;
            r.ix = wr.ix; r.iy = wr.iy; r.iz = wr.iz;
            if (sp <= 0) return true;
            e = stack.get(--sp); // below a return entry: a TLAS node or an instance entry
        }
        if ((e & 0xC0000000u) == kLeafTag && !in_blas) {
            // a TLAS leaf (instances first .. first + n - 1 of the leaf list): the first
            // instance is entered in this step, the others wait on the stack
            const uint32_t first = e & 0x03FFFFFFu;
#pragma unroll 1
            for (uint32_t q = (e >> 26) & 0xFu; q > 0; --q)
                if (sp < kStack) stack.put(sp++, kInstTag | __ldg(s.tlas_inst + first + q));
            e = kInstTag | __ldg(s.tlas_inst + first);
        }
        if ((e & 0xC0000000u) == kLeafTag) {
            const uint32_t first = e & 0x03FFFFFFu, cnt_tri = ((e >> 26) & 0xFu) + 1u;
#pragma unroll 1
            for (uint32_t q = 0; q < cnt_tri; ++q) {
                const float4* tp = reinterpret_cast<const float4*>(s.tris + first + q);
                const float4 a = __ldg(tp), b = __ldg(tp + 1), cc = __ldg(tp + 2);
                if (COUNT) cnt.tris++;
                float t, u, v;
                if (!intersect_tri(r, a, b, cc, tmin, best, t, u, v)) continue;
                const uint32_t prim = __float_as_uint(a.w);
                if (SHADOW) {
                    h.inst = cur_inst;
                    sp = 0;
                    return true;
                }
                if (!closer(t, cur_inst, prim, h.t, h.inst, h.prim)) continue;
                if (!cur_opaque && ah && !anyhit_accept(s, cur_geom, prim, *ah)) continue;
                h.t = t; h.u = u; h.v = v; h.inst = cur_inst; h.prim = prim;
                best = t;
            }
            return sp <= 0;
        }
        if (e & kInstTag) {
            cur_inst = e & ~kInstTag;
            const InstanceRec* ip = s.inst + cur_inst;
            InstanceRec in;
            in.w2o0 = __ldg(&ip->w2o0);
            in.w2o1 = __ldg(&ip->w2o1);
            in.w2o2 = __ldg(&ip->w2o2);
            const uint4 meta = __ldg(reinterpret_cast<const uint4*>(ip) + 3);
            if (COUNT) cnt.insts++;
            if (meta.z & 2u) return sp <= 0; // hidden (dummy BLAS, rt.cpp:156)
            cur_geom = meta.y;
            cur_opaque = (meta.z & 1u) != 0;
            to_object(in, wr.ox, wr.oy, wr.oz, wr.dx, wr.dy, wr.dz, r);
            in_blas = true;
            if (sp + 2 > kStack) return sp <= 0;
            stack.put(sp++, kPopTag);
            e = meta.x; // the BLAS root, visited in this step
        }
        Node4 n;
        float tn[4];
        const int mask = box4_dir(r, reinterpret_cast<const float4*>((in_blas ? s.blas_nodes : s.tlas_nodes) + e), tmin,
                                  best, tn, n.child, n.cnt);
        if (COUNT) cnt.nodes++;
        // children to visit, as (entry distance, stack entry); misses get -inf. The child
        // links are stack entries already: node indices, and leaf entries (triangles in a
        // BLAS, instances in the TLAS) sorted with the inner children by distance. Empty
        // children have inverted boxes and never hit.
        float it[4];
        uint32_t ic[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            it[c] = ((mask >> c) & 1) ? tn[c] : __int_as_float(0xff800000);
            ic[c] = (uint32_t)lanei(n.child, c);
        }
        // sort by entry distance (fixed network, registers only), then push. Closest-hit rays
        // sort descending, so the nearest child ends on top of the stack; shadow rays (ended by
        // any hit) sort ascending and take the farthest child first, which visits fewer nodes
        // per ray than nearest-first on the 256-icosphere frame (23 against 26).
#define KF_CSWAP(a, b)                                                                                     \
    if (SHADOW ? it[a] > it[b] : it[a] < it[b]) {                                                          \
        const float tf = it[a];                                                                            \
        it[a] = it[b];                                                                                     \
        it[b] = tf;                                                                                        \
        const uint32_t tu = ic[a];                                                                         \
        ic[a] = ic[b];                                                                                     \
        ic[b] = tu;                                                                                        \
    }
        KF_CSWAP(0, 1)
        KF_CSWAP(2, 3)
        KF_CSWAP(0, 2)
        KF_CSWAP(1, 3)
        KF_CSWAP(1, 2)
#undef KF_CSWAP
        if (sp + 4 <= kSmemStack) { // all four fit the shared part of the stack
            uint32_t* top = stack.sm + sp * kThreadsTrace;
#pragma unroll
            for (int c = 0; c < 4; ++c)
                if (it[c] != __int_as_float(0xff800000)) {
                    *top = ic[c];
                    top += kThreadsTrace;
                    ++sp;
                }
        } else {
#pragma unroll
            for (int c = 0; c < 4; ++c)
                if (it[c] != __int_as_float(0xff800000) && sp < kStack) stack.put(sp++, ic[c]);
        }
        return sp <= 0;
    }
};

// smem: the block's shared stack area (kSmemStack * kThreadsTrace words).
template <bool SHADOW, bool COUNT>
__device__ bool trace(const SceneDev& s, uint32_t root, uint32_t* smem, float ox, float oy, float oz, float dx,
                      float dy, float dz, float tmin, float tmax, HitOut& h, TraceCounters& cnt,
                      AnyHitCtx* ah = nullptr) {
    Tracer<SHADOW, COUNT> t;
    t.stack.sm = smem + threadIdx.x;
    t.init(root, ox, oy, oz, dx, dy, dz, tmin, tmax);
    t.cnt = cnt;
#pragma unroll 1
    while (!t.step(s, ah)) {
    }
    cnt = t.cnt;
    h = t.h;
    return h.inst != kMiss;
}

__device__ __forceinline__ uint32_t lanemask_lt() { return (1u << (threadIdx.x & 31)) - 1u; }

// Warp-aggregated append: one atomic per warp, positions by ballot prefix.
// Must be reached by all 32 lanes (warp-uniform control flow).
__device__ __forceinline__ uint32_t warp_append(bool pred, uint32_t* counter) {
    const uint32_t m = __ballot_sync(kFull, pred);
    uint32_t base = 0;
    if (m) {
        if ((threadIdx.x & 31) == 0) base = atomicAdd(counter, (uint32_t)__popc(m));
        base = __shfl_sync(kFull, base, 0);
    }
    return base + __popc(m & lanemask_lt());
}

__device__ __forceinline__ void warp_add_stat(unsigned long long* p, uint32_t v) {
    for (int off = 16; off; off >>= 1) v += __shfl_xor_sync(kFull, v, off);
    if ((threadIdx.x & 31) == 0 && v) atomicAdd(p, (unsigned long long)v);
}

// mat4 (column-major) * vec4, columns summed in order.
__device__ __forceinline__ void mat4_mul(const float* m, const float v[4], float out[4]) {
#pragma unroll
    for (int r = 0; r < 4; ++r) out[r] = m[0 * 4 + r] * v[0] + m[1 * 4 + r] * v[1] + m[2 * 4 + r] * v[2] + m[3 * 4 + r] * v[3];
}

// Batched launches: the item of global path G (items sorted by path_start, item 0 starts at 0).
__device__ __forceinline__ uint32_t find_item(const BatchDev& b, uint64_t G) {
    uint32_t lo = 0, hi = b.num_items;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (b.items[mid].path_start <= G) lo = mid;
        else hi = mid;
    }
    return lo;
}

// The view a path belongs to: single-view frames use the scene's own TLAS root; batched
// ones the root of the path's item (paths carry their item in w.path_item).
template <bool BATCH> struct View {
    const FrameDev* f;
    const ItemDev* it;
    uint64_t g; // path index within the view
};
template <bool BATCH>
__device__ __forceinline__ View<BATCH> view_of(const FrameDev* fp, const BatchDev& b, const WaveDev& w,
                                               uint64_t chunk_start, uint32_t p) {
    View<BATCH> v;
    if (BATCH) {
        v.it = b.items + w.path_item[p];
        v.f = &v.it->f;
        v.g = chunk_start + p - v.it->path_start;
    } else {
        v.it = nullptr;
        v.f = fp;
        v.g = chunk_start + p;
    }
    return v;
}
template <bool BATCH> __device__ __forceinline__ uint32_t root_of(const SceneDev& s, const View<BATCH>& v) {
    if (BATCH) return v.it->root;
    return s.has_tlas ? 0u : kNoRoot;
}

// ---------------------------------------------------------------------------
// Ray generation (PathTrace.rgen:30-75).
// ---------------------------------------------------------------------------
// Queue order of a sample's pixels: bands of kTileH rows, each cut into kTileW-wide column
// blocks (narrower at the right edge), a block's pixels row by row — a warp's 32 camera rays
// cover a 4x8 tile instead of 32 pixels of one row, and stay coherent downstream (4x8
// measured fastest of 2x16 .. 16x4 on the 256-icosphere frame). idx is the position within
// the sample, the result the row-major pixel index (a bijection for any size).
constexpr uint32_t kTileW = 4, kTileH = 8;
__device__ __forceinline__ uint32_t tiled_pixel(uint32_t idx, uint32_t width, uint32_t height) {
    const uint32_t band = width * kTileH;
    const uint32_t rb = idx / band;
    const uint32_t hb = min(kTileH, height - rb * kTileH);
    const uint32_t r = idx - rb * band;
    const uint32_t cb = r / (kTileW * hb);
    const uint32_t wb = min(kTileW, width - cb * kTileW);
    const uint32_t k = r - cb * kTileW * hb;
    return (rb * kTileH + k / wb) * width + cb * kTileW + k % wb;
}

template <bool BATCH>
__global__ void k_raygen(const FrameDev* __restrict__ fp, BatchDev b, WaveDev w, uint64_t chunk_start,
                         uint32_t chunk_n) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; // queue position
    if (j == 0) w.counters[0] = chunk_n;
    if (j >= chunk_n) return;
    uint64_t g = chunk_start + j;
    uint64_t view_start = 0; // global index of the view's first path
    const FrameDev* fsel = fp;
    uint32_t item = 0;
    if (BATCH) {
        item = find_item(b, g);
        fsel = &b.items[item].f;
        view_start = b.items[item].path_start;
    }
    const FrameDev& f = *fsel;
    g -= view_start;
    uint32_t sample, pix;
    if (view_start >= chunk_start && view_start + (uint64_t)f.npix * f.pc.spp <= chunk_start + chunk_n) {
        // the whole view in this chunk: a pixel's samples are queued one after the other,
        // pixels in tile order, so a warp's camera rays start in 4 neighbouring pixels
        // (+5 % over queuing each sample's pixels in tile order)
        uint32_t t;
        split_path(g, f.pc.spp, t, sample);
        pix = tiled_pixel(t, f.width, f.height);
    } else {
        split_path(g, f.npix, sample, pix);
        // a sample whose pixels all lie in this chunk is queued in tile order
        const uint64_t row0 = view_start + (uint64_t)sample * f.npix;
        if (row0 >= chunk_start && row0 + f.npix <= chunk_start + chunk_n) pix = tiled_pixel(pix, f.width, f.height);
    }
    // the path id p (the index of all per-path state) stays the row-major one
    const uint64_t row = view_start + (uint64_t)sample * f.npix;
    const uint32_t p = (uint32_t)(row + pix - chunk_start);
    if (BATCH) w.path_item[p] = (uint16_t)item;
    const uint32_t px = pix % f.width, py = pix / f.width;
    PathKey pk{make_uint2(f.seed ^ pix, f.camera_index), sample, f.frame};
    Stream js;
    js.init(0, KF_RNG_JITTER);
    const float jx = js.next(pk);
    const float jy = js.next(pk);
    const float posx = (float)px + jx, posy = (float)py + jy;
    const float nx = posx / (float)f.width, ny = posy / (float)f.height;
    const float dxn = nx * 2.0f - 1.0f, dyn = ny * 2.0f - 1.0f;
    const float aperture = f.cam.position[3];
    const float focus = f.cam.front[3];
    float offx = 0.0f, offy = 0.0f;
    if (aperture > 0.0f) { // diskSampling (Sampling.glsl:124-134)
        Stream ls;
        ls.init(0, KF_RNG_LENS);
        float qx, qy;
        do {
            const float a = ls.next(pk), b = ls.next(pk);
            qx = 2.0f * a - 1.0f;
            qy = 2.0f * b - 1.0f;
        } while (qx * qx + qy * qy >= 1.0f);
        offx = aperture / 2.0f * qx;
        offy = aperture / 2.0f * qy;
    }
    const float tin[4] = {dxn, dyn, 1.0f, 1.0f};
    float target[4];
    mat4_mul(f.cam.proj_inv, tin, target);
    float origin[4], dir[4];
    if (aperture > 0.0f) {
        const float oin[4] = {offx, offy, 0.0f, 1.0f};
        mat4_mul(f.cam.view_inv, oin, origin);
        const v3 tv = mk(target[0], target[1], target[2]) * focus - mk(offx, offy, 0.0f);
        const v3 nd = normalize(tv);
        const float din[4] = {nd.x, nd.y, nd.z, 0.0f};
        mat4_mul(f.cam.view_inv, din, dir);
    } else {
        const float oin[4] = {0.0f, 0.0f, 0.0f, 1.0f};
        mat4_mul(f.cam.view_inv, oin, origin);
        const v3 nd = normalize(mk(target[0], target[1], target[2]));
        const float din[4] = {nd.x, nd.y, nd.z, 0.0f};
        mat4_mul(f.cam.view_inv, din, dir);
    }
    w.q_o[0][j] = make_float4(origin[0], origin[1], origin[2], __uint_as_float(p));
    w.q_d[0][j] = make_float4(dir[0], dir[1], dir[2], 0.0f);
    w.weight[p] = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
    w.radiance[chunk_start + p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
}

// ---------------------------------------------------------------------------
// Closest-hit extension (traceRayEXT with tMin 0.001, tMax 10000).
// ---------------------------------------------------------------------------
template <bool COUNT, bool BATCH>
__global__ void __launch_bounds__(128) k_extend(SceneDev s, const FrameDev* __restrict__ fp, BatchDev b, WaveDev w,
                                                int cur, uint32_t depth, uint64_t chunk_start) {
    __shared__ uint32_t s_stack[kSmemStack * kThreadsTrace];
    const uint32_t count = w.counters[cur];
    const float4* __restrict__ qo = w.q_o[cur];
    const float4* __restrict__ qd = w.q_d[cur];
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&w.stats[depth == 0 ? 0 : 1], (unsigned long long)count);
    TraceCounters cnt{0, 0, 0};
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const float4 o = qo[i], d = qd[i];
        HitOut h;
        const View<BATCH> v = view_of<BATCH>(fp, b, w, chunk_start, __float_as_uint(o.w));
        AnyHitCtx ah;
        ah.f = v.f;
        ah.g = v.g;
        ah.st.init(depth, KF_RNG_ANYHIT);
        trace<false, COUNT>(s, root_of<BATCH>(s, v), s_stack, o.x, o.y, o.z, d.x, d.y, d.z, KF_T_MIN, KF_T_MAX, h,
                            cnt, &ah);
        w.hit[i] = make_float4(h.t, h.u, h.v, __uint_as_float(h.inst));
        w.hit_prim[i] = h.prim;
        if (depth == 0 && w.primary) {
            const uint32_t p = __float_as_uint(o.w);
            kf_hit ph;
            ph.t = h.t; ph.u = h.u; ph.v = h.v; ph.prim = h.prim;
            ph.instance = (BATCH && h.inst != kMiss) ? h.inst - v.it->inst_base : h.inst; // scene-local id
            ph.pad[0] = ph.pad[1] = ph.pad[2] = 0;
            w.primary[chunk_start + p] = ph;
        }
    }
    if (COUNT) {
        const uint32_t active = __activemask();
        if (active == kFull) {
            warp_add_stat(&w.stats[3], cnt.nodes);
            warp_add_stat(&w.stats[4], cnt.tris);
            warp_add_stat(&w.stats[5], cnt.insts);
        } else {
            atomicAdd(&w.stats[3], (unsigned long long)cnt.nodes);
            atomicAdd(&w.stats[4], (unsigned long long)cnt.tris);
            atomicAdd(&w.stats[5], (unsigned long long)cnt.insts);
        }
    }
}

// ---------------------------------------------------------------------------
// Shader library (base/Random.glsl, base/Sampling.glsl).
// ---------------------------------------------------------------------------
__device__ __forceinline__ v3 getPerpendicularVector(v3 u) { // Random.glsl:58-65
    const v3 a = mk(fabsf(u.x), fabsf(u.y), fabsf(u.z));
    const uint32_t xm = ((a.x - a.y) < 0.0f && (a.x - a.z) < 0.0f) ? 1u : 0u;
    const uint32_t ym = (a.y - a.z) < 0.0f ? (1u ^ xm) : 0u;
    const uint32_t zm = 1u ^ (xm | ym);
    return cross(u, mk((float)xm, (float)ym, (float)zm));
}
__device__ __forceinline__ float Schlick(float cosine, float ior) { // Random.glsl:68-73
    float r0 = (1.0f - ior) / (1.0f + ior);
    r0 *= r0;
    return r0 + (1.0f - r0) * kpow5(1.0f - cosine);
}
__device__ __forceinline__ float ggxD(float NdotH, float a2) { // Random.glsl:75-79
    const float d = fmaxf(NdotH * NdotH * (a2 - 1.0f) + 1.0f, 1e-6f);
    return a2 / (d * d * KF_REF_PI);
}
__device__ __forceinline__ float G1(float d, float a2) { return (2.0f * d) / (d + sqrtf(a2 + (1.0f - a2) * (d * d))); }
__device__ __forceinline__ float GeometricShadowing(float NdotV, float NdotL, float a2) {
    return G1(NdotL, a2) * G1(NdotV, a2);
}
__device__ __forceinline__ v3 schlickFresnel(v3 f0, float lDotH) { // Random.glsl:133-136
    const float e = (-5.55473f * lDotH - 6.98316f) * lDotH;
    return f0 + (splat(1.0f) - f0) * kexp2(e);
}
__device__ __forceinline__ v3 sampleGGX(float u0, float u1, float a2, v3 N) { // Random.glsl:83-101
    const v3 B = getPerpendicularVector(N);
    const v3 T = cross(B, N);
    const float cosThetaH = sqrtf(clampf((1.0f - u0) / ((a2 - 1.0f) * u0 + 1.0f), 0.0f, 1.0f));
    const float sinThetaH = sqrtf(clampf(1.0f - cosThetaH * cosThetaH, 0.0f, 1.0f));
    const float phiH = u1 * KF_REF_PI * 2.0f;
    float sp, cp;
    ksincos(phiH, sp, cp);
    return T * (sinThetaH * cp) + B * (sinThetaH * sp) + N * cosThetaH;
}
__device__ __forceinline__ v3 transformLocalToWorld(v3 dir, v3 n) { // Sampling.glsl:6-23
    v3 tangent;
    if (fabsf(n.x) > fabsf(n.y))
        tangent = mk(n.z, 0.0f, -n.x) / sqrtf(n.x * n.x + n.z * n.z);
    else
        tangent = mk(0.0f, -n.z, n.y) / sqrtf(n.y * n.y + n.z * n.z);
    const v3 bitangent = cross(n, tangent);
    return dir.x * tangent + dir.y * bitangent + dir.z * n;
}
__device__ __forceinline__ v3 cosineHemisphereSampling(float u0, float u1, v3 n) { // Sampling.glsl:25-35
    const float sq = sqrtf(1.0f - u1);
    const float ang = 2.0f * KF_REF_PI * u0;
    float sa, ca;
    ksincos(ang, sa, ca);
    return transformLocalToWorld(mk(ca * sq, sa * sq, sqrtf(u1)), n);
}
__device__ __forceinline__ v3 uniformSphereSampling(Stream& st, const PathKey& pk) { // Sampling.glsl:72-83
    v3 p;
    do {
        const float a = st.next(pk), b = st.next(pk), c = st.next(pk);
        p = mk(a, b, c) * 2.0f - splat(1.0f);
    } while (dot(p, p) >= 1.0f);
    return p;
}

// Environment lookup of PathTrace.rmiss:14-29: texture(environmentMap, vec3(-d.y, d.z, -d.x)).
// Face selection by the major axis and face coordinates (sc, tc) of the Vulkan / GL cube
// rules; bilinear within the face, clamp to edge. env: 6 faces of env_size^2 texels.
// Texture and environment lookups are not inlined: k_shade is bound by instruction fetch
// (its largest stall is "no instruction"), and one copy each keeps the kernel smaller.
__device__ __noinline__ v3 env_lookup(const float4* env, uint32_t env_size, v3 d) {
    const float rx = -d.y, ry = d.z, rz = -d.x;
    const float ax = fabsf(rx), ay = fabsf(ry), az = fabsf(rz);
    uint32_t face;
    float sc, tc, ma;
    if (ax >= ay && ax >= az) {
        ma = ax;
        face = rx >= 0.0f ? 0u : 1u;
        sc = rx >= 0.0f ? -rz : rz;
        tc = -ry;
    } else if (ay >= az) {
        ma = ay;
        face = ry >= 0.0f ? 2u : 3u;
        sc = rx;
        tc = ry >= 0.0f ? rz : -rz;
    } else {
        ma = az;
        face = rz >= 0.0f ? 4u : 5u;
        sc = rz >= 0.0f ? rx : -rx;
        tc = -ry;
    }
    const uint32_t n = env_size;
    const float fs = 0.5f * (sc / ma + 1.0f), ft = 0.5f * (tc / ma + 1.0f);
    const float x = fs * (float)n - 0.5f, y = ft * (float)n - 0.5f;
    const float fx0 = floorf(x), fy0 = floorf(y);
    const float wx = x - fx0, wy = y - fy0;
    const int ix = (int)fx0, iy = (int)fy0, hi = (int)n - 1;
    const uint32_t x0 = (uint32_t)min(max(ix, 0), hi), x1 = (uint32_t)min(max(ix + 1, 0), hi);
    const uint32_t y0 = (uint32_t)min(max(iy, 0), hi), y1 = (uint32_t)min(max(iy + 1, 0), hi);
    const float4* fp = env + (size_t)face * n * n;
    const float4 t00 = __ldg(fp + (size_t)y0 * n + x0), t10 = __ldg(fp + (size_t)y0 * n + x1);
    const float4 t01 = __ldg(fp + (size_t)y1 * n + x0), t11 = __ldg(fp + (size_t)y1 * n + x1);
    const v3 top = mk(t00.x, t00.y, t00.z) * (1.0f - wx) + mk(t10.x, t10.y, t10.z) * wx;
    const v3 bot = mk(t01.x, t01.y, t01.z) * (1.0f - wx) + mk(t11.x, t11.y, t11.z) * wx;
    return top * (1.0f - wy) + bot * wy;
}

// Texture lookup: bilinear, repeat, optional sRGB decode (vkCore.hpp:585,619-637).
__device__ __noinline__ v3 texture_rgb(const SceneDev& s, int id, float u, float v) {
    if (id < 0 || (uint32_t)id >= s.num_textures) return splat(1.0f);
    const uint4 ti = __ldg(s.tex_info + id);
    const float x = u * (float)ti.y - 0.5f;
    const float y = v * (float)ti.z - 0.5f;
    const float fx0 = floorf(x), fy0 = floorf(y);
    const float ax = x - fx0, ay = y - fy0;
    const long long ix = (long long)fx0, iy = (long long)fy0;
    auto wrap = [](long long i, uint32_t n) {
        long long m = i % (long long)n;
        return (uint32_t)(m < 0 ? m + n : m);
    };
    const uint32_t x0 = wrap(ix, ti.y), x1 = wrap(ix + 1, ti.y);
    const uint32_t y0 = wrap(iy, ti.z), y1 = wrap(iy + 1, ti.z);
    const uchar4 t00 = __ldg(s.texels + ti.x + (size_t)y0 * ti.y + x0);
    const uchar4 t10 = __ldg(s.texels + ti.x + (size_t)y0 * ti.y + x1);
    const uchar4 t01 = __ldg(s.texels + ti.x + (size_t)y1 * ti.y + x0);
    const uchar4 t11 = __ldg(s.texels + ti.x + (size_t)y1 * ti.y + x1);
    auto dec = [&](unsigned char b) { return ti.w ? __ldg(s.srgb_decode + b) : (float)b / 255.0f; };
    float out[3];
    const unsigned char c00[3] = {t00.x, t00.y, t00.z}, c10[3] = {t10.x, t10.y, t10.z};
    const unsigned char c01[3] = {t01.x, t01.y, t01.z}, c11[3] = {t11.x, t11.y, t11.z};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const float top = dec(c00[c]) * (1.0f - ax) + dec(c10[c]) * ax;
        const float bot = dec(c01[c]) * (1.0f - ax) + dec(c11[c]) * ax;
        out[c] = top * (1.0f - ay) + bot * ay;
    }
    return mk(out[0], out[1], out[2]);
}

struct Shading {
    float f, a2;
    v3 diffuseColor, specularColor, transmissionColor;
    bool isInside;
};

// calcDirectContribution (PathTrace.rchit:103-171).
__device__ v3 calcDirectContribution(Stream& st, const PathKey& pk, v3 L, v3 V, v3 N, v3 lightEmission,
                                     const Shading& sh) {
    v3 weight = splat(0.0f);
    const float a2 = sh.a2, f = sh.f;
    if (sh.transmissionColor != splat(0.0f)) {
        if (sh.isInside) {
            weight = splat(0.0f);
        } else {
            const float NdotV0 = dot(N, V);
            const v3 refractedL = refract(-V, N, 1.0f / f);
            const float reflectProb = refractedL != splat(0.0f) ? Schlick(NdotV0, f) : 1.0f;
            if (st.next(pk) <= reflectProb) {
                const v3 H = normalize(L + V);
                const float NdotL = dot(N, L);
                const float NdotH = dot(N, H);
                const float HdotV = dot(H, V);
                const float NdotV = fmaxf(dot(N, V), 1e-6f);
                const float LdotH = dot(L, H);
                const float D = ggxD(NdotH, a2);
                const float G = GeometricShadowing(NdotL, NdotV, a2);
                const v3 F = schlickFresnel(sh.transmissionColor, LdotH);
                weight = D * F * G * HdotV / NdotH * NdotV;
            } else {
                weight = splat(0.0f);
            }
        }
    } else {
        const v3 H = normalize(L + V);
        const float NdotL = dot(N, L);
        const float NdotH = dot(N, H);
        const float HdotV = dot(H, V);
        const float NdotV = fmaxf(dot(N, V), 1e-6f);
        const float LdotH = dot(L, H);
        const float D = ggxD(NdotH, a2);
        const float G = GeometricShadowing(NdotL, NdotV, a2);
        const v3 F = schlickFresnel(sh.specularColor, LdotH);
        const float diffuseLum = length(sh.diffuseColor);
        const float specularLum = length(sh.specularColor);
        float probDiffuse = diffuseLum / (diffuseLum + specularLum);
        if (diffuseLum == 0.0f && specularLum == 0.0f) probDiffuse = 0.5f;
        const v3 diffuseWeight = sh.diffuseColor * splat(NdotL);
        const v3 specularWeight = D * F * G * HdotV / NdotH * NdotV;
        weight = st.next(pk) < probDiffuse ? diffuseWeight * probDiffuse : specularWeight * (1.0f - probDiffuse);
    }
    return lightEmission * weight;
}

// Light slots of a view: the scene's own (single-view frame) or its item's (batched).
struct SceneLights {
    const SceneDev& s;
    __device__ __forceinline__ uint32_t group(uint32_t j) const { return s.slot_group[j]; }
    __device__ __forceinline__ uint32_t index(uint32_t j) const { return s.slot_index[j]; }
    __device__ __forceinline__ const kf_dir_light_ubo* dlight() const { return s.dlight; }
    __device__ __forceinline__ const kf_point_lights_ubo* plights() const { return s.plights; }
    __device__ __forceinline__ const kf_active_lights_ubo* alights() const { return s.alights; }
};
struct ItemLights {
    const ItemDev* it;
    __device__ __forceinline__ uint32_t group(uint32_t j) const { return it->slot_group[j]; }
    __device__ __forceinline__ uint32_t index(uint32_t j) const { return it->slot_index[j]; }
    __device__ __forceinline__ const kf_dir_light_ubo* dlight() const { return it->dlight; }
    __device__ __forceinline__ const kf_point_lights_ubo* plights() const { return it->plights; }
    __device__ __forceinline__ const kf_active_lights_ubo* alights() const { return it->alights; }
};

// One light slot's sample: returns true if a shadow ray is needed (NdotL > 0 and a
// non-zero contribution), with its direction, length and contribution.
template <class LS>
__device__ bool light_sample(const SceneDev& s, const LS& ls, uint32_t slot, uint32_t depth, const PathKey& pk,
                             v3 worldPos, v3 N, v3 V, const Shading& sh, v3& Lout, float& tmax, v3& contrib) {
    const uint32_t group = ls.group(slot), li = ls.index(slot);
    Stream st;
    v3 L, lightEmission;
    float maxDist;
    if (group == 0) { // traceDirectionalLight (rchit:204-223)
        const kf_dir_light_ubo* dl = ls.dlight();
        st.init(depth, KF_RNG_DIRLIGHT);
        lightEmission = ld3(dl->rgbs) * dl->rgbs[3];
        if (lightEmission == splat(0.0f)) return false;
        L = -ld3(dl->direction);
        if (dl->direction[3] != 0.0f) {
            const float a = st.next(pk), b = st.next(pk), c = st.next(pk);
            L = normalize(L + dl->direction[3] * mk(a, b, c));
        }
        maxDist = KF_DIR_LIGHT_TMAX;
    } else if (group == 1) { // tracePointLights (rchit:227-258)
        const kf_point_lights_ubo* pl = ls.plights();
        st.init(depth, KF_RNG_POINT0 + li);
        if (!(pl->rgbs[li][3] > 0.0f)) return false;
        const float lum = length(ld3(pl->rgbs[li]) * pl->rgbs[li][3]);
        if (lum == 0.0f) return false;
        v3 lpos = ld3(pl->posr[li]);
        if (pl->posr[li][3] != 0.0f) {
            const v3 perturb = uniformSphereSampling(st, pk);
            lpos = lpos + pl->posr[li][3] * normalize(perturb);
        }
        L = lpos - worldPos;
        const float d = length(L);
        L = normalize(L);
        lightEmission = ld3(pl->rgbs[li]) * pl->rgbs[li][3] / d / d;
        maxDist = d;
    } else { // traceActiveLights (rchit:262-316)
        const kf_active_lights_ubo* al = ls.alights();
        st.init(depth, KF_RNG_ACTIVE0 + li);
        if (!(al->front[li][3] > 0.0f)) return false;
        const float lum = length(ld3(al->rgbs[li]) * al->rgbs[li][3]);
        if (lum == 0.0f) return false;
        const float softness = al->sftp[li][0];
        v3 lpos = ld3(al->position[li]);
        if (softness != 0.0f) {
            const v3 perturb = uniformSphereSampling(st, pk);
            lpos = lpos + softness * normalize(perturb);
        }
        L = lpos - worldPos;
        const float d = length(L);
        L = normalize(L);
        const float fov = al->sftp[li][1];
        const v3 alightDir = normalize(ld3(al->front[li]));
        const float halfAngle = clampf(fov, 0.0f, KF_REF_PI) / 2.0f;
        const float cos_ = dot(alightDir, -L);
        if (!(cos_ > kcos(halfAngle))) return false;
        const int texID = (int)al->sftp[li][2];
        v3 color = ld3(al->rgbs[li]);
        if (texID >= 0) {
            // proj * view * vec4(worldPos, 1) = (proj * view) * vec4(...)
            const float* P = al->proj[li];
            const float* Vw = al->view[li];
            float pv[16];
#pragma unroll
            for (int c = 0; c < 4; ++c)
#pragma unroll
                for (int r = 0; r < 4; ++r)
                    pv[c * 4 + r] = P[0 * 4 + r] * Vw[c * 4 + 0] + P[1 * 4 + r] * Vw[c * 4 + 1] +
                                    P[2 * 4 + r] * Vw[c * 4 + 2] + P[3 * 4 + r] * Vw[c * 4 + 3];
            const float wp[4] = {worldPos.x, worldPos.y, worldPos.z, 1.0f};
            float tc[4];
            mat4_mul(pv, wp, tc);
            const float ww = tc[3];
            for (int k = 0; k < 4; ++k) tc[k] = tc[k] / ww;
            color = color * texture_rgb(s, texID, tc[0] * 0.5f + 0.5f, tc[1] * 0.5f + 0.5f);
        }
        lightEmission = color * al->rgbs[li][3] / d / d;
        maxDist = d;
    }
    // traceShadowRay (rchit:175-200): only NdotL > 0 traces; the lobe draw is the
    // next draw of this light's stream.
    if (!(dot(N, L) > 0.0f)) return false;
    contrib = calcDirectContribution(st, pk, L, V, N, lightEmission, sh);
    if (contrib == splat(0.0f)) return false;
    Lout = L;
    tmax = maxDist;
    return true;
}

// ---------------------------------------------------------------------------
// Shade: miss / emission / PrincipledBSDF (rchit:322-468), light samples, RR.
// ---------------------------------------------------------------------------
// ---------------------------------------------------------------------------
// Rays that missed (PathTrace.rmiss:12-31): environment map, else clear colour, added with
// the path weight; the path ends. The rays that hit are listed in w.sel for k_shade, so
// that its warps shade hits only.
// ---------------------------------------------------------------------------
template <bool BATCH>
__device__ __forceinline__ void miss_path(const SceneDev& s, const FrameDev* fp, const BatchDev& b, const WaveDev& w,
                                          int cur, uint32_t depth, uint64_t chunk_start, uint32_t i) {
    const float4 qo = w.q_o[cur][i], qd = w.q_d[cur][i];
    const uint32_t p = __float_as_uint(qo.w);
    const uint64_t g = chunk_start + p;
    const View<BATCH> vw = view_of<BATCH>(fp, b, w, chunk_start, p);
    const FrameDev& f = *vw.f;
    const float4* env = BATCH ? vw.it->env : s.env;
    const uint32_t env_size = BATCH ? vw.it->env_size : s.env_size;
    const float4 w4 = w.weight[p];
    const v3 wold = mk(w4.x, w4.y, w4.z);
    const float4 col4 = w.radiance[g];
    v3 color = mk(col4.x, col4.y, col4.z);
    const v3 emission = (f.pc.use_env_map && env) ? env_lookup(env, env_size, mk(qd.x, qd.y, qd.z))
                                                   : ld3(f.pc.clear_color) * f.pc.clear_color[3];
    color = color + emission * wold;
    w.radiance[g] = make_float4(color.x, color.y, color.z, 0.0f);
    w.req[p] = 0;
    if (depth == 0 && vw.g < f.npix) { // sample 0 of the first bounce
        const uint32_t pix = (uint32_t)vw.g;
        (BATCH ? vw.it->depth : w.depth)[pix] = 0.0f;
        uint4* aov_seg = BATCH ? vw.it->seg : w.seg;
        if (aov_seg) aov_seg[pix] = make_uint4(kMiss, kMiss, kMiss, 0u);
    }
}

// One block of kMissThreads takes tiles of kMissThreads * kMissPer rays, kMissPer consecutive
// rays per thread; the hits of a tile get their list positions from one atomic per tile (a
// block scan), not one per warp, and stay in queue order (the order k_shade appends the next
// bounce's rays in, which keeps neighbouring rays together).
constexpr uint32_t kMissThreads = 128, kMissPer = 4;
template <bool BATCH>
__global__ void __launch_bounds__(kMissThreads) k_miss(SceneDev s, const FrameDev* __restrict__ fp, BatchDev b,
                                                       WaveDev w, int cur, uint32_t depth, uint64_t chunk_start) {
    __shared__ uint32_t s_cnt[kMissThreads / 32];
    __shared__ uint32_t s_base;
    const uint32_t count = w.counters[cur];
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    constexpr uint32_t tile = kMissThreads * kMissPer;
    for (uint32_t base = blockIdx.x * tile; base < count; base += gridDim.x * tile) {
        uint32_t hitm = 0, missm = 0, nh = 0;
#pragma unroll
        for (uint32_t q = 0; q < kMissPer; ++q) {
            const uint32_t i = base + threadIdx.x * kMissPer + q;
            if (i < count) {
                if (__float_as_uint(w.hit[i].w) == kMiss) {
                    missm |= 1u << q;
                } else {
                    hitm |= 1u << q;
                    ++nh;
                }
            }
        }
        uint32_t x = nh; // inclusive scan over the warp
#pragma unroll
        for (uint32_t o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(kFull, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) s_cnt[warp] = x;
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t t = 0;
            for (uint32_t k = 0; k < kMissThreads / 32; ++k) t += s_cnt[k];
            s_base = t ? atomicAdd(&w.counters[5], t) : 0u;
        }
        __syncthreads();
        uint32_t pos = s_base + x - nh;
        for (uint32_t k = 0; k < warp; ++k) pos += s_cnt[k];
        __syncthreads(); // s_cnt and s_base are rewritten by the next tile
#pragma unroll
        for (uint32_t q = 0; q < kMissPer; ++q)
            if (hitm & (1u << q)) w.sel[pos++] = base + threadIdx.x * kMissPer + q;
#pragma unroll 1
        for (uint32_t q = 0; q < kMissPer; ++q)
            if (missm & (1u << q)) miss_path<BATCH>(s, fp, b, w, cur, depth, chunk_start, base + threadIdx.x * kMissPer + q);
    }
}

// Blocks of the shading kernels (k_shade, k_nee); k_shade's block scan keeps one count per warp.
constexpr uint32_t kShadeThreads = 128, kShadeWarps = kShadeThreads / 32;

template <bool BATCH>
// 4 resident blocks per SM (128 registers, no spill) measured fastest; unbounded it takes 148.
__global__ void __launch_bounds__(kShadeThreads, 4) k_shade(SceneDev s, const FrameDev* __restrict__ fp, BatchDev b, WaveDev w,
                                               int cur, uint32_t depth, uint64_t chunk_start) {
    const uint32_t count = w.counters[5]; // rays of this bounce that hit (k_miss takes the others)
    const int nxt = cur ^ 1;
    const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const uint32_t stride = gridDim.x * blockDim.x;
    __shared__ uint32_t s_cnt[2][kShadeWarps], s_base[2]; // per tile parity: the block scan of continuing paths
    uint32_t par = 0;
    for (uint32_t bbase = blockIdx.x * blockDim.x; bbase < count; bbase += stride, par ^= 1) {
        const uint32_t base = bbase + (threadIdx.x & ~31u);
        const bool valid = base + lane < count;
        const uint32_t i = valid ? w.sel[base + lane] : 0u; // queue position of the ray
        uint32_t p = 0;
        uint64_t g = 0;
        PathKey pk;
        bool is_mat = false, cont = false;
        v3 worldPos = splat(0.0f), N = splat(0.0f), V = splat(0.0f), L = splat(0.0f);
        v3 wnew = splat(0.0f), wcont = splat(0.0f);
        Shading sh;
        sh.f = 1.0f; sh.a2 = 0.0f;
        sh.diffuseColor = sh.specularColor = sh.transmissionColor = splat(0.0f);
        sh.isInside = false;
        View<BATCH> vw{fp, nullptr, 0};
        if (valid) {
            const float4 qo = w.q_o[cur][i], qd = w.q_d[cur][i];
            p = __float_as_uint(qo.w);
            g = chunk_start + p; // radiance index (the batch's path space)
            vw = view_of<BATCH>(fp, b, w, chunk_start, p);
            const FrameDev& f = *vw.f;
            uint32_t sample, pix;
            split_path(vw.g, f.npix, sample, pix);
            pk = PathKey{make_uint2(f.seed ^ pix, f.camera_index), sample, f.frame};
            float4* aov_albedo = BATCH ? vw.it->albedo : w.albedo;
            float4* aov_normal = BATCH ? vw.it->normal : w.normal;
            float* aov_depth = BATCH ? vw.it->depth : w.depth;
            const float4 hv = w.hit[i];
            const uint32_t inst = __float_as_uint(hv.w); // never kMiss here
            const float4 w4 = w.weight[p];
            const v3 wold = mk(w4.x, w4.y, w4.z);
            float4 col4 = w.radiance[g];
            v3 color = mk(col4.x, col4.y, col4.z);
            const v3 rayD = mk(qd.x, qd.y, qd.z);
            {
                const uint32_t prim = w.hit_prim[i];
                const InstanceRec* ip = s.inst + inst;
                const float4 m0 = __ldg(&ip->w2o0), m1 = __ldg(&ip->w2o1), m2 = __ldg(&ip->w2o2);
                const uint32_t geom = __ldg(&ip->geometry);
                const uint4 gi = __ldg(s.geom + geom);
                const uint32_t tri = gi.y + prim;
                const uint32_t i0 = __ldg(s.indices + 3 * (size_t)tri + 0) + gi.x;
                const uint32_t i1 = __ldg(s.indices + 3 * (size_t)tri + 1) + gi.x;
                const uint32_t i2 = __ldg(s.indices + 3 * (size_t)tri + 2) + gi.x;
                const float4 a0 = __ldg(s.verts + 3 * (size_t)i0), a1 = __ldg(s.verts + 3 * (size_t)i0 + 1),
                             a2v = __ldg(s.verts + 3 * (size_t)i0 + 2);
                const float4 b0 = __ldg(s.verts + 3 * (size_t)i1), b1 = __ldg(s.verts + 3 * (size_t)i1 + 1),
                             b2 = __ldg(s.verts + 3 * (size_t)i1 + 2);
                const float4 c0 = __ldg(s.verts + 3 * (size_t)i2), c1 = __ldg(s.verts + 3 * (size_t)i2 + 1),
                             c2 = __ldg(s.verts + 3 * (size_t)i2 + 2);
                const kf_material_gpu mat = s.materials[__ldg(s.matidx + tri)];
                const v3 emission = ld3(mat.emission) * mat.emission[3];
                if (emission != splat(0.0f)) {
                    // emissive hit ends the path (rchit:330-335)
                    color = color + (ld3(mat.emission) * mat.emission[3]) * wold;
                    w.radiance[g] = make_float4(color.x, color.y, color.z, 0.0f);
                } else {
                    // getShadingData (rchit:66-98); unpackVertex: pos = d0.xyz,
                    // normal = (d0.w, d1.x, d1.y), uv = (d2.y, d2.z)
                    const float bx = 1.0f - hv.y - hv.z, by = hv.y, bz = hv.z;
                    const v3 n0 = mk(a0.w, a1.x, a1.y), n1 = mk(b0.w, b1.x, b1.y), n2 = mk(c0.w, c1.x, c1.y);
                    const v3 ln = n0 * bx + n1 * by + n2 * bz;
                    const v3 wn = mk(ln.x * m0.x + ln.y * m1.x + ln.z * m2.x, ln.x * m0.y + ln.y * m1.y + ln.z * m2.y,
                                     ln.x * m0.z + ln.y * m1.z + ln.z * m2.z);
                    N = normalize(wn);
                    const v3 rayO = mk(qo.x, qo.y, qo.z);
                    worldPos = rayO + rayD * hv.x;
                    const float uvx = a2v.y * bx + b2.y * by + c2.y * bz;
                    const float uvy = a2v.z * bx + b2.z * by + c2.z * bz;
                    // facing in object space: front when dir opposes (v1-v0)x(v2-v0)
                    bool backface;
                    {
                        const float odx = m0.x * rayD.x + m0.y * rayD.y + m0.z * rayD.z;
                        const float ody = m1.x * rayD.x + m1.y * rayD.y + m1.z * rayD.z;
                        const float odz = m2.x * rayD.x + m2.y * rayD.y + m2.z * rayD.z;
                        const v3 e1 = mk(b0.x, b0.y, b0.z) - mk(a0.x, a0.y, a0.z);
                        const v3 e2 = mk(c0.x, c0.y, c0.z) - mk(a0.x, a0.y, a0.z);
                        backface = dot(mk(odx, ody, odz), cross(e1, e2)) > 0.0f;
                    }
                    v3 baseColor = ld3(mat.diffuse);
                    if (mat.diffuse_tex >= 0) baseColor = texture_rgb(s, mat.diffuse_tex, uvx, uvy);
                    baseColor = baseColor / KF_REF_PI;
                    const float metallic =
                        mat.metallic_tex >= 0 ? texture_rgb(s, mat.metallic_tex, uvx, uvy).x : mat.metallic;
                    const float roughness =
                        mat.roughness_tex >= 0 ? texture_rgb(s, mat.roughness_tex, uvx, uvy).x : mat.roughness;
                    const float a2 = roughness * roughness;
                    const float transmission = mat.transmission_tex >= 0
                                                   ? texture_rgb(s, mat.transmission_tex, uvx, uvy).x
                                                   : mat.transmission;
                    const float fi = fmaxf(mat.ior, 1e-5f);
                    const float diffuse_weight =
                        (1.0f - clampf(metallic, 0.0f, 1.0f)) * (1.0f - clampf(transmission, 0.0f, 1.0f));
                    const float final_transmission =
                        clampf(transmission, 0.0f, 1.0f) * (1.0f - clampf(metallic, 0.0f, 1.0f));
                    const float specular_weight = (1.0f - final_transmission);
                    v3 weight = splat(0.0f);
                    V = normalize(-rayD);
                    const bool isInside = backface;
                    N = isInside ? -N : N;
                    L = splat(0.0f);
                    const float NdotV = dot(N, V);
                    const v3 diffuseColor = diffuse_weight * baseColor;
                    const v3 specularColor =
                        specular_weight * (baseColor * metallic + (mat.specular * 0.08f * splat(1.0f)) * (1.0f - metallic));
                    const v3 transmissionColor = transmission * baseColor;
                    const float diffuseLum = length(diffuseColor);
                    const float specularLum = length(specularColor);
                    float probDiffuse = diffuseLum / (diffuseLum + specularLum);
                    if (diffuseLum == 0.0f && specularLum == 0.0f) {
                        if (baseColor == splat(0.0f)) {
                            if (diffuse_weight == 1.0f) probDiffuse = 1.0f;
                            else if (diffuse_weight == 0.0f) probDiffuse = 0.0f;
                            else probDiffuse = 0.5f;
                        } else
                            probDiffuse = 0.0f;
                    } else {
                        probDiffuse *= specular_weight;
                    }
                    Stream bs;
                    bs.init(depth, KF_RNG_BSDF);
                    const bool chooseDiffuse = bs.next(pk) < probDiffuse;
                    if (chooseDiffuse) {
                        const float u0 = bs.next(pk), u1 = bs.next(pk);
                        L = cosineHemisphereSampling(u0, u1, N);
                        const float NdotL = clampf(dot(N, L), 0.0f, 1.0f);
                        weight = KF_REF_PI * diffuseColor * NdotL / probDiffuse;
                    }
                    if (!chooseDiffuse) {
                        if (final_transmission == 0.0f) {
                            const float u0 = bs.next(pk), u1 = bs.next(pk);
                            const v3 H = sampleGGX(u0, u1, a2, N);
                            const float HdotV = dot(H, V);
                            L = 2.0f * HdotV * H - V;
                            const float NoV = fmaxf(dot(N, V), 1e-7f);
                            const float NoL = dot(N, L);
                            const float NoH = fmaxf(dot(N, H), 1e-7f);
                            const float VoH = fmaxf(dot(V, H), 1e-7f);
                            if (NoL >= 0.0f) {
                                const float G = GeometricShadowing(NoV, NoL, a2);
                                const v3 F = schlickFresnel(specularColor, VoH);
                                weight = KF_REF_PI * F * G * VoH / (NoH * NoV * (1.0f - probDiffuse));
                            } else
                                weight = splat(0.0f);
                        } else {
                            const float ior = isInside ? 1.0f / fi : fi;
                            const float _dot = isInside ? NdotV * ior : NdotV;
                            const v3 refractedL = refract(-V, N, 1.0f / fi);
                            const float reflectProb = refractedL != splat(0.0f) ? Schlick(_dot, fi) : 1.0f;
                            if (bs.next(pk) >= reflectProb) {
                                L = refractedL;
                                weight = KF_REF_PI * transmissionColor / (1.0f - probDiffuse);
                            } else {
                                L = reflect(-V, N);
                                weight = KF_REF_PI * transmissionColor / (1.0f - probDiffuse);
                            }
                        }
                    }
                    sh.f = fi;
                    sh.a2 = a2;
                    sh.diffuseColor = diffuseColor;
                    sh.specularColor = specularColor;
                    sh.transmissionColor = transmissionColor;
                    sh.isInside = isInside;
                    // AOVs of sample 0, first bounce (rgen:114-117)
                    if (depth == 0 && sample == 0) {
                        aov_albedo[pix] = make_float4(baseColor.x, baseColor.y, baseColor.z, 1.0f);
                        aov_normal[pix] = make_float4(N.x, N.y, N.z, 1.0f);
                    }
                    // rgen:110  weight *= ray.weight
                    wnew = wold * weight;
                    if (wnew != splat(0.0f)) {
                        is_mat = true;
                        bool alive = true;
                        wcont = wnew;
                        if (f.pc.russian_roulette && depth >= f.pc.rr_min_bounces) { // rgen:124-138
                            const float pr = fmaxf(wnew.x, fmaxf(wnew.y, wnew.z));
                            Stream rs;
                            rs.init(depth, KF_RNG_RR);
                            const float rnd = rs.next(pk);
                            if (rnd > pr)
                                alive = false;
                            else
                                wcont = wnew * (1.0f / pr);
                        }
                        cont = alive && (depth + 1 <= f.pc.max_path_depth);
                    }
                }
            }
            if (depth == 0 && sample == 0) {
                aov_depth[pix] = hv.x;
                uint4* aov_seg = BATCH ? vw.it->seg : w.seg;
                if (aov_seg) {
                    const uint32_t gidx = __ldg(&s.inst[inst].geometry);
                    const uint32_t prim = w.hit_prim[i];
                    const uint32_t midx = __ldg(s.matidx + __ldg(s.geom + gidx).y + prim);
                    aov_seg[pix] = BATCH ? make_uint4(inst - vw.it->inst_base, gidx - vw.it->geom_base, midx, prim)
                                         : make_uint4(inst, gidx, midx, prim);
                }
            }
        }
        // what the light samples of this hit need, for k_nee (hit-list order)
        if (valid) {
            float4* rec = w.nee_in + (size_t)6 * (base + lane);
            rec[0] = make_float4(worldPos.x, worldPos.y, worldPos.z,
                                 __uint_as_float(p | (is_mat ? 0x80000000u : 0u) | (sh.isInside ? 0x40000000u : 0u)));
            rec[1] = make_float4(N.x, N.y, N.z, sh.f);
            rec[2] = make_float4(V.x, V.y, V.z, sh.a2);
            rec[3] = make_float4(sh.diffuseColor.x, sh.diffuseColor.y, sh.diffuseColor.z, wnew.x);
            rec[4] = make_float4(sh.specularColor.x, sh.specularColor.y, sh.specularColor.z, wnew.y);
            rec[5] = make_float4(sh.transmissionColor.x, sh.transmissionColor.y, sh.transmissionColor.z, wnew.z);
        }
        // next rays in hit-list order: one atomic per block tile
        const uint32_t m = __ballot_sync(kFull, cont);
        if (lane == 0) s_cnt[par][wid] = __popc(m);
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t t = 0;
            for (uint32_t k = 0; k < kShadeWarps; ++k) t += s_cnt[par][k];
            s_base[par] = t ? atomicAdd(&w.counters[nxt], t) : 0u;
        }
        __syncthreads();
        uint32_t pos = s_base[par] + __popc(m & lanemask_lt());
        for (uint32_t k = 0; k < wid; ++k) pos += s_cnt[par][k];
        if (cont) {
            w.q_o[nxt][pos] = make_float4(worldPos.x, worldPos.y, worldPos.z, __uint_as_float(p));
            w.q_d[nxt][pos] = make_float4(L.x, L.y, L.z, 0.0f);
            w.weight[p] = make_float4(wcont.x, wcont.y, wcont.z, 0.0f);
        }
    }
}

// ---------------------------------------------------------------------------
// Light samples of the hits (traceDirectionalLight / tracePointLights / traceActiveLights,
// rchit:204-316, after the BSDF sample as in rchit:457-460): one warp-uniform loop over the
// light slots, one ballot per slot. A kernel of its own, beside k_shade: each of the two is
// small enough for the instruction cache.
// ---------------------------------------------------------------------------
template <bool BATCH>
__global__ void __launch_bounds__(kShadeThreads) k_nee(SceneDev s, const FrameDev* __restrict__ fp, BatchDev b, WaveDev w,
                                             uint32_t depth, uint64_t chunk_start) {
    const uint32_t count = w.counters[5];
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t bbase = blockIdx.x * blockDim.x; bbase < count; bbase += stride) {
        const uint32_t base = bbase + (threadIdx.x & ~31u);
        const bool valid = base + lane < count;
        uint32_t p = 0;
        bool is_mat = false;
        v3 worldPos = splat(0.0f), N = splat(0.0f), V = splat(0.0f), wnew = splat(0.0f);
        Shading sh;
        sh.f = 1.0f; sh.a2 = 0.0f;
        sh.diffuseColor = sh.specularColor = sh.transmissionColor = splat(0.0f);
        sh.isInside = false;
        View<BATCH> vw{fp, nullptr, 0};
        PathKey pk{make_uint2(0, 0), 0, 0};
        if (valid) {
            const float4* rec = w.nee_in + (size_t)6 * (base + lane);
            const float4 r0 = rec[0], r1 = rec[1], r2 = rec[2], r3 = rec[3], r4 = rec[4], r5 = rec[5];
            const uint32_t bits = __float_as_uint(r0.w);
            p = bits & 0x3FFFFFFFu;
            is_mat = (bits & 0x80000000u) != 0;
            sh.isInside = (bits & 0x40000000u) != 0;
            worldPos = mk(r0.x, r0.y, r0.z);
            N = mk(r1.x, r1.y, r1.z);
            sh.f = r1.w;
            V = mk(r2.x, r2.y, r2.z);
            sh.a2 = r2.w;
            sh.diffuseColor = mk(r3.x, r3.y, r3.z);
            sh.specularColor = mk(r4.x, r4.y, r4.z);
            sh.transmissionColor = mk(r5.x, r5.y, r5.z);
            wnew = mk(r3.w, r4.w, r5.w);
            vw = view_of<BATCH>(fp, b, w, chunk_start, p);
            const FrameDev& f = *vw.f;
            pk = path_key(f, vw.g);
        }
        uint64_t req = 0;
        const uint32_t nslots =
            BATCH ? __reduce_max_sync(kFull, valid ? vw.it->num_slots : 0u) : s.num_slots;
        for (uint32_t j = 0; j < nslots; ++j) {
            v3 Ls = splat(0.0f), c = splat(0.0f);
            float tmax = 0.0f;
            bool emit;
            if (BATCH)
                emit = is_mat && j < vw.it->num_slots &&
                       light_sample(s, ItemLights{vw.it}, j, depth, pk, worldPos, N, V, sh, Ls, tmax, c);
            else
                emit = is_mat && light_sample(s, SceneLights{s}, j, depth, pk, worldPos, N, V, sh, Ls, tmax, c);
            // each light slot has its own shadow queue, so a shadow-traversal warp takes rays
            // towards one light from neighbouring points; one atomic per warp and slot (a
            // block-wide scan instead waited at two barriers per slot for the warp with the
            // longest light sampling)
            const uint32_t pos = warp_append(emit, &w.scount[j]);
            if (emit) {
                const size_t q = (size_t)j * w.chunk_cap + pos;
                w.sq_o[q] = make_float4(worldPos.x, worldPos.y, worldPos.z, tmax);
                w.sq_d[q] = make_float4(Ls.x, Ls.y, Ls.z, __uint_as_float((j << 26) | p));
                w.contrib[(size_t)j * w.chunk_cap + p] = make_float4(c.x, c.y, c.z, 0.0f);
                w.vis[(size_t)j * w.chunk_cap + p] = 0;
                req |= 1ull << j;
            }
        }
        if (valid) {
            w.req[p] = req;
            if (req) w.nee_w[p] = make_float4(wnew.x, wnew.y, wnew.z, 0.0f);
        }
    }
}

// ---------------------------------------------------------------------------
// Shadow rays: any hit in [0.001, tmax] (rchit:175-200, PathTraceShadow.rmiss).
// ---------------------------------------------------------------------------
// Shadow queues: slot j's rays are sq_o / sq_d[j * chunk_cap + k], k < scount[j]. Kernels
// number the rays slot after slot; shadow_prefix puts the prefix sums of the counts in
// shared memory (all threads of the block must call it) and returns the total.
constexpr uint32_t kMaxSlots = 64;
static_assert(1 + KF_MAX_POINT_LIGHTS + KF_MAX_ACTIVE_LIGHTS <= kMaxSlots, "light slots exceed the shadow queues");
__device__ __forceinline__ uint32_t shadow_prefix(const WaveDev& w, uint32_t* s_pre) {
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (uint32_t j = 0; j < w.nslot; ++j) {
            s_pre[j] = t;
            t += w.scount[j];
        }
        s_pre[w.nslot] = t;
    }
    __syncthreads();
    return s_pre[w.nslot];
}
// Queue entry of shadow ray i (i < the total).
__device__ __forceinline__ uint32_t shadow_entry(const WaveDev& w, const uint32_t* s_pre, uint32_t i) {
    uint32_t j = 0;
    while (i >= s_pre[j + 1]) ++j;
    return j * w.chunk_cap + (i - s_pre[j]);
}

template <bool COUNT, bool BATCH>
__global__ void __launch_bounds__(128) k_shadow(SceneDev s, BatchDev b, WaveDev w) {
    __shared__ uint32_t s_stack[kSmemStack * kThreadsTrace];
    __shared__ uint32_t s_pre[kMaxSlots + 1];
    const uint32_t count = shadow_prefix(w, s_pre);
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&w.stats[2], (unsigned long long)count);
    TraceCounters cnt{0, 0, 0};
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const uint32_t e = shadow_entry(w, s_pre, i);
        const float4 o = w.sq_o[e], d = w.sq_d[e];
        const uint32_t tag = __float_as_uint(d.w);
        const uint32_t slot = tag >> 26, p = tag & ((1u << 26) - 1u);
        const uint32_t root = BATCH ? b.items[w.path_item[p]].root : (s.has_tlas ? 0u : kNoRoot);
        HitOut h;
        const bool occluded =
            trace<true, COUNT>(s, root, s_stack, o.x, o.y, o.z, d.x, d.y, d.z, KF_T_MIN, o.w, h, cnt);
        if (!occluded) w.vis[(size_t)slot * w.chunk_cap + p] = 1;
    }
    if (COUNT) {
        atomicAdd(&w.stats[6], (unsigned long long)cnt.nodes);
        atomicAdd(&w.stats[7], (unsigned long long)cnt.tris);
        atomicAdd(&w.stats[8], (unsigned long long)cnt.insts);
    }
}

// ---------------------------------------------------------------------------
// Persistent traversal with dynamic ray fetch. Each warp keeps up to 32 rays in
// flight; whenever fewer than refill_below lanes are busy, the idle lanes take
// the next rays of the queue (one ballot, one atomic per warp), so a warp does
// not idle behind its slowest ray. Results are identical to k_extend / k_shadow:
// each ray runs the same Tracer steps, only the interleaving changes.
// ---------------------------------------------------------------------------
// refill_below: a warp fetches rays when fewer lanes than this are busy; steps: traversal
// steps between fetches (both tunable, kf_config.dyn_refill_below / dyn_steps).
// Occupancy: 7 resident blocks per SM for closest-hit rays (72 registers, 2 bytes of spill)
// and 9 for shadow rays (56 registers, no spill) measured fastest on the 256-icosphere frame.
template <bool SHADOW, bool COUNT, bool BATCH>
__global__ void __launch_bounds__(128, SHADOW ? 9 : 7)
    k_trace_dyn(SceneDev s, const FrameDev* __restrict__ fp, BatchDev b, WaveDev w, int cur, uint32_t depth,
                uint64_t chunk_start, uint32_t refill_below, int steps) {
    __shared__ uint32_t s_stack[kSmemStack * kThreadsTrace];
    __shared__ uint32_t s_pre[SHADOW ? kMaxSlots + 1 : 1];
    const uint32_t count = SHADOW ? shadow_prefix(w, s_pre) : w.counters[cur];
    uint32_t* fetch = w.counters + (SHADOW ? 4 : 3);
    if (blockIdx.x == 0 && threadIdx.x == 0)
        atomicAdd(&w.stats[SHADOW ? 2 : (depth == 0 ? 0 : 1)], (unsigned long long)count);
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t single_root = s.has_tlas ? 0u : kNoRoot;
    Tracer<SHADOW, COUNT> t;
    t.stack.sm = s_stack + threadIdx.x;
    t.cnt = TraceCounters{0, 0, 0};
    AnyHitCtx ah;
    ah.f = fp;
    ah.g = 0;
    ah.st.init(depth, KF_RNG_ANYHIT);
    bool active = false;
    bool exhausted = false;
    uint32_t idx = 0;
    for (;;) {
        uint32_t act = __ballot_sync(kFull, active);
        if (!exhausted && (uint32_t)__popc(act) < refill_below) {
            const bool need = !active;
            const uint32_t m = __ballot_sync(kFull, need);
            uint32_t base = 0;
            if (lane == 0) base = atomicAdd(fetch, (uint32_t)__popc(m));
            base = __shfl_sync(kFull, base, 0);
            if (base + (uint32_t)__popc(m) >= count) exhausted = true;
            if (need) {
                const uint32_t j = base + __popc(m & lanemask_lt());
                if (j < count) {
                    idx = SHADOW ? shadow_entry(w, s_pre, j) : j;
                    if (SHADOW) {
                        const float4 o = w.sq_o[idx], d = w.sq_d[idx];
                        const uint32_t p = __float_as_uint(d.w) & ((1u << 26) - 1u);
                        const uint32_t root = BATCH ? b.items[w.path_item[p]].root : single_root;
                        t.init(root, o.x, o.y, o.z, d.x, d.y, d.z, KF_T_MIN, o.w);
                    } else {
                        const float4 o = w.q_o[cur][j], d = w.q_d[cur][j];
                        const View<BATCH> v = view_of<BATCH>(fp, b, w, chunk_start, __float_as_uint(o.w));
                        ah.f = v.f;
                        ah.g = v.g;
                        ah.st.init(depth, KF_RNG_ANYHIT);
                        t.init(BATCH ? v.it->root : single_root, o.x, o.y, o.z, d.x, d.y, d.z, KF_T_MIN, KF_T_MAX);
                    }
                    active = true;
                }
            }
            act = __ballot_sync(kFull, active);
        }
        if (act == 0) break;
        if (active) {
            bool done = false;
#pragma unroll 1
            for (int k = 0; k < steps && !done; ++k) done = t.step(s, SHADOW ? nullptr : &ah);
            if (done) {
                if (SHADOW) {
                    if (t.h.inst == kMiss) {
                        const uint32_t tag = __float_as_uint(w.sq_d[idx].w);
                        w.vis[(size_t)(tag >> 26) * w.chunk_cap + (tag & ((1u << 26) - 1u))] = 1;
                    }
                } else {
                    w.hit[idx] = make_float4(t.h.t, t.h.u, t.h.v, __uint_as_float(t.h.inst));
                    w.hit_prim[idx] = t.h.prim;
                    if (depth == 0 && w.primary) {
                        const uint32_t p = __float_as_uint(w.q_o[cur][idx].w);
                        kf_hit ph;
                        ph.t = t.h.t; ph.u = t.h.u; ph.v = t.h.v; ph.prim = t.h.prim;
                        ph.instance = (BATCH && t.h.inst != kMiss)
                                          ? t.h.inst - b.items[w.path_item[p]].inst_base // scene-local id
                                          : t.h.inst;
                        ph.pad[0] = ph.pad[1] = ph.pad[2] = 0;
                        w.primary[chunk_start + p] = ph;
                    }
                }
                active = false;
            }
        }
    }
    if (COUNT) {
        warp_add_stat(&w.stats[SHADOW ? 6 : 3], t.cnt.nodes);
        warp_add_stat(&w.stats[SHADOW ? 7 : 4], t.cnt.tris);
        warp_add_stat(&w.stats[SHADOW ? 8 : 5], t.cnt.insts);
    }
}

// ---------------------------------------------------------------------------
// Gather: shadow_color = traceDirectionalLight + tracePointLights + traceActiveLights
// (rchit:457-460), color += shadow_color * weight (rgen:111).
// ---------------------------------------------------------------------------
template <bool BATCH>
__global__ void k_gather(SceneDev s, BatchDev b, WaveDev w, int cur, uint64_t chunk_start) {
    const uint32_t count = w.counters[cur];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const uint32_t p = __float_as_uint(w.q_o[cur][i].w);
        uint64_t req = w.req[p];
        if (!req) continue;
        const uint8_t* slot_group = BATCH ? b.items[w.path_item[p]].slot_group : nullptr;
        v3 D = splat(0.0f), P = splat(0.0f), A = splat(0.0f);
        while (req) {
            const uint32_t j = __ffsll((long long)req) - 1;
            req &= req - 1;
            if (!w.vis[(size_t)j * w.chunk_cap + p]) continue;
            const float4 c4 = w.contrib[(size_t)j * w.chunk_cap + p];
            const v3 c = mk(c4.x, c4.y, c4.z);
            const uint32_t grp = BATCH ? slot_group[j] : s.slot_group[j];
            if (grp == 0) D = c;
            else if (grp == 1) P = P + c;
            else A = A + c;
        }
        const v3 shadow = (D + P) + A;
        const float4 wn = w.nee_w[p];
        const uint64_t g = chunk_start + p;
        const float4 col = w.radiance[g];
        const v3 color = mk(col.x, col.y, col.z) + shadow * mk(wn.x, wn.y, wn.z);
        w.radiance[g] = make_float4(color.x, color.y, color.z, 0.0f);
    }
}

// ---------------------------------------------------------------------------
// Per-pixel resolve: finalColor = colors / spp (rgen:140-144) and the running
// mean over frames (rgen:151-163); FP64 sum of finalColor alongside.
// ---------------------------------------------------------------------------
__global__ void k_resolve(const FrameDev* __restrict__ fp, const float4* __restrict__ radiance, uint32_t npix,
                          uint32_t spp, float4* accum, dbl4* sum64) {
    const uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
    if (pix >= npix) return;
    const int32_t frame_count = fp->pc.frame_count;
    v3 colors = splat(0.0f);
    for (uint32_t sidx = 0; sidx < spp; ++sidx) {
        const float4 c = radiance[(size_t)sidx * npix + pix];
        colors = colors + mk(c.x, c.y, c.z);
    }
    const v3 fin = colors / (float)spp;
    if (frame_count <= 0) {
        accum[pix] = make_float4(fin.x, fin.y, fin.z, 1.0f);
        sum64[pix] = make_dbl4(fin.x, fin.y, fin.z, 1.0);
    } else {
        const float4 old = accum[pix];
        const float a = 1.0f / (float)(frame_count + 1);
        // mix(x, y, a) = x * (1 - a) + y * a
        accum[pix] = make_float4(old.x * (1.0f - a) + fin.x * a, old.y * (1.0f - a) + fin.y * a,
                                 old.z * (1.0f - a) + fin.z * a, 1.0f);
        const dbl4 s = sum64[pix];
        sum64[pix] = make_dbl4(s.x + fin.x, s.y + fin.y, s.z + fin.z, s.w + 1.0);
    }
}

__constant__ float c_srgb_thresh[256];

__device__ __forceinline__ unsigned char srgb8(float v) {
    if (!(v > 0.0f)) return 0;
    int lo = 0;
#pragma unroll
    for (int step = 128; step >= 1; step >>= 1)
        if (c_srgb_thresh[lo + step] <= v) lo += step;
    return (unsigned char)lo;
}

// Linear RGBA32F -> B8G8R8A8 sRGB (config.hpp:144, PostProcessing.frag:11-17).
__global__ void k_srgb(const float4* __restrict__ img, uint32_t npix, uchar4* out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npix) return;
    const float4 c = img[i];
    out[i] = make_uchar4(srgb8(c.z), srgb8(c.y), srgb8(c.x), 255);
}

// FP64 relative MSE: sum over rgb of (x - r)^2 / (r^2 + eps), per-block partials then one final block.
__global__ void k_relmse_partial(const float4* __restrict__ x, const float4* __restrict__ ref, uint64_t n, double eps,
                                 double* partial) {
    double acc = 0.0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const float4 a = x[i], b = ref[i];
        const double d0 = (double)a.x - b.x, d1 = (double)a.y - b.y, d2 = (double)a.z - b.z;
        acc += d0 * d0 / ((double)b.x * b.x + eps) + d1 * d1 / ((double)b.y * b.y + eps) +
               d2 * d2 / ((double)b.z * b.z + eps);
    }
    __shared__ double sm[256];
    sm[threadIdx.x] = acc;
    __syncthreads();
    for (int off = blockDim.x / 2; off; off >>= 1) {
        if ((int)threadIdx.x < off) sm[threadIdx.x] += sm[threadIdx.x + off];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = sm[0];
}
__global__ void k_relmse_final(const double* partial, uint32_t blocks, uint64_t n, double* out) {
    __shared__ double sm[256];
    double acc = 0.0;
    for (uint32_t i = threadIdx.x; i < blocks; i += blockDim.x) acc += partial[i];
    sm[threadIdx.x] = acc;
    __syncthreads();
    for (int off = blockDim.x / 2; off; off >>= 1) {
        if ((int)threadIdx.x < off) sm[threadIdx.x] += sm[threadIdx.x + off];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = sm[0] / (3.0 * (double)n);
}

} // namespace

void launch_raygen(const FrameDev* f, const BatchDev& b, const WaveDev& w, uint64_t chunk_start, uint32_t chunk_n,
                   cudaStream_t st) {
    const unsigned grid = (chunk_n + 255) / 256;
    if (b.items)
        k_raygen<true><<<grid, 256, 0, st>>>(f, b, w, chunk_start, chunk_n);
    else
        k_raygen<false><<<grid, 256, 0, st>>>(f, b, w, chunk_start, chunk_n);
    KF_CUDA_CHECK(cudaGetLastError());
}
void launch_extend(const SceneDev& s, const FrameDev* f, const BatchDev& b, const WaveDev& w, int cur,
                   uint32_t depth, uint64_t chunk_start, uint32_t grid, bool count_mode, cudaStream_t st) {
    if (b.items) {
        if (count_mode)
            k_extend<true, true><<<grid, 128, 0, st>>>(s, f, b, w, cur, depth, chunk_start);
        else
            k_extend<false, true><<<grid, 128, 0, st>>>(s, f, b, w, cur, depth, chunk_start);
    } else {
        if (count_mode)
            k_extend<true, false><<<grid, 128, 0, st>>>(s, f, b, w, cur, depth, chunk_start);
        else
            k_extend<false, false><<<grid, 128, 0, st>>>(s, f, b, w, cur, depth, chunk_start);
    }
    KF_CUDA_CHECK(cudaGetLastError());
}
void launch_shade(const SceneDev& s, const FrameDev* f, const BatchDev& b, const WaveDev& w, int cur,
                  uint32_t depth, uint64_t chunk_start, uint32_t grid, cudaStream_t st) {
    if (b.items)
        k_shade<true><<<grid, kShadeThreads, 0, st>>>(s, f, b, w, cur, depth, chunk_start);
    else
        k_shade<false><<<grid, kShadeThreads, 0, st>>>(s, f, b, w, cur, depth, chunk_start);
    KF_CUDA_CHECK(cudaGetLastError());
}
void launch_miss(const SceneDev& s, const FrameDev* f, const BatchDev& b, const WaveDev& w, int cur,
                 uint32_t depth, uint64_t chunk_start, uint32_t grid, cudaStream_t st) {
    if (b.items)
        k_miss<true><<<grid, kMissThreads, 0, st>>>(s, f, b, w, cur, depth, chunk_start);
    else
        k_miss<false><<<grid, kMissThreads, 0, st>>>(s, f, b, w, cur, depth, chunk_start);
    KF_CUDA_CHECK(cudaGetLastError());
}
void launch_nee(const SceneDev& s, const FrameDev* f, const BatchDev& b, const WaveDev& w, uint32_t depth,
                uint64_t chunk_start, uint32_t grid, cudaStream_t st) {
    if (b.items)
        k_nee<true><<<grid, kShadeThreads, 0, st>>>(s, f, b, w, depth, chunk_start);
    else
        k_nee<false><<<grid, kShadeThreads, 0, st>>>(s, f, b, w, depth, chunk_start);
    KF_CUDA_CHECK(cudaGetLastError());
}
void launch_shadow(const SceneDev& s, const BatchDev& b, const WaveDev& w, uint32_t grid, bool count_mode,
                   cudaStream_t st) {
    if (b.items) {
        if (count_mode)
            k_shadow<true, true><<<grid, 128, 0, st>>>(s, b, w);
        else
            k_shadow<false, true><<<grid, 128, 0, st>>>(s, b, w);
    } else {
        if (count_mode)
            k_shadow<true, false><<<grid, 128, 0, st>>>(s, b, w);
        else
            k_shadow<false, false><<<grid, 128, 0, st>>>(s, b, w);
    }
    KF_CUDA_CHECK(cudaGetLastError());
}

template <bool BATCH>
static void trace_dyn_dispatch(const SceneDev& s, const FrameDev* f, const BatchDev& b, const WaveDev& w, int cur,
                               uint32_t depth, uint64_t chunk_start, bool shadow, uint32_t grid, bool count_mode,
                               uint32_t rb, int ns, cudaStream_t st) {
    if (shadow) {
        if (count_mode)
            k_trace_dyn<true, true, BATCH><<<grid, 128, 0, st>>>(s, f, b, w, cur, depth, chunk_start, rb, ns);
        else
            k_trace_dyn<true, false, BATCH><<<grid, 128, 0, st>>>(s, f, b, w, cur, depth, chunk_start, rb, ns);
    } else {
        if (count_mode)
            k_trace_dyn<false, true, BATCH><<<grid, 128, 0, st>>>(s, f, b, w, cur, depth, chunk_start, rb, ns);
        else
            k_trace_dyn<false, false, BATCH><<<grid, 128, 0, st>>>(s, f, b, w, cur, depth, chunk_start, rb, ns);
    }
}
void launch_trace_dyn(const SceneDev& s, const FrameDev* f, const BatchDev& b, const WaveDev& w, int cur,
                      uint32_t depth, uint64_t chunk_start, bool shadow, uint32_t grid, bool count_mode,
                      uint32_t refill_below, uint32_t steps, cudaStream_t st) {
    const uint32_t rb = std::min(std::max(refill_below, 1u), 32u);
    const int ns = (int)std::min(std::max(steps, 1u), 64u);
    if (b.items)
        trace_dyn_dispatch<true>(s, f, b, w, cur, depth, chunk_start, shadow, grid, count_mode, rb, ns, st);
    else
        trace_dyn_dispatch<false>(s, f, b, w, cur, depth, chunk_start, shadow, grid, count_mode, rb, ns, st);
    KF_CUDA_CHECK(cudaGetLastError());
}

uint32_t trace_dyn_blocks_per_sm(bool shadow) {
    int a = 0;
    if (shadow)
        KF_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_trace_dyn<true, false, false>, 128, 0));
    else
        KF_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_trace_dyn<false, false, false>, 128, 0));
    return (uint32_t)std::max(1, a);
}

void launch_gather(const SceneDev& s, const BatchDev& b, const WaveDev& w, int cur, uint64_t chunk_start,
                   uint32_t grid, cudaStream_t st) {
    if (b.items)
        k_gather<true><<<grid, 256, 0, st>>>(s, b, w, cur, chunk_start);
    else
        k_gather<false><<<grid, 256, 0, st>>>(s, b, w, cur, chunk_start);
    KF_CUDA_CHECK(cudaGetLastError());
}
void launch_resolve(const FrameDev* f, const float4* radiance, uint32_t npix, uint32_t spp, float4* accum,
                    dbl4* sum64, cudaStream_t st) {
    k_resolve<<<(npix + 255) / 256, 256, 0, st>>>(f, radiance, npix, spp, accum, sum64);
    KF_CUDA_CHECK(cudaGetLastError());
}
void launch_srgb(const float4* img, uint32_t npix, uchar4* out, cudaStream_t st) {
    k_srgb<<<(npix + 255) / 256, 256, 0, st>>>(img, npix, out);
    KF_CUDA_CHECK(cudaGetLastError());
}
void upload_srgb_thresholds(const float* thresh256) {
    KF_CUDA_CHECK(cudaMemcpyToSymbol(c_srgb_thresh, thresh256, sizeof(float) * 256));
}
void launch_relmse(const float4* x, const float4* ref, uint64_t n, double eps, double* partial, uint32_t blocks,
                   double* out, cudaStream_t st) {
    k_relmse_partial<<<blocks, 256, 0, st>>>(x, ref, n, eps, partial);
    k_relmse_final<<<1, 256, 0, st>>>(partial, blocks, n, out);
    KF_CUDA_CHECK(cudaGetLastError());
}

} // namespace kf

// ---------------------------------------------------------------------------
// kf_relmse_noalloc: the relative-MSE reduction for callers that cannot call
// cudaMalloc (an embedding application whose device memory belongs to its own
// pool allocator, or a frame loop that must not take the implicit device-wide
// synchronisation of cudaMalloc / cudaFree). The per-block FP64 partials live
// in this file-scope device array instead of allocated scratch. Every GPU that
// loads the library holds it (32 KiB + 8 B) until the process exits.
// ---------------------------------------------------------------------------
namespace {
constexpr uint32_t kNoAllocMaxBlocks = 4096;
constexpr uint64_t kNoAllocMaxPixels = 268435456ull; // 2^28: the stated per-call limit
static __device__ __align__(256) double g_relmse_scratch[kNoAllocMaxBlocks + 1];
} // namespace

namespace kf {
void set_last_error(const std::string& msg);
}

extern "C" KF_API int kf_relmse_noalloc(const float* x_dev, const float* ref_dev, uint64_t num_pixels, double eps,
                                        void* stream, double* out) {
    if (!x_dev || !ref_dev || !out || num_pixels == 0) {
        kf::set_last_error("kf_relmse_noalloc: null pointer or zero pixels");
        return KF_ERR_INVALID_ARGUMENT;
    }
    if (((uintptr_t)x_dev & 15) != 0 || ((uintptr_t)ref_dev & 15) != 0) { // float4 pixel loads
        kf::set_last_error("kf_relmse_noalloc: images must be 16-byte aligned");
        return KF_ERR_INVALID_ARGUMENT;
    }
    if (num_pixels > kNoAllocMaxPixels) {
        kf::set_last_error("kf_relmse_noalloc: more than 268435456 pixels per call exceed the limit of its static "
                           "scratch; use kf_relmse");
        return KF_ERR_LIMIT;
    }
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) {
        kf::set_last_error("kf_relmse_noalloc: no current CUDA device");
        return KF_ERR_NO_DEVICE;
    }
    // The host-side name of the array is not a device address: ask the runtime for the
    // address on the current device, on every call (it is cheap beside the launches and
    // the synchronisation, and stays right if the device's context was re-created). The
    // first call on a device loads the module there.
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_relmse_scratch);
    if (e != cudaSuccess || !p) {
        kf::set_last_error(std::string("kf_relmse_noalloc: cudaGetSymbolAddress failed: ") + cudaGetErrorString(e));
        return KF_ERR_CUDA;
    }
    double* scratch = static_cast<double*>(p);
    // k_relmse_partial is a grid-stride loop: 4 blocks per SM fill the GPU, at most one
    // block per 256 pixels, and never more blocks than the array holds partials
    const uint64_t want = std::min<uint64_t>((num_pixels + 255) / 256, (uint64_t)sms * 4);
    const uint32_t blocks = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(want, kNoAllocMaxBlocks));
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // every partial in [0, blocks) and the result slot are written before they are read,
    // so nothing needs clearing between calls
    kf::k_relmse_partial<<<blocks, 256, 0, st>>>(reinterpret_cast<const float4*>(x_dev),
                                                  reinterpret_cast<const float4*>(ref_dev), num_pixels, eps,
                                                  scratch);
    kf::k_relmse_final<<<1, 256, 0, st>>>(scratch, blocks, num_pixels, scratch + kNoAllocMaxBlocks);
    e = cudaGetLastError();
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(out, scratch + kNoAllocMaxBlocks, sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        kf::set_last_error(std::string("kf_relmse_noalloc: ") + cudaGetErrorString(e));
        return KF_ERR_CUDA;
    }
    return KF_OK;
}
