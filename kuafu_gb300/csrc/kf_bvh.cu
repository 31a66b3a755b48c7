// kf_bvh.cu — GPU construction of the acceleration structures that replace
// kuafu's driver-built BLAS/TLAS (src/core/rt/rt.cpp:142-495).
//
// Pipeline per structure (one BLAS per geometry, one TLAS over instances):
//   1. centroid bounds        (block reduction)
//   2. 30-bit Morton codes    (Karras, "Maximizing Parallelism in the
//                              Construction of BVHs, Octrees, and k-d Trees", HPG 2012)
//   3. stable LSD radix sort  (8-bit digits, per-tile histograms + one scan)
//   4. binary radix tree      (Karras 2012: one thread per internal node)
//   5. bottom-up AABB refit   (atomic arrival counters, second child proceeds)
//   6. BVH2 -> BVH4 collapse  (top-down, expand the child of largest surface
//                              area until four children; small subtrees become
//                              leaves over contiguous primitive ranges)
// Leaves address contiguous ranges of the Morton-sorted primitive order, so the
// caller reorders primitive payloads once (triangles / instance ids).
//
// Alternative to steps 4-5 (bvh_builder = 2): PLOC, parallel locally-ordered clustering
// (Meister and Bittner, "Parallel Locally-Ordered Clustering for Bounding Volume Hierarchy
// Construction", TVCG 2018). The clusters start as the Morton-sorted primitives; in every
// round each cluster finds, among the clusters at most `radius` positions away in the
// array, the one whose merged box has the smallest surface area; pairs that chose each
// other merge into a new node; the array is compacted in order. Ties are broken by the
// pair's positions, so the globally best pair always chooses itself and every round
// merges. The leaves are then numbered in depth-first order, which makes every subtree a
// contiguous primitive range for step 6.
#include "kf_bvh.h"

#include <algorithm>
#include <array>
#include <cstdlib>
#include <cstdio>
#include <vector>

#include "kf_device.cuh"
#include "kf_util.h"

namespace kf {

namespace {

constexpr int kSortThreads = 256;
constexpr int kSortItems = 8;
constexpr int kSortTile = kSortThreads * kSortItems;

__device__ __forceinline__ uint32_t expand_bits10(uint32_t v) {
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

__device__ __forceinline__ void atomic_min_f(float* addr, float v) {
    if (v >= 0.0f)
        atomicMin(reinterpret_cast<int*>(addr), __float_as_int(v));
    else
        atomicMax(reinterpret_cast<unsigned int*>(addr), __float_as_uint(v));
}
__device__ __forceinline__ void atomic_max_f(float* addr, float v) {
    if (v >= 0.0f)
        atomicMax(reinterpret_cast<int*>(addr), __float_as_int(v));
    else
        atomicMin(reinterpret_cast<unsigned int*>(addr), __float_as_uint(v));
}

// Centroid bounds: bounds[0..2] = min, bounds[3..5] = max (initialised by the caller).
__global__ void k_centroid_bounds(const float4* __restrict__ lo, const float4* __restrict__ hi, int n,
                                  float* bounds) {
    float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 a = lo[i], b = hi[i];
        const float c[3] = {(a.x + b.x) * 0.5f, (a.y + b.y) * 0.5f, (a.z + b.z) * 0.5f};
        for (int k = 0; k < 3; ++k) {
            mn[k] = fminf(mn[k], c[k]);
            mx[k] = fmaxf(mx[k], c[k]);
        }
    }
    for (int k = 0; k < 3; ++k) {
        for (int off = 16; off; off >>= 1) {
            mn[k] = fminf(mn[k], __shfl_xor_sync(0xFFFFFFFFu, mn[k], off));
            mx[k] = fmaxf(mx[k], __shfl_xor_sync(0xFFFFFFFFu, mx[k], off));
        }
    }
    if ((threadIdx.x & 31) == 0) {
        for (int k = 0; k < 3; ++k) {
            atomic_min_f(&bounds[k], mn[k]);
            atomic_max_f(&bounds[3 + k], mx[k]);
        }
    }
}

__global__ void k_morton(const float4* __restrict__ lo, const float4* __restrict__ hi, int n,
                         const float* __restrict__ bounds, uint32_t* keys, uint32_t* vals) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 a = lo[i], b = hi[i];
    const float c[3] = {(a.x + b.x) * 0.5f, (a.y + b.y) * 0.5f, (a.z + b.z) * 0.5f};
    uint32_t q[3];
    for (int k = 0; k < 3; ++k) {
        const float ext = bounds[3 + k] - bounds[k];
        float u = ext > 0.0f ? (c[k] - bounds[k]) / ext : 0.0f;
        u = fminf(fmaxf(u * 1024.0f, 0.0f), 1023.0f);
        q[k] = (uint32_t)u;
    }
    keys[i] = expand_bits10(q[0]) * 4u + expand_bits10(q[1]) * 2u + expand_bits10(q[2]);
    vals[i] = (uint32_t)i;
}

// ---- stable LSD radix sort (8-bit digits) ----
__global__ void k_sort_hist(const uint32_t* __restrict__ keys, int n, int shift, int num_tiles, uint32_t* counts) {
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const int base = blockIdx.x * kSortTile;
    for (int r = 0; r < kSortItems; ++r) {
        const int i = base + r * kSortThreads + threadIdx.x;
        if (i < n) atomicAdd(&h[(keys[i] >> shift) & 0xFFu], 1u);
    }
    __syncthreads();
    counts[threadIdx.x * num_tiles + blockIdx.x] = h[threadIdx.x];
}

// Exclusive scan of `m` counters in one block of 1024 threads.
__global__ void k_sort_scan(uint32_t* counts, int m) {
    __shared__ uint32_t part[1024];
    const int per = (m + 1023) / 1024;
    const int b = threadIdx.x * per;
    uint32_t s = 0;
    for (int k = 0; k < per; ++k)
        if (b + k < m) s += counts[b + k];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
        uint32_t v = threadIdx.x >= (unsigned)off ? part[threadIdx.x - off] : 0u;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    uint32_t run = threadIdx.x ? part[threadIdx.x - 1] : 0u;
    for (int k = 0; k < per; ++k)
        if (b + k < m) {
            const uint32_t c = counts[b + k];
            counts[b + k] = run;
            run += c;
        }
}

__global__ void k_sort_scatter(const uint32_t* __restrict__ keys_in, const uint32_t* __restrict__ vals_in,
                               uint32_t* keys_out, uint32_t* vals_out, int n, int shift, int num_tiles,
                               const uint32_t* __restrict__ offsets) {
    __shared__ uint32_t wcount[kSortThreads / 32][256];
    __shared__ uint32_t running[256];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    running[threadIdx.x] = offsets[threadIdx.x * num_tiles + blockIdx.x];
    const int base = blockIdx.x * kSortTile;
    const uint32_t lt = (1u << lane) - 1u;
    for (int r = 0; r < kSortItems; ++r) {
        for (int w = 0; w < kSortThreads / 32; ++w) wcount[w][threadIdx.x] = 0;
        __syncthreads();
        const int i = base + r * kSortThreads + threadIdx.x;
        const bool valid = i < n;
        uint32_t key = 0, val = 0, d = 256;
        if (valid) {
            key = keys_in[i];
            val = vals_in[i];
            d = (key >> shift) & 0xFFu;
        }
        const uint32_t peers = __match_any_sync(0xFFFFFFFFu, d);
        const uint32_t rank = __popc(peers & lt);
        if (valid && rank == 0) wcount[warp][d] = __popc(peers);
        __syncthreads();
        {
            uint32_t run = running[threadIdx.x];
            for (int w = 0; w < kSortThreads / 32; ++w) {
                const uint32_t c = wcount[w][threadIdx.x];
                wcount[w][threadIdx.x] = run;
                run += c;
            }
            running[threadIdx.x] = run;
        }
        __syncthreads();
        if (valid) {
            const uint32_t pos = wcount[warp][d] + rank;
            keys_out[pos] = key;
            vals_out[pos] = val;
        }
        __syncthreads();
    }
}

// ---- Karras 2012 binary radix tree ----
__device__ __forceinline__ int delta(const uint32_t* keys, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    const uint32_t a = keys[i], b = keys[j];
    if (a == b) return 32 + __clz((uint32_t)(i ^ j));
    return __clz(a ^ b);
}

// Node indexing: internal nodes 0..n-2, leaf i at (n-1)+i.
__global__ void k_karras(const uint32_t* __restrict__ keys, int n, int* left, int* right, int* parent, int2* range) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    const int d = (delta(keys, n, i, i + 1) - delta(keys, n, i, i - 1)) >= 0 ? 1 : -1;
    const int dmin = delta(keys, n, i, i - d);
    int lmax = 2;
    while (delta(keys, n, i, i + lmax * d) > dmin) lmax <<= 1;
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
        if (delta(keys, n, i, i + (l + t) * d) > dmin) l += t;
    const int j = i + l * d;
    const int dnode = delta(keys, n, i, j);
    int s = 0;
    int t = l;
    do {
        t = (t + 1) >> 1;
        if (delta(keys, n, i, i + (s + t) * d) > dnode) s += t;
    } while (t > 1);
    const int gamma = i + s * d + min(d, 0);
    const int lo = min(i, j), hi = max(i, j);
    const int lc = (lo == gamma) ? (n - 1) + gamma : gamma;
    const int rc = (hi == gamma + 1) ? (n - 1) + gamma + 1 : gamma + 1;
    left[i] = lc;
    right[i] = rc;
    range[i] = make_int2(lo, hi);
    parent[lc] = i;
    parent[rc] = i;
    if (i == 0) parent[0] = -1;
}

__global__ void k_leaf_boxes(const float4* __restrict__ lo, const float4* __restrict__ hi,
                             const uint32_t* __restrict__ order, int n, float4* blo, float4* bhi) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t p = order[i];
    blo[(n - 1) + i] = lo[p];
    bhi[(n - 1) + i] = hi[p];
}

__global__ void k_refit(int n, const int* __restrict__ left, const int* __restrict__ right,
                        const int* __restrict__ parent, float4* blo, float4* bhi, int* flags) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int node = parent[(n - 1) + i];
    while (node >= 0) {
        __threadfence();
        if (atomicAdd(&flags[node], 1) == 0) return;
        __threadfence();
        const int l = left[node], r = right[node];
        const float4 al = __ldcg(&blo[l]), ah = __ldcg(&bhi[l]);
        const float4 bl = __ldcg(&blo[r]), bh = __ldcg(&bhi[r]);
        __stcg(&blo[node], make_float4(fminf(al.x, bl.x), fminf(al.y, bl.y), fminf(al.z, bl.z), 0.0f));
        __stcg(&bhi[node], make_float4(fmaxf(ah.x, bh.x), fmaxf(ah.y, bh.y), fmaxf(ah.z, bh.z), 0.0f));
        node = parent[node];
    }
}

__device__ __forceinline__ float surface_area(float4 lo, float4 hi) {
    const float dx = hi.x - lo.x, dy = hi.y - lo.y, dz = hi.z - lo.z;
    return dx * dy + dy * dz + dz * dx;
}

__device__ __forceinline__ int range_size(int node, int n, const int2* range) {
    if (node >= n - 1) return 1;
    const int2 r = range[node];
    return r.y - r.x + 1;
}
__device__ __forceinline__ int range_first(int node, int n, const int2* range) {
    if (node >= n - 1) return node - (n - 1);
    return range[node].x;
}

// Collapse one level of the frontier: item k turns BVH2 node `src[k]` into
// BVH4 node `dst[k]`.
__global__ void k_collapse(int n, int max_leaf, const int* __restrict__ left, const int* __restrict__ right,
                           const int2* __restrict__ range, const float4* __restrict__ blo,
                           const float4* __restrict__ bhi, const int* __restrict__ src, const int* __restrict__ dst,
                           int count, int* next_src, int* next_dst, int* next_count, int* node_count, Node4* out) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    const int s = src[k];
    int ch[4];
    int nc = 2;
    ch[0] = left[s];
    ch[1] = right[s];
    while (nc < 4) {
        int best = -1;
        float best_sa = -1.0f;
        for (int c = 0; c < nc; ++c) {
            const int node = ch[c];
            if (node >= n - 1 || range_size(node, n, range) <= max_leaf) continue;
            const float sa = surface_area(blo[node], bhi[node]);
            if (sa > best_sa) {
                best_sa = sa;
                best = c;
            }
        }
        if (best < 0) break;
        const int node = ch[best];
        ch[best] = left[node];
        ch[nc++] = right[node];
    }
    Node4 o;
    float lx[4], hx[4], ly[4], hy[4], lz[4], hz[4];
    int cc[4], cn[4];
    for (int c = 0; c < 4; ++c) {
        if (c >= nc) {
            lx[c] = ly[c] = lz[c] = INFINITY;
            hx[c] = hy[c] = hz[c] = -INFINITY;
            cc[c] = 0;
            cn[c] = -1;
            continue;
        }
        const int node = ch[c];
        const float4 a = blo[node], b = bhi[node];
        lx[c] = a.x; ly[c] = a.y; lz[c] = a.z;
        hx[c] = b.x; hy[c] = b.y; hz[c] = b.z;
        const int rs = range_size(node, n, range);
        if (node >= n - 1 || rs <= max_leaf) {
            cc[c] = leaf_child(range_first(node, n, range), rs);
            cn[c] = rs;
        } else {
            const int slot = atomicAdd(node_count, 1);
            const int q = atomicAdd(next_count, 1);
            next_src[q] = node;
            next_dst[q] = slot;
            cc[c] = slot;
            cn[c] = 0;
        }
    }
    o.lox = make_float4(lx[0], lx[1], lx[2], lx[3]);
    o.hix = make_float4(hx[0], hx[1], hx[2], hx[3]);
    o.loy = make_float4(ly[0], ly[1], ly[2], ly[3]);
    o.hiy = make_float4(hy[0], hy[1], hy[2], hy[3]);
    o.loz = make_float4(lz[0], lz[1], lz[2], lz[3]);
    o.hiz = make_float4(hz[0], hz[1], hz[2], hz[3]);
    o.child = make_int4(cc[0], cc[1], cc[2], cc[3]);
    o.cnt = make_int4(cn[0], cn[1], cn[2], cn[3]);
    out[dst[k]] = o;
}

// A structure whose primitives all fit one leaf: a single node with one leaf child.
__global__ void k_single_leaf(const float4* __restrict__ lo, const float4* __restrict__ hi, int n, Node4* out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    float4 a = make_float4(INFINITY, INFINITY, INFINITY, 0.0f), b = make_float4(-INFINITY, -INFINITY, -INFINITY, 0.0f);
    for (int i = 0; i < n; ++i) {
        a.x = fminf(a.x, lo[i].x); a.y = fminf(a.y, lo[i].y); a.z = fminf(a.z, lo[i].z);
        b.x = fmaxf(b.x, hi[i].x); b.y = fmaxf(b.y, hi[i].y); b.z = fmaxf(b.z, hi[i].z);
    }
    Node4 o;
    o.lox = make_float4(a.x, INFINITY, INFINITY, INFINITY);
    o.hix = make_float4(b.x, -INFINITY, -INFINITY, -INFINITY);
    o.loy = make_float4(a.y, INFINITY, INFINITY, INFINITY);
    o.hiy = make_float4(b.y, -INFINITY, -INFINITY, -INFINITY);
    o.loz = make_float4(a.z, INFINITY, INFINITY, INFINITY);
    o.hiz = make_float4(b.z, -INFINITY, -INFINITY, -INFINITY);
    o.child = make_int4(leaf_child(0, n), 0, 0, 0);
    o.cnt = make_int4(n, -1, -1, -1);
    out[0] = o;
}

__global__ void k_identity(uint32_t* order, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) order[i] = (uint32_t)i;
}

// ---- PLOC rounds ----
// nn[i] = the position j != i within `radius` of i whose cluster merged with cl[i] has the
// smallest surface area. Ties (coincident boxes) go to the nearer position, then to the
// pair starting at an even position, then to the lower pair: a total order on pairs that
// both ends share, so the best pair always chooses itself, and runs of equal clusters pair
// off as (2k, 2k + 1) and halve in one round.
__global__ void k_ploc_nn(const int* __restrict__ cl, int m, const float4* __restrict__ blo,
                          const float4* __restrict__ bhi, int radius, int* nn) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    const int ci = cl[i];
    const float4 a0 = blo[ci], a1 = bhi[ci];
    float best = INFINITY;
    int bj = -1, bd = 0x7FFFFFFF, bodd = 2, bl = 0x7FFFFFFF;
    const int j0 = max(0, i - radius), j1 = min(m - 1, i + radius);
    for (int j = j0; j <= j1; ++j) {
        if (j == i) continue;
        const int cj = cl[j];
        const float4 b0 = blo[cj], b1 = bhi[cj];
        const float4 lo = make_float4(fminf(a0.x, b0.x), fminf(a0.y, b0.y), fminf(a0.z, b0.z), 0.0f);
        const float4 hi = make_float4(fmaxf(a1.x, b1.x), fmaxf(a1.y, b1.y), fmaxf(a1.z, b1.z), 0.0f);
        const float sa = surface_area(lo, hi);
        const int l = min(i, j), d = abs(i - j), odd = l & 1;
        if (sa < best ||
            (sa == best && (d < bd || (d == bd && (odd < bodd || (odd == bodd && l < bl)))))) {
            best = sa;
            bj = j;
            bd = d;
            bodd = odd;
            bl = l;
        }
    }
    nn[i] = bj;
}

// Fallback rounds (inputs on which the greedy rounds stall): neighbours (2k, 2k + 1) pair up.
__global__ void k_ploc_pairs(int m, int* nn) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    const int j = i ^ 1;
    nn[i] = j < m ? j : -1;
}

// Mutual nearest neighbours merge: the lower position makes internal node
// (n - 2 - k) for the k-th merge (the root, made last, gets node 0; children always have
// larger indices than their parent) and keeps it; the higher one drops out.
__global__ void k_ploc_merge(int* cl, int m, const int* __restrict__ nn, int n, int* left, int* right, float4* blo,
                             float4* bhi, int* merges, uint32_t* keep, uint32_t* offs) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    const int j = nn[i];
    uint32_t k = 1;
    if (j >= 0 && nn[j] == i) {
        if (i < j) {
            const int id = (n - 2) - atomicAdd(merges, 1);
            const int a = cl[i], b = cl[j];
            left[id] = a;
            right[id] = b;
            const float4 a0 = blo[a], a1 = bhi[a], b0 = blo[b], b1 = bhi[b];
            blo[id] = make_float4(fminf(a0.x, b0.x), fminf(a0.y, b0.y), fminf(a0.z, b0.z), 0.0f);
            bhi[id] = make_float4(fmaxf(a1.x, b1.x), fmaxf(a1.y, b1.y), fmaxf(a1.z, b1.z), 0.0f);
            cl[i] = id;
        } else {
            k = 0;
        }
    }
    keep[i] = k;
    offs[i] = k;
}

// cl_out[offs[i]] = cl[i] for the kept clusters (offs: exclusive scan of keep)
__global__ void k_ploc_compact(const int* __restrict__ cl, int m, const uint32_t* __restrict__ keep,
                               const uint32_t* __restrict__ offs, int* cl_out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < m && keep[i]) cl_out[offs[i]] = cl[i];
}

__global__ void k_iota_leaves(int* cl, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) cl[i] = (n - 1) + i;
}

} // namespace

void radix_sort_pairs(uint32_t* keys, uint32_t* vals, uint32_t* keys_tmp, uint32_t* vals_tmp, uint32_t* counts,
                      int n, int bits, cudaStream_t st) {
    if (n <= 1) return;
    const int tiles = (n + kSortTile - 1) / kSortTile;
    uint32_t *ki = keys, *vi = vals, *ko = keys_tmp, *vo = vals_tmp;
    int passes = 0;
    for (int shift = 0; shift < bits; shift += 8) {
        k_sort_hist<<<tiles, kSortThreads, 0, st>>>(ki, n, shift, tiles, counts);
        k_sort_scan<<<1, 1024, 0, st>>>(counts, 256 * tiles);
        k_sort_scatter<<<tiles, kSortThreads, 0, st>>>(ki, vi, ko, vo, n, shift, tiles, counts);
        std::swap(ki, ko);
        std::swap(vi, vo);
        ++passes;
    }
    if (passes & 1) {
        KF_CUDA_CHECK(cudaMemcpyAsync(keys, ki, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, st));
        KF_CUDA_CHECK(cudaMemcpyAsync(vals, vi, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, st));
    }
}

size_t radix_sort_count_words(int n) {
    const int tiles = (n + kSortTile - 1) / kSortTile;
    return (size_t)256 * std::max(tiles, 1);
}

// PLOC binary tree over the n Morton-sorted primitives (order: sorted primitive ids, on
// return in depth-first leaf order): internal nodes 0..n-2 (root 0), leaf p at (n-1)+p
// for position p of `order`, range[] the contiguous leaf positions of every internal node,
// boxes of all 2n-1 nodes in blo / bhi. Same layout as the Karras path.
static void ploc_tree(const float4* plo, const float4* phi, int n, uint32_t* order, int* left, int* right,
                      int2* range, float4* blo, float4* bhi, cudaStream_t st) {
    constexpr int kRadius = 16;
    const int tb = 256;
    TempAlloc arena(st);
    int* cl = arena.alloc<int>(n);
    int* cl2 = arena.alloc<int>(n);
    int* nn = arena.alloc<int>(n);
    uint32_t* keep = arena.alloc<uint32_t>(n);
    uint32_t* offs = arena.alloc<uint32_t>(n);
    int* merges = arena.alloc<int>(1);
    k_leaf_boxes<<<(n + tb - 1) / tb, tb, 0, st>>>(plo, phi, order, n, blo, bhi);
    k_iota_leaves<<<(n + tb - 1) / tb, tb, 0, st>>>(cl, n);
    KF_CUDA_CHECK(cudaMemsetAsync(merges, 0, sizeof(int), st));
    // greedy rounds reduce the clusters by about a third each; after kGreedyRounds the
    // rest pair up in order, which halves them every round and ends on any input
    constexpr int kGreedyRounds = 64;
    int m = n, rounds = 0;
    while (m > 1) {
        KF_REQUIRE(++rounds <= kGreedyRounds + 40, KF_ERR_INTERNAL, "PLOC clustering did not converge");
        const unsigned g = (unsigned)((m + tb - 1) / tb);
        if (rounds <= kGreedyRounds)
            k_ploc_nn<<<g, tb, 0, st>>>(cl, m, blo, bhi, kRadius, nn);
        else
            k_ploc_pairs<<<g, tb, 0, st>>>(m, nn);
        k_ploc_merge<<<g, tb, 0, st>>>(cl, m, nn, n, left, right, blo, bhi, merges, keep, offs);
        k_sort_scan<<<1, 1024, 0, st>>>(offs, m);
        k_ploc_compact<<<g, tb, 0, st>>>(cl, m, keep, offs, cl2);
        KF_CUDA_CHECK(cudaGetLastError());
        uint32_t last[2];
        KF_CUDA_CHECK(cudaMemcpyAsync(&last[0], offs + (m - 1), sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        KF_CUDA_CHECK(cudaMemcpyAsync(&last[1], keep + (m - 1), sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        KF_CUDA_CHECK(cudaStreamSynchronize(st));
        const int m2 = (int)(last[0] + last[1]);
        KF_REQUIRE(m2 < m, KF_ERR_INTERNAL, "PLOC round without a merge");
        m = m2;
        std::swap(cl, cl2);
    }
    // depth-first leaf numbering on the host: leaf counts bottom-up (children have larger
    // indices than their parent), first positions top-down
    std::vector<int> hl(n - 1), hr(n - 1);
    std::vector<uint32_t> ho(n);
    KF_CUDA_CHECK(cudaMemcpyAsync(hl.data(), left, sizeof(int) * (n - 1), cudaMemcpyDeviceToHost, st));
    KF_CUDA_CHECK(cudaMemcpyAsync(hr.data(), right, sizeof(int) * (n - 1), cudaMemcpyDeviceToHost, st));
    KF_CUDA_CHECK(cudaMemcpyAsync(ho.data(), order, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, st));
    KF_CUDA_CHECK(cudaStreamSynchronize(st));
    auto count = [&](int node, const std::vector<int>& cnt) { return node >= n - 1 ? 1 : cnt[node]; };
    std::vector<int> cnt(n - 1), first(2 * n - 1);
    for (int id = n - 2; id >= 0; --id) cnt[id] = count(hl[id], cnt) + count(hr[id], cnt);
    first[0] = 0;
    for (int id = 0; id < n - 1; ++id) {
        first[hl[id]] = first[id];
        first[hr[id]] = first[id] + count(hl[id], cnt);
    }
    std::vector<int2> hrange(n - 1);
    std::vector<uint32_t> new_order(n);
    auto leaf_id = [&](int node) { return node >= n - 1 ? (n - 1) + first[node] : node; };
    for (int id = 0; id < n - 1; ++id) {
        hrange[id] = make_int2(first[id], first[id] + cnt[id] - 1);
        for (int c : {hl[id], hr[id]})
            if (c >= n - 1) new_order[first[c]] = ho[c - (n - 1)];
        hl[id] = leaf_id(hl[id]);
        hr[id] = leaf_id(hr[id]);
    }
    KF_CUDA_CHECK(cudaMemcpyAsync(left, hl.data(), sizeof(int) * (n - 1), cudaMemcpyHostToDevice, st));
    KF_CUDA_CHECK(cudaMemcpyAsync(right, hr.data(), sizeof(int) * (n - 1), cudaMemcpyHostToDevice, st));
    KF_CUDA_CHECK(cudaMemcpyAsync(range, hrange.data(), sizeof(int2) * (n - 1), cudaMemcpyHostToDevice, st));
    KF_CUDA_CHECK(cudaMemcpyAsync(order, new_order.data(), sizeof(uint32_t) * n, cudaMemcpyHostToDevice, st));
    // leaf boxes in the new leaf order (the internal boxes are unions of the same leaves)
    k_leaf_boxes<<<(n + tb - 1) / tb, tb, 0, st>>>(plo, phi, order, n, blo, bhi);
    KF_CUDA_CHECK(cudaGetLastError());
    KF_CUDA_CHECK(cudaStreamSynchronize(st)); // the host vectors are freed on return
}

int build_wide_bvh(const float4* plo, const float4* phi, int n, int max_leaf, DeviceBuffer<Node4>& nodes_out,
                   DeviceBuffer<uint32_t>& order_out, cudaStream_t st, bool ploc) {
    if (n <= 0) {
        nodes_out.resize(0, st);
        order_out.resize(0, st);
        return 0;
    }
    order_out.resize(n, st);
    if (n <= max_leaf) {
        nodes_out.resize(1, st);
        k_single_leaf<<<1, 32, 0, st>>>(plo, phi, n, nodes_out.ptr);
        k_identity<<<(n + 255) / 256, 256, 0, st>>>(order_out.ptr, n);
        KF_CUDA_CHECK(cudaGetLastError());
        return 1;
    }
    TempAlloc arena(st);
    float* bounds = arena.alloc<float>(8);
    uint32_t* keys = arena.alloc<uint32_t>(n);
    uint32_t* keys_tmp = arena.alloc<uint32_t>(n);
    uint32_t* vals_tmp = arena.alloc<uint32_t>(n);
    uint32_t* counts = arena.alloc<uint32_t>(radix_sort_count_words(n));
    int* left = arena.alloc<int>(n);
    int* right = arena.alloc<int>(n);
    int* parent = arena.alloc<int>(2 * n);
    int2* range = arena.alloc<int2>(n);
    float4* blo = arena.alloc<float4>(2 * n);
    float4* bhi = arena.alloc<float4>(2 * n);
    int* flags = arena.alloc<int>(n);
    int* fa_src = arena.alloc<int>(n);
    int* fa_dst = arena.alloc<int>(n);
    int* fb_src = arena.alloc<int>(n);
    int* fb_dst = arena.alloc<int>(n);
    int* ctr = arena.alloc<int>(4); // [0] next frontier count, [1] node count

    const float init[8] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY, 0.0f, 0.0f};
    KF_CUDA_CHECK(cudaMemcpyAsync(bounds, init, sizeof(init), cudaMemcpyHostToDevice, st));
    const int tb = 256;
    const int gb = std::min((n + tb - 1) / tb, 1024);
    k_centroid_bounds<<<gb, tb, 0, st>>>(plo, phi, n, bounds);
    k_morton<<<(n + tb - 1) / tb, tb, 0, st>>>(plo, phi, n, bounds, keys, order_out.ptr);
    radix_sort_pairs(keys, order_out.ptr, keys_tmp, vals_tmp, counts, n, 32, st);
    if (!ploc) {
        k_karras<<<(n - 1 + tb - 1) / tb, tb, 0, st>>>(keys, n, left, right, parent, range);
        k_leaf_boxes<<<(n + tb - 1) / tb, tb, 0, st>>>(plo, phi, order_out.ptr, n, blo, bhi);
        KF_CUDA_CHECK(cudaMemsetAsync(flags, 0, sizeof(int) * n, st));
        k_refit<<<(n + tb - 1) / tb, tb, 0, st>>>(n, left, right, parent, blo, bhi, flags);
    } else {
        ploc_tree(plo, phi, n, order_out.ptr, left, right, range, blo, bhi, st);
    }

    // Collapse: frontier starts with the BVH2 root (internal node 0) -> BVH4 node 0.
    // Worst case node count for a 4-wide tree over n leaves is below n.
    nodes_out.resize(n, st);
    const int zero_one[4] = {0, 1, 0, 0};
    KF_CUDA_CHECK(cudaMemcpyAsync(ctr, zero_one, sizeof(zero_one), cudaMemcpyHostToDevice, st));
    const int root_src = 0, root_dst = 0;
    KF_CUDA_CHECK(cudaMemcpyAsync(fa_src, &root_src, sizeof(int), cudaMemcpyHostToDevice, st));
    KF_CUDA_CHECK(cudaMemcpyAsync(fa_dst, &root_dst, sizeof(int), cudaMemcpyHostToDevice, st));
    int count = 1;
    int levels = 0;
    while (count > 0) {
        KF_CUDA_CHECK(cudaMemsetAsync(ctr, 0, sizeof(int), st));
        k_collapse<<<(count + 127) / 128, 128, 0, st>>>(n, max_leaf, left, right, range, blo, bhi, fa_src, fa_dst,
                                                        count, fb_src, fb_dst, ctr, ctr + 1, nodes_out.ptr);
        KF_CUDA_CHECK(cudaGetLastError());
        int h[2];
        KF_CUDA_CHECK(cudaMemcpyAsync(h, ctr, sizeof(h), cudaMemcpyDeviceToHost, st));
        KF_CUDA_CHECK(cudaStreamSynchronize(st));
        count = h[0];
        std::swap(fa_src, fb_src);
        std::swap(fa_dst, fb_dst);
        if (++levels > 4 * 64) {
            throw KfError(KF_ERR_INTERNAL, "BVH collapse did not terminate");
        }
    }
    int total = 0;
    KF_CUDA_CHECK(cudaMemcpyAsync(&total, ctr + 1, sizeof(int), cudaMemcpyDeviceToHost, st));
    KF_CUDA_CHECK(cudaStreamSynchronize(st));
    return total;
}

// ---------------------------------------------------------------------------
// Host SAH builder (cost = C_node + sum_i SA_i / SA * N_i): nodes of at most kSweepMax
// primitives try every split of the centroid-sorted order on each axis (a full sweep);
// larger nodes take 32 bins per axis over the centroid bounds (Wald 2007, "On fast
// construction of SAH-based bounding volume hierarchies"). Then the 4-wide collapse of the
// binary tree, each node's four children chosen by SAH cost (a dynamic program).
// ---------------------------------------------------------------------------
namespace {

struct HBox {
    float lo[3], hi[3];
    void reset() {
        for (int k = 0; k < 3; ++k) {
            lo[k] = INFINITY;
            hi[k] = -INFINITY;
        }
    }
    void grow(const HBox& b) {
        for (int k = 0; k < 3; ++k) {
            lo[k] = std::min(lo[k], b.lo[k]);
            hi[k] = std::max(hi[k], b.hi[k]);
        }
    }
    float area() const {
        const float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
        if (!(dx >= 0.0f) || !(dy >= 0.0f) || !(dz >= 0.0f)) return 0.0f;
        return 2.0f * (dx * dy + dy * dz + dz * dx);
    }
};

struct BNode {
    HBox box;
    int left, right; // -1: leaf
    int first, count;
};

constexpr int kSweepMax = 4096;

struct SahBuilder {
    const float* lo;
    const float* hi;
    int max_leaf;
    std::vector<uint32_t> idx;
    std::vector<float> cen; // 3 per primitive
    std::vector<BNode> nodes;
    std::vector<uint32_t> sweep_order[3]; // scratch of the full sweep (consumed before recursing)
    std::vector<float> sweep_area;

    // Best SAH split of idx[begin, end) over all centroid-sorted orders: on success the range
    // is left in the winning axis's order and the split position is returned, else -1.
    int sweep_split(int begin, int end) {
        const int n = end - begin;
        float best_cost = INFINITY;
        int best_axis = -1, best_at = 0;
        sweep_area.resize(n);
        for (int axis = 0; axis < 3; ++axis) {
            std::vector<uint32_t>& o = sweep_order[axis];
            o.assign(idx.begin() + begin, idx.begin() + end);
            std::sort(o.begin(), o.end(), [&](uint32_t a, uint32_t b) {
                const float ca = cen[3 * a + axis], cb = cen[3 * b + axis];
                return ca < cb || (ca == cb && a < b);
            });
            HBox acc;
            acc.reset();
            for (int i = n - 1; i > 0; --i) {
                acc.grow(prim_box(o[i]));
                sweep_area[i] = acc.area();
            }
            acc.reset();
            for (int i = 0; i < n - 1; ++i) {
                acc.grow(prim_box(o[i]));
                const float cost = acc.area() * (float)(i + 1) + sweep_area[i + 1] * (float)(n - i - 1);
                // equal costs (coincident boxes): the split nearest the middle
                if (cost < best_cost ||
                    (cost == best_cost && std::abs(2 * (i + 1) - n) < std::abs(2 * best_at - n))) {
                    best_cost = cost;
                    best_axis = axis;
                    best_at = i + 1;
                }
            }
        }
        if (best_axis < 0) return -1;
        std::copy(sweep_order[best_axis].begin(), sweep_order[best_axis].end(), idx.begin() + begin);
        return begin + best_at;
    }

    HBox prim_box(uint32_t p) const {
        HBox b;
        for (int k = 0; k < 3; ++k) {
            b.lo[k] = lo[3 * p + k];
            b.hi[k] = hi[3 * p + k];
        }
        return b;
    }

    int build(int begin, int end, int depth) {
        const int node = (int)nodes.size();
        nodes.push_back(BNode{});
        HBox box, cb;
        box.reset();
        cb.reset();
        for (int i = begin; i < end; ++i) {
            box.grow(prim_box(idx[i]));
            for (int k = 0; k < 3; ++k) {
                cb.lo[k] = std::min(cb.lo[k], cen[3 * idx[i] + k]);
                cb.hi[k] = std::max(cb.hi[k], cen[3 * idx[i] + k]);
            }
        }
        const int n = end - begin;
        if (n <= max_leaf) { // leaves never exceed max_leaf (traversal encodes <= 16 triangles)
            nodes[node] = BNode{box, -1, -1, begin, n};
            return node;
        }
        if (n <= kSweepMax && depth < 48) {
            int mid = sweep_split(begin, end);
            if (mid <= begin || mid >= end) mid = begin + n / 2;
            const int l = build(begin, mid, depth + 1);
            const int r = build(mid, end, depth + 1);
            nodes[node] = BNode{box, l, r, begin, n};
            return node;
        }
        constexpr int kBins = 32;
        float best_cost = INFINITY;
        int best_axis = -1, best_bin = 0;
        // from depth 48 on only median splits: bounds the recursion for any input
        for (int axis = 0; axis < 3 && depth < 48; ++axis) {
            const float ext = cb.hi[axis] - cb.lo[axis];
            if (!(ext > 0.0f)) continue;
            HBox bb[kBins];
            int bc[kBins];
            for (int b = 0; b < kBins; ++b) {
                bb[b].reset();
                bc[b] = 0;
            }
            const float scale = kBins / ext;
            for (int i = begin; i < end; ++i) {
                const uint32_t p = idx[i];
                int b = (int)((cen[3 * p + axis] - cb.lo[axis]) * scale);
                b = std::min(std::max(b, 0), kBins - 1);
                bb[b].grow(prim_box(p));
                ++bc[b];
            }
            float right_area[kBins];
            int right_count[kBins];
            HBox acc;
            acc.reset();
            int cnt = 0;
            for (int b = kBins - 1; b > 0; --b) {
                acc.grow(bb[b]);
                cnt += bc[b];
                right_area[b] = acc.area();
                right_count[b] = cnt;
            }
            acc.reset();
            cnt = 0;
            for (int b = 0; b < kBins - 1; ++b) {
                acc.grow(bb[b]);
                cnt += bc[b];
                if (cnt == 0 || right_count[b + 1] == 0) continue;
                const float cost = acc.area() * (float)cnt + right_area[b + 1] * (float)right_count[b + 1];
                if (cost < best_cost) {
                    best_cost = cost;
                    best_axis = axis;
                    best_bin = b;
                }
            }
        }
        int mid;
        if (best_axis < 0) { // all centroids coincide: split the range in half
            mid = begin + n / 2;
        } else {
            const float ext = cb.hi[best_axis] - cb.lo[best_axis];
            const float scale = kBins / ext;
            auto it = std::partition(idx.begin() + begin, idx.begin() + end, [&](uint32_t p) {
                int b = (int)((cen[3 * p + best_axis] - cb.lo[best_axis]) * scale);
                b = std::min(std::max(b, 0), kBins - 1);
                return b <= best_bin;
            });
            mid = (int)(it - idx.begin());
            if (mid == begin || mid == end) mid = begin + n / 2;
        }
        const int l = build(begin, mid, depth + 1);
        const int r = build(mid, end, depth + 1);
        nodes[node] = BNode{box, l, r, begin, n};
        return node;
    }
};

} // namespace

int build_wide_bvh_sah_host(const float* lo, const float* hi, int n, int max_leaf, std::vector<Node4>& out,
                            std::vector<uint32_t>& order) {
    out.clear();
    order.clear();
    if (n <= 0) return 0;
    SahBuilder B;
    B.lo = lo;
    B.hi = hi;
    B.max_leaf = std::max(1, max_leaf);
    B.idx.resize(n);
    B.cen.resize(3 * (size_t)n);
    for (int i = 0; i < n; ++i) {
        B.idx[i] = (uint32_t)i;
        for (int k = 0; k < 3; ++k) B.cen[3 * (size_t)i + k] = 0.5f * (lo[3 * (size_t)i + k] + hi[3 * (size_t)i + k]);
    }
    B.nodes.reserve(2 * (size_t)n);
    const int root = B.build(0, n, 0);
    order = B.idx;
    // SAH-optimal choice of each 4-wide node's children among the binary subtree below it
    // (a dynamic program over the binary tree, as for the wide BVHs of Ylitie, Karras and
    // Laine 2017): U(m) = cost of m as one child (leaf: SA x kTri x count; inner: F(m)),
    // G(m, j) = the cheapest cover of m's subtree by at most j children, F(m) = SA x 1 +
    // min over k of G(left, k) + G(right, 4 - k). Costs in surface area, node step = 1.
    constexpr float kTri = 0.3f; // a triangle test against a 4-box node step (0.1..2 measured alike)
    const size_t nb = B.nodes.size();
    std::vector<std::array<float, 5>> G(nb);
    std::vector<std::array<int8_t, 5>> cut(nb); // G(m, j): 0 = m whole, k = k to the left
    for (size_t mi = nb; mi-- > 0;) { // children are numbered after their parent
        const BNode& m = B.nodes[mi];
        const float sa = m.box.area();
        if (m.left < 0) {
            for (int j = 1; j <= 4; ++j) {
                G[mi][j] = sa * kTri * (float)m.count;
                cut[mi][j] = 0;
            }
            continue;
        }
        float f = INFINITY;
        for (int k = 1; k <= 3; ++k) f = std::min(f, G[m.left][k] + G[m.right][4 - k]);
        const float u = sa + f;
        G[mi][1] = u;
        cut[mi][1] = 0;
        for (int j = 2; j <= 4; ++j) {
            G[mi][j] = u;
            cut[mi][j] = 0;
            for (int k = 1; k < j; ++k) {
                const float c = G[m.left][k] + G[m.right][j - k];
                if (c < G[mi][j]) {
                    G[mi][j] = c;
                    cut[mi][j] = (int8_t)k;
                }
            }
        }
    }
    // the children of binary node b as a 4-wide node: the cover that gives F(b)
    auto children_of = [&](int b, int* ch) {
        int nc = 0;
        std::vector<std::pair<int, int>> todo; // (node, units allowed)
        const BNode& bn = B.nodes[b];
        int bk = 1;
        float best = INFINITY;
        for (int k = 1; k <= 3; ++k) {
            const float c = G[bn.left][k] + G[bn.right][4 - k];
            if (c < best) {
                best = c;
                bk = k;
            }
        }
        todo.push_back({bn.right, 4 - bk});
        todo.push_back({bn.left, bk});
        while (!todo.empty()) {
            const auto [m, j] = todo.back();
            todo.pop_back();
            const int k = cut[m][j];
            if (k == 0) {
                ch[nc++] = m;
            } else {
                todo.push_back({B.nodes[m].right, j - k});
                todo.push_back({B.nodes[m].left, k});
            }
        }
        return nc;
    };
    // 4-wide collapse, breadth first so that the root is node 0
    struct Item {
        int bnode, slot;
    };
    std::vector<Item> queue{{root, 0}};
    out.resize(1);
    for (size_t qi = 0; qi < queue.size(); ++qi) {
        const BNode& bn = B.nodes[queue[qi].bnode];
        int ch[4];
        int nc = 0;
        if (bn.left < 0) {
            ch[nc++] = queue[qi].bnode; // a structure that fits one leaf: one leaf child
        } else {
            nc = children_of(queue[qi].bnode, ch);
        }
        float lx[4], hx[4], ly[4], hy[4], lz[4], hz[4];
        int cc[4], cn[4];
        for (int c = 0; c < 4; ++c) {
            if (c >= nc) {
                lx[c] = ly[c] = lz[c] = INFINITY;
                hx[c] = hy[c] = hz[c] = -INFINITY;
                cc[c] = 0;
                cn[c] = -1;
                continue;
            }
            const BNode& b = B.nodes[ch[c]];
            lx[c] = b.box.lo[0]; ly[c] = b.box.lo[1]; lz[c] = b.box.lo[2];
            hx[c] = b.box.hi[0]; hy[c] = b.box.hi[1]; hz[c] = b.box.hi[2];
            if (b.left < 0) {
                cc[c] = leaf_child(b.first, b.count);
                cn[c] = b.count;
            } else {
                const int slot = (int)out.size();
                out.emplace_back();
                queue.push_back(Item{ch[c], slot});
                cc[c] = slot;
                cn[c] = 0;
            }
        }
        Node4 o;
        o.lox = make_float4(lx[0], lx[1], lx[2], lx[3]);
        o.hix = make_float4(hx[0], hx[1], hx[2], hx[3]);
        o.loy = make_float4(ly[0], ly[1], ly[2], ly[3]);
        o.hiy = make_float4(hy[0], hy[1], hy[2], hy[3]);
        o.loz = make_float4(lz[0], lz[1], lz[2], lz[3]);
        o.hiz = make_float4(hz[0], hz[1], hz[2], hz[3]);
        o.child = make_int4(cc[0], cc[1], cc[2], cc[3]);
        o.cnt = make_int4(cn[0], cn[1], cn[2], cn[3]);
        out[queue[qi].slot] = o;
    }
    return (int)out.size();
}

} // namespace kf
