// kf_bvh.h — GPU wide-BVH construction (BLAS over triangles, TLAS over instances).
#pragma once

#include "kf_device.cuh"
#include "kf_util.h"

namespace kf {

// Stable LSD radix sort of (key, value) pairs on the low `bits` bits of the keys.
// `counts` must hold radix_sort_count_words(n) words.
void radix_sort_pairs(uint32_t* keys, uint32_t* vals, uint32_t* keys_tmp, uint32_t* vals_tmp, uint32_t* counts,
                      int n, int bits, cudaStream_t st);
size_t radix_sort_count_words(int n);

// Builds a 4-wide BVH over n primitive boxes [plo[i], phi[i]] (device pointers).
// On return `order` holds the primitive permutation leaves address (leaf child
// = first position in `order`, cnt = number of consecutive entries) and `nodes`
// the node pool with the root at index 0. Returns the number of nodes.
// ploc: the binary tree by locally-ordered clustering over the Morton order (Meister and
// Bittner 2018) instead of the Karras radix tree; same outputs.
int build_wide_bvh(const float4* plo, const float4* phi, int n, int max_leaf, DeviceBuffer<Node4>& nodes,
                   DeviceBuffer<uint32_t>& order, cudaStream_t st, bool ploc = false);

// The same 4-wide layout built on the host by SAH (surface area heuristic: every split of
// the sorted centroids for nodes of up to 4096 primitives, 32 bins per axis above) and
// collapsed from the binary tree with each node's children chosen by SAH cost: fewer node
// visits per ray than the Morton-order builds, at host build cost. lo / hi: n x 3 floats.
// Returns the number of nodes (root at 0).
int build_wide_bvh_sah_host(const float* lo, const float* hi, int n, int max_leaf, std::vector<Node4>& nodes,
                            std::vector<uint32_t>& order);

} // namespace kf
