// kf_conv.cu — tcgen05 tensor-core kernels of the learned denoiser:
//
//   * implicit 3x3 convolution (forward and backward-data): NHWC BF16 activations,
//     per K step one 4D TMA box of 128 output pixels x 32 input channels shifted by
//     the filter tap (shifts fall on W / H, the 64-byte channel slice stays aligned;
//     out-of-image taps read TMA's zero fill = zero padding) and one 3D TMA box of
//     weights, tcgen05.mma kind::f16 (M = 128, N = output channels) accumulating in
//     TMEM, epilogue tcgen05.ld -> + bias -> ReLU -> BF16 NHWC store (into a channel
//     slice, so skip concatenation costs nothing);
//   * K-major GEMM D += A * B^T (weight gradients): 2D TMA, 128-byte swizzle,
//     split-K with FP32 atomics in the epilogue.
//
// One CTA of 128 threads per output tile: warp 0 lane 0 issues TMA into a 2-, 3- or
// 4-stage mbarrier ring, warp 1 lane 0 issues the MMAs, all four warps drain TMEM. Every
// wait is bounded (~1 s of SM clock); on expiry the kernel records an error code,
// drains its own copies and frees its TMEM.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstring>
#include <mutex>

#include "kf_conv.h"
#include "kf_tc.cuh"
#include "kf_util.h"

namespace kf {

__device__ uint32_t g_tc_error;

namespace {

constexpr long long kWaitBudget = 2000000000ll; // SM cycles (~1 s)

struct TcParams {
    int N, H, W, Cin; // conv: A tensor NHWC
    int Cout;         // valid output channels
    int bw, bh;       // conv output tile (bw * bh = 128)
    int tiles_x, tiles_y;
    int n_tile;       // N columns per CTA
    int kchunks;      // conv: Cin / CK
    const float* bias;
    int relu;
    __nv_bfloat16* out;
    int out_cstride, out_coff;
    float* outf;      // gemm output (atomic add); conv: FP32 output instead of BF16 when set
    int ldo, M_valid, N_valid;
    int k_iters, k_per_split;
    uint32_t tmem_cols;
};

__device__ __forceinline__ void set_error(uint32_t code) { atomicCAS(&g_tc_error, 0u, code); }

// MODE 0: implicit conv3x3 (4D A, 3D B); MODE 1: GEMM (2D A, 2D B).
template <int MODE, int SWZ, int kStages>
__global__ void __launch_bounds__(128, 1) k_tc(const __grid_constant__ CUtensorMap tmA,
                                               const __grid_constant__ CUtensorMap tmB, const TcParams p) {
    constexpr int CK = SWZ / 2;                     // BF16 elements per K chunk (one swizzle row)
    constexpr uint32_t LAYOUT = SWZ == 128 ? 2u : (SWZ == 64 ? 4u : 6u);
    constexpr uint32_t SBO = 8u * SWZ;              // 8 rows of SWZ bytes
    constexpr uint32_t A_BYTES = 128u * SWZ;
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const uint32_t B_BYTES = ((uint32_t)p.n_tile * SWZ + 1023u) & ~1023u;
    uint8_t* sA = smem;
    uint8_t* sB = smem + kStages * A_BYTES;
    uint64_t* full = reinterpret_cast<uint64_t*>(sB + kStages * B_BYTES);
    uint64_t* empty = full + kStages;
    uint64_t* done = empty + kStages;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 1);
    float* sbias = reinterpret_cast<float*>(tmem_slot + 4); // the tile's bias (0 where none)

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    // ---- tile coordinates ----
    int n_img = 0, x0 = 0, y0 = 0, m0 = 0;
    const int n0 = blockIdx.y * p.n_tile;
    int k_begin = 0, k_end = p.k_iters;
    if (MODE == 0) {
        const int t = blockIdx.x;
        const int per_img = p.tiles_x * p.tiles_y;
        n_img = t / per_img;
        const int r = t % per_img;
        y0 = (r / p.tiles_x) * p.bh;
        x0 = (r % p.tiles_x) * p.bw;
    } else {
        m0 = blockIdx.x * 128;
        k_begin = blockIdx.z * p.k_per_split;
        k_end = min(p.k_iters, k_begin + p.k_per_split);
    }
    const int nk = max(0, k_end - k_begin);

    if (warp == 0) tc::tmem_alloc(tmem_slot, p.tmem_cols);
    if (MODE == 0)
        for (int i = threadIdx.x; i < p.n_tile; i += blockDim.x)
            sbias[i] = (p.bias && n0 + i < p.Cout) ? p.bias[n0 + i] : 0.0f;
    if (threadIdx.x == 32) {
        for (int s = 0; s < kStages; ++s) {
            tc::mbar_init(&full[s], 1);
            tc::mbar_init(&empty[s], 1);
        }
        tc::mbar_init(done, 1);
        tc::fence_barrier_init();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0 && lane == 0) {
        // ---- producer: TMA ----
        bool ok = true;
        for (int i = 0; i < nk && ok; ++i) {
            const int s = i % kStages;
            if (i >= kStages && !tc::mbar_wait(&empty[s], ((i / kStages) - 1) & 1, kWaitBudget)) {
                set_error(1);
                ok = false;
                break;
            }
            const uint32_t b_bytes = (uint32_t)p.n_tile * SWZ;
            tc::mbar_arrive_expect_tx(&full[s], A_BYTES + b_bytes);
            const int k = k_begin + i;
            if (MODE == 0) {
                const int tap = k / p.kchunks, ch = (k % p.kchunks) * CK;
                const int dy = tap / 3 - 1, dx = tap % 3 - 1;
                tc::tma_load_4d(sA + s * A_BYTES, &tmA, &full[s], ch, x0 + dx, y0 + dy, n_img);
                tc::tma_load_3d(sB + s * B_BYTES, &tmB, &full[s], ch, n0, tap);
            } else {
                tc::tma_load_2d(sA + s * A_BYTES, &tmA, &full[s], k * CK, m0);
                tc::tma_load_2d(sB + s * B_BYTES, &tmB, &full[s], k * CK, n0);
            }
        }
        // drain: the last use of every stage must have landed before the CTA may exit
        for (int s = 0; s < kStages && s < nk; ++s) {
            const int last = ((nk - 1 - s) / kStages) * kStages + s;
            if (!tc::mbar_wait(&full[s], (last / kStages) & 1, kWaitBudget)) set_error(2);
        }
    } else if (warp == 1 && lane == 0) {
        // ---- MMA issuer ----
        const uint32_t idesc = tc::idesc_bf16(128, (uint32_t)p.n_tile);
        for (int i = 0; i < nk; ++i) {
            const int s = i % kStages;
            if (!tc::mbar_wait(&full[s], (i / kStages) & 1, kWaitBudget)) {
                set_error(3);
                break;
            }
            tc::fence_after_sync();
            const uint32_t a_addr = tc::smem_u32(sA + s * A_BYTES);
            const uint32_t b_addr = tc::smem_u32(sB + s * B_BYTES);
#pragma unroll
            for (int kk = 0; kk < CK / 16; ++kk) {
                const uint64_t ad = tc::smem_desc(a_addr + kk * 32, SBO, LAYOUT);
                const uint64_t bd = tc::smem_desc(b_addr + kk * 32, SBO, LAYOUT);
                tc::mma_bf16(tmem, ad, bd, idesc, (i > 0 || kk > 0) ? 1u : 0u);
            }
            tc::mma_commit(&empty[s]);
        }
        tc::mma_commit(done);
    }

    // ---- epilogue: all 4 warps, warp w owns TMEM lanes [32w, 32w + 32) ----
    const bool ready = (nk == 0) ? true : tc::mbar_wait(done, 0, kWaitBudget);
    if (!ready) set_error(4);
    __syncwarp();
    tc::fence_after_sync();
    const int row = warp * 32 + lane;
    if (MODE == 0) {
        const int px = x0 + (row % p.bw), py = y0 + (row / p.bw);
        const bool valid = ready && nk > 0 && px < p.W && py < p.H;
        const size_t base = ((size_t)((size_t)n_img * p.H + py) * p.W + px) * p.out_cstride + p.out_coff;
        // 16 columns per TMEM wait: two loads in flight; bias from shared memory
        auto emit8 = [&](const uint32_t(&r)[8], int c) {
            const int co = n0 + c;
            if (!valid || co >= p.Cout) return;
            float v[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                v[j] = __uint_as_float(r[j]);
                if (p.bias && co + j < p.Cout) v[j] += sbias[c + j];
                if (p.relu) v[j] = fmaxf(v[j], 0.0f);
            }
            if (p.outf) { // FP32 output (a network head)
                for (int j = 0; j < 8 && co + j < p.Cout; ++j) p.outf[base + co + j] = v[j];
                return;
            }
            __nv_bfloat16* dst = p.out + base;
            if (co + 8 <= p.Cout && ((p.out_coff + co) & 7) == 0 && (p.out_cstride & 7) == 0) {
                __nv_bfloat162 q[4];
#pragma unroll
                for (int j = 0; j < 4; ++j) q[j] = __floats2bfloat162_rn(v[2 * j], v[2 * j + 1]);
                *reinterpret_cast<uint4*>(dst + co) = *reinterpret_cast<const uint4*>(q);
            } else {
                for (int j = 0; j < 8 && co + j < p.Cout; ++j) dst[co + j] = __float2bfloat16_rn(v[j]);
            }
        };
        for (int c = 0; c < p.n_tile; c += 16) {
            uint32_t r0[8], r1[8];
            tc::tmem_ld8(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c, r0);
            tc::tmem_ld8(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(c + 8), r1);
            tc::tmem_ld_wait();
            emit8(r0, c);
            emit8(r1, c + 8);
        }
    } else {
        const int m = m0 + row;
        const bool valid = ready && nk > 0 && m < p.M_valid;
        for (int c = 0; c < p.n_tile; c += 8) {
            uint32_t r[8];
            tc::tmem_ld8(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c, r);
            tc::tmem_ld_wait();
            if (!valid) continue;
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const int n = n0 + c + j;
                if (n < p.N_valid) atomicAdd(p.outf + (size_t)m * p.ldo + n, __uint_as_float(r[j]));
            }
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, p.tmem_cols);
}

// ---------------------------------------------------------------------------
// Halo convolution: persistent, warp-specialised, for images at least 96 pixels wide.
//
// A tile is R output rows x 128 pixels x n_tile output channels: R accumulators of
// n_tile TMEM columns, double-buffered so the epilogue of one tile overlaps the MMAs of
// the next. Per chunk of CK input channels one 4D TMA box brings the tile's input halo,
// (R + 2) rows x 130 pixels, into shared memory as [row][pixel][CK channels]: one swizzled
// K-major row of CK x 2 bytes (32- or 64-byte swizzle) per pixel, so TMA moves 32- or
// 64-byte pieces of the NHWC input (16-byte pieces deliver half the bytes per second).
// The A operand of tap (dy, dx) for output row r is that buffer viewed from row r + dy,
// pixel dx on: the descriptor's start address moves by whole rows. The tensor cores apply
// the swizzle to the absolute shared-memory address, as TMA does when it writes a box at
// a 1024-byte aligned address, so a view starting at any row reads the rows TMA wrote
// (the descriptor's base-offset field stays 0). The halo is read from L2 once per chunk
// and used by all 9 taps (the per-tap kernel above reads 9 shifted boxes). The weights of a
// chunk (9 blocks of n_tile rows of CK channels, swizzled, ordered [dx][dy = 2, 1, 0] so
// that one MMA covers up to STACK output rows: halo_chunk_mmas) stream with the halo by TMA,
// or, when one chunk covers all input channels, are loaded once per CTA.
//
// The epilogue writes 16 channels of a pixel with one 32-byte store and can also do the
// 2x2 average pooling that follows some layers (rows are paired inside a tile, the right
// neighbour is the next lane), saving the pass that would read the layer's output again.
//
// Warp 0 lane 0: TMA producer (a ring of STAGES stages). Warp 1 lane 0: MMA issuer.
// Warps 2-9: epilogue, warp w owning TMEM lanes [32 (w % 4), +32) = tile pixels, warps 2-5
// the first half of the channels and warps 6-9 the second.
// Every wait is bounded; on expiry the kernel records an error code, lets its own
// copies and MMAs finish and frees its TMEM.
// ---------------------------------------------------------------------------
constexpr int kHaloW = 130;     // 128 output pixels + 2 halo pixels
// Halo stages in flight (STAGES): 3, or 2 where a third does not fit 227 KB (8-row
// tiles, or 32-channel chunks with streamed weights).
constexpr int kHaloThreads = 320;  // producer warp, MMA warp, 8 epilogue warps

// 8 or 16 FP32 values stored as BF16 with one 16- or 32-byte store (dst 16- / 32-byte aligned)
__device__ __forceinline__ void st_bf16x8(__nv_bfloat16* dst, const float (&v)[8]) {
    __nv_bfloat162 q2[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) q2[q] = __floats2bfloat162_rn(v[2 * q], v[2 * q + 1]);
    *reinterpret_cast<uint4*>(dst) = *reinterpret_cast<const uint4*>(q2);
}
__device__ __forceinline__ void st_bf16x16(__nv_bfloat16* dst, const float (&v0)[8], const float (&v1)[8]) {
    __nv_bfloat162 q2[8];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        q2[q] = __floats2bfloat162_rn(v0[2 * q], v0[2 * q + 1]);
        q2[4 + q] = __floats2bfloat162_rn(v1[2 * q], v1[2 * q + 1]);
    }
    const uint32_t* w = reinterpret_cast<const uint32_t*>(q2);
    asm volatile("st.global.v8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"l"(dst), "r"(w[0]), "r"(w[1]),
                 "r"(w[2]), "r"(w[3]), "r"(w[4]), "r"(w[5]), "r"(w[6]), "r"(w[7])
                 : "memory");
}

struct HaloParams {
    int N, H, W, Cin, Cout;
    int n_tile, R, kchunks;
    int tiles_x, tiles_y, num_tiles;
    int w_resident;          // 1: the weights of all input channels are one chunk, loaded once
    int stack;               // output rows one MMA covers (1..3, stack x n_tile <= 256)
    uint32_t halo_bytes;     // bytes of one halo box
    uint32_t halo_stride;    // its slot in shared memory (1024-aligned)
    uint32_t w_bytes;        // bytes of one chunk of weights (9 x n_tile x CK)
    uint32_t w_stride;
    uint32_t tmem_cols;
    const float* bias;
    int relu;
    __nv_bfloat16* out;
    int out_cstride, out_coff;
    float* outf;
    __nv_bfloat16* pool_out;   // fused 2x2 average pooling into a dense [N][H/2][W/2][Cout] tensor, or null
};

// Constants of the MMA sequence that depend on n_tile: weight block offsets (in
// descriptor units of 16 bytes), instruction descriptors for 1..3 stacked rows, and the
// TMEM column of each output row.
struct HaloMmaConsts {
    uint32_t boff[9];
    uint32_t idesc[3];
    uint32_t dcol[8];
};

// The MMAs of one chunk, unrolled at compile time (the single issuing thread then spends a
// few instructions per MMA; built from a table at run time they took half again as long).
// Halo row hr with shift dx feeds output rows hr - 2 .. hr (tap dy = hr - r); their
// accumulators are adjacent TMEM columns and their weight blocks ([dx][dy = 2, 1, 0])
// adjacent rows, so one MMA of N = rows x n_tile covers up to STACK of them and the A
// operand is read once per (hr, dx, kk) instead of once per output row. The loop runs
// over halo rows outermost, so consecutive MMAs accumulate into the same columns. In a
// tile's first chunk the row a halo row reaches first (r = hr, at dx = 0, kk = 0) starts
// its accumulator with a non-accumulating MMA of its own.
template <int CK, int R, int STACK, bool FIRST>
__device__ __forceinline__ void halo_chunk_mmas(uint64_t ad0, uint64_t bd0, uint32_t acc, const HaloMmaConsts& k) {
    constexpr uint32_t W_ROW = CK * 2, HALO_ROW = kHaloW * W_ROW;
#pragma unroll
    for (int hr = 0; hr < R + 2; ++hr) {
#pragma unroll
        for (int dx = 0; dx < 3; ++dx) {
#pragma unroll
            for (int kk = 0; kk < CK / 16; ++kk) {
                const uint64_t ad = ad0 + (((uint32_t)hr * HALO_ROW + (uint32_t)dx * W_ROW + kk * 32) >> 4);
                const int lo = hr - 2 > 0 ? hr - 2 : 0;
                int hi = hr < R - 1 ? hr : R - 1;
                if (FIRST && dx == 0 && kk == 0 && hi == hr) {
                    tc::mma_bf16(acc + k.dcol[hr], ad, bd0 + k.boff[dx * 3 + 2] + kk * 2, k.idesc[0], 0u);
                    --hi;
                }
#pragma unroll
                for (int r0 = lo; r0 <= hi; r0 += STACK) {
                    const int r1 = r0 + STACK - 1 < hi ? r0 + STACK - 1 : hi;
                    tc::mma_bf16(acc + k.dcol[r0], ad, bd0 + k.boff[dx * 3 + 2 - (hr - r0)] + kk * 2,
                                 k.idesc[r1 - r0], 1u);
                }
            }
        }
    }
}

template <int CK, int R, int STACK, int STAGES>
__global__ void __launch_bounds__(kHaloThreads, 1) k_conv_halo(const __grid_constant__ CUtensorMap tmX,
                                                                 const __grid_constant__ CUtensorMap tmW,
                                                                 const HaloParams p) {
    constexpr uint32_t W_ROW = CK * 2;                 // bytes per pixel row and weight row (the swizzle width)
    constexpr uint32_t W_LAYOUT = CK == 32 ? 4u : 6u;  // 64 B / 32 B swizzle
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint8_t* halo = smem;
    uint8_t* wst = halo + STAGES * p.halo_stride;
    const int w_slots = p.w_resident ? 1 : STAGES;
    uint64_t* full = reinterpret_cast<uint64_t*>(wst + w_slots * p.w_stride);
    uint64_t* empty = full + STAGES;
    uint64_t* acc_full = empty + STAGES;
    uint64_t* acc_empty = acc_full + 2;
    uint64_t* wbar = acc_empty + 2;
    uint64_t* mma_done = wbar + 1;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(mma_done + 1);
    float* sbias = reinterpret_cast<float*>(tmem_slot + 4);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int n0 = blockIdx.y * p.n_tile;
    const int acc_cols = p.R * p.n_tile;

    if (warp == 0) tc::tmem_alloc(tmem_slot, p.tmem_cols);
    for (int i = threadIdx.x; i < p.n_tile; i += blockDim.x)
        sbias[i] = (p.bias && n0 + i < p.Cout) ? p.bias[n0 + i] : 0.0f;
    if (threadIdx.x == 32) {
        for (int s = 0; s < STAGES; ++s) {
            tc::mbar_init(&full[s], 1);
            tc::mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            tc::mbar_init(&acc_full[b], 1);
            tc::mbar_init(&acc_empty[b], 8);
        }
        tc::mbar_init(wbar, 1);
        tc::mbar_init(mma_done, 1);
        tc::fence_barrier_init();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tmem_slot;

    auto tile_origin = [&](int t, int& n_img, int& y0, int& x0) {
        const int per_img = p.tiles_x * p.tiles_y;
        n_img = t / per_img;
        const int r = t % per_img;
        y0 = (r / p.tiles_x) * p.R;
        x0 = (r % p.tiles_x) * 128;
    };

    if (warp == 0 && lane == 0) {
        // ---- producer ----
        bool ok = true;
        // the weights of a chunk in shared memory as 9 blocks of n_tile rows in the order
        // [dx][dy = 2, 1, 0]: the blocks of the taps one halo row and shift give the
        // output rows r, r + 1, r + 2 (dy = j - r) are adjacent, one stacked B operand
        auto load_weights = [&](uint8_t* dst, uint64_t* bar, int c) {
#pragma unroll 1
            for (int tap = 0; tap < 9; ++tap) {
                const int blk = (tap % 3) * 3 + (2 - tap / 3);
                tc::tma_load_3d(dst + (uint32_t)blk * p.n_tile * W_ROW, &tmW, bar, c * CK, n0, tap);
            }
        };
        if (p.w_resident) {
            tc::mbar_arrive_expect_tx(wbar, p.w_bytes);
            load_weights(wst, wbar, 0);
        }
        uint32_t it = 0;
        for (int t = blockIdx.x; t < p.num_tiles && ok; t += gridDim.x) {
            int n_img, y0, x0;
            tile_origin(t, n_img, y0, x0);
            for (int c = 0; c < p.kchunks; ++c, ++it) {
                const uint32_t s = it % STAGES;
                if (it >= (uint32_t)STAGES &&
                    !tc::mbar_wait(&empty[s], ((it / STAGES) - 1) & 1, kWaitBudget)) {
                    set_error(11);
                    ok = false;
                    break;
                }
                tc::mbar_arrive_expect_tx(&full[s], p.halo_bytes + (p.w_resident ? 0u : p.w_bytes));
                tc::tma_load_4d(halo + s * p.halo_stride, &tmX, &full[s], c * CK, x0 - 1, y0 - 1, n_img);
                if (!p.w_resident) load_weights(wst + s * p.w_stride, &full[s], c);
            }
        }
        // drain: every issued copy must have landed before the CTA may exit
        for (uint32_t s = 0; s < (uint32_t)STAGES && s < it; ++s) {
            const uint32_t last = ((it - 1 - s) / STAGES) * STAGES + s;
            if (!tc::mbar_wait(&full[s], (last / STAGES) & 1, kWaitBudget)) set_error(12);
        }
        if (p.w_resident && !tc::mbar_wait(wbar, 0, kWaitBudget)) set_error(13);
    } else if (warp == 1 && lane == 0) {
        // ---- MMA issuer ----
        const uint32_t halo0 = tc::smem_u32(halo), w0 = tc::smem_u32(wst);
        // per-CTA constants of the unrolled MMA sequence (halo_chunk_mmas)
        HaloMmaConsts k;
#pragma unroll
        for (int b = 0; b < 9; ++b) k.boff[b] = (uint32_t)(b * p.n_tile) * W_ROW >> 4;
#pragma unroll
        for (int q = 0; q < 3; ++q) k.idesc[q] = tc::idesc_bf16(128, (uint32_t)((q + 1) * p.n_tile));
#pragma unroll
        for (int r = 0; r < R; ++r) k.dcol[r] = (uint32_t)(r * p.n_tile);
        bool ok = !p.w_resident || tc::mbar_wait(wbar, 0, kWaitBudget);
        if (!ok) set_error(14);
        uint32_t it = 0, j = 0;
        for (int t = blockIdx.x; t < p.num_tiles && ok; t += gridDim.x, ++j) {
            const uint32_t b = j & 1;
            if (j >= 2 && !tc::mbar_wait(&acc_empty[b], ((j / 2) - 1) & 1, kWaitBudget)) {
                set_error(15);
                break;
            }
            tc::fence_after_sync();
            const uint32_t acc = tmem + b * (uint32_t)acc_cols;
            for (int c = 0; c < p.kchunks; ++c, ++it) {
                const uint32_t s = it % STAGES;
                if (!tc::mbar_wait(&full[s], (it / STAGES) & 1, kWaitBudget)) {
                    set_error(16);
                    ok = false;
                    break;
                }
                tc::fence_after_sync();
                const uint32_t ha = halo0 + s * p.halo_stride;
                const uint32_t wa = w0 + (p.w_resident ? 0u : s * p.w_stride);
                const uint64_t ad0 = tc::smem_desc(ha, 8u * W_ROW, W_LAYOUT);
                const uint64_t bd0 = tc::smem_desc(wa, 8u * W_ROW, W_LAYOUT);
                if (c == 0)
                    halo_chunk_mmas<CK, R, STACK, true>(ad0, bd0, acc, k);
                else
                    halo_chunk_mmas<CK, R, STACK, false>(ad0, bd0, acc, k);
                tc::mma_commit(&empty[s]);
            }
            if (!ok) break;
            tc::mma_commit(&acc_full[b]);
        }
        // every MMA of this CTA completes before the TMEM is freed
        tc::mma_commit(mma_done);
        if (!tc::mbar_wait(mma_done, 0, kWaitBudget)) set_error(17);
    } else if (warp >= 2) {
        // ---- epilogue: 8 warps, two per TMEM lane group, each taking half the channels ----
        const int lg = warp & 3;                 // TMEM lane group of this warp
        const int px_in_tile = lg * 32 + lane;
        const int half = (warp - 2) >> 2;
        const int cb = half * (p.n_tile / 2), ce = cb + p.n_tile / 2;  // multiples of 8
        // 32-byte stores need 32-byte aligned rows: the tensor, the channel stride and slice
        const bool wide = !p.outf && p.out && ((uintptr_t)p.out & 31) == 0 && (p.out_cstride & 15) == 0;
        const bool pool_wide = p.pool_out && ((uintptr_t)p.pool_out & 31) == 0 && (p.Cout & 15) == 0 &&
                               (n0 & 15) == 0;
        uint32_t j = 0;
        for (int t = blockIdx.x; t < p.num_tiles; t += gridDim.x, ++j) {
            const uint32_t b = j & 1;
            const bool ready = tc::mbar_wait(&acc_full[b], (j / 2) & 1, kWaitBudget);
            __syncwarp();
            if (!ready) {
                set_error(18);
                break;
            }
            tc::fence_after_sync();
            int n_img, y0, x0;
            tile_origin(t, n_img, y0, x0);
            const int px = x0 + px_in_tile;
            // one output row's 8 channels [cc, cc + 8) of this pixel (BF16 or FP32)
            auto emit8 = [&](const float(&v)[8], int py, int cc) {
                const int co = n0 + cc;
                if (!(px < p.W && py < p.H) || co >= p.Cout) return;
                const size_t base = ((size_t)((size_t)n_img * p.H + py) * p.W + px) * p.out_cstride + p.out_coff;
                if (p.outf) {
                    for (int q = 0; q < 8 && co + q < p.Cout; ++q) p.outf[base + co + q] = v[q];
                    return;
                }
                __nv_bfloat162 q2[4];
#pragma unroll
                for (int q = 0; q < 4; ++q) q2[q] = __floats2bfloat162_rn(v[2 * q], v[2 * q + 1]);
                const uint4 packed = *reinterpret_cast<const uint4*>(q2);
                __nv_bfloat16* dst = p.out + base + co;
                if (co + 8 <= p.Cout && ((p.out_coff + co) & 7) == 0 && (p.out_cstride & 7) == 0)
                    *reinterpret_cast<uint4*>(dst) = packed;
                else
                    for (int q = 0; q < 8 && co + q < p.Cout; ++q) dst[q] = __float2bfloat16_rn(v[q]);
            };
            // 16 channels [cc, cc + 16): one 32-byte store (a whole L2 sector) when aligned
            auto emit16 = [&](const float(&v0)[8], const float(&v1)[8], int py, int cc) {
                const int co = n0 + cc;
                if (wide && co + 16 <= p.Cout && ((p.out_coff + co) & 15) == 0) {
                    if (!(px < p.W && py < p.H)) return;
                    const size_t base = ((size_t)((size_t)n_img * p.H + py) * p.W + px) * p.out_cstride + p.out_coff;
                    st_bf16x16(p.out + base + co, v0, v1);
                    return;
                }
                emit8(v0, py, cc);
                emit8(v1, py, cc + 8);
            };
            auto act = [&](uint32_t raw, int cc) {
                const float v = __uint_as_float(raw) + sbias[cc];
                return p.relu ? fmaxf(v, 0.0f) : v;
            };
            const uint32_t lanes = (uint32_t)(lg * 32) << 16;
            if (!p.pool_out) {
                for (int r = 0; r < p.R; ++r) {
                    const uint32_t col0 = (b * (uint32_t)p.R + (uint32_t)r) * (uint32_t)p.n_tile;
                    for (int c = cb; c < ce; c += 16) { // two TMEM loads per wait
                        uint32_t r0[8], r1[8];
                        const bool two = c + 16 <= ce;
                        tc::tmem_ld8(tmem + lanes + col0 + (uint32_t)c, r0);
                        if (two) tc::tmem_ld8(tmem + lanes + col0 + (uint32_t)(c + 8), r1);
                        tc::tmem_ld_wait();
                        float v0[8], v1[8];
#pragma unroll
                        for (int q = 0; q < 8; ++q) {
                            v0[q] = act(r0[q], c + q);
                            v1[q] = two ? act(r1[q], c + 8 + q) : 0.0f;
                        }
                        if (two)
                            emit16(v0, v1, y0 + r, c);
                        else
                            emit8(v0, y0 + r, c);
                    }
                }
            } else {
                // rows in pairs (R and y0 are even): the 2x2 average of the BF16 outputs, as the
                // separate pooling pass computes it ((a + b) + c) + d over (2y, 2x), (2y, 2x+1),
                // (2y+1, 2x), (2y+1, 2x+1); the right neighbour is the next lane
                const int Hh = p.H / 2, Wh = p.W / 2;
                for (int r = 0; r < p.R; r += 2) {
                    const int py = y0 + r;
                    const uint32_t col0 = (b * (uint32_t)p.R + (uint32_t)r) * (uint32_t)p.n_tile;
                    for (int c = cb; c < ce; c += 16) {
                        const bool two = c + 16 <= ce;
                        uint32_t ra[16], rc[16];
                        tc::tmem_ld8(tmem + lanes + col0 + (uint32_t)c, *reinterpret_cast<uint32_t(*)[8]>(ra));
                        tc::tmem_ld8(tmem + lanes + col0 + (uint32_t)(p.n_tile + c),
                                     *reinterpret_cast<uint32_t(*)[8]>(rc));
                        if (two) {
                            tc::tmem_ld8(tmem + lanes + col0 + (uint32_t)(c + 8),
                                         *reinterpret_cast<uint32_t(*)[8]>(ra + 8));
                            tc::tmem_ld8(tmem + lanes + col0 + (uint32_t)(p.n_tile + c + 8),
                                         *reinterpret_cast<uint32_t(*)[8]>(rc + 8));
                        }
                        tc::tmem_ld_wait();
                        float va[16], vc[16], pooled[16];
#pragma unroll
                        for (int q = 0; q < 16; ++q) {
                            const bool live = q < 8 || two;
                            va[q] = live ? act(ra[q], c + q) : 0.0f;
                            vc[q] = live ? act(rc[q], c + q) : 0.0f;
                            const float a = __bfloat162float(__float2bfloat16_rn(va[q]));
                            const float cv = __bfloat162float(__float2bfloat16_rn(vc[q]));
                            const float bv = __shfl_xor_sync(0xFFFFFFFFu, a, 1);
                            const float dv = __shfl_xor_sync(0xFFFFFFFFu, cv, 1);
                            pooled[q] = 0.25f * (((a + bv) + cv) + dv);
                        }
                        const float(&va0)[8] = *reinterpret_cast<const float(*)[8]>(va);
                        const float(&va1)[8] = *reinterpret_cast<const float(*)[8]>(va + 8);
                        const float(&vc0)[8] = *reinterpret_cast<const float(*)[8]>(vc);
                        const float(&vc1)[8] = *reinterpret_cast<const float(*)[8]>(vc + 8);
                        if (two) {
                            emit16(va0, va1, py, c);
                            emit16(vc0, vc1, py + 1, c);
                        } else {
                            emit8(va0, py, c);
                            emit8(vc0, py + 1, c);
                        }
                        const int co = n0 + c;
                        if ((lane & 1) == 0 && px + 1 < p.W && py + 1 < p.H && co < p.Cout) {
                            const size_t pb = ((size_t)((size_t)n_img * Hh + py / 2) * Wh + px / 2) * p.Cout + co;
                            const float(&p0)[8] = *reinterpret_cast<const float(*)[8]>(pooled);
                            const float(&p1)[8] = *reinterpret_cast<const float(*)[8]>(pooled + 8);
                            if (two && pool_wide && co + 16 <= p.Cout && (co & 15) == 0)
                                st_bf16x16(p.pool_out + pb, p0, p1);
                            else {
                                st_bf16x8(p.pool_out + pb, p0);
                                if (two && co + 8 < p.Cout) st_bf16x8(p.pool_out + pb + 8, p1);
                            }
                        }
                    }
                }
            }
            tc::fence_before_sync();
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(&acc_empty[b]);
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, p.tmem_cols);
}

// ---- host: tensor maps ----
PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    KF_REQUIRE(fn, KF_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
    return fn;
}

CUtensorMap make_map(const void* base, int rank, const uint64_t* dims, const uint64_t* strides_bytes,
                     const uint32_t* box, CUtensorMapSwizzle swz) {
    CUtensorMap m;
    std::memset(&m, 0, sizeof(m));
    uint32_t estr[5] = {1, 1, 1, 1, 1};
    const CUresult r = encode_fn()(&m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, (cuuint32_t)rank, const_cast<void*>(base),
                                   reinterpret_cast<const cuuint64_t*>(dims),
                                   reinterpret_cast<const cuuint64_t*>(strides_bytes),
                                   reinterpret_cast<const cuuint32_t*>(box), estr, CU_TENSOR_MAP_INTERLEAVE_NONE, swz,
                                   CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        char msg[256];
        std::snprintf(msg, sizeof(msg),
                      "cuTensorMapEncodeTiled rejected a tensor layout (CUresult %d, rank %d, dims %llu x %llu, "
                      "box %u x %u)",
                      (int)r, rank, (unsigned long long)dims[0], (unsigned long long)dims[1], box[0], box[1]);
        throw KfError(KF_ERR_INVALID_ARGUMENT, msg);
    }
    return m;
}

uint32_t pow2_at_least(uint32_t v) {
    uint32_t c = 32;
    while (c < v) c <<= 1;
    return c;
}

template <int MODE, int SWZ, int kStages> size_t smem_bytes(int n_tile) {
    const size_t a = 128u * SWZ, b = (((size_t)n_tile * SWZ) + 1023) & ~size_t(1023);
    return 1024 + kStages * (a + b) + 256 + 4u * (size_t)n_tile;
}

template <int MODE, int SWZ, int kStages>
void launch_tc(dim3 grid, const CUtensorMap& a, const CUtensorMap& b, const TcParams& p, cudaStream_t st) {
    const size_t sm = smem_bytes<MODE, SWZ, kStages>(p.n_tile);
    static bool configured = false;
    if (!configured) {
        KF_CUDA_CHECK(cudaFuncSetAttribute(k_tc<MODE, SWZ, kStages>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)smem_bytes<MODE, SWZ, kStages>(256)));
        configured = true;
    }
    k_tc<MODE, SWZ, kStages><<<grid, 128, sm, st>>>(a, b, p);
    KF_CUDA_CHECK(cudaGetLastError());
}

// Shape of a halo-convolution launch: rows per tile R, channels per chunk CK, and the
// shared memory it takes. Larger R first (less halo per output row, fewer weight
// reloads per pixel), then larger CK; both accumulators must fit the 512 TMEM columns.
struct HaloShape {
    int R = 0, CK = 0, stages = 3;
    bool w_resident = false;
    uint32_t halo_bytes = 0, halo_stride = 0, w_bytes = 0, w_stride = 0;
    size_t smem = 0;
};

int halo_stack(int n_tile) { return std::min(3, 256 / n_tile); }

bool halo_shape(int Cin, int n_tile, HaloShape& out) {
    for (int R : {8, 4, 2, 1}) {
        if (2 * R * n_tile > 512) continue;
        const int S = halo_stack(n_tile);
        if (!((R >= 4 && S == 3) || (R == 2 && S >= 2) || (R == 1 && S == 1))) continue;
        // 32-channel chunks first (64-byte TMA pieces, half the chunk round trips), with three
        // stages or, where those do not fit, two; then 16-channel chunks
        for (const auto& [CK, stages] : {std::pair{32, 3}, std::pair{32, 2}, std::pair{16, 3}, std::pair{16, 2}}) {
            if (Cin % CK) continue;
            if (R == 8 && stages == 3) continue; // an 8-row halo leaves room for two
            HaloShape h;
            h.R = R;
            h.CK = CK;
            h.stages = stages;
            h.w_resident = Cin == CK;
            h.halo_bytes = (uint32_t)((R + 2) * kHaloW * CK * 2);
            h.halo_stride = (h.halo_bytes + 1023u) & ~1023u;
            h.w_bytes = (uint32_t)(9 * n_tile * CK * 2);
            h.w_stride = (h.w_bytes + 1023u) & ~1023u;
            h.smem = 1024 + (size_t)stages * h.halo_stride +
                     (size_t)(h.w_resident ? 1 : stages) * h.w_stride + 256 + 4u * (size_t)n_tile;
            if (h.smem <= 227u * 1024u) {
                out = h;
                return true;
            }
        }
    }
    return false;
}

int num_sms() {
    int dev = 0, n = 0;
    KF_CUDA_CHECK(cudaGetDevice(&dev));
    KF_CUDA_CHECK(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev));
    return std::max(1, n);
}

template <int CK, int R, int STACK, int STAGES>
void launch_halo(dim3 grid, const CUtensorMap& x, const CUtensorMap& w, const HaloParams& p, size_t smem,
                 cudaStream_t st) {
    static bool configured = false;
    if (!configured) {
        KF_CUDA_CHECK(cudaFuncSetAttribute(k_conv_halo<CK, R, STACK, STAGES>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024));
        configured = true;
    }
    k_conv_halo<CK, R, STACK, STAGES><<<grid, kHaloThreads, smem, st>>>(x, w, p);
    KF_CUDA_CHECK(cudaGetLastError());
}

// One instantiation per (rows per tile, stacked rows, stages): R = 8 comes with n_tile <= 32
// and R = 4 with n_tile <= 64, so STACK = 3; R = 2 with n_tile <= 128 (STACK 2 or 3); R = 1
// with n_tile > 128 (STACK 1). halo_shape takes no other pair.
template <int CK, int STAGES>
bool launch_halo_stages(dim3 grid, const CUtensorMap& x, const CUtensorMap& w, const HaloParams& p, size_t smem,
                        cudaStream_t st) {
    if (p.R == 8 && p.stack == 3 && STAGES == 2) launch_halo<CK, 8, 3, 2>(grid, x, w, p, smem, st);
    else if (p.R == 4 && p.stack == 3) launch_halo<CK, 4, 3, STAGES>(grid, x, w, p, smem, st);
    else if (p.R == 2 && p.stack == 2) launch_halo<CK, 2, 2, STAGES>(grid, x, w, p, smem, st);
    else if (p.R == 2 && p.stack == 3) launch_halo<CK, 2, 3, STAGES>(grid, x, w, p, smem, st);
    else if (p.R == 1 && p.stack == 1) launch_halo<CK, 1, 1, STAGES>(grid, x, w, p, smem, st);
    else return false;
    return true;
}
template <int CK> void launch_halo_ck(dim3 grid, const CUtensorMap& x, const CUtensorMap& w, const HaloParams& p,
                                      int stages, size_t smem, cudaStream_t st) {
    const bool ok = stages == 2 ? launch_halo_stages<CK, 2>(grid, x, w, p, smem, st)
                                : launch_halo_stages<CK, 3>(grid, x, w, p, smem, st);
    if (!ok) throw KfError(KF_ERR_INTERNAL, "conv3x3: no halo kernel for this tile shape");
}

// The halo kernel for images at least 96 pixels wide. Returns 0 when no shape
// fits (the caller takes the per-tile kernel), 1 when it ran, 2 when it also did the fused work.
int conv3x3_halo(const __nv_bfloat16* x, int N, int H, int W, int Cin, const __nv_bfloat16* w, int Cout_rows,
                 const float* bias, int Cout, bool relu, __nv_bfloat16* y, int y_cstride, int y_coff,
                 cudaStream_t st, float* y_f32, const ConvFuse* fuse) {
    const int n_tile = Cout_rows <= 256 ? Cout_rows : 128;
    HaloShape h;
    // a tile is 128 pixels of one row: from 96 pixels wide on, at most a quarter of its
    // rows are padding (the per-tile kernel takes narrower images)
    if (W < 96 || !halo_shape(Cin, n_tile, h)) return 0;
    // input NHWC: dims (Cin, W, H, N), a box of CK channels x 130 pixels x (R + 2) rows,
    // swizzled like the weights (CK x 2 bytes per row)
    const uint64_t xdims[4] = {(uint64_t)Cin, (uint64_t)W, (uint64_t)H, (uint64_t)N};
    const uint64_t xstr[3] = {(uint64_t)Cin * 2, (uint64_t)W * Cin * 2, (uint64_t)H * W * Cin * 2};
    const uint32_t xbox[4] = {(uint32_t)h.CK, (uint32_t)kHaloW, (uint32_t)h.R + 2, 1};
    const CUtensorMap mx = make_map(x, 4, xdims, xstr, xbox,
                                    h.CK == 32 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_32B);
    const uint64_t wdims[3] = {(uint64_t)Cin, (uint64_t)Cout_rows, 9};
    const uint64_t wstr[2] = {(uint64_t)Cin * 2, (uint64_t)Cout_rows * Cin * 2};
    const uint32_t wbox[3] = {(uint32_t)h.CK, (uint32_t)n_tile, 1};  // one tap per copy
    const CUtensorMap mw = make_map(w, 3, wdims, wstr, wbox,
                                    h.CK == 32 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_32B);
    HaloParams p{};
    p.N = N; p.H = H; p.W = W; p.Cin = Cin; p.Cout = Cout;
    p.n_tile = n_tile;
    p.R = h.R;
    p.kchunks = Cin / h.CK;
    p.tiles_x = (W + 127) / 128;
    p.tiles_y = (H + h.R - 1) / h.R;
    p.num_tiles = p.tiles_x * p.tiles_y * N;
    p.w_resident = h.w_resident ? 1 : 0;
    p.stack = halo_stack(n_tile);
    p.halo_bytes = h.halo_bytes;
    p.halo_stride = h.halo_stride;
    p.w_bytes = h.w_bytes;
    p.w_stride = h.w_stride;
    p.tmem_cols = pow2_at_least((uint32_t)(2 * h.R * n_tile));
    p.bias = bias;
    p.relu = relu ? 1 : 0;
    p.out = y;
    p.outf = y_f32;
    p.out_cstride = y_cstride;
    p.out_coff = y_coff;
    bool fused = false;
    // pooling pairs rows inside a tile (R even) and reads the right neighbour's lane
    if (fuse && fuse->pool_out && y && !y_f32 && Cout % 8 == 0 && n_tile % 8 == 0 && h.R % 2 == 0 && H % 2 == 0 &&
        W % 2 == 0) {
        p.pool_out = fuse->pool_out;
        fused = true;
    }
    const int slices = (Cout_rows + n_tile - 1) / n_tile;
    const int per_slice = std::max(1, num_sms() / slices);
    const dim3 grid((unsigned)std::min(p.num_tiles, per_slice), (unsigned)slices, 1);
    if (h.CK == 32)
        launch_halo_ck<32>(grid, mx, mw, p, h.stages, h.smem, st);
    else
        launch_halo_ck<16>(grid, mx, mw, p, h.stages, h.smem, st);
    return fused ? 2 : 1;
}

} // namespace

bool conv3x3_bf16(const __nv_bfloat16* x, int N, int H, int W, int Cin, const __nv_bfloat16* w, int Cout_rows,
                  const float* bias, int Cout, bool relu, __nv_bfloat16* y, int y_cstride, int y_coff,
                  cudaStream_t st, float* y_f32, const ConvFuse* fuse) {
    KF_REQUIRE(N > 0 && H > 0 && W > 0, KF_ERR_INVALID_ARGUMENT, "conv3x3: empty tensor");
    KF_REQUIRE(y || y_f32, KF_ERR_INVALID_ARGUMENT, "conv3x3: no output tensor");
    KF_REQUIRE((Cin % 32 == 0 && Cin > 0) || Cin == 16, KF_ERR_INVALID_ARGUMENT,
               "conv3x3: input channels must be 16 or a multiple of 32");
    KF_REQUIRE(Cout > 0 && Cout <= Cout_rows && Cout_rows % 16 == 0, KF_ERR_INVALID_ARGUMENT,
               "conv3x3: weight rows must be a multiple of 16 covering the output channels");
    KF_REQUIRE(y_coff >= 0 && y_coff + Cout <= y_cstride, KF_ERR_INVALID_ARGUMENT, "conv3x3: output slice");
    // the epilogue stores 8 BF16 channels as one 16-byte word where the slice allows it
    KF_REQUIRE(((uintptr_t)x & 15) == 0 && ((uintptr_t)w & 15) == 0 && ((uintptr_t)y & 15) == 0 &&
                   ((uintptr_t)y_f32 & 3) == 0,
               KF_ERR_INVALID_ARGUMENT, "conv3x3: tensors must be 16-byte aligned (FP32 output: 4-byte)");
    KF_REQUIRE(!fuse || !fuse->pool_out || (((uintptr_t)fuse->pool_out & 15) == 0 && Cout % 8 == 0),
               KF_ERR_INVALID_ARGUMENT, "conv3x3: pooled output must be 16-byte aligned with Cout % 8 == 0");
    const int halo = conv3x3_halo(x, N, H, W, Cin, w, Cout_rows, bias, Cout, relu, y, y_cstride, y_coff, st, y_f32,
                                  fuse);
    if (halo) return halo == 2;
    KF_REQUIRE(Cin % 32 == 0, KF_ERR_INVALID_ARGUMENT,
               "conv3x3: 16 input channels need an image the halo kernel takes (at least 96 wide)");
    // narrow images: one CTA per tile of bw x bh = 128 pixels, 9 tap-shifted boxes per chunk
    int bw = 128;
    while (bw > W && bw > 8) bw >>= 1;
    const int bh = 128 / bw;
    const uint64_t adims[4] = {(uint64_t)Cin, (uint64_t)W, (uint64_t)H, (uint64_t)N};
    const uint64_t astr[3] = {(uint64_t)Cin * 2, (uint64_t)W * Cin * 2, (uint64_t)H * W * Cin * 2};
    const uint32_t abox[4] = {32, (uint32_t)bw, (uint32_t)bh, 1};
    const CUtensorMap ma = make_map(x, 4, adims, astr, abox, CU_TENSOR_MAP_SWIZZLE_64B);
    const int n_tile = Cout_rows <= 256 ? Cout_rows : 128;
    const uint64_t bdims[3] = {(uint64_t)Cin, (uint64_t)Cout_rows, 9};
    const uint64_t bstr[2] = {(uint64_t)Cin * 2, (uint64_t)Cout_rows * Cin * 2};
    const uint32_t bbox[3] = {32, (uint32_t)n_tile, 1};
    const CUtensorMap mb = make_map(w, 3, bdims, bstr, bbox, CU_TENSOR_MAP_SWIZZLE_64B);
    TcParams p{};
    p.N = N; p.H = H; p.W = W; p.Cin = Cin; p.Cout = Cout;
    p.bw = bw; p.bh = bh;
    p.tiles_x = (W + bw - 1) / bw;
    p.tiles_y = (H + bh - 1) / bh;
    p.n_tile = n_tile;
    p.kchunks = Cin / 32;
    p.k_iters = 9 * p.kchunks;
    p.k_per_split = p.k_iters;
    p.bias = bias;
    p.relu = relu ? 1 : 0;
    p.out = y;
    p.outf = y_f32;
    p.out_cstride = y_cstride;
    p.out_coff = y_coff;
    p.tmem_cols = pow2_at_least((uint32_t)n_tile);
    const dim3 grid((unsigned)(p.tiles_x * p.tiles_y * N), (unsigned)((Cout_rows + n_tile - 1) / n_tile), 1);
    // short K loops (Cin <= 64: 9 or 18 steps) take a 2-stage ring: half the shared memory,
    // twice the resident CTAs, so one CTA's epilogue overlaps the others' loads and MMAs
    if (p.k_iters <= 18)
        launch_tc<0, 64, 2>(grid, ma, mb, p, st);
    else
        launch_tc<0, 64, 3>(grid, ma, mb, p, st);
    return false;
}

void gemm_bf16_tn(const __nv_bfloat16* a, int M, const __nv_bfloat16* b, int N, int K, float* d, int ldd, int splits,
                  cudaStream_t st) {
    KF_REQUIRE(M > 0 && N > 0 && K > 0, KF_ERR_INVALID_ARGUMENT, "gemm: empty operand");
    KF_REQUIRE(K % 8 == 0, KF_ERR_INVALID_ARGUMENT, "gemm: K must be a multiple of 8 (16-byte rows)");
    KF_REQUIRE(((uintptr_t)a & 15) == 0 && ((uintptr_t)b & 15) == 0, KF_ERR_INVALID_ARGUMENT,
               "gemm: operands must be 16-byte aligned");
    KF_REQUIRE(d && ((uintptr_t)d & 3) == 0 && ldd >= N, KF_ERR_INVALID_ARGUMENT,
               "gemm: output must be 4-byte aligned with ldd >= n");
    const int n_tile = N <= 256 ? ((N + 15) / 16) * 16 : 128;
    const uint64_t adims[2] = {(uint64_t)K, (uint64_t)M};
    const uint64_t astr[1] = {(uint64_t)K * 2};
    const uint32_t abox[2] = {64, 128};
    const CUtensorMap ma = make_map(a, 2, adims, astr, abox, CU_TENSOR_MAP_SWIZZLE_128B);
    const uint64_t bdims[2] = {(uint64_t)K, (uint64_t)N};
    const uint64_t bstr[1] = {(uint64_t)K * 2};
    const uint32_t bbox[2] = {64, (uint32_t)n_tile};
    const CUtensorMap mb = make_map(b, 2, bdims, bstr, bbox, CU_TENSOR_MAP_SWIZZLE_128B);
    TcParams p{};
    p.n_tile = n_tile;
    p.outf = d;
    p.ldo = ldd;
    p.M_valid = M;
    p.N_valid = N;
    p.k_iters = (K + 63) / 64;
    const int sp = std::max(1, std::min(splits, p.k_iters));
    p.k_per_split = (p.k_iters + sp - 1) / sp;
    p.tmem_cols = pow2_at_least((uint32_t)n_tile);
    const dim3 grid((unsigned)((M + 127) / 128), (unsigned)((N + n_tile - 1) / n_tile),
                    (unsigned)((p.k_iters + p.k_per_split - 1) / p.k_per_split));
    launch_tc<1, 128, 4>(grid, ma, mb, p, st);
}

namespace {
// One thread waits on an mbarrier that nothing arrives on, through the same bounded wait the
// tensor-core kernels use: it gives up after `budget` SM cycles and records `code`.
__global__ void k_wait_probe(long long budget, uint32_t code) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        tc::mbar_init(&bar, 1);
        tc::fence_barrier_init();
        if (!tc::mbar_wait(&bar, 0, budget)) set_error(code);
    }
}
} // namespace

void tc_wait_probe(long long budget_cycles, cudaStream_t st) {
    KF_REQUIRE(budget_cycles > 0 && budget_cycles <= kWaitBudget, KF_ERR_INVALID_ARGUMENT,
               "wait probe: budget must be in (0, 2e9] cycles");
    k_wait_probe<<<1, 32, 0, st>>>(budget_cycles, kWaitProbeError);
    KF_CUDA_CHECK(cudaGetLastError());
}

uint32_t tc_take_error() {
    uint32_t e = 0, z = 0;
    KF_CUDA_CHECK(cudaMemcpyFromSymbol(&e, g_tc_error, sizeof(e)));
    KF_CUDA_CHECK(cudaMemcpyToSymbol(g_tc_error, &z, sizeof(z)));
    return e;
}

} // namespace kf
