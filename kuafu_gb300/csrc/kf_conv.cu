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

} // namespace

void conv3x3_bf16(const __nv_bfloat16* x, int N, int H, int W, int Cin, const __nv_bfloat16* w, int Cout_rows,
                  const float* bias, int Cout, bool relu, __nv_bfloat16* y, int y_cstride, int y_coff,
                  cudaStream_t st, float* y_f32) {
    KF_REQUIRE(N > 0 && H > 0 && W > 0, KF_ERR_INVALID_ARGUMENT, "conv3x3: empty tensor");
    KF_REQUIRE(y || y_f32, KF_ERR_INVALID_ARGUMENT, "conv3x3: no output tensor");
    KF_REQUIRE(Cin % 32 == 0 && Cin > 0, KF_ERR_INVALID_ARGUMENT, "conv3x3: input channels must be a multiple of 32");
    KF_REQUIRE(Cout > 0 && Cout <= Cout_rows && Cout_rows % 16 == 0, KF_ERR_INVALID_ARGUMENT,
               "conv3x3: weight rows must be a multiple of 16 covering the output channels");
    KF_REQUIRE(y_coff >= 0 && y_coff + Cout <= y_cstride, KF_ERR_INVALID_ARGUMENT, "conv3x3: output slice");
    KF_REQUIRE(((uintptr_t)x & 15) == 0 && ((uintptr_t)w & 15) == 0, KF_ERR_INVALID_ARGUMENT,
               "conv3x3: tensors must be 16-byte aligned");
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
}

void gemm_bf16_tn(const __nv_bfloat16* a, int M, const __nv_bfloat16* b, int N, int K, float* d, int ldd, int splits,
                  cudaStream_t st) {
    KF_REQUIRE(M > 0 && N > 0 && K > 0, KF_ERR_INVALID_ARGUMENT, "gemm: empty operand");
    KF_REQUIRE(K % 8 == 0, KF_ERR_INVALID_ARGUMENT, "gemm: K must be a multiple of 8 (16-byte rows)");
    KF_REQUIRE(((uintptr_t)a & 15) == 0 && ((uintptr_t)b & 15) == 0, KF_ERR_INVALID_ARGUMENT,
               "gemm: operands must be 16-byte aligned");
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

uint32_t tc_take_error() {
    uint32_t e = 0, z = 0;
    KF_CUDA_CHECK(cudaMemcpyFromSymbol(&e, g_tc_error, sizeof(e)));
    KF_CUDA_CHECK(cudaMemcpyToSymbol(g_tc_error, &z, sizeof(z)));
    return e;
}

} // namespace kf
