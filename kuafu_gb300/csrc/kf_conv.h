// kf_conv.h — tensor-core convolution / GEMM launchers (kf_conv.cu).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace kf {

// Work a convolution can take over from the pass that follows it: 2x2 average pooling of
// its BF16 output into a dense [N][H/2][W/2][Cout] tensor. The values equal those of the
// separate pass (both read the BF16-rounded outputs).
struct ConvFuse {
    __nv_bfloat16* pool_out = nullptr;
};

// y[n, y, x, y_coff + co] = act(bias[co] + sum_{tap, ci} x[n, y+dy, x+dx, ci] * w[tap][co][ci])
// NHWC BF16, zero padding, FP32 accumulation on tcgen05. w is [9][Cout_rows][Cin] with
// Cout_rows a multiple of 16 (rows >= Cout are computed and dropped); Cin % 32 == 0, or
// Cin == 16 for images at least 96 wide.
// With y_f32 set, the output is written there in FP32 (same strides) and y is unused.
// Returns true when it also did the fused work asked for in `fuse` (the persistent halo
// kernel does it for suitable shapes; otherwise the caller runs the separate pass).
bool conv3x3_bf16(const __nv_bfloat16* x, int N, int H, int W, int Cin, const __nv_bfloat16* w, int Cout_rows,
                  const float* bias, int Cout, bool relu, __nv_bfloat16* y, int y_cstride, int y_coff,
                  cudaStream_t st, float* y_f32 = nullptr, const ConvFuse* fuse = nullptr);

// d[m][n] += sum_k a[m][k] * b[n][k]   (BF16 K-major operands, FP32 atomics; split-K over `splits`)
void gemm_bf16_tn(const __nv_bfloat16* a, int M, const __nv_bfloat16* b, int N, int K, float* d, int ldd, int splits,
                  cudaStream_t st);

// Reads and clears the error word the tensor-core kernels set when a bounded wait expires.
uint32_t tc_take_error();
// Error word a wait probe leaves when its wait gives up.
constexpr uint32_t kWaitProbeError = 99;
// Launches a kernel whose wait on a barrier that nothing arrives on gives up after
// budget_cycles SM cycles and sets the error word to kWaitProbeError (no fault: the
// context stays usable).
void tc_wait_probe(long long budget_cycles, cudaStream_t st);

} // namespace kf
