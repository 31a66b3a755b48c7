// kf_tone.cuh — the denoiser's working space: g(x) = asinh(x / kTone) of linear radiance
// and its inverse. g'(x) = 1 / sqrt(x^2 + kTone^2), so errors in g space weigh like the
// relMSE metric (x - ref)^2 / (ref^2 + 1e-2).
#pragma once

namespace kf {

constexpr float kTone = 0.1f;
__device__ __forceinline__ float tone(float x) { return asinhf(fmaxf(x, 0.0f) * (1.0f / kTone)); }
__device__ __forceinline__ float untone(float y) { return kTone * sinhf(fmaxf(y, 0.0f)); }

} // namespace kf
