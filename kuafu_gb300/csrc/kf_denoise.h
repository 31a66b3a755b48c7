// kf_denoise.h — learned U-Net denoiser (kf_denoise.cu).
#pragma once

#include <cstddef>
#include <cstdint>

struct kf_renderer_s;
struct kf_scene_s;
struct kf_camera_s;
struct kf_denoiser_s;

namespace kf {

using kf_denoiser_impl = ::kf_denoiser_s;

kf_denoiser_impl* denoiser_create(kf_renderer_s* r, uint32_t seed);
void denoiser_destroy(kf_denoiser_impl* d);
size_t denoiser_num_params(const kf_denoiser_impl* d);
uint32_t denoiser_num_views(const kf_denoiser_impl* d);
kf_renderer_s* denoiser_renderer(const kf_denoiser_impl* d);
void denoiser_get_params(kf_denoiser_impl* d, float* out, size_t n);
void denoiser_set_params(kf_denoiser_impl* d, const float* in, size_t n);

// Tensor-level entry points (device pointers): feat [n][h][w][32] BF16, out [n][h][w][4] FP32,
// tgt [n][h][w] float4 linear radiance. h and w divisible by 16.
// base (optional): FP32 [n][h][w] float4 residual added to the network output.
void denoiser_forward(kf_denoiser_impl* d, const void* feat, const void* base, int n, int h, int w, void* out);
float denoiser_train_step(kf_denoiser_impl* d, const void* feat, const void* base, const float* tgt, int n, int h,
                          int w, float lr, float* grads_out, bool apply_update);

// The network input kf_denoiser_apply builds from the camera's current frame (padded to 16).
void denoiser_camera_features(kf_denoiser_impl* d, kf_camera_s* c, void* feat, float* base);
// Renders training pairs of a camera: one frame of low_spp[i] samples per input and one
// target (high_frames x high_spp, FP64 accumulation) that all num_inputs inputs share.
void denoiser_add_view(kf_denoiser_impl* d, kf_scene_s* s, kf_camera_s* c, const uint32_t* low_spp,
                       uint32_t num_inputs, uint32_t high_spp, uint32_t high_frames);
// Adam over random crops of the training views; returns the mean loss of the iterations.
float denoiser_train(kf_denoiser_impl* d, uint32_t iters, uint32_t batch, uint32_t crop, float lr);
// Denoises the camera's accumulated radiance into its denoised target.
void denoiser_apply(kf_denoiser_impl* d, kf_camera_s* c);
// context.cpp:651-670: the denoised image replaces the presented one. Here the BGRA
// frame is re-encoded from the denoised target; the running mean stays as rendered.
void present_denoised(kf_renderer_s* r, kf_camera_s* c);

} // namespace kf
