// kf_denoise.cu — the learned denoiser that replaces kuafu's OptiX pass
// (src/core/denoiser.cpp:257-316, context.cpp:651-670): a 5-level U-Net of 3x3
// convolutions (32 / 64 / 96 / 128 / 160 channels) over noisy radiance, albedo,
// normal and depth, trained on low-spp / high-spp pairs this tracer renders.
//
// Every convolution (forward, backward-data) and every weight gradient runs on the
// tcgen05 kernels of kf_conv.cu (BF16 operands, FP32 accumulation). Activations
// and activation gradients are BF16 NHWC; master weights, weight gradients and
// Adam moments are FP32. Skip connections are written by the encoder straight
// into the channel slice of the decoder's concatenation buffer.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

#include "kf_conv.h"
#include "kf_denoise.h"
#include "kf_host.h"
#include "kf_tone.cuh"

namespace kf {

namespace {

using bf16 = __nv_bfloat16;

// ---------------------------------------------------------------------------
// Elementwise kernels (HBM-bound, NHWC with channel stride / offset). Channel counts,
// strides and offsets of pooled / upsampled tensors are multiples of 8, so each thread
// moves 8 channels (16 bytes) per access.
// ---------------------------------------------------------------------------
struct F8 {
    float v[8];
};
__device__ __forceinline__ F8 ld8(const bf16* p) {
    const uint4 q = *reinterpret_cast<const uint4*>(p);
    const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&q);
    F8 f;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float2 t = __bfloat1622float2(h[k]);
        f.v[2 * k] = t.x;
        f.v[2 * k + 1] = t.y;
    }
    return f;
}
__device__ __forceinline__ void st8(bf16* p, const F8& f) {
    uint4 q;
    __nv_bfloat162* h = reinterpret_cast<__nv_bfloat162*>(&q);
#pragma unroll
    for (int k = 0; k < 4; ++k) h[k] = __floats2bfloat162_rn(f.v[2 * k], f.v[2 * k + 1]);
    *reinterpret_cast<uint4*>(p) = q;
}

// y (dense, H/2 x W/2) = 2x2 average of x[slice] (H x W)
__global__ void k_pool_fwd(const bf16* __restrict__ x, int xs, int xo, int C, int N, int H, int W, bf16* y) {
    const int Ho = H / 2, Wo = W / 2, G = C / 8;
    const size_t total = (size_t)N * Ho * Wo * G;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const int g = (int)(i % G);
        const size_t pix = i / G; // (n, yh, xw) of the output
        const int xw = (int)(pix % Wo);
        const size_t ny = pix / Wo; // n * Ho + yh
        const size_t row0 = (2 * ny) * W + 2 * xw; // n * H + 2 yh == 2 * (n * Ho + yh)
        F8 a = ld8(x + row0 * xs + xo + 8 * g), b = ld8(x + (row0 + 1) * xs + xo + 8 * g);
        const F8 c = ld8(x + (row0 + W) * xs + xo + 8 * g), d = ld8(x + (row0 + W + 1) * xs + xo + 8 * g);
#pragma unroll
        for (int k = 0; k < 8; ++k) a.v[k] = 0.25f * (((a.v[k] + b.v[k]) + c.v[k]) + d.v[k]);
        st8(y + pix * C + 8 * g, a);
    }
}

// gx (dense, H x W) = broadcast(gy / 4) + gskip[slice] (optional)
__global__ void k_pool_bwd_add(const bf16* __restrict__ gy, const bf16* __restrict__ gskip, int ss, int so, int C,
                               int N, int H, int W, bf16* gx) {
    const int G = C / 8;
    const size_t total = (size_t)N * H * W * G;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const int g = (int)(i % G);
        const size_t pix = i / G;
        const int xw = (int)(pix % W);
        const size_t ny = pix / W; // n * H + y
        const size_t low = (ny / 2) * (W / 2) + xw / 2;
        F8 v = ld8(gy + low * C + 8 * g);
#pragma unroll
        for (int k = 0; k < 8; ++k) v.v[k] *= 0.25f;
        if (gskip) {
            const F8 sk = ld8(gskip + pix * ss + so + 8 * g);
#pragma unroll
            for (int k = 0; k < 8; ++k) v.v[k] += sk.v[k];
        }
        st8(gx + pix * C + 8 * g, v);
    }
}

// nearest 2x upsampling of x (dense, H/2 x W/2) into y[slice] (H x W)
__global__ void k_up_fwd(const bf16* __restrict__ x, int C, int N, int H, int W, bf16* y, int ys, int yo) {
    const int Ho = H / 2, Wo = W / 2, G = C / 8;
    const size_t total = (size_t)N * Ho * Wo * G;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const int g = (int)(i % G);
        const size_t pix = i / G;
        const int xw = (int)(pix % Wo);
        const size_t ny = pix / Wo;
        const uint4 q = *reinterpret_cast<const uint4*>(x + pix * C + 8 * g);
        const size_t row0 = (2 * ny) * W + 2 * xw;
        *reinterpret_cast<uint4*>(y + row0 * ys + yo + 8 * g) = q;
        *reinterpret_cast<uint4*>(y + (row0 + 1) * ys + yo + 8 * g) = q;
        *reinterpret_cast<uint4*>(y + (row0 + W) * ys + yo + 8 * g) = q;
        *reinterpret_cast<uint4*>(y + (row0 + W + 1) * ys + yo + 8 * g) = q;
    }
}

// gx (dense, H/2 x W/2) = sum of the 2x2 block of gy[slice] (H x W)
__global__ void k_up_bwd(const bf16* __restrict__ gy, int gs, int go, int C, int N, int H, int W, bf16* gx) {
    const int Ho = H / 2, Wo = W / 2, G = C / 8;
    const size_t total = (size_t)N * Ho * Wo * G;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const int g = (int)(i % G);
        const size_t pix = i / G;
        const int xw = (int)(pix % Wo);
        const size_t ny = pix / Wo;
        const size_t row0 = (2 * ny) * W + 2 * xw;
        F8 a = ld8(gy + row0 * gs + go + 8 * g), b = ld8(gy + (row0 + 1) * gs + go + 8 * g);
        const F8 c = ld8(gy + (row0 + W) * gs + go + 8 * g), d = ld8(gy + (row0 + W + 1) * gs + go + 8 * g);
#pragma unroll
        for (int k = 0; k < 8; ++k) a.v[k] = ((a.v[k] + b.v[k]) + c.v[k]) + d.v[k];
        st8(gx + pix * C + 8 * g, a);
    }
}

// dz[p][c] = (c < C) ? gy[p][c] * (relu ? y[p][c] > 0 : 1) : 0   for c < Ck (dense, Ck channels)
__global__ void k_relu_mask(const bf16* __restrict__ gy, int gs, int go, const bf16* __restrict__ y, int ys, int yo,
                            int C, int Ck, size_t P, int relu, bf16* dz) {
    const bool vec = (C % 8) == 0 && (gs % 8) == 0 && (go % 8) == 0 && (!relu || ((ys % 8) == 0 && (yo % 8) == 0));
    if (vec) {
        const int G = Ck / 8, Gc = C / 8;
        const size_t total = P * G;
        for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
            const int g = (int)(i % G);
            const size_t p = i / G;
            F8 v;
            if (g < Gc) {
                v = ld8(gy + p * gs + go + 8 * g);
                if (relu) {
                    const F8 m = ld8(y + p * ys + yo + 8 * g);
#pragma unroll
                    for (int k = 0; k < 8; ++k)
                        if (!(m.v[k] > 0.0f)) v.v[k] = 0.0f;
                }
            } else {
#pragma unroll
                for (int k = 0; k < 8; ++k) v.v[k] = 0.0f;
            }
            st8(dz + p * Ck + 8 * g, v);
        }
        return;
    }
    const size_t total = P * Ck;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const int c = (int)(i % Ck);
        const size_t p = i / Ck;
        float v = 0.0f;
        if (c < C) {
            v = __bfloat162float(gy[p * gs + go + c]);
            if (relu && !(__bfloat162float(y[p * ys + yo + c]) > 0.0f)) v = 0.0f;
        }
        dz[i] = __float2bfloat16_rn(v);
    }
}

// db[c] += sum_p dz[p][c]
__global__ void k_bias_grad(const bf16* __restrict__ dz, int Ck, int C, size_t P, float* db) {
    const int c = blockIdx.y;
    float s = 0.0f;
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < P; p += (size_t)gridDim.x * blockDim.x)
        s += __bfloat162float(dz[p * Ck + c]);
    for (int off = 16; off; off >>= 1) s += __shfl_xor_sync(0xFFFFFFFFu, s, off);
    __shared__ float sm[32];
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        s = threadIdx.x < (blockDim.x >> 5) ? sm[threadIdx.x] : 0.0f;
        for (int off = 16; off; off >>= 1) s += __shfl_xor_sync(0xFFFFFFFFu, s, off);
        if (threadIdx.x == 0 && c < C) atomicAdd(db + c, s);
    }
}

// t[c][p] = x[n, y+dy, x+dx, c] (0 outside the image and for P <= p < Pk): the K-major
// operand of one filter tap's weight gradient, rows padded to Pk (a multiple of 8).
__global__ void k_shift_transpose(const bf16* __restrict__ x, int xs, int xo, int C, int N, int H, int W, int dy,
                                  int dx, size_t Pk, bf16* t) {
    __shared__ bf16 tile[32][33];
    const size_t P = (size_t)N * H * W;
    const size_t p0 = (size_t)blockIdx.x * 32;
    const int c0 = blockIdx.y * 32;
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        const size_t p = p0 + k;
        const int c = c0 + threadIdx.x;
        bf16 v = __float2bfloat16_rn(0.0f);
        if (p < P && c < C) {
            const int xw = (int)(p % W);
            const size_t r = p / W;
            const int yh = (int)(r % H);
            const int n = (int)(r / H);
            const int sy = yh + dy, sx = xw + dx;
            if (sy >= 0 && sy < H && sx >= 0 && sx < W) v = x[(((size_t)n * H + sy) * W + sx) * xs + xo + c];
        }
        tile[k][threadIdx.x] = v;
    }
    __syncthreads();
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        const int c = c0 + k;
        const size_t p = p0 + threadIdx.x;
        if (c < C && p < Pk) t[(size_t)c * Pk + p] = tile[threadIdx.x][k];
    }
}

// Adam on FP32 master weights (Kingma & Ba 2015).
__global__ void k_adam(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                       size_t n, float lr, float b1, float b2, float eps, float bc1, float bc2) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.0f - b1) * gi;
        const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        w[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
    }
}

// BF16 forward weights wf[tap][co][ci] (rows >= cout zero) and backward-data weights
// wb[8 - tap][ci][co] (co >= cout zero) from FP32 master W[tap][co][ci].
__global__ void k_pack_layer(const float* __restrict__ W, int cin, int cout, int rows, int cout_k, bf16* wf, bf16* wb) {
    const size_t total = (size_t)9 * rows * cin;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const int ci = (int)(i % cin);
        const size_t r = i / cin;
        const int co = (int)(r % rows);
        const int tap = (int)(r / rows);
        const float v = co < cout ? W[((size_t)tap * cout + co) * cin + ci] : 0.0f;
        wf[i] = __float2bfloat16_rn(v);
        if (co < cout_k) wb[((size_t)(8 - tap) * cin + ci) * cout_k + co] = __float2bfloat16_rn(v);
    }
}

// out[r][c] = in[r][c] for c < cout of rows of cin channels (BF16).
__global__ void k_slice_cin(const bf16* __restrict__ in, int rows, int cin, int cout, bf16* out) {
    const size_t total = (size_t)rows * cout;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x)
        out[i] = in[(i / cout) * cin + i % cout];
}

// The network works on g(x) = tone(x) of linear radiance (kf_tone.cuh).

// Network input from render targets: g(radiance), albedo (base colour of the first hit of
// sample 0), normal, hit distance t / (1 + t), log2(samples) / 8; CH channels (32, or 16
// for the inference path whose first convolution takes 16), the rest zero. base (optional)
// receives g(radiance) in FP32: the residual the network corrects. Pixels of the padded
// tensor outside (H, W) are zero.
template <int CH>
__global__ void k_pack_features(const float4* __restrict__ rad, const float4* __restrict__ alb,
                                const float4* __restrict__ nrm, const float* __restrict__ dep, float spp_feature,
                                int H, int W, int Hp, int Wp, bf16* out, float4* base) {
    const size_t total = (size_t)Hp * Wp;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const int x = (int)(i % Wp), y = (int)(i / Wp);
        float f[32];
        for (int c = 0; c < 32; ++c) f[c] = 0.0f;
        if (x < W && y < H) {
            const size_t s = (size_t)y * W + x;
            const float4 r = rad[s], a = alb[s], n = nrm[s];
            const float d = dep[s];
            f[0] = tone(r.x);
            f[1] = tone(r.y);
            f[2] = tone(r.z);
            f[3] = a.x;
            f[4] = a.y;
            f[5] = a.z;
            f[6] = n.x;
            f[7] = n.y;
            f[8] = n.z;
            f[9] = d / (1.0f + d);
            f[10] = spp_feature;
        }
        bf16* o = out + i * CH;
#pragma unroll
        for (int g = 0; g < CH / 8; ++g) {
            F8 q;
#pragma unroll
            for (int k = 0; k < 8; ++k) q.v[k] = f[8 * g + k];
            st8(o + 8 * g, q);
        }
        if (base) base[i] = make_float4(f[0], f[1], f[2], 0.0f);
    }
}

// head[p].xyz += base[p].xyz (the residual connection around the network)
__global__ void k_add_base(float4* __restrict__ head, const float4* __restrict__ base, size_t P) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < P; i += (size_t)gridDim.x * blockDim.x) {
        const float4 b = base[i];
        float4 h = head[i];
        h.x += b.x;
        h.y += b.y;
        h.z += b.z;
        head[i] = h;
    }
}

// denoised linear radiance = g^-1(prediction + g(radiance)) for the (H, W) window: the
// residual add and the unpack in one pass, g(radiance) recomputed from the render target
// (the same function of the same value the feature pass applies, so the same bits)
__global__ void k_unpack_residual(const float4* __restrict__ pred, const float4* __restrict__ rad, int H, int W,
                                  int Wp, float4* out) {
    const size_t total = (size_t)H * W;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const int x = (int)(i % W), y = (int)(i / W);
        const float4 p = pred[(size_t)y * Wp + x], r = rad[i];
        out[i] = make_float4(untone(p.x + tone(r.x)), untone(p.y + tone(r.y)), untone(p.z + tone(r.z)), 1.0f);
    }
}


// L = mean|p - t| + lambda * mean(|dx p - dx t| + |dy p - dy t|) in g space, p the FP32
// prediction [P][4], t = g(target); writes dL/dp as the BF16 [P][32] gradient of the head.
__global__ void k_loss(const float* __restrict__ pred, const float4* __restrict__ target, int N, int H, int W,
                       float lambda, float* loss, bf16* gpred) {
    const size_t total = (size_t)N * H * W;
    const float inv = 1.0f / (float)(total * 3);
    float acc = 0.0f;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const int x = (int)(i % W);
        const int y = (int)((i / W) % H);
        const float4 t4 = target[i];
        const float tv[3] = {tone(t4.x), tone(t4.y), tone(t4.z)};
        bf16* g = gpred + i * 32;
        for (int c = 0; c < 3; ++c) {
            auto P = [&](size_t j) { return pred[j * 4 + c]; };
            auto T = [&](size_t j) {
                const float4 q = target[j];
                return tone(c == 0 ? q.x : (c == 1 ? q.y : q.z));
            };
            const float p = P(i);
            float d = p - tv[c];
            acc += fabsf(d);
            float gr = (d > 0.0f ? 1.0f : (d < 0.0f ? -1.0f : 0.0f));
            // forward differences touching pixel i: (i, i+1) and (i-1, i) in x, same in y
            if (x + 1 < W) {
                const float e = (P(i + 1) - p) - (T(i + 1) - tv[c]);
                acc += lambda * fabsf(e);
                gr -= lambda * (e > 0.0f ? 1.0f : (e < 0.0f ? -1.0f : 0.0f));
            }
            if (x > 0) {
                const float e = (p - P(i - 1)) - (tv[c] - T(i - 1));
                gr += lambda * (e > 0.0f ? 1.0f : (e < 0.0f ? -1.0f : 0.0f));
            }
            if (y + 1 < H) {
                const float e = (P(i + W) - p) - (T(i + W) - tv[c]);
                acc += lambda * fabsf(e);
                gr -= lambda * (e > 0.0f ? 1.0f : (e < 0.0f ? -1.0f : 0.0f));
            }
            if (y > 0) {
                const float e = (p - P(i - W)) - (tv[c] - T(i - W));
                gr += lambda * (e > 0.0f ? 1.0f : (e < 0.0f ? -1.0f : 0.0f));
            }
            g[c] = __float2bfloat16_rn(gr * inv);
        }
        for (int c = 3; c < 32; ++c) g[c] = __float2bfloat16_rn(0.0f);
    }
    for (int off = 16; off; off >>= 1) acc += __shfl_xor_sync(0xFFFFFFFFu, acc, off);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, acc * inv);
}

// A training target from the FP64 accumulation: sum of the frames' pixel means / frames.
__global__ void k_target_from_sum64(const dbl4* __restrict__ sum, size_t n, float4* out) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const dbl4 v = sum[i];
        const double inv = v.w > 0.0 ? 1.0 / v.w : 0.0;
        out[i] = make_float4((float)(v.x * inv), (float)(v.y * inv), (float)(v.z * inv), 1.0f);
    }
}

// crop gather: features [n][H][W][32], residual bases and targets -> batch [b][c][c]
__global__ void k_gather_crops(const bf16* __restrict__ feat, const float4* __restrict__ base,
                               const float4* __restrict__ tgt, int H, int W, const int4* __restrict__ crops, int B,
                               int c, bf16* bf, float4* bb, float4* bt) {
    const size_t total = (size_t)B * c * c;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const int x = (int)(i % c);
        const int y = (int)((i / c) % c);
        const int b = (int)(i / ((size_t)c * c));
        const int4 cr = crops[b]; // {input, y0, x0, target}
        const size_t src = ((size_t)cr.x * H + cr.y + y) * W + cr.z + x;
        const size_t src_t = ((size_t)cr.w * H + cr.y + y) * W + cr.z + x;
        const uint4* s = reinterpret_cast<const uint4*>(feat + src * 32);
        uint4* d = reinterpret_cast<uint4*>(bf + i * 32);
        for (int k = 0; k < 4; ++k) d[k] = s[k];
        bb[i] = base[src];
        bt[i] = tgt[src_t];
    }
}

inline unsigned grid_for(size_t n) { return (unsigned)std::min<size_t>((n + 255) / 256, 152 * 32); }
inline int pad32(int c) { return (c + 31) / 32 * 32; }
inline int pad16(int c) { return (c + 15) / 16 * 16; }

} // namespace

// ---------------------------------------------------------------------------
// Network
// ---------------------------------------------------------------------------
struct TRef {
    bf16* p;
    int cs, co, c; // channel stride, offset, count
};

struct Layer {
    int cin, cout, rows, cout_k;
    bool relu;
    size_t w_off, b_off;   // offsets in the FP32 parameter vector
    size_t wf_off, wb_off; // offsets in the BF16 packed weight buffers
};

struct Acts {
    int n = 0, h = 0, w = 0;
    DeviceBuffer<bf16> buf; // one arena for every activation and activation gradient
    DeviceBuffer<float> head; // FP32 network output [P][4] (log1p radiance, 0)
    std::vector<size_t> off;
    bf16* at(int k) { return buf.ptr + off[k]; }
};

// tensor ids in Acts
enum {
    T_IN, T_E0A, T_CAT0, T_P0, T_E1A, T_CAT1, T_P1, T_E2A, T_CAT2, T_P2, T_E3A, T_CAT3, T_P3, T_E4A, T_E4B, T_D3A, T_D3B,
    T_D2A, T_D2B, T_D1A, T_D1B, T_D0A, T_D0B, T_OUT,
    // gradients
    G_OUT, G_D0B, G_D0A, G_CAT0, G_D1B, G_D1A, G_CAT1, G_D2B, G_D2A, G_CAT2, G_D3B, G_D3A, G_CAT3, G_E4B, G_E4A, G_P3,
    G_E3B, G_E3A, G_P2, G_E2B, G_E2A, G_P1, G_E1B, G_E1A, G_P0, G_E0B, G_E0A, G_DZ, G_T, G_ZT,
    T_COUNT
};

} // namespace kf

// The object behind the C-ABI's kf_denoiser handle.
struct kf_denoiser_s {
    kf_renderer_s* r = nullptr;
    std::vector<kf::Layer> L;
    size_t nparams = 0, nwf = 0, nwb = 0;
    kf::DeviceBuffer<float> params, grads, m, v;
    kf::DeviceBuffer<__nv_bfloat16> wf, wb;
    kf::DeviceBuffer<__nv_bfloat16> wf0_16; // first layer, input channels 0..15 (inference)
    kf::DeviceBuffer<float> loss;
    int step = 0;
    bool packed = false;
    kf::Acts acts;
    // dataset: ds_n inputs (features + residual base), ds_targets targets; input k is
    // paired with target ds_tgt_of[k]. Capacities grow by doubling.
    int ds_h = 0, ds_w = 0, ds_n = 0, ds_targets = 0;
    size_t ds_cap_in = 0, ds_cap_tgt = 0;
    std::vector<int> ds_tgt_of;
    kf::DeviceBuffer<__nv_bfloat16> ds_feat;
    kf::DeviceBuffer<float4> ds_base, ds_tgt;
    kf::DeviceBuffer<__nv_bfloat16> batch_feat;
    kf::DeviceBuffer<float4> batch_base, batch_tgt;
    kf::DeviceBuffer<int4> crops;
    std::mt19937 rng{1234};
};

namespace kf {

namespace {

// (cin, cout, relu) of the 19 convolutions in order (encoder, bottleneck, decoder, head)
const int kLayers[19][3] = {{32, 32, 1},   {32, 32, 1},   {32, 64, 1},   {64, 64, 1},   {64, 96, 1},
                            {96, 96, 1},   {96, 128, 1},  {128, 128, 1}, {128, 160, 1}, {160, 160, 1},
                            {288, 128, 1}, {128, 128, 1}, {224, 96, 1},  {96, 96, 1},   {160, 64, 1},
                            {64, 64, 1},   {96, 32, 1},   {32, 32, 1},   {32, 3, 0}};

void build_layers(kf_denoiser_impl& d) {
    d.L.clear();
    size_t po = 0, fo = 0, bo = 0;
    for (const auto& l : kLayers) {
        Layer x;
        x.cin = l[0];
        x.cout = l[1];
        x.relu = l[2] != 0;
        x.rows = pad16(x.cout);
        x.cout_k = pad32(x.cout);
        x.w_off = po;
        po += (size_t)9 * x.cout * x.cin;
        x.b_off = po;
        po += (size_t)x.cout;
        x.wf_off = fo;
        fo += ((size_t)9 * x.rows * x.cin + 7) / 8 * 8;
        x.wb_off = bo;
        bo += ((size_t)9 * x.cin * x.cout_k + 7) / 8 * 8;
        d.L.push_back(x);
    }
    d.nparams = po;
    d.nwf = fo;
    d.nwb = bo;
}

void init_params(kf_denoiser_impl& d, uint32_t seed, cudaStream_t st) {
    std::vector<float> h(d.nparams, 0.0f);
    std::mt19937 g(seed);
    for (const Layer& l : d.L) {
        std::normal_distribution<float> nd(0.0f, std::sqrt(2.0f / (9.0f * (float)l.cin)));
        const float scale = l.relu ? 1.0f : 0.1f;
        for (size_t i = 0; i < (size_t)9 * l.cout * l.cin; ++i) h[l.w_off + i] = nd(g) * scale;
    }
    d.params.upload(h.data(), h.size(), st);
    d.grads.resize(d.nparams, st);
    d.m.resize(d.nparams, st);
    d.v.resize(d.nparams, st);
    KF_CUDA_CHECK(cudaMemsetAsync(d.m.ptr, 0, d.m.bytes(), st));
    KF_CUDA_CHECK(cudaMemsetAsync(d.v.ptr, 0, d.v.bytes(), st));
    d.wf.resize(d.nwf, st);
    d.wb.resize(d.nwb, st);
    KF_CUDA_CHECK(cudaMemsetAsync(d.wb.ptr, 0, d.wb.bytes(), st));
    d.loss.resize(4, st);
    d.packed = false;
    d.step = 0;
}

void pack(kf_denoiser_impl& d, cudaStream_t st) {
    for (const Layer& l : d.L) {
        const size_t n = (size_t)9 * l.rows * l.cin;
        k_pack_layer<<<grid_for(n), 256, 0, st>>>(d.params.ptr + l.w_off, l.cin, l.cout, l.rows, l.cout_k,
                                                  d.wf.ptr + l.wf_off, d.wb.ptr + l.wb_off);
    }
    // the first convolution's weights of input channels 0..15 alone: the inference path
    // feeds it 16-channel features (channels 11..31 of the input are always zero)
    const Layer& l0 = d.L[0];
    d.wf0_16.resize((size_t)9 * l0.rows * 16, st);
    k_slice_cin<<<grid_for((size_t)9 * l0.rows * 16), 256, 0, st>>>(d.wf.ptr + l0.wf_off, 9 * l0.rows, l0.cin, 16,
                                                                   d.wf0_16.ptr);
    KF_CUDA_CHECK(cudaGetLastError());
    d.packed = true;
}

// channel counts and spatial level of every tensor
struct TDesc {
    int c, level;
};
const TDesc kT[T_COUNT] = {
    {32, 0}, {32, 0}, {96, 0}, {32, 1}, {64, 1}, {160, 1}, {64, 2}, {96, 2}, {224, 2}, {96, 3}, {128, 3}, {288, 3},
    {128, 4}, {160, 4}, {160, 4}, {128, 3}, {128, 3}, {96, 2}, {96, 2}, {64, 1}, {64, 1}, {32, 0}, {32, 0}, {32, 0},
    // gradients
    {32, 0}, {32, 0}, {32, 0}, {96, 0}, {64, 1}, {64, 1}, {160, 1}, {96, 2}, {96, 2}, {224, 2}, {128, 3}, {128, 3},
    {288, 3}, {160, 4}, {160, 4}, {128, 4}, {128, 3}, {128, 3}, {96, 3}, {96, 2}, {96, 2}, {64, 2}, {64, 1}, {64, 1},
    {32, 1}, {32, 0}, {32, 0},
    {0, 0}, {0, 0}, {0, 0}};

void ensure_acts(kf_denoiser_impl& d, int n, int h, int w, cudaStream_t st) {
    Acts& a = d.acts;
    if (a.n == n && a.h == h && a.w == w) return;
    KF_REQUIRE(h % 16 == 0 && w % 16 == 0, KF_ERR_INVALID_ARGUMENT, "denoiser tensors need H and W divisible by 16");
    a.off.assign(T_COUNT, 0);
    size_t total = 0;
    const size_t P0 = (size_t)n * h * w;
    for (int k = 0; k < G_DZ; ++k) {
        a.off[k] = total;
        total += (P0 >> (2 * kT[k].level)) * kT[k].c;
        total = (total + 127) / 128 * 128;
    }
    // scratch: masked gradient (P0 x 160 max at any level), transposed operands
    size_t dz_max = 0, t_max = 0, zt_max = 0;
    int level[19] = {0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 3, 3, 2, 2, 1, 1, 0, 0, 0};
    for (int i = 0; i < 19; ++i) {
        const size_t P = P0 >> (2 * level[i]);
        const size_t Pk = (P + 7) / 8 * 8;
        dz_max = std::max(dz_max, P * (size_t)pad32(kLayers[i][1]));
        t_max = std::max(t_max, Pk * (size_t)kLayers[i][0]);
        zt_max = std::max(zt_max, Pk * (size_t)kLayers[i][1]);
    }
    a.off[G_DZ] = total;
    total += (dz_max + 127) / 128 * 128;
    a.off[G_T] = total;
    total += (t_max + 127) / 128 * 128;
    a.off[G_ZT] = total;
    total += (zt_max + 127) / 128 * 128;
    a.buf.resize(total, st);
    KF_CUDA_CHECK(cudaMemsetAsync(a.buf.ptr, 0, a.buf.bytes(), st));
    a.head.resize(P0 * 4, st);
    KF_CUDA_CHECK(cudaMemsetAsync(a.head.ptr, 0, a.head.bytes(), st));
    a.n = n;
    a.h = h;
    a.w = w;
}

struct Ctx {
    kf_denoiser_impl& d;
    cudaStream_t st;
    int n, h, w;
    int H(int level) const { return h >> level; }
    int W(int level) const { return w >> level; }
    size_t P(int level) const { return (size_t)n * H(level) * W(level); }
};

// The convolution, and (when `fuse` is given) the pooling / upsampling pass after it: the
// persistent conv kernel does that work in its epilogue where it can, else the pass runs here.
bool conv_fwd(Ctx& c, int li, int level, TRef x, TRef y, const ConvFuse* fuse = nullptr) {
    const Layer& l = c.d.L[li];
    return conv3x3_bf16(x.p, c.n, c.H(level), c.W(level), x.cs, c.d.wf.ptr + l.wf_off, l.rows,
                        c.d.params.ptr + l.b_off, l.cout, l.relu, y.p, y.cs, y.co, c.st, nullptr, fuse);
}

// Backward of y = act(conv(x) + b): accumulates dW, db; writes gx (if gx.p) = dL/dx.
void conv_bwd(Ctx& c, int li, int level, TRef x, TRef y, TRef gy, TRef gx) {
    const Layer& l = c.d.L[li];
    Acts& a = c.d.acts;
    const size_t P = c.P(level);
    bf16* dz = a.at(G_DZ);
    k_relu_mask<<<grid_for(P * l.cout_k), 256, 0, c.st>>>(gy.p, gy.cs, gy.co, y.p, y.cs, y.co, l.cout, l.cout_k, P,
                                                         l.relu ? 1 : 0, dz);
    k_bias_grad<<<dim3((unsigned)std::min<size_t>((P + 255) / 256, 64), (unsigned)l.cout_k), 256, 0, c.st>>>(
        dz, l.cout_k, l.cout, P, c.d.grads.ptr + l.b_off);
    // dZ^T [cout][Pk]
    const size_t Pk = (P + 7) / 8 * 8;
    bf16* zt = a.at(G_ZT);
    k_shift_transpose<<<dim3((unsigned)((Pk + 31) / 32), (unsigned)((l.cout + 31) / 32)), dim3(32, 8), 0, c.st>>>(
        dz, l.cout_k, 0, l.cout, c.n, c.H(level), c.W(level), 0, 0, Pk, zt);
    bf16* t = a.at(G_T);
    const int splits = (int)std::max<size_t>(1, std::min<size_t>(64, P / 8192));
    for (int tap = 0; tap < 9; ++tap) {
        const int dy = tap / 3 - 1, dx = tap % 3 - 1;
        k_shift_transpose<<<dim3((unsigned)((Pk + 31) / 32), (unsigned)((l.cin + 31) / 32)), dim3(32, 8), 0, c.st>>>(
            x.p, x.cs, x.co, l.cin, c.n, c.H(level), c.W(level), dy, dx, Pk, t);
        gemm_bf16_tn(zt, l.cout, t, l.cin, (int)Pk, c.d.grads.ptr + l.w_off + (size_t)tap * l.cout * l.cin, l.cin,
                     splits, c.st);
    }
    if (gx.p) {
        conv3x3_bf16(dz, c.n, c.H(level), c.W(level), l.cout_k, c.d.wb.ptr + l.wb_off, l.cin, nullptr, l.cin, false,
                     gx.p, gx.cs, gx.co, c.st);
    }
    KF_CUDA_CHECK(cudaGetLastError());
}

TRef T(Acts& a, int k) { return TRef{a.at(k), kT[k].c, 0, kT[k].c}; }
TRef S(Acts& a, int k, int off, int cnt) { return TRef{a.at(k), kT[k].c, off, cnt}; }

void pool_fwd(Ctx& c, TRef x, int level, TRef y) {
    const size_t n = c.P(level + 1) * x.c / 8;
    k_pool_fwd<<<grid_for(n), 256, 0, c.st>>>(x.p, x.cs, x.co, x.c, c.n, c.H(level), c.W(level), y.p);
}
void up_fwd(Ctx& c, TRef x, int level_hi, TRef y) {
    const size_t n = c.P(level_hi + 1) * x.c / 8;
    k_up_fwd<<<grid_for(n), 256, 0, c.st>>>(x.p, x.c, c.n, c.H(level_hi), c.W(level_hi), y.p, y.cs, y.co);
}
// conv into y, then 2x2 pooling of y into `pooled` (at level + 1)
void conv_pool(Ctx& c, int li, int level, TRef x, TRef y, TRef pooled) {
    ConvFuse f;
    f.pool_out = pooled.p;
    if (!conv_fwd(c, li, level, x, y, &f)) pool_fwd(c, y, level, pooled);
}
// conv into y, then nearest 2x upsampling of y into the channel slice `up` (at level - 1).
// A separate pass: both forms are bound by the same HBM writes of the four copies, and
// written from the conv epilogue (32-byte stores) the layer grew by what the pass takes.
void conv_up(Ctx& c, int li, int level, TRef x, TRef y, TRef up) {
    conv_fwd(c, li, level, x, y);
    up_fwd(c, y, level - 1, up);
}

// prediction (in a.head) = network(T_IN) + base (FP32 residual, optional). in16: T_IN holds
// 16-channel features (the first convolution then reads half the bytes and does half the
// MMAs; channels 16..31 of the 32-channel input are zero, so the values are the same).
void forward(Ctx& c, const float4* base, bool in16 = false) {
    Acts& a = c.d.acts;
    if (in16) {
        const Layer& l = c.d.L[0];
        conv3x3_bf16(a.at(T_IN), c.n, c.h, c.w, 16, c.d.wf0_16.ptr, l.rows, c.d.params.ptr + l.b_off, l.cout, l.relu,
                     a.at(T_E0A), 32, 0, c.st);
    } else {
        conv_fwd(c, 0, 0, T(a, T_IN), T(a, T_E0A));
    }
    conv_pool(c, 1, 0, T(a, T_E0A), S(a, T_CAT0, 64, 32), T(a, T_P0));
    conv_fwd(c, 2, 1, T(a, T_P0), T(a, T_E1A));
    conv_pool(c, 3, 1, T(a, T_E1A), S(a, T_CAT1, 96, 64), T(a, T_P1));
    conv_fwd(c, 4, 2, T(a, T_P1), T(a, T_E2A));
    conv_pool(c, 5, 2, T(a, T_E2A), S(a, T_CAT2, 128, 96), T(a, T_P2));
    conv_fwd(c, 6, 3, T(a, T_P2), T(a, T_E3A));
    conv_pool(c, 7, 3, T(a, T_E3A), S(a, T_CAT3, 160, 128), T(a, T_P3));
    conv_fwd(c, 8, 4, T(a, T_P3), T(a, T_E4A));
    conv_up(c, 9, 4, T(a, T_E4A), T(a, T_E4B), S(a, T_CAT3, 0, 160));
    conv_fwd(c, 10, 3, T(a, T_CAT3), T(a, T_D3A));
    conv_up(c, 11, 3, T(a, T_D3A), T(a, T_D3B), S(a, T_CAT2, 0, 128));
    conv_fwd(c, 12, 2, T(a, T_CAT2), T(a, T_D2A));
    conv_up(c, 13, 2, T(a, T_D2A), T(a, T_D2B), S(a, T_CAT1, 0, 96));
    conv_fwd(c, 14, 1, T(a, T_CAT1), T(a, T_D1A));
    conv_up(c, 15, 1, T(a, T_D1A), T(a, T_D1B), S(a, T_CAT0, 0, 64));
    conv_fwd(c, 16, 0, T(a, T_CAT0), T(a, T_D0A));
    conv_fwd(c, 17, 0, T(a, T_D0A), T(a, T_D0B));
    {
        const Layer& l = c.d.L[18];
        conv3x3_bf16(a.at(T_D0B), c.n, c.h, c.w, 32, c.d.wf.ptr + l.wf_off, l.rows, c.d.params.ptr + l.b_off, l.cout,
                     false, nullptr, 4, 0, c.st, a.head.ptr);
    }
    if (base)
        k_add_base<<<grid_for(c.P(0)), 256, 0, c.st>>>(reinterpret_cast<float4*>(a.head.ptr), base, c.P(0));
    KF_CUDA_CHECK(cudaGetLastError());
}

void pool_bwd_add(Ctx& c, TRef gy_low, TRef gskip, int level_hi, TRef gx) {
    const size_t n = c.P(level_hi) * gx.c / 8;
    k_pool_bwd_add<<<grid_for(n), 256, 0, c.st>>>(gy_low.p, gskip.p, gskip.cs, gskip.co, gx.c, c.n, c.H(level_hi),
                                                   c.W(level_hi), gx.p);
}
void up_bwd(Ctx& c, TRef gy_slice, int level_hi, TRef gx_low) {
    const size_t n = c.P(level_hi + 1) * gx_low.c / 8;
    k_up_bwd<<<grid_for(n), 256, 0, c.st>>>(gy_slice.p, gy_slice.cs, gy_slice.co, gx_low.c, c.n, c.H(level_hi),
                                             c.W(level_hi), gx_low.p);
}

void backward(Ctx& c) {
    Acts& a = c.d.acts;
    TRef none{nullptr, 0, 0, 0};
    conv_bwd(c, 18, 0, T(a, T_D0B), TRef{a.at(T_OUT), 32, 0, 3}, T(a, G_OUT), T(a, G_D0B));
    conv_bwd(c, 17, 0, T(a, T_D0A), T(a, T_D0B), T(a, G_D0B), T(a, G_D0A));
    conv_bwd(c, 16, 0, T(a, T_CAT0), T(a, T_D0A), T(a, G_D0A), T(a, G_CAT0));
    up_bwd(c, S(a, G_CAT0, 0, 64), 0, T(a, G_D1B));
    conv_bwd(c, 15, 1, T(a, T_D1A), T(a, T_D1B), T(a, G_D1B), T(a, G_D1A));
    conv_bwd(c, 14, 1, T(a, T_CAT1), T(a, T_D1A), T(a, G_D1A), T(a, G_CAT1));
    up_bwd(c, S(a, G_CAT1, 0, 96), 1, T(a, G_D2B));
    conv_bwd(c, 13, 2, T(a, T_D2A), T(a, T_D2B), T(a, G_D2B), T(a, G_D2A));
    conv_bwd(c, 12, 2, T(a, T_CAT2), T(a, T_D2A), T(a, G_D2A), T(a, G_CAT2));
    up_bwd(c, S(a, G_CAT2, 0, 128), 2, T(a, G_D3B));
    conv_bwd(c, 11, 3, T(a, T_D3A), T(a, T_D3B), T(a, G_D3B), T(a, G_D3A));
    conv_bwd(c, 10, 3, T(a, T_CAT3), T(a, T_D3A), T(a, G_D3A), T(a, G_CAT3));
    up_bwd(c, S(a, G_CAT3, 0, 160), 3, T(a, G_E4B));
    conv_bwd(c, 9, 4, T(a, T_E4A), T(a, T_E4B), T(a, G_E4B), T(a, G_E4A));
    conv_bwd(c, 8, 4, T(a, T_P3), T(a, T_E4A), T(a, G_E4A), T(a, G_P3));
    pool_bwd_add(c, T(a, G_P3), S(a, G_CAT3, 160, 128), 3, T(a, G_E3B));
    conv_bwd(c, 7, 3, T(a, T_E3A), S(a, T_CAT3, 160, 128), T(a, G_E3B), T(a, G_E3A));
    conv_bwd(c, 6, 3, T(a, T_P2), T(a, T_E3A), T(a, G_E3A), T(a, G_P2));
    pool_bwd_add(c, T(a, G_P2), S(a, G_CAT2, 128, 96), 2, T(a, G_E2B));
    conv_bwd(c, 5, 2, T(a, T_E2A), S(a, T_CAT2, 128, 96), T(a, G_E2B), T(a, G_E2A));
    conv_bwd(c, 4, 2, T(a, T_P1), T(a, T_E2A), T(a, G_E2A), T(a, G_P1));
    pool_bwd_add(c, T(a, G_P1), S(a, G_CAT1, 96, 64), 1, T(a, G_E1B));
    conv_bwd(c, 3, 1, T(a, T_E1A), S(a, T_CAT1, 96, 64), T(a, G_E1B), T(a, G_E1A));
    conv_bwd(c, 2, 1, T(a, T_P0), T(a, T_E1A), T(a, G_E1A), T(a, G_P0));
    pool_bwd_add(c, T(a, G_P0), S(a, G_CAT0, 64, 32), 0, T(a, G_E0B));
    conv_bwd(c, 1, 0, T(a, T_E0A), S(a, T_CAT0, 64, 32), T(a, G_E0B), T(a, G_E0A));
    conv_bwd(c, 0, 0, T(a, T_IN), T(a, T_E0A), T(a, G_E0A), none);
}

} // namespace

// ---------------------------------------------------------------------------
// Public operations
// ---------------------------------------------------------------------------
kf_denoiser_impl* denoiser_create(kf_renderer_s* r, uint32_t seed) {
    auto d = new kf_denoiser_impl();
    d->r = r;
    build_layers(*d);
    init_params(*d, seed, r->stream);
    d->rng.seed(seed ^ 0x5bd1e995u);
    return d;
}
void denoiser_destroy(kf_denoiser_impl* d) { delete d; }
size_t denoiser_num_params(const kf_denoiser_impl* d) { return d->nparams; }
uint32_t denoiser_num_views(const kf_denoiser_impl* d) { return (uint32_t)d->ds_n; }
kf_renderer_s* denoiser_renderer(const kf_denoiser_impl* d) { return d->r; }

void denoiser_get_params(kf_denoiser_impl* d, float* out, size_t n) {
    KF_REQUIRE(n >= d->nparams, KF_ERR_OUT_OF_RANGE, "parameter buffer too small");
    KF_CUDA_CHECK(cudaMemcpyAsync(out, d->params.ptr, d->nparams * 4, cudaMemcpyDeviceToHost, d->r->stream));
    KF_CUDA_CHECK(cudaStreamSynchronize(d->r->stream));
}
void denoiser_set_params(kf_denoiser_impl* d, const float* in, size_t n) {
    KF_REQUIRE(n == d->nparams, KF_ERR_INVALID_ARGUMENT, "parameter count mismatch");
    KF_CUDA_CHECK(cudaMemcpyAsync(d->params.ptr, in, d->nparams * 4, cudaMemcpyHostToDevice, d->r->stream));
    KF_CUDA_CHECK(cudaMemsetAsync(d->m.ptr, 0, d->m.bytes(), d->r->stream));
    KF_CUDA_CHECK(cudaMemsetAsync(d->v.ptr, 0, d->v.bytes(), d->r->stream));
    KF_CUDA_CHECK(cudaStreamSynchronize(d->r->stream));
    d->packed = false;
    d->step = 0;
}

// out: [n, h, w, 4] FP32 device buffer (channels 0..2 = prediction in g space, 3 = 0);
// base: optional FP32 residual [n, h, w] float4 added to the network output.
void denoiser_forward(kf_denoiser_impl* d, const void* feat, const void* base, int n, int h, int w, void* out) {
    cudaStream_t st = d->r->stream;
    ensure_acts(*d, n, h, w, st);
    if (!d->packed) pack(*d, st);
    KF_CUDA_CHECK(cudaMemcpyAsync(d->acts.at(T_IN), feat, (size_t)n * h * w * 32 * 2, cudaMemcpyDeviceToDevice, st));
    Ctx c{*d, st, n, h, w};
    forward(c, static_cast<const float4*>(base));
    if (out)
        KF_CUDA_CHECK(cudaMemcpyAsync(out, d->acts.head.ptr, (size_t)n * h * w * 16, cudaMemcpyDeviceToDevice, st));
}

float denoiser_train_step(kf_denoiser_impl* d, const void* feat, const void* base, const float* tgt, int n, int h,
                          int w, float lr, float* grads_out, bool apply_update) {
    cudaStream_t st = d->r->stream;
    denoiser_forward(d, feat, base, n, h, w, nullptr);
    Acts& a = d->acts;
    KF_CUDA_CHECK(cudaMemsetAsync(d->loss.ptr, 0, sizeof(float), st));
    const size_t P = (size_t)n * h * w;
    k_loss<<<grid_for(P), 256, 0, st>>>(a.head.ptr, reinterpret_cast<const float4*>(tgt), n, h, w, 0.5f, d->loss.ptr,
                                        a.at(G_OUT));
    KF_CUDA_CHECK(cudaMemsetAsync(d->grads.ptr, 0, d->grads.bytes(), st));
    Ctx c{*d, st, n, h, w};
    backward(c);
    if (grads_out)
        KF_CUDA_CHECK(cudaMemcpyAsync(grads_out, d->grads.ptr, d->nparams * 4, cudaMemcpyDeviceToDevice, st));
    if (apply_update) {
        ++d->step;
        const float b1 = 0.9f, b2 = 0.999f;
        const float bc1 = 1.0f - std::pow(b1, (float)d->step), bc2 = 1.0f - std::pow(b2, (float)d->step);
        k_adam<<<grid_for(d->nparams), 256, 0, st>>>(d->params.ptr, d->grads.ptr, d->m.ptr, d->v.ptr, d->nparams, lr,
                                                     b1, b2, 1e-8f, bc1, bc2);
        d->packed = false;
    }
    float loss = 0.0f;
    KF_CUDA_CHECK(cudaMemcpyAsync(&loss, d->loss.ptr, sizeof(float), cudaMemcpyDeviceToHost, st));
    KF_CUDA_CHECK(cudaStreamSynchronize(st));
    return loss;
}

// Features (and residual base) of a camera's current render targets, padded to [1][Hp][Wp].
static void camera_features(kf_camera_s* c, uint32_t samples, bf16* out, float4* base, int Hp, int Wp,
                            cudaStream_t st, bool ch16 = false) {
    const float spp_feature = std::log2((float)std::max(samples, 1u)) / 8.0f;
    const unsigned grid = grid_for((size_t)Hp * Wp);
    if (ch16)
        k_pack_features<16><<<grid, 256, 0, st>>>(c->accum.ptr, c->albedo.ptr, c->normal.ptr, c->depth.ptr,
                                                  spp_feature, c->target_h, c->target_w, Hp, Wp, out, base);
    else
        k_pack_features<32><<<grid, 256, 0, st>>>(c->accum.ptr, c->albedo.ptr, c->normal.ptr, c->depth.ptr,
                                                  spp_feature, c->target_h, c->target_w, Hp, Wp, out, base);
    KF_CUDA_CHECK(cudaGetLastError());
}

namespace {
// kuafu's frame state, restored when a training render leaves its scope
struct FrameStateGuard {
    kf_renderer_s* r;
    uint32_t accumulate;
    explicit FrameStateGuard(kf_renderer_s* rr) : r(rr), accumulate(rr->cfg.accumulate_frames) {}
    ~FrameStateGuard() {
        r->frame_count = -1;
        r->cfg.accumulate_frames = accumulate;
    }
};

template <class T> void grow(DeviceBuffer<T>& b, size_t old_n, size_t new_n, cudaStream_t st) {
    DeviceBuffer<T> nb;
    nb.resize(new_n, st);
    if (old_n) KF_CUDA_CHECK(cudaMemcpyAsync(nb.ptr, b.ptr, old_n * sizeof(T), cudaMemcpyDeviceToDevice, st));
    KF_CUDA_CHECK(cudaStreamSynchronize(st));
    b = std::move(nb);
}
} // namespace

void denoiser_add_view(kf_denoiser_impl* d, kf_scene_s* s, kf_camera_s* c, const uint32_t* low_spp,
                       uint32_t num_inputs, uint32_t high_spp, uint32_t high_frames) {
    kf_renderer_s* r = d->r;
    cudaStream_t st = r->stream;
    KF_REQUIRE(c->width % 16 == 0 && c->height % 16 == 0, KF_ERR_INVALID_ARGUMENT,
               "training views need width and height divisible by 16");
    if (d->ds_n == 0) {
        d->ds_h = c->height;
        d->ds_w = c->width;
    }
    KF_REQUIRE(c->width == d->ds_w && c->height == d->ds_h, KF_ERR_INVALID_ARGUMENT,
               "all training views must have the same size");
    const size_t npix = (size_t)c->width * c->height;
    const size_t k = (size_t)d->ds_n, t = (size_t)d->ds_targets;
    if (k + num_inputs > d->ds_cap_in) {
        const size_t cap = std::max<size_t>({k + num_inputs, 2 * d->ds_cap_in, 8});
        grow(d->ds_feat, npix * 32 * k, npix * 32 * cap, st);
        grow(d->ds_base, npix * k, npix * cap, st);
        d->ds_cap_in = cap;
    }
    if (t + 1 > d->ds_cap_tgt) {
        const size_t cap = std::max<size_t>({t + 1, 2 * d->ds_cap_tgt, 8});
        grow(d->ds_tgt, npix * t, npix * cap, st);
        d->ds_cap_tgt = cap;
    }
    FrameStateGuard guard(r);
    r->cfg.accumulate_frames = 1;
    // noisy inputs: one frame of low_spp[i] samples each (every render takes a new frame
    // index, so the inputs' random streams and the target's are independent)
    for (uint32_t i = 0; i < num_inputs; ++i) {
        r->frame_count = -1;
        render_frame(r, s, c, low_spp[i]);
        camera_features(c, low_spp[i], d->ds_feat.ptr + npix * 32 * (k + i), d->ds_base.ptr + npix * (k + i),
                        c->height, c->width, st);
    }
    // target: high_frames frames of high_spp samples, averaged from the FP64 accumulation
    r->frame_count = -1;
    for (uint32_t f = 0; f < high_frames; ++f) render_frame(r, s, c, high_spp);
    k_target_from_sum64<<<grid_for(npix), 256, 0, st>>>(c->sum64.ptr, npix, d->ds_tgt.ptr + npix * t);
    KF_CUDA_CHECK(cudaGetLastError());
    KF_CUDA_CHECK(cudaStreamSynchronize(st));
    for (uint32_t i = 0; i < num_inputs; ++i) d->ds_tgt_of.push_back((int)t);
    d->ds_n += (int)num_inputs;
    ++d->ds_targets;
}

float denoiser_train(kf_denoiser_impl* d, uint32_t iters, uint32_t batch, uint32_t crop, float lr) {
    KF_REQUIRE(d->ds_n > 0, KF_ERR_STATE, "the denoiser has no training views");
    KF_REQUIRE(crop % 16 == 0 && (int)crop <= d->ds_h && (int)crop <= d->ds_w && batch > 0, KF_ERR_INVALID_ARGUMENT,
               "crop must be a multiple of 16 no larger than the training views");
    cudaStream_t st = d->r->stream;
    const size_t per = (size_t)crop * crop;
    d->batch_feat.resize(per * 32 * batch, st);
    d->batch_base.resize(per * batch, st);
    d->batch_tgt.resize(per * batch, st);
    d->crops.resize(batch, st);
    std::vector<int4> cr(batch);
    double acc = 0.0;
    for (uint32_t it = 0; it < iters; ++it) {
        for (uint32_t b = 0; b < batch; ++b) {
            cr[b].x = (int)(d->rng() % (uint32_t)d->ds_n);
            cr[b].y = (int)(d->rng() % (uint32_t)(d->ds_h - crop + 1));
            cr[b].z = (int)(d->rng() % (uint32_t)(d->ds_w - crop + 1));
            cr[b].w = d->ds_tgt_of[(size_t)cr[b].x];
        }
        d->crops.upload(cr.data(), batch, st);
        k_gather_crops<<<grid_for(per * batch), 256, 0, st>>>(d->ds_feat.ptr, d->ds_base.ptr, d->ds_tgt.ptr, d->ds_h,
                                                              d->ds_w, d->crops.ptr, (int)batch, (int)crop,
                                                              d->batch_feat.ptr, d->batch_base.ptr, d->batch_tgt.ptr);
        acc += denoiser_train_step(d, d->batch_feat.ptr, d->batch_base.ptr,
                                   reinterpret_cast<const float*>(d->batch_tgt.ptr), (int)batch, (int)crop, (int)crop,
                                   lr, nullptr, true);
    }
    return iters ? (float)(acc / iters) : 0.0f;
}

void denoiser_camera_features(kf_denoiser_impl* d, kf_camera_s* c, void* feat, float* base) {
    kf_renderer_s* r = d->r;
    const int Hp = (c->target_h + 15) / 16 * 16, Wp = (c->target_w + 15) / 16 * 16;
    const uint32_t frames = (r->cfg.accumulate_frames && r->frame_count >= 0) ? (uint32_t)r->frame_count + 1u : 1u;
    camera_features(c, frames * std::max(r->stats.last_spp, 1u), static_cast<bf16*>(feat),
                    reinterpret_cast<float4*>(base), Hp, Wp, r->stream);
}

void denoiser_apply(kf_denoiser_impl* d, kf_camera_s* c) {
    kf_renderer_s* r = d->r;
    cudaStream_t st = r->stream;
    KF_REQUIRE(c->has_frame, KF_ERR_STATE, "the camera has no frame to denoise");
    const int Hp = (c->target_h + 15) / 16 * 16, Wp = (c->target_w + 15) / 16 * 16;
    ensure_acts(*d, 1, Hp, Wp, st);
    if (!d->packed) pack(*d, st);
    const uint32_t frames = (r->cfg.accumulate_frames && r->frame_count >= 0) ? (uint32_t)r->frame_count + 1u : 1u;
    // frames the halo convolution takes (at least 96 wide) use the 16-channel input
    const bool in16 = Wp >= 96;
    camera_features(c, frames * std::max(r->stats.last_spp, 1u), d->acts.at(T_IN), nullptr, Hp, Wp, st, in16);
    Ctx cx{*d, st, 1, Hp, Wp};
    forward(cx, nullptr, in16);
    const size_t npix = (size_t)c->target_w * c->target_h;
    if (c->denoised.count != npix) c->denoised.resize(npix, st);
    k_unpack_residual<<<grid_for(npix), 256, 0, st>>>(reinterpret_cast<const float4*>(d->acts.head.ptr),
                                                      c->accum.ptr, c->target_h, c->target_w, Wp, c->denoised.ptr);
    KF_CUDA_CHECK(cudaGetLastError());
}

} // namespace kf

namespace kf {

void present_denoised(kf_renderer_s* r, kf_camera_s* c) {
    denoiser_apply(r->denoiser, c);
    launch_srgb(c->denoised.ptr, (uint32_t)c->denoised.count, c->bgra.ptr, r->stream);
    KF_CUDA_CHECK(cudaGetLastError());
}

} // namespace kf
