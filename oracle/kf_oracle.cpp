// kf_oracle.cpp — CPU oracle (TEST INFRASTRUCTURE ONLY; the product never links it).
//
// A scalar C++ restatement of kuafu's ray-tracing shaders, kept line-for-line
// close to the GLSL so that a reader can check it against:
//   resources/shaders/PathTrace.rgen      (ray generation, bounce loop, accumulation)
//   resources/shaders/PathTrace.rchit     (shading data, PrincipledBSDF, light loops)
//   resources/shaders/PathTrace.rahit     (stochastic alpha)
//   resources/shaders/PathTrace.rmiss     (clear colour)
//   resources/shaders/PathTraceShadow.rmiss
//   resources/shaders/base/Random.glsl, base/Sampling.glsl
// The closed Vulkan traversal (traceRayEXT) is replaced by a watertight
// ray/triangle test (Woop, Benthin, Wald 2013) over all triangles or over a
// per-geometry CPU BVH with a conservative slab test (Ize 2013).
//
// Two random-number modes:
//   PHILOX  — the product's counter-based Philox4x32-10 sub-streams (kf_types.h);
//   TEA_LCG — kuafu's own tea()/lcg()/rnd() sequence with clockARB() pinned,
//             drawing in exactly the order the shaders draw.
// Two precisions: FP32 (parity with the GPU) and FP64 (converged references).
//
// Build: g++ -O2 -ffp-contract=off -fPIC -shared -pthread (see oracle/build.py).
// Floating-point contraction is off so every a*b+c rounds twice, as on the GPU
// side (-fmad=false); fused operations appear only as explicit std::fma calls.

#include "kf_oracle.h"

#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <thread>
#include <vector>

namespace {

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy
// as 1, 2, 3", SC'11). Multipliers and Weyl constants are those of the paper.
// ---------------------------------------------------------------------------
inline void philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        if (r > 0) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c1 ^ k0, n1 = lo1, n2 = hi0 ^ c3 ^ k1, n3 = lo0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

inline float u24(uint32_t x) { return (float)(x >> 8) * (1.0f / 16777216.0f); }

// kuafu's generator (base/Random.glsl:7-39).
inline uint32_t tea(uint32_t val0, uint32_t val1) {
    uint32_t v0 = val0, v1 = val1, s0 = 0;
    for (uint32_t n = 0; n < 16; n++) {
        s0 += 0x9e3779b9u;
        v0 += ((v1 << 4) + 0xa341316cu) ^ (v1 + s0) ^ ((v1 >> 5) + 0xc8013ea4u);
        v1 += ((v0 << 4) + 0xad90777du) ^ (v0 + s0) ^ ((v0 >> 5) + 0x7e95761eu);
    }
    return v0;
}
inline uint32_t lcg(uint32_t& prev) {
    prev = 1664525u * prev + 1013904223u;
    return prev & 0x00FFFFFFu;
}
inline float rnd_lcg(uint32_t& prev) { return (float)lcg(prev) / (float)0x01000000; }

// ---------------------------------------------------------------------------
// Deterministic single-precision transcendentals. The shaders call cos/sin
// (sampling directions, spot-cone test) and pow (Schlick terms). To make the
// GPU and CPU bit-identical both sides evaluate the same published method:
// Cody-Waite reduction by pi/2 in three float parts (Cody & Waite, "Software
// Manual for the Elementary Functions", 1980) followed by the Taylor series
// of sin / cos on [-pi/4, pi/4]; exp2 by x = k + f, |f| <= 1/2, and the Taylor
// series of e^(f ln 2). Constants are the exact values rounded to float
// (derived with mpmath). Accuracy <= 2 ulp over the ranges the shaders use.
// ---------------------------------------------------------------------------
constexpr float kPio2Hi = 0x1.921fb6p+0f;
constexpr float kPio2Mid = -0x1.777a5cp-25f;
constexpr float kPio2Lo = -0x1.ee59dap-50f;
constexpr float kTwoOverPi = 0x1.45f306p-1f;

inline float poly_sin(float r) {
    float r2 = r * r;
    float p = std::fma(r2, 0x1.71de3ap-19f, -0x1.a01a02p-13f);
    p = std::fma(r2, p, 0x1.111112p-7f);
    p = std::fma(r2, p, -0x1.555556p-3f);
    return std::fma(r * r2, p, r);
}
inline float poly_cos(float r) {
    float r2 = r * r;
    float p = std::fma(r2, -0x1.27e4fcp-22f, 0x1.a01a02p-16f);
    p = std::fma(r2, p, -0x1.6c16c2p-10f);
    p = std::fma(r2, p, 0x1.555556p-5f);
    p = std::fma(r2, p, -0.5f);
    return std::fma(r2, p, 1.0f);
}
inline float reduce_pio2(float x, int& q) {
    float k = std::nearbyint(x * kTwoOverPi);
    float r = std::fma(-k, kPio2Hi, x);
    r = std::fma(-k, kPio2Mid, r);
    r = std::fma(-k, kPio2Lo, r);
    q = ((int)k) & 3;
    return r;
}
inline float kf_sin(float x) {
    int q;
    float r = reduce_pio2(x, q);
    switch (q) {
        case 0: return poly_sin(r);
        case 1: return poly_cos(r);
        case 2: return -poly_sin(r);
        default: return -poly_cos(r);
    }
}
inline float kf_cos(float x) {
    int q;
    float r = reduce_pio2(x, q);
    switch (q) {
        case 0: return poly_cos(r);
        case 1: return -poly_sin(r);
        case 2: return -poly_cos(r);
        default: return poly_sin(r);
    }
}
inline float kf_exp2(float x) {
    if (!(x > -126.0f)) return (x != x) ? x : 0.0f;
    if (x > 127.0f) return INFINITY;
    float k = std::nearbyint(x);
    float f = x - k;
    float p = 0x1.ffcbfcp-17f;
    p = std::fma(p, f, 0x1.430912p-13f);
    p = std::fma(p, f, 0x1.5d87fep-10f);
    p = std::fma(p, f, 0x1.3b2ab6p-7f);
    p = std::fma(p, f, 0x1.c6b08ep-5f);
    p = std::fma(p, f, 0x1.ebfbe0p-3f);
    p = std::fma(p, f, 0x1.62e430p-1f);
    p = std::fma(p, f, 1.0f);
    int ki = (int)k;
    uint32_t bits = (uint32_t)(ki + 127) << 23;
    float scale;
    std::memcpy(&scale, &bits, 4);
    return p * scale;
}
// pow(x, 5.0) of Random.glsl:72 is evaluated as ((x*x)*(x*x))*x.
inline float kf_pow5(float x) {
    float x2 = x * x;
    return (x2 * x2) * x;
}

// Math dispatch per precision: FP32 uses the deterministic functions above,
// FP64 uses libm in double.
template <class R> struct M;
template <> struct M<float> {
    static float sin(float x) { return kf_sin(x); }
    static float cos(float x) { return kf_cos(x); }
    static float exp2(float x) { return kf_exp2(x); }
    static float pow5(float x) { return kf_pow5(x); }
    static float sqrt(float x) { return std::sqrt(x); }
};
template <> struct M<double> {
    static double sin(double x) { return std::sin(x); }
    static double cos(double x) { return std::cos(x); }
    static double exp2(double x) { return std::exp2(x); }
    static double pow5(double x) { double x2 = x * x; return (x2 * x2) * x; }
    static double sqrt(double x) { return std::sqrt(x); }
};

// ---------------------------------------------------------------------------
// GLSL vector semantics (component-wise, left-to-right evaluation).
// ---------------------------------------------------------------------------
template <class R> struct V3 {
    R x, y, z;
    V3() : x(0), y(0), z(0) {}
    V3(R a) : x(a), y(a), z(a) {}
    V3(R a, R b, R c) : x(a), y(b), z(c) {}
    R operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
template <class R> inline V3<R> operator+(V3<R> a, V3<R> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class R> inline V3<R> operator-(V3<R> a, V3<R> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class R> inline V3<R> operator-(V3<R> a) { return {-a.x, -a.y, -a.z}; }
template <class R> inline V3<R> operator*(V3<R> a, V3<R> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <class R> inline V3<R> operator*(V3<R> a, R s) { return {a.x * s, a.y * s, a.z * s}; }
template <class R> inline V3<R> operator*(R s, V3<R> a) { return {s * a.x, s * a.y, s * a.z}; }
template <class R> inline V3<R> operator/(V3<R> a, R s) { return {a.x / s, a.y / s, a.z / s}; }
template <class R> inline bool operator==(V3<R> a, V3<R> b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
template <class R> inline bool operator!=(V3<R> a, V3<R> b) { return !(a == b); }
template <class R> inline R dot(V3<R> a, V3<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class R> inline V3<R> cross(V3<R> a, V3<R> b) {
    return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y};
}
template <class R> inline R length(V3<R> a) { return M<R>::sqrt(dot(a, a)); }
// normalize(v) = v * (1 / length(v))
template <class R> inline V3<R> normalize(V3<R> a) { R inv = R(1) / length(a); return a * inv; }
template <class R> inline R clampf(R x, R lo, R hi) { return std::min(std::max(x, lo), hi); }
template <class R> inline V3<R> reflect(V3<R> I, V3<R> N) { return I - (R(2) * dot(N, I)) * N; }
template <class R> inline V3<R> refract(V3<R> I, V3<R> N, R eta) {
    R d = dot(N, I);
    R k = R(1) - eta * eta * (R(1) - d * d);
    if (k < R(0)) return V3<R>(R(0));
    return eta * I - (eta * d + M<R>::sqrt(k)) * N;
}
template <class R> inline V3<R> cvt(V3<float> v) { return {(R)v.x, (R)v.y, (R)v.z}; }
template <class R> inline V3<float> tof(V3<R> v) { return {(float)v.x, (float)v.y, (float)v.z}; }

// mat4 (column-major) * vec4: sum over columns in order 0..3.
template <class R> inline void mat4_mul(const float* m, const R v[4], R out[4]) {
    for (int r = 0; r < 4; ++r)
        out[r] = (R)m[0 * 4 + r] * v[0] + (R)m[1 * 4 + r] * v[1] + (R)m[2 * 4 + r] * v[2] + (R)m[3 * 4 + r] * v[3];
}

// (A * B)[c][r] = sum_k A[k][r] * B[c][k], k in order 0..3.
template <class R> inline void mat4_mul_mat4(const float* a, const float* b, R out[16]) {
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r)
            out[c * 4 + r] = (R)a[0 * 4 + r] * (R)b[c * 4 + 0] + (R)a[1 * 4 + r] * (R)b[c * 4 + 1] +
                             (R)a[2 * 4 + r] * (R)b[c * 4 + 2] + (R)a[3 * 4 + r] * (R)b[c * 4 + 3];
}

constexpr float kRefPi = KF_REF_PI;

// ---------------------------------------------------------------------------
// Random streams.
// ---------------------------------------------------------------------------
struct Rng {
    uint32_t mode = KF_ORACLE_RNG_PHILOX;
    // philox
    uint32_t key[2] = {0, 0};
    uint32_t sample = 0, frame = 0, depth = 0;
    uint32_t counter[256];
    // tea/lcg
    uint32_t pixel_seed = 0; // `seed` in rgen (jitter)
    uint32_t ray_seed = 0;   // `ray.seed`

    void set_depth(uint32_t d) {
        depth = d;
        std::memset(counter, 0, sizeof(counter));
    }
    float philox_draw(uint32_t purpose) {
        uint32_t idx = counter[purpose]++;
        uint32_t ctr[4] = {sample, frame, (depth << 8) | purpose, idx >> 2};
        uint32_t out[4];
        philox4x32_10(ctr, key, out);
        return u24(out[idx & 3]);
    }
    float jitter() { return mode == KF_ORACLE_RNG_PHILOX ? philox_draw(KF_RNG_JITTER) : rnd_lcg(pixel_seed); }
    float next(uint32_t purpose) { return mode == KF_ORACLE_RNG_PHILOX ? philox_draw(purpose) : rnd_lcg(ray_seed); }
};

// ---------------------------------------------------------------------------
// Scene acceleration (replaces the Vulkan BLAS/TLAS of src/core/rt/rt.cpp).
// ---------------------------------------------------------------------------
struct Ray32 {
    float o[3], d[3];
    int kx, ky, kz;
    float Sx, Sy, Sz;
    float inv[3];
};

inline void ray_setup(Ray32& r) {
    int kz = 0;
    if (std::fabs(r.d[1]) > std::fabs(r.d[kz])) kz = 1;
    if (std::fabs(r.d[2]) > std::fabs(r.d[kz])) kz = 2;
    int kx = kz + 1; if (kx == 3) kx = 0;
    int ky = kx + 1; if (ky == 3) ky = 0;
    if (r.d[kz] < 0.0f) std::swap(kx, ky);
    r.kx = kx; r.ky = ky; r.kz = kz;
    r.Sx = r.d[kx] / r.d[kz];
    r.Sy = r.d[ky] / r.d[kz];
    r.Sz = 1.0f / r.d[kz];
    for (int i = 0; i < 3; ++i) r.inv[i] = 1.0f / r.d[i];
}

// Watertight ray/triangle intersection (Woop, Benthin, Wald, JCGT 2(1), 2013),
// both facings accepted (TRIANGLE_FACING_CULL_DISABLE, rt.cpp:134).
inline bool intersect_tri(const Ray32& r, const float* v0, const float* v1, const float* v2, float tmin, float tmax,
                          float& t_out, float& u_out, float& v_out) {
    const int kx = r.kx, ky = r.ky, kz = r.kz;
    const float Ax0 = v0[0] - r.o[0], Ay0 = v0[1] - r.o[1], Az0 = v0[2] - r.o[2];
    const float Bx0 = v1[0] - r.o[0], By0 = v1[1] - r.o[1], Bz0 = v1[2] - r.o[2];
    const float Cx0 = v2[0] - r.o[0], Cy0 = v2[1] - r.o[1], Cz0 = v2[2] - r.o[2];
    const float A[3] = {Ax0, Ay0, Az0}, B[3] = {Bx0, By0, Bz0}, C[3] = {Cx0, Cy0, Cz0};
    const float Ax = A[kx] - r.Sx * A[kz];
    const float Ay = A[ky] - r.Sy * A[kz];
    const float Bx = B[kx] - r.Sx * B[kz];
    const float By = B[ky] - r.Sy * B[kz];
    const float Cx = C[kx] - r.Sx * C[kz];
    const float Cy = C[ky] - r.Sy * C[kz];
    float U = Cx * By - Cy * Bx;
    float V = Ax * Cy - Ay * Cx;
    float W = Bx * Ay - By * Ax;
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        double CxBy = (double)Cx * (double)By, CyBx = (double)Cy * (double)Bx;
        U = (float)(CxBy - CyBx);
        double AxCy = (double)Ax * (double)Cy, AyCx = (double)Ay * (double)Cx;
        V = (float)(AxCy - AyCx);
        double BxAy = (double)Bx * (double)Ay, ByAx = (double)By * (double)Ax;
        W = (float)(BxAy - ByAx);
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    const float det = U + V + W;
    if (det == 0.0f) return false;
    const float Az = r.Sz * A[kz];
    const float Bz = r.Sz * B[kz];
    const float Cz = r.Sz * C[kz];
    const float T = U * Az + V * Bz + W * Cz;
    const float t = T / det;
    if (!(t >= tmin && t <= tmax)) return false;
    t_out = t;
    u_out = V / det;
    v_out = W / det;
    return true;
}

// Conservative slab test: far distances widened by 1 + 2*gamma(3) (Ize,
// "Robust BVH Ray Traversal", JCGT 2(2), 2013).
constexpr float kBoxWiden = 1.0f + 2.0f * (3.0f * 0x1.0p-24f) / (1.0f - 3.0f * 0x1.0p-24f);
// the closest hit so far is widened as well, so a box holding a triangle whose t ties it
// (rounded entry distance a few ulp beyond) is still opened and the tie rule decides
constexpr float kTmaxWiden = 1.0f + 0x1.0p-19f;
inline bool box_hit(const Ray32& r, const float* lo, const float* hi, float tmin, float tmax) {
    float tn = tmin, tf = INFINITY;
    for (int a = 0; a < 3; ++a) {
        float nearp = r.inv[a] >= 0.0f ? lo[a] : hi[a];
        float farp = r.inv[a] >= 0.0f ? hi[a] : lo[a];
        float t0 = (nearp - r.o[a]) * r.inv[a];
        float t1 = (farp - r.o[a]) * r.inv[a];
        tn = std::fmax(tn, t0);
        tf = std::fmin(tf, t1);
    }
    return tn <= std::fmin(tf * kBoxWiden, tmax * kTmaxWiden);
}

struct BvhNode {
    float lo[3], hi[3];
    int left, right; // internal: child indices; leaf: left = -1
    int start, count;
};

struct GeomAccel {
    std::vector<BvhNode> nodes;
    std::vector<uint32_t> prims;
    std::vector<float> tri; // 9 floats per triangle (object space)
};

void build_bvh(GeomAccel& ga, const kf_flat_geometry& g) {
    const uint32_t n = g.num_triangles;
    ga.tri.resize((size_t)n * 9);
    std::vector<float> cen((size_t)n * 3);
    for (uint32_t i = 0; i < n; ++i) {
        for (int k = 0; k < 3; ++k) {
            const float* p = g.vertices[g.indices[3 * i + k]].pos;
            for (int a = 0; a < 3; ++a) ga.tri[(size_t)i * 9 + k * 3 + a] = p[a];
        }
        for (int a = 0; a < 3; ++a)
            cen[i * 3 + a] = (ga.tri[i * 9 + a] + ga.tri[i * 9 + 3 + a] + ga.tri[i * 9 + 6 + a]) / 3.0f;
    }
    ga.prims.resize(n);
    for (uint32_t i = 0; i < n; ++i) ga.prims[i] = i;
    ga.nodes.clear();
    if (n == 0) return;
    struct Item { int node, start, count; };
    std::vector<Item> stack;
    ga.nodes.push_back(BvhNode{});
    stack.push_back({0, 0, (int)n});
    while (!stack.empty()) {
        Item it = stack.back();
        stack.pop_back();
        BvhNode nd;
        for (int a = 0; a < 3; ++a) { nd.lo[a] = INFINITY; nd.hi[a] = -INFINITY; }
        float clo[3] = {INFINITY, INFINITY, INFINITY}, chi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (int i = it.start; i < it.start + it.count; ++i) {
            uint32_t p = ga.prims[i];
            for (int k = 0; k < 3; ++k)
                for (int a = 0; a < 3; ++a) {
                    nd.lo[a] = std::min(nd.lo[a], ga.tri[p * 9 + k * 3 + a]);
                    nd.hi[a] = std::max(nd.hi[a], ga.tri[p * 9 + k * 3 + a]);
                }
            for (int a = 0; a < 3; ++a) {
                clo[a] = std::min(clo[a], cen[p * 3 + a]);
                chi[a] = std::max(chi[a], cen[p * 3 + a]);
            }
        }
        if (it.count <= 4) {
            nd.left = nd.right = -1;
            nd.start = it.start;
            nd.count = it.count;
            ga.nodes[it.node] = nd;
            continue;
        }
        int axis = 0;
        for (int a = 1; a < 3; ++a)
            if (chi[a] - clo[a] > chi[axis] - clo[axis]) axis = a;
        int mid = it.start + it.count / 2;
        std::nth_element(ga.prims.begin() + it.start, ga.prims.begin() + mid, ga.prims.begin() + it.start + it.count,
                         [&](uint32_t a, uint32_t b) {
                             float ca = cen[a * 3 + axis], cb = cen[b * 3 + axis];
                             return ca < cb || (ca == cb && a < b);
                         });
        int l = (int)ga.nodes.size();
        ga.nodes.push_back(BvhNode{});
        int rr = (int)ga.nodes.size();
        ga.nodes.push_back(BvhNode{});
        nd.left = l;
        nd.right = rr;
        nd.start = nd.count = 0;
        ga.nodes[it.node] = nd;
        stack.push_back({l, it.start, mid - it.start});
        stack.push_back({rr, mid, it.start + it.count - mid});
    }
}

struct SceneAccel {
    const kf_flat_scene* s = nullptr;
    std::vector<GeomAccel> geoms;
    bool use_bvh = false;
};

struct HitRec {
    float t = 0, u = 0, v = 0;
    uint32_t inst = 0xFFFFFFFFu, prim = 0;
};

inline bool closer(float t, uint32_t inst, uint32_t prim, const HitRec& h) {
    if (h.inst == 0xFFFFFFFFu) return true;
    if (t < h.t) return true;
    if (t == h.t) return inst < h.inst || (inst == h.inst && prim < h.prim);
    return false;
}

// Object-space ray of an instance: o' = W2O * (o, 1), d' = W2O * (d, 0).
inline void to_object(const kf_flat_instance& in, const float* o, const float* d, Ray32& r) {
    const float* m = in.world_to_object;
    for (int i = 0; i < 3; ++i) {
        r.o[i] = m[i * 4 + 0] * o[0] + m[i * 4 + 1] * o[1] + m[i * 4 + 2] * o[2] + m[i * 4 + 3];
        r.d[i] = m[i * 4 + 0] * d[0] + m[i * 4 + 1] * d[1] + m[i * 4 + 2] * d[2];
    }
    ray_setup(r);
}

// Any-hit callback state (PathTrace.rahit:30-48).
struct AnyHit {
    Rng* rng = nullptr;
};

inline bool anyhit_accept(const SceneAccel& sa, uint32_t inst, uint32_t prim, AnyHit* ah) {
    const kf_flat_scene& s = *sa.s;
    const kf_flat_geometry& g = s.geometries[s.instances[inst].geometry_index];
    if (g.opaque) return true;
    const kf_material_gpu& mat = s.materials[g.mat_index[prim]];
    if (mat.alpha == 0.0f) return false;
    if (ah && ah->rng && ah->rng->next(KF_RNG_ANYHIT) > mat.alpha) return false;
    return true;
}

// Closest hit (shadow == false) or any hit (shadow == true: TerminateOnFirstHit | Opaque).
bool trace(const SceneAccel& sa, const float o[3], const float d[3], float tmin, float tmax, bool shadow, HitRec& hit,
           AnyHit* ah) {
    const kf_flat_scene& s = *sa.s;
    hit = HitRec{};
    float tbest = tmax;
    for (uint32_t ii = 0; ii < s.num_instances; ++ii) {
        const kf_flat_instance& in = s.instances[ii];
        const kf_flat_geometry& g = s.geometries[in.geometry_index];
        if (g.hide_render || g.num_triangles == 0) continue;
        Ray32 r;
        to_object(in, o, d, r);
        if (!sa.use_bvh) {
            for (uint32_t p = 0; p < g.num_triangles; ++p) {
                const float* v0 = g.vertices[g.indices[3 * p + 0]].pos;
                const float* v1 = g.vertices[g.indices[3 * p + 1]].pos;
                const float* v2 = g.vertices[g.indices[3 * p + 2]].pos;
                float t, u, v;
                if (!intersect_tri(r, v0, v1, v2, tmin, tbest, t, u, v)) continue;
                if (!closer(t, ii, p, hit)) continue;
                if (!shadow && !anyhit_accept(sa, ii, p, ah)) continue;
                hit.t = t; hit.u = u; hit.v = v; hit.inst = ii; hit.prim = p;
                tbest = t;
                if (shadow) return true;
            }
        } else {
            const GeomAccel& ga = sa.geoms[in.geometry_index];
            int stack[128];
            int sp = 0;
            stack[sp++] = 0;
            while (sp) {
                const BvhNode& nd = ga.nodes[stack[--sp]];
                if (!box_hit(r, nd.lo, nd.hi, tmin, tbest)) continue;
                if (nd.left < 0) {
                    for (int i = nd.start; i < nd.start + nd.count; ++i) {
                        uint32_t p = ga.prims[i];
                        const float* tv = &ga.tri[(size_t)p * 9];
                        float t, u, v;
                        if (!intersect_tri(r, tv, tv + 3, tv + 6, tmin, tbest, t, u, v)) continue;
                        if (!closer(t, ii, p, hit)) continue;
                        if (!shadow && !anyhit_accept(sa, ii, p, ah)) continue;
                        hit.t = t; hit.u = u; hit.v = v; hit.inst = ii; hit.prim = p;
                        tbest = t;
                        if (shadow) return true;
                    }
                } else {
                    stack[sp++] = nd.left;
                    stack[sp++] = nd.right;
                }
            }
        }
    }
    return hit.inst != 0xFFFFFFFFu;
}

// ---------------------------------------------------------------------------
// Texture lookup (sampler2D with linear filter, repeat, sRGB decode:
// vkCore.hpp:585,619-637).
// ---------------------------------------------------------------------------
struct SrgbTables {
    float decode[256];
    float thresh[256]; // thresh[k] = smallest linear value that encodes to >= k (k = 1..255)
    SrgbTables() {
        for (int i = 0; i < 256; ++i) {
            double c = i / 255.0;
            double l = c <= 0.04045 ? c / 12.92 : std::pow((c + 0.055) / 1.055, 2.4);
            decode[i] = (float)l;
        }
        thresh[0] = -INFINITY;
        for (int k = 1; k < 256; ++k) {
            double c = (k - 0.5) / 255.0;
            double l = c <= 0.04045 ? c / 12.92 : std::pow((c + 0.055) / 1.055, 2.4);
            thresh[k] = (float)l;
        }
    }
};
const SrgbTables& srgb_tables() {
    static SrgbTables t;
    return t;
}

inline uint8_t srgb_encode8(float v) {
    const SrgbTables& T = srgb_tables();
    if (!(v > 0.0f)) return 0;
    int lo = 0, hi = 255; // largest k with thresh[k] <= v
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (T.thresh[mid] <= v) lo = mid; else hi = mid - 1;
    }
    return (uint8_t)lo;
}

template <class R> V3<R> texture_rgb(const kf_flat_scene& s, int id, R u, R v) {
    if (id < 0 || (uint32_t)id >= s.num_textures) return V3<R>(R(1));
    const kf_texture_desc& tx = s.textures[id];
    const SrgbTables& T = srgb_tables();
    float x = (float)u * (float)tx.width - 0.5f;
    float y = (float)v * (float)tx.height - 0.5f;
    float fx0 = std::floor(x), fy0 = std::floor(y);
    float ax = x - fx0, ay = y - fy0;
    long ix = (long)fx0, iy = (long)fy0;
    auto wrap = [](long i, uint32_t n) { long m = i % (long)n; return (uint32_t)(m < 0 ? m + n : m); };
    uint32_t x0 = wrap(ix, tx.width), x1 = wrap(ix + 1, tx.width);
    uint32_t y0 = wrap(iy, tx.height), y1 = wrap(iy + 1, tx.height);
    float out[3];
    for (int c = 0; c < 3; ++c) {
        auto tex = [&](uint32_t xx, uint32_t yy) {
            uint8_t b = tx.rgba8[((size_t)yy * tx.width + xx) * 4 + c];
            return tx.srgb ? T.decode[b] : (float)b / 255.0f;
        };
        float top = tex(x0, y0) * (1.0f - ax) + tex(x1, y0) * ax;
        float bot = tex(x0, y1) * (1.0f - ax) + tex(x1, y1) * ax;
        out[c] = top * (1.0f - ay) + bot * ay;
    }
    return V3<R>((R)out[0], (R)out[1], (R)out[2]);
}

// PathTrace.rmiss:14-29: texture(environmentMap, vec3(-d.y, d.z, -d.x)) of a cube map.
// Face by the major axis, face coordinates (sc, tc) of the Vulkan / GL cube-map rules
// (Vulkan spec "Cube Map Face Selection"), bilinear within the face, clamp to edge.
// Evaluated in float whatever the oracle precision (a texture unit filters in float).
static void env_lookup(const kf_flat_scene& s, const float d[3], float out[3]) {
    const float rx = -d[1], ry = d[2], rz = -d[0];
    const float ax = std::fabs(rx), ay = std::fabs(ry), az = std::fabs(rz);
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
    const uint32_t n = s.env_size;
    const float fs = 0.5f * (sc / ma + 1.0f), ft = 0.5f * (tc / ma + 1.0f);
    const float x = fs * (float)n - 0.5f, y = ft * (float)n - 0.5f;
    const float fx0 = std::floor(x), fy0 = std::floor(y);
    const float wx = x - fx0, wy = y - fy0;
    const int ix = (int)fx0, iy = (int)fy0, hi = (int)n - 1;
    auto cl = [hi](int i) { return (size_t)std::min(std::max(i, 0), hi); };
    const size_t x0 = cl(ix), x1 = cl(ix + 1), y0 = cl(iy), y1 = cl(iy + 1);
    const float* fp = s.env_rgba32f + (size_t)face * n * n * 4;
    for (int c = 0; c < 3; ++c) {
        const float top = fp[(y0 * n + x0) * 4 + c] * (1.0f - wx) + fp[(y0 * n + x1) * 4 + c] * wx;
        const float bot = fp[(y1 * n + x0) * 4 + c] * (1.0f - wx) + fp[(y1 * n + x1) * 4 + c] * wx;
        out[c] = top * (1.0f - wy) + bot * wy;
    }
}

// ---------------------------------------------------------------------------
// Shader library (base/Random.glsl, base/Sampling.glsl).
// ---------------------------------------------------------------------------
template <class R> inline V3<R> getPerpendicularVector(V3<R> u) { // Random.glsl:58-65
    V3<R> a(std::fabs(u.x), std::fabs(u.y), std::fabs(u.z));
    uint32_t xm = ((a.x - a.y) < R(0) && (a.x - a.z) < R(0)) ? 1u : 0u;
    uint32_t ym = (a.y - a.z) < R(0) ? (1u ^ xm) : 0u;
    uint32_t zm = 1u ^ (xm | ym);
    return cross(u, V3<R>((R)xm, (R)ym, (R)zm));
}
template <class R> inline R Schlick(R cosine, R ior) { // Random.glsl:68-73
    R r0 = (R(1) - ior) / (R(1) + ior);
    r0 *= r0;
    return r0 + (R(1) - r0) * M<R>::pow5(R(1) - cosine);
}
template <class R> inline R ggxNormalDistribution(R NdotH, R a2) { // Random.glsl:75-79
    R d = std::max(NdotH * NdotH * (a2 - R(1)) + R(1), R(1e-6f));
    return a2 / (d * d * R(kRefPi));
}
template <class R> inline V3<R> sampleGGX(R u0, R u1, R a2, V3<R> N) { // Random.glsl:83-101
    V3<R> B = getPerpendicularVector(N);
    V3<R> T = cross(B, N);
    R cosThetaH = M<R>::sqrt(clampf((R(1) - u0) / ((a2 - R(1)) * u0 + R(1)), R(0), R(1)));
    R sinThetaH = M<R>::sqrt(clampf(R(1) - cosThetaH * cosThetaH, R(0), R(1)));
    R phiH = u1 * R(kRefPi) * R(2);
    return T * (sinThetaH * M<R>::cos(phiH)) + B * (sinThetaH * M<R>::sin(phiH)) + N * cosThetaH;
}
template <class R> inline R G1(R d, R a2) { // Random.glsl:117-121
    return (R(2) * d) / (d + M<R>::sqrt(a2 + (R(1) - a2) * (d * d)));
}
template <class R> inline R GeometricShadowing(R NdotV, R NdotL, R a2) { // Random.glsl:123-127
    return G1(NdotL, a2) * G1(NdotV, a2);
}
template <class R> inline V3<R> schlickFresnel(V3<R> f0, R lDotH) { // Random.glsl:133-136
    R e = (R(-5.55473f) * lDotH - R(6.98316f)) * lDotH;
    return f0 + (V3<R>(R(1)) - f0) * M<R>::exp2(e);
}
template <class R> inline V3<R> transformLocalToWorld(V3<R> dir, V3<R> n) { // Sampling.glsl:6-23
    V3<R> tangent;
    if (std::fabs(n.x) > std::fabs(n.y))
        tangent = V3<R>(n.z, R(0), -n.x) / M<R>::sqrt(n.x * n.x + n.z * n.z);
    else
        tangent = V3<R>(R(0), -n.z, n.y) / M<R>::sqrt(n.y * n.y + n.z * n.z);
    V3<R> bitangent = cross(n, tangent);
    return dir.x * tangent + dir.y * bitangent + dir.z * n;
}
template <class R> inline V3<R> cosineHemisphereSampling(R u0, R u1, V3<R> n) { // Sampling.glsl:25-35
    R sq = M<R>::sqrt(R(1) - u1);
    R ang = R(2) * R(kRefPi) * u0;
    V3<R> direction(M<R>::cos(ang) * sq, M<R>::sin(ang) * sq, M<R>::sqrt(u1));
    return transformLocalToWorld(direction, n);
}
template <class R> inline V3<R> uniformSphereSampling(Rng& rng, uint32_t purpose) { // Sampling.glsl:72-83
    V3<R> p;
    do {
        R a = (R)rng.next(purpose), b = (R)rng.next(purpose), c = (R)rng.next(purpose);
        p = V3<R>(a, b, c) * R(2) - V3<R>(R(1));
    } while (dot(p, p) >= R(1));
    return p;
}

template <class R> inline void diskSampling(Rng& rng, uint32_t purpose, R& qx, R& qy) { // Sampling.glsl:124-134
    do {
        R a = (R)rng.next(purpose), b = (R)rng.next(purpose);
        qx = R(2) * a - R(1);
        qy = R(2) * b - R(1);
    } while (qx * qx + qy * qy >= R(1));
}

// ---------------------------------------------------------------------------
// Closest-hit shader (PathTrace.rchit).
// ---------------------------------------------------------------------------
template <class R> struct Payload { // base/Ray.glsl:1-14
    V3<R> direction, albedo, normal, emission, origin, weight;
    uint32_t depth = 0;
    V3<R> shadow_color;
};

struct Ctx {
    const SceneAccel* sa;
    const kf_flat_scene* s;
    const kf_push_constants* pc;
    uint64_t rays_shadow = 0, rays_extension = 0;
};

template <class R> struct Shading {
    R f, a2;
    V3<R> diffuseColor, specularColor, transmissionColor;
    bool isInside;
};

// calcDirectContribution (PathTrace.rchit:103-171).
template <class R>
V3<R> calcDirectContribution(Rng& rng, uint32_t purpose, V3<R> L, V3<R> V, V3<R> N, V3<R> lightEmission,
                             const Shading<R>& sh) {
    V3<R> weight(R(0));
    const R a2 = sh.a2, f = sh.f;
    if (sh.transmissionColor != V3<R>(R(0))) {
        if (sh.isInside) {
            weight = V3<R>(R(0));
        } else {
            R NdotV0 = dot(N, V);
            V3<R> refractedL = refract(-V, N, R(1) / f);
            R reflectProb = refractedL != V3<R>(R(0)) ? Schlick(NdotV0, f) : R(1);
            if ((R)rng.next(purpose) <= reflectProb) {
                V3<R> H = normalize(L + V);
                R NdotL = dot(N, L);
                R NdotH = dot(N, H);
                R HdotV = dot(H, V);
                R NdotV = std::max(dot(N, V), R(1e-6f));
                R LdotH = dot(L, H);
                R D = ggxNormalDistribution(NdotH, a2);
                R G = GeometricShadowing(NdotL, NdotV, a2);
                V3<R> F = schlickFresnel(sh.transmissionColor, LdotH);
                weight = D * F * G * HdotV / NdotH * NdotV;
            } else {
                weight = V3<R>(R(0));
            }
        }
    } else {
        V3<R> H = normalize(L + V);
        R NdotL = dot(N, L);
        R NdotH = dot(N, H);
        R HdotV = dot(H, V);
        R NdotV = std::max(dot(N, V), R(1e-6f));
        R LdotH = dot(L, H);
        R D = ggxNormalDistribution(NdotH, a2);
        R G = GeometricShadowing(NdotL, NdotV, a2);
        V3<R> F = schlickFresnel(sh.specularColor, LdotH);
        R diffuseLum = length(sh.diffuseColor);
        R specularLum = length(sh.specularColor);
        R probDiffuse = diffuseLum / (diffuseLum + specularLum);
        if (diffuseLum == R(0) && specularLum == R(0)) probDiffuse = R(0.5f);
        V3<R> diffuseWeight = sh.diffuseColor * V3<R>(NdotL);
        V3<R> specularWeight = D * F * G * HdotV / NdotH * NdotV;
        weight = (R)rng.next(purpose) < probDiffuse ? diffuseWeight * probDiffuse : specularWeight * (R(1) - probDiffuse);
    }
    return lightEmission * weight;
}

// traceShadowRay (PathTrace.rchit:175-200).
template <class R>
V3<R> traceShadowRay(Ctx& cx, Rng& rng, uint32_t purpose, V3<R> worldPos, V3<R> L, V3<R> V, V3<R> N, R maxDist,
                     V3<R> lightEmission, const Shading<R>& sh) {
    bool isShadowed = true;
    R NdotL = dot(N, L);
    if (NdotL > R(0)) {
        V3<float> o = tof(worldPos), d = tof(L);
        float og[3] = {o.x, o.y, o.z}, dg[3] = {d.x, d.y, d.z};
        HitRec h;
        cx.rays_shadow++;
        isShadowed = trace(*cx.sa, og, dg, KF_T_MIN, (float)maxDist, true, h, nullptr);
    }
    return isShadowed ? V3<R>(R(0)) : calcDirectContribution(rng, purpose, L, V, N, lightEmission, sh);
}

template <class R> V3<R> vec4xyz(const float* v) { return V3<R>((R)v[0], (R)v[1], (R)v[2]); }

template <class R>
V3<R> traceDirectionalLight(Ctx& cx, Rng& rng, const Payload<R>& ray, V3<R> worldPos, V3<R> N, const Shading<R>& sh) {
    const kf_dir_light_ubo& dl = cx.s->dlight;
    V3<R> lightEmission = vec4xyz<R>(dl.rgbs) * (R)dl.rgbs[3];
    if (lightEmission == V3<R>(R(0))) return V3<R>(R(0));
    V3<R> L = -vec4xyz<R>(dl.direction);
    V3<R> V = normalize(-ray.direction);
    if (dl.direction[3] != 0.0f) {
        R a = (R)rng.next(KF_RNG_DIRLIGHT), b = (R)rng.next(KF_RNG_DIRLIGHT), c = (R)rng.next(KF_RNG_DIRLIGHT);
        V3<R> perturb(a, b, c);
        L = normalize(L + (R)dl.direction[3] * perturb);
    }
    R maxDist = R(KF_DIR_LIGHT_TMAX);
    return traceShadowRay(cx, rng, KF_RNG_DIRLIGHT, worldPos, L, V, N, maxDist, lightEmission, sh);
}

template <class R>
V3<R> tracePointLights(Ctx& cx, Rng& rng, const Payload<R>& ray, V3<R> worldPos, V3<R> N, const Shading<R>& sh) {
    const kf_point_lights_ubo& pl = cx.s->plights;
    V3<R> ret(R(0));
    for (uint32_t i = 0; i < KF_MAX_POINT_LIGHTS; ++i)
        if (pl.rgbs[i][3] > 0.0f) {
            R lum = length(vec4xyz<R>(pl.rgbs[i]) * (R)pl.rgbs[i][3]);
            if (lum == R(0)) continue;
            const uint32_t purpose = KF_RNG_POINT0 + i;
            V3<R> V = normalize(-ray.direction);
            V3<R> lpos = vec4xyz<R>(pl.posr[i]);
            if (pl.posr[i][3] != 0.0f) {
                V3<R> perturb = uniformSphereSampling<R>(rng, purpose);
                lpos = lpos + (R)pl.posr[i][3] * normalize(perturb);
            }
            V3<R> L = lpos - worldPos;
            R d = length(L);
            L = normalize(L);
            V3<R> lightEmission = vec4xyz<R>(pl.rgbs[i]) * (R)pl.rgbs[i][3] / d / d;
            ret = ret + traceShadowRay(cx, rng, purpose, worldPos, L, V, N, d, lightEmission, sh);
        }
    return ret;
}

template <class R>
V3<R> traceActiveLights(Ctx& cx, Rng& rng, const Payload<R>& ray, V3<R> worldPos, V3<R> N, const Shading<R>& sh) {
    const kf_active_lights_ubo& al = cx.s->alights;
    V3<R> ret(R(0));
    for (uint32_t i = 0; i < KF_MAX_ACTIVE_LIGHTS; ++i)
        if (al.front[i][3] > 0.0f) {
            R lum = length(vec4xyz<R>(al.rgbs[i]) * (R)al.rgbs[i][3]);
            if (lum == R(0)) continue;
            const uint32_t purpose = KF_RNG_ACTIVE0 + i;
            V3<R> V = normalize(-ray.direction);
            R softness = (R)al.sftp[i][0];
            V3<R> lpos = vec4xyz<R>(al.position[i]);
            if (softness != R(0)) {
                V3<R> perturb = uniformSphereSampling<R>(rng, purpose);
                lpos = lpos + softness * normalize(perturb);
            }
            V3<R> L = lpos - worldPos;
            R d = length(L);
            L = normalize(L);
            R fov = (R)al.sftp[i][1];
            V3<R> alightDir = normalize(vec4xyz<R>(al.front[i]));
            R halfAngle = clampf(fov, R(0), R(kRefPi)) / R(2);
            R cos_ = dot(alightDir, -L);
            if (cos_ > M<R>::cos(halfAngle)) {
                int texID = (int)al.sftp[i][2];
                V3<R> color = vec4xyz<R>(al.rgbs[i]);
                if (texID >= 0) {
                    // proj * view * vec4(worldPos, 1) parses as (proj * view) * vec4(...)
                    R wp[4] = {worldPos.x, worldPos.y, worldPos.z, R(1)};
                    R pv[16], tc[4];
                    mat4_mul_mat4<R>(al.proj[i], al.view[i], pv);
                    for (int r = 0; r < 4; ++r)
                        tc[r] = pv[0 * 4 + r] * wp[0] + pv[1 * 4 + r] * wp[1] + pv[2 * 4 + r] * wp[2] + pv[3 * 4 + r] * wp[3];
                    R w = tc[3];
                    for (int k = 0; k < 4; ++k) tc[k] = tc[k] / w;
                    R uvx = tc[0] * R(0.5f) + R(0.5f), uvy = tc[1] * R(0.5f) + R(0.5f);
                    color = color * texture_rgb<R>(*cx.s, texID, uvx, uvy);
                }
                V3<R> lightEmission = color * (R)al.rgbs[i][3] / d / d;
                ret = ret + traceShadowRay(cx, rng, purpose, worldPos, L, V, N, d, lightEmission, sh);
            }
        }
    return ret;
}

// rchit main (PathTrace.rchit:322-468). `backface` is gl_HitKindEXT == BackFacing.
template <class R>
void closestHit(Ctx& cx, Rng& rng, Payload<R>& ray, const HitRec& h, const float wo[3], const float wd[3]) {
    const kf_flat_scene& s = *cx.s;
    const kf_flat_instance& in = s.instances[h.inst];
    const kf_flat_geometry& g = s.geometries[in.geometry_index];
    // getShadingData (rchit:66-98)
    const uint32_t i0 = g.indices[3 * h.prim + 0], i1 = g.indices[3 * h.prim + 1], i2 = g.indices[3 * h.prim + 2];
    const kf_vertex &v0 = g.vertices[i0], &v1 = g.vertices[i1], &v2 = g.vertices[i2];
    const R bx = R(1) - (R)h.u - (R)h.v, by = (R)h.u, bz = (R)h.v;
    V3<R> n0 = vec4xyz<R>(v0.normal), n1 = vec4xyz<R>(v1.normal), n2 = vec4xyz<R>(v2.normal);
    V3<R> localNormal = n0 * bx + n1 * by + n2 * bz;
    const float* m = in.world_to_object; // rows of the 3x4
    // vec3(localNormal * gl_WorldToObjectEXT): component j = dot(localNormal, column j)
    V3<R> wn((R)localNormal.x * (R)m[0] + localNormal.y * (R)m[4] + localNormal.z * (R)m[8],
             localNormal.x * (R)m[1] + localNormal.y * (R)m[5] + localNormal.z * (R)m[9],
             localNormal.x * (R)m[2] + localNormal.y * (R)m[6] + localNormal.z * (R)m[10]);
    V3<R> N = normalize(wn);
    V3<R> rayO((R)wo[0], (R)wo[1], (R)wo[2]), rayD((R)wd[0], (R)wd[1], (R)wd[2]);
    V3<R> worldPos = rayO + rayD * (R)h.t;
    R uvx = (R)v0.uv[0] * bx + (R)v1.uv[0] * by + (R)v2.uv[0] * bz;
    R uvy = (R)v0.uv[1] * bx + (R)v1.uv[1] * by + (R)v2.uv[1] * bz;
    const kf_material_gpu& mat = s.materials[g.mat_index[h.prim]];

    // Facing: front-facing when the object-space direction opposes (v1-v0)x(v2-v0).
    bool backface;
    {
        float od[3];
        for (int i = 0; i < 3; ++i) od[i] = m[i * 4 + 0] * wd[0] + m[i * 4 + 1] * wd[1] + m[i * 4 + 2] * wd[2];
        V3<float> e1 = V3<float>(v1.pos[0], v1.pos[1], v1.pos[2]) - V3<float>(v0.pos[0], v0.pos[1], v0.pos[2]);
        V3<float> e2 = V3<float>(v2.pos[0], v2.pos[1], v2.pos[2]) - V3<float>(v0.pos[0], v0.pos[1], v0.pos[2]);
        V3<float> ng = cross(e1, e2);
        backface = dot(V3<float>(od[0], od[1], od[2]), ng) > 0.0f;
    }

    V3<R> emission = vec4xyz<R>(mat.emission) * (R)mat.emission[3];
    if (emission != V3<R>(R(0))) {
        ray.depth = cx.pc->max_path_depth + 1;
        ray.emission = vec4xyz<R>(mat.emission) * (R)mat.emission[3];
        return;
    }
    V3<R> baseColor = vec4xyz<R>(mat.diffuse);
    if (mat.diffuse_tex >= 0) baseColor = texture_rgb<R>(s, mat.diffuse_tex, uvx, uvy);
    baseColor = baseColor / R(kRefPi);
    R metallic = mat.metallic_tex >= 0 ? texture_rgb<R>(s, mat.metallic_tex, uvx, uvy).x : (R)mat.metallic;
    R roughness = mat.roughness_tex >= 0 ? texture_rgb<R>(s, mat.roughness_tex, uvx, uvy).x : (R)mat.roughness;
    R a2 = roughness * roughness;
    R transmission =
        mat.transmission_tex >= 0 ? texture_rgb<R>(s, mat.transmission_tex, uvx, uvy).x : (R)mat.transmission;
    R f = std::max((R)mat.ior, R(1e-5f));
    R diffuse_weight = (R(1) - clampf(metallic, R(0), R(1))) * (R(1) - clampf(transmission, R(0), R(1)));
    R final_transmission = clampf(transmission, R(0), R(1)) * (R(1) - clampf(metallic, R(0), R(1)));
    R specular_weight = (R(1) - final_transmission);
    V3<R> weight(R(0));
    V3<R> V = normalize(-ray.direction);
    bool isInside = backface;
    N = isInside ? -N : N;
    V3<R> L(R(0));
    R NdotV = dot(N, V);
    V3<R> diffuseColor = diffuse_weight * baseColor;
    V3<R> specularColor =
        specular_weight * (baseColor * metallic + ((R)mat.specular * R(0.08f) * V3<R>(R(1))) * (R(1) - metallic));
    V3<R> transmissionColor = transmission * baseColor;
    R diffuseLum = length(diffuseColor);
    R specularLum = length(specularColor);
    R probDiffuse = diffuseLum / (diffuseLum + specularLum);
    if (diffuseLum == R(0) && specularLum == R(0)) {
        if (baseColor == V3<R>(R(0))) {
            if (diffuse_weight == R(1)) probDiffuse = R(1);
            else if (diffuse_weight == R(0)) probDiffuse = R(0);
            else probDiffuse = R(0.5f);
        } else
            probDiffuse = R(0);
    } else {
        probDiffuse *= specular_weight;
    }
    bool chooseDiffuse = (R)rng.next(KF_RNG_BSDF) < probDiffuse;
    if (chooseDiffuse) {
        R u0 = (R)rng.next(KF_RNG_BSDF), u1 = (R)rng.next(KF_RNG_BSDF);
        L = cosineHemisphereSampling(u0, u1, N);
        R NdotL = clampf(dot(N, L), R(0), R(1));
        weight = R(kRefPi) * diffuseColor * NdotL / probDiffuse;
    }
    if (!chooseDiffuse) {
        if (final_transmission == R(0)) {
            R u0 = (R)rng.next(KF_RNG_BSDF), u1 = (R)rng.next(KF_RNG_BSDF);
            V3<R> H = sampleGGX(u0, u1, a2, N);
            R HdotV = dot(H, V);
            L = R(2) * HdotV * H - V;
            R NoV = std::max(dot(N, V), R(1e-7f));
            R NoL = dot(N, L);
            R NoH = std::max(dot(N, H), R(1e-7f));
            R VoH = std::max(dot(V, H), R(1e-7f));
            if (NoL >= R(0)) {
                R G = GeometricShadowing(NoV, NoL, a2);
                V3<R> F = schlickFresnel(specularColor, VoH);
                weight = R(kRefPi) * F * G * VoH / (NoH * NoV * (R(1) - probDiffuse));
            } else
                weight = V3<R>(R(0));
        } else {
            R ior = isInside ? R(1) / f : f;
            R _dot = isInside ? NdotV * ior : NdotV;
            V3<R> refractedL = refract(-V, N, R(1) / f);
            R reflectProb = refractedL != V3<R>(R(0)) ? Schlick(_dot, f) : R(1);
            if ((R)rng.next(KF_RNG_BSDF) >= reflectProb) {
                L = refractedL;
                weight = R(kRefPi) * transmissionColor / (R(1) - probDiffuse);
            } else {
                L = reflect(-V, N);
                weight = R(kRefPi) * transmissionColor / (R(1) - probDiffuse);
            }
        }
    }
    Shading<R> sh{f, a2, diffuseColor, specularColor, transmissionColor, isInside};
    // rchit:457-460 sums the three light loops; with kuafu's single tea/lcg stream their
    // order matters, and it is the left-to-right order glslang emits
    const V3<R> dir_part = traceDirectionalLight(cx, rng, ray, worldPos, N, sh);
    const V3<R> point_part = tracePointLights(cx, rng, ray, worldPos, N, sh);
    const V3<R> active_part = traceActiveLights(cx, rng, ray, worldPos, N, sh);
    ray.shadow_color = dir_part + point_part + active_part;
    ray.origin = worldPos;
    ray.direction = L;
    ray.emission = V3<R>(R(0));
    ray.weight = weight;
    ray.albedo = baseColor;
    ray.normal = N;
}

// ---------------------------------------------------------------------------
// Ray generation (PathTrace.rgen main) for one pixel.
// ---------------------------------------------------------------------------
template <class R>
void render_pixel(Ctx& cx, const kf_oracle_view& view, uint32_t px, uint32_t py, uint32_t out_index,
                  uint32_t crop_pixels, kf_oracle_out* out) {
    const kf_push_constants& pc = view.pc;
    const kf_camera_ubo& cam = *view.camera;
    const uint32_t mapping = py * view.width + px;
    Rng rng;
    rng.mode = view.rng_mode;
    rng.key[0] = view.seed ^ mapping;
    rng.key[1] = view.camera_index;
    rng.frame = view.frame;
    // clockARB() is called at rgen:23 (seed), rgen:28 (timeStart) and rgen:32 once per
    // sample; the pinned clock returns tea_clock + call index.
    rng.pixel_seed = tea(mapping, view.tea_clock);
    V3<R> colors(R(0)), albedo(R(0)), normal(R(0));
    for (uint32_t i = 0; i < pc.spp; ++i) {
        rng.sample = i;
        rng.ray_seed = tea(mapping, view.tea_clock + 2u + i);
        rng.set_depth(0);
        Payload<R> ray;
        R jx = (R)rng.jitter();
        R jy = (R)rng.jitter();
        R posx = (R)px + jx, posy = (R)py + jy;
        R nx = posx / (R)view.width, ny = posy / (R)view.height;
        R dx = nx * R(2) - R(1), dy = ny * R(2) - R(1);
        R aperture = (R)cam.position[3];
        R focusDistance = (R)cam.front[3];
        R offx = 0, offy = 0;
        if (view.rng_mode == KF_ORACLE_RNG_TEA_LCG || aperture > R(0)) {
            R qx, qy;
            diskSampling<R>(rng, KF_RNG_LENS, qx, qy);
            offx = aperture / R(2) * qx;
            offy = aperture / R(2) * qy;
        }
        R tgt_in[4] = {dx, dy, R(1), R(1)}, target[4];
        mat4_mul<R>(cam.proj_inv, tgt_in, target);
        R origin[4], direction[4];
        if (aperture > R(0)) {
            R o_in[4] = {offx, offy, R(0), R(1)};
            mat4_mul<R>(cam.view_inv, o_in, origin);
            V3<R> tv = V3<R>(target[0], target[1], target[2]) * focusDistance - V3<R>(offx, offy, R(0));
            V3<R> nd = normalize(tv);
            R d_in[4] = {nd.x, nd.y, nd.z, R(0)};
            mat4_mul<R>(cam.view_inv, d_in, direction);
        } else {
            R o_in[4] = {R(0), R(0), R(0), R(1)};
            mat4_mul<R>(cam.view_inv, o_in, origin);
            V3<R> nd = normalize(V3<R>(target[0], target[1], target[2]));
            R d_in[4] = {nd.x, nd.y, nd.z, R(0)};
            mat4_mul<R>(cam.view_inv, d_in, direction);
        }
        ray.direction = V3<R>(direction[0], direction[1], direction[2]);
        ray.origin = V3<R>(origin[0], origin[1], origin[2]);
        ray.weight = V3<R>(R(0));
        ray.emission = V3<R>(R(1));
        ray.albedo = V3<R>(R(0));
        ray.normal = V3<R>(R(0));
        ray.shadow_color = V3<R>(R(0));
        V3<R> weight(R(1)), color(R(0));
        uint32_t traces = 0;
        AnyHit ah;
        ah.rng = &rng;
        for (ray.depth = 0; ray.depth <= pc.max_path_depth; ++ray.depth) {
            rng.set_depth(ray.depth);
            const uint32_t depth_at_trace = ray.depth;
            V3<float> of = tof(ray.origin), dfv = tof(ray.direction);
            float og[3] = {of.x, of.y, of.z}, dg[3] = {dfv.x, dfv.y, dfv.z};
            HitRec h;
            bool hit = trace(*cx.sa, og, dg, KF_T_MIN, KF_T_MAX, false, h, &ah);
            traces++;
            if (depth_at_trace == 0) {
                if (out->primary_hits) {
                    kf_hit& ph = out->primary_hits[(size_t)i * crop_pixels + out_index];
                    ph.t = h.t; ph.u = h.u; ph.v = h.v; ph.instance = h.inst; ph.prim = h.prim;
                    ph.pad[0] = ph.pad[1] = ph.pad[2] = 0;
                }
            } else {
                cx.rays_extension++;
            }
            if (!hit) {
                // PathTrace.rmiss:12-31: environment map, else clear colour
                if (pc.use_env_map && cx.s->env_rgba32f && cx.s->env_size) {
                    float e[3];
                    env_lookup(*cx.s, dg, e);
                    ray.emission = V3<R>((R)e[0], (R)e[1], (R)e[2]);
                } else {
                    ray.emission = V3<R>((R)pc.clear_color[0], (R)pc.clear_color[1], (R)pc.clear_color[2]) *
                                   (R)pc.clear_color[3];
                }
                ray.depth = pc.max_path_depth + 1;
            } else {
                closestHit<R>(cx, rng, ray, h, og, dg);
            }
            color = color + ray.emission * weight;
            weight = weight * ray.weight;
            color = color + ray.shadow_color * weight;
            ray.shadow_color = V3<R>(R(0));
            if (i == 0 && ray.depth == 0) {
                albedo = ray.albedo;
                normal = ray.normal;
            }
            if (weight == V3<R>(R(0))) break;
            if (pc.russian_roulette && ray.depth >= pc.rr_min_bounces) {
                R p = std::max(weight.x, std::max(weight.y, weight.z));
                R rand = (R)rng.next(KF_RNG_RR);
                if (rand > p) break;
                weight = weight * (R(1) / p);
            }
        }
        if (out->path_radiance) {
            float* pr = out->path_radiance + ((size_t)i * crop_pixels + out_index) * 3;
            pr[0] = (float)color.x; pr[1] = (float)color.y; pr[2] = (float)color.z;
        }
        if (out->path_depths) out->path_depths[(size_t)i * crop_pixels + out_index] = traces;
        colors = colors + color;
    }
    V3<R> finalColor = colors / (R)pc.spp;
    if (out->pixel_color) {
        float* p = out->pixel_color + (size_t)out_index * 3;
        p[0] = (float)finalColor.x; p[1] = (float)finalColor.y; p[2] = (float)finalColor.z;
    }
    if (out->pixel_color64) {
        double* p = out->pixel_color64 + (size_t)out_index * 3;
        p[0] = (double)finalColor.x; p[1] = (double)finalColor.y; p[2] = (double)finalColor.z;
    }
    if (out->albedo) {
        float* p = out->albedo + (size_t)out_index * 3;
        p[0] = (float)albedo.x; p[1] = (float)albedo.y; p[2] = (float)albedo.z;
    }
    if (out->normal) {
        float* p = out->normal + (size_t)out_index * 3;
        p[0] = (float)normal.x; p[1] = (float)normal.y; p[2] = (float)normal.z;
    }
}

void prepare_accel(SceneAccel& sa, const kf_flat_scene* s, bool use_bvh) {
    sa.s = s;
    sa.use_bvh = use_bvh;
    if (use_bvh) {
        sa.geoms.resize(s->num_geometries);
        for (uint32_t g = 0; g < s->num_geometries; ++g) build_bvh(sa.geoms[g], s->geometries[g]);
    }
}

// double-precision 4x4 inverse by cofactors (used for camera matrices).
void inverse4(const double* m, double* inv) {
    double a[16];
    std::memcpy(a, m, sizeof(a));
    double r[16];
    r[0] = a[5] * a[10] * a[15] - a[5] * a[11] * a[14] - a[9] * a[6] * a[15] + a[9] * a[7] * a[14] + a[13] * a[6] * a[11] - a[13] * a[7] * a[10];
    r[4] = -a[4] * a[10] * a[15] + a[4] * a[11] * a[14] + a[8] * a[6] * a[15] - a[8] * a[7] * a[14] - a[12] * a[6] * a[11] + a[12] * a[7] * a[10];
    r[8] = a[4] * a[9] * a[15] - a[4] * a[11] * a[13] - a[8] * a[5] * a[15] + a[8] * a[7] * a[13] + a[12] * a[5] * a[11] - a[12] * a[7] * a[9];
    r[12] = -a[4] * a[9] * a[14] + a[4] * a[10] * a[13] + a[8] * a[5] * a[14] - a[8] * a[6] * a[13] - a[12] * a[5] * a[10] + a[12] * a[6] * a[9];
    r[1] = -a[1] * a[10] * a[15] + a[1] * a[11] * a[14] + a[9] * a[2] * a[15] - a[9] * a[3] * a[14] - a[13] * a[2] * a[11] + a[13] * a[3] * a[10];
    r[5] = a[0] * a[10] * a[15] - a[0] * a[11] * a[14] - a[8] * a[2] * a[15] + a[8] * a[3] * a[14] + a[12] * a[2] * a[11] - a[12] * a[3] * a[10];
    r[9] = -a[0] * a[9] * a[15] + a[0] * a[11] * a[13] + a[8] * a[1] * a[15] - a[8] * a[3] * a[13] - a[12] * a[1] * a[11] + a[12] * a[3] * a[9];
    r[13] = a[0] * a[9] * a[14] - a[0] * a[10] * a[13] - a[8] * a[1] * a[14] + a[8] * a[2] * a[13] + a[12] * a[1] * a[10] - a[12] * a[2] * a[9];
    r[2] = a[1] * a[6] * a[15] - a[1] * a[7] * a[14] - a[5] * a[2] * a[15] + a[5] * a[3] * a[14] + a[13] * a[2] * a[7] - a[13] * a[3] * a[6];
    r[6] = -a[0] * a[6] * a[15] + a[0] * a[7] * a[14] + a[4] * a[2] * a[15] - a[4] * a[3] * a[14] - a[12] * a[2] * a[7] + a[12] * a[3] * a[6];
    r[10] = a[0] * a[5] * a[15] - a[0] * a[7] * a[13] - a[4] * a[1] * a[15] + a[4] * a[3] * a[13] + a[12] * a[1] * a[7] - a[12] * a[3] * a[5];
    r[14] = -a[0] * a[5] * a[14] + a[0] * a[6] * a[13] + a[4] * a[1] * a[14] - a[4] * a[2] * a[13] - a[12] * a[1] * a[6] + a[12] * a[2] * a[5];
    r[3] = -a[1] * a[6] * a[11] + a[1] * a[7] * a[10] + a[5] * a[2] * a[11] - a[5] * a[3] * a[10] - a[9] * a[2] * a[7] + a[9] * a[3] * a[6];
    r[7] = a[0] * a[6] * a[11] - a[0] * a[7] * a[10] - a[4] * a[2] * a[11] + a[4] * a[3] * a[10] + a[8] * a[2] * a[7] - a[8] * a[3] * a[6];
    r[11] = -a[0] * a[5] * a[11] + a[0] * a[7] * a[9] + a[4] * a[1] * a[11] - a[4] * a[3] * a[9] - a[8] * a[1] * a[7] + a[8] * a[3] * a[5];
    r[15] = a[0] * a[5] * a[10] - a[0] * a[6] * a[9] - a[4] * a[1] * a[10] + a[4] * a[2] * a[9] + a[8] * a[1] * a[6] - a[8] * a[2] * a[5];
    double det = a[0] * r[0] + a[1] * r[4] + a[2] * r[8] + a[3] * r[12];
    for (int i = 0; i < 16; ++i) inv[i] = r[i] / det;
}

} // namespace

// ---------------------------------------------------------------------------
// C API
// ---------------------------------------------------------------------------
extern "C" {

// The references a flat scene holds stay inside its arrays: vertex indices, material
// indices and instance geometry indices (the product refuses such a scene before its
// upload with KF_ERR_OUT_OF_RANGE; here it is return code 3).
static bool scene_consistent(const kf_flat_scene* s) {
    for (uint32_t i = 0; i < s->num_instances; ++i)
        if (s->instances[i].geometry_index >= s->num_geometries) return false;
    for (uint32_t gi = 0; gi < s->num_geometries; ++gi) {
        const kf_flat_geometry& g = s->geometries[gi];
        for (uint32_t t = 0; t < g.num_triangles; ++t) {
            if (g.mat_index[t] >= s->num_materials) return false;
            for (int k = 0; k < 3; ++k)
                if (g.indices[3 * t + k] >= g.num_vertices) return false;
        }
    }
    return true;
}

int kf_oracle_render(const kf_flat_scene* scene, const kf_oracle_view* view, kf_oracle_out* out) {
    if (!scene || !view || !out || !view->camera || view->width == 0 || view->height == 0) return 1;
    if (!scene_consistent(scene)) return 3;
    const uint32_t cw = view->crop_w ? view->crop_w : view->width;
    const uint32_t ch = view->crop_h ? view->crop_h : view->height;
    if (view->x0 + cw > view->width || view->y0 + ch > view->height) return 2;
    SceneAccel sa;
    prepare_accel(sa, scene, view->use_bvh != 0);
    const uint32_t crop_pixels = cw * ch;
    unsigned nt = view->threads ? view->threads : std::max(1u, std::thread::hardware_concurrency());
    std::atomic<uint32_t> next_row{0};
    std::atomic<uint64_t> rs{0}, re{0};
    auto worker = [&]() {
        Ctx cx;
        cx.sa = &sa;
        cx.s = scene;
        cx.pc = &view->pc;
        for (;;) {
            uint32_t row = next_row.fetch_add(1);
            if (row >= ch) break;
            for (uint32_t x = 0; x < cw; ++x) {
                uint32_t oi = row * cw + x;
                if (view->precision == KF_ORACLE_FP64)
                    render_pixel<double>(cx, *view, view->x0 + x, view->y0 + row, oi, crop_pixels, out);
                else
                    render_pixel<float>(cx, *view, view->x0 + x, view->y0 + row, oi, crop_pixels, out);
            }
        }
        rs += cx.rays_shadow;
        re += cx.rays_extension;
    };
    std::vector<std::thread> th;
    for (unsigned t = 1; t < nt; ++t) th.emplace_back(worker);
    worker();
    for (auto& t : th) t.join();
    out->rays_primary = (uint64_t)crop_pixels * view->pc.spp;
    out->rays_extension = re.load();
    out->rays_shadow = rs.load();
    return 0;
}

int kf_oracle_trace(const kf_flat_scene* scene, const float* rays, uint32_t n, uint32_t use_bvh, kf_hit* out) {
    if (!scene || (!rays && n) || (!out && n)) return 1;
    if (!scene_consistent(scene)) return 3;
    SceneAccel sa;
    prepare_accel(sa, scene, use_bvh != 0);
    for (uint32_t i = 0; i < n; ++i) {
        const float* r = rays + (size_t)i * 8;
        HitRec h;
        trace(sa, r, r + 4, r[3], r[7], false, h, nullptr);
        out[i].t = h.t; out[i].u = h.u; out[i].v = h.v; out[i].instance = h.inst; out[i].prim = h.prim;
        out[i].pad[0] = out[i].pad[1] = out[i].pad[2] = 0;
    }
    return 0;
}

void kf_oracle_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    philox4x32_10(ctr, key, out);
}
uint32_t kf_oracle_tea(uint32_t v0, uint32_t v1) { return tea(v0, v1); }
float kf_oracle_rnd_lcg(uint32_t* state) { return rnd_lcg(*state); }
float kf_oracle_uniform(uint32_t seed, uint32_t pixel, uint32_t camera, uint32_t sample, uint32_t frame,
                        uint32_t depth, uint32_t purpose, uint32_t draw) {
    uint32_t ctr[4] = {sample, frame, (depth << 8) | purpose, draw >> 2};
    uint32_t key[2] = {seed ^ pixel, camera};
    uint32_t out[4];
    philox4x32_10(ctr, key, out);
    return u24(out[draw & 3]);
}
float kf_oracle_sin(float x) { return kf_sin(x); }
float kf_oracle_cos(float x) { return kf_cos(x); }
float kf_oracle_exp2(float x) { return kf_exp2(x); }

int kf_oracle_intersect(const float org[3], const float dir[3], const float v0[3], const float v1[3],
                        const float v2[3], float tmin, float tmax, float* t, float* u, float* v) {
    Ray32 r;
    for (int i = 0; i < 3; ++i) { r.o[i] = org[i]; r.d[i] = dir[i]; }
    ray_setup(r);
    return intersect_tri(r, v0, v1, v2, tmin, tmax, *t, *u, *v) ? 1 : 0;
}
void kf_oracle_sample_ggx(float u0, float u1, float a2, const float n[3], float out[3]) {
    V3<float> h = sampleGGX(u0, u1, a2, V3<float>(n[0], n[1], n[2]));
    out[0] = h.x; out[1] = h.y; out[2] = h.z;
}
void kf_oracle_cosine_hemisphere(float u0, float u1, const float n[3], float out[3]) {
    V3<float> h = cosineHemisphereSampling(u0, u1, V3<float>(n[0], n[1], n[2]));
    out[0] = h.x; out[1] = h.y; out[2] = h.z;
}
float kf_oracle_schlick(float cosine, float ior) { return Schlick(cosine, ior); }
float kf_oracle_ggx_d(float ndoth, float a2) { return ggxNormalDistribution(ndoth, a2); }
float kf_oracle_g1(float d, float a2) { return G1(d, a2); }
void kf_oracle_schlick_fresnel(const float f0[3], float ldoth, float out[3]) {
    V3<float> r = schlickFresnel(V3<float>(f0[0], f0[1], f0[2]), ldoth);
    out[0] = r.x; out[1] = r.y; out[2] = r.z;
}

// Camera UBO as kuafu's host code builds it: view = glm::lookAt(pos, pos + front, up)
// (camera.cpp:92-94), projection from intrinsics (camera.cpp:111-124, near 0.1, far 100),
// inverses in double rounded to float (glm is not vendored; its float inverse is replaced).
void kf_oracle_camera_ubo(const float position[3], const float front[3], const float up[3], float width,
                          float height, float fx, float fy, float cx, float cy, float skew, kf_camera_ubo* out) {
    std::memset(out, 0, sizeof(*out));
    // lookAt (right-handed): f = normalize(center - eye), s = normalize(cross(f, up)), u = cross(s, f)
    V3<float> eye(position[0], position[1], position[2]);
    V3<float> center = eye + V3<float>(front[0], front[1], front[2]);
    V3<float> upv(up[0], up[1], up[2]);
    auto nrm = [](V3<float> v) { float inv = 1.0f / std::sqrt(dot(v, v)); return v * inv; };
    V3<float> f = nrm(center - eye);
    V3<float> s = nrm(cross(f, upv));
    V3<float> u = cross(s, f);
    float* V = out->view;
    for (int i = 0; i < 16; ++i) V[i] = (i % 5 == 0) ? 1.0f : 0.0f;
    V[0 * 4 + 0] = s.x; V[1 * 4 + 0] = s.y; V[2 * 4 + 0] = s.z;
    V[0 * 4 + 1] = u.x; V[1 * 4 + 1] = u.y; V[2 * 4 + 1] = u.z;
    V[0 * 4 + 2] = -f.x; V[1 * 4 + 2] = -f.y; V[2 * 4 + 2] = -f.z;
    V[3 * 4 + 0] = -dot(s, eye);
    V[3 * 4 + 1] = -dot(u, eye);
    V[3 * 4 + 2] = dot(f, eye);
    const float nearp = 0.1f, farp = 100.0f;
    float* P = out->proj;
    for (int i = 0; i < 16; ++i) P[i] = 0.0f;
    P[0 * 4 + 0] = (2.0f * fx) / width;
    P[1 * 4 + 0] = -2.0f * skew / width;
    P[1 * 4 + 1] = -(2.0f * fy) / height;
    P[2 * 4 + 0] = -2.0f * cx / width + 1.0f;
    P[2 * 4 + 1] = -2.0f * cy / height + 1.0f;
    P[2 * 4 + 2] = -farp / (farp - nearp);
    P[2 * 4 + 3] = -1.0f;
    P[3 * 4 + 2] = -farp * nearp / (farp - nearp);
    P[3 * 4 + 3] = 0.0f;
    double md[16], mi[16];
    for (int i = 0; i < 16; ++i) md[i] = V[i];
    inverse4(md, mi);
    for (int i = 0; i < 16; ++i) out->view_inv[i] = (float)mi[i];
    for (int i = 0; i < 16; ++i) md[i] = P[i];
    inverse4(md, mi);
    for (int i = 0; i < 16; ++i) out->proj_inv[i] = (float)mi[i];
    out->position[0] = eye.x; out->position[1] = eye.y; out->position[2] = eye.z; out->position[3] = 0.0f;
    out->front[0] = front[0]; out->front[1] = front[1]; out->front[2] = front[2]; out->front[3] = 5.0f;
    for (int i = 0; i < 4; ++i) out->pad1[i] = out->pad2[i] = 1.0f;
}

uint8_t kf_oracle_srgb8(float linear) { return srgb_encode8(linear); }

void kf_oracle_perpendicular(const float u[3], float out[3]) {
    V3<float> r = getPerpendicularVector(V3<float>(u[0], u[1], u[2]));
    out[0] = r.x; out[1] = r.y; out[2] = r.z;
}
void kf_oracle_uniform_sphere_lcg(uint32_t* state, float out[3]) {
    Rng rng;
    rng.mode = KF_ORACLE_RNG_TEA_LCG;
    rng.ray_seed = *state;
    V3<float> p = uniformSphereSampling<float>(rng, 0);
    *state = rng.ray_seed;
    out[0] = p.x; out[1] = p.y; out[2] = p.z;
}
void kf_oracle_disk_lcg(uint32_t* state, float out[2]) {
    Rng rng;
    rng.mode = KF_ORACLE_RNG_TEA_LCG;
    rng.ray_seed = *state;
    diskSampling<float>(rng, 0, out[0], out[1]);
    *state = rng.ray_seed;
}

// The icosphere of the benchmark scenes: the icosahedron (golden-ratio vertices, 20 faces),
// every face split into four `level` times with edge midpoints pushed to the unit sphere
// (in double), then Geometry::recalculateNormals (geometry.cpp:268-295): the unit face
// normals summed per vertex in face order (degenerate faces skipped) and renormalised, in
// float, with glm::normalize = v * (1 / length(v)). uv are the spherical angles.
int kf_oracle_icosphere(int level, kf_vertex* v, uint32_t vcap, uint32_t* idx, uint32_t icap, uint32_t* nv,
                        uint32_t* ni) {
    if (level < 0 || level > 8 || !nv || !ni) return 1;
    const double g = (1.0 + std::sqrt(5.0)) / 2.0;
    std::vector<std::array<double, 3>> P = {{-1, g, 0}, {1, g, 0},   {-1, -g, 0}, {1, -g, 0},
                                            {0, -1, g}, {0, 1, g},   {0, -1, -g}, {0, 1, -g},
                                            {g, 0, -1}, {g, 0, 1},   {-g, 0, -1}, {-g, 0, 1}};
    auto unit = [](std::array<double, 3> p) {
        const double n = std::sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
        return std::array<double, 3>{p[0] / n, p[1] / n, p[2] / n};
    };
    for (auto& p : P) p = unit(p);
    std::vector<uint32_t> F = {0, 11, 5, 0, 5, 1, 0, 1, 7, 0, 7, 10, 0, 10, 11, 1, 5, 9, 5, 11, 4, 11, 10, 2,
                               10, 7, 6, 7, 1, 8, 3, 9, 4, 3, 4, 2, 3, 2, 6, 3, 6, 8, 3, 8, 9, 4, 9, 5,
                               2, 4, 11, 6, 2, 10, 8, 6, 7, 9, 8, 1};
    for (int l = 0; l < level; ++l) {
        std::map<uint64_t, uint32_t> mids;
        auto mid = [&](uint32_t a, uint32_t b) -> uint32_t {
            const uint64_t key = ((uint64_t)std::min(a, b) << 32) | std::max(a, b);
            auto it = mids.find(key);
            if (it != mids.end()) return it->second;
            P.push_back(unit({(P[a][0] + P[b][0]) * 0.5, (P[a][1] + P[b][1]) * 0.5, (P[a][2] + P[b][2]) * 0.5}));
            return mids[key] = (uint32_t)P.size() - 1;
        };
        std::vector<uint32_t> next;
        next.reserve(F.size() * 4);
        for (size_t f = 0; f < F.size(); f += 3) {
            const uint32_t a = F[f], b = F[f + 1], c = F[f + 2];
            const uint32_t ab = mid(a, b), bc = mid(b, c), ca = mid(c, a);
            const uint32_t sub[12] = {a, ab, ca, b, bc, ab, c, ca, bc, ab, bc, ca};
            next.insert(next.end(), sub, sub + 12);
        }
        F.swap(next);
    }
    *nv = (uint32_t)P.size();
    *ni = (uint32_t)F.size();
    if (vcap == 0 && icap == 0) return 0;
    if (!v || !idx || vcap < P.size() || icap < F.size()) return 2;
    const double pi = 3.14159265358979323846;
    for (size_t i = 0; i < P.size(); ++i) {
        kf_vertex& o = v[i];
        std::memset(&o, 0, sizeof(o));
        for (int k = 0; k < 3; ++k) o.pos[k] = (float)P[i][k];
        o.uv[0] = (float)(0.5 + std::atan2(P[i][1], P[i][0]) / (2.0 * pi));
        o.uv[1] = (float)(0.5 - std::asin(std::max(-1.0, std::min(1.0, P[i][2]))) / pi);
    }
    auto normalize = [](V3<float> a) { const float inv = 1.0f / std::sqrt(dot(a, a)); return a * inv; };
    for (size_t f = 0; f < F.size(); f += 3) {
        kf_vertex& A = v[F[f]];
        kf_vertex& B = v[F[f + 1]];
        kf_vertex& C = v[F[f + 2]];
        const V3<float> pa(A.pos[0], A.pos[1], A.pos[2]), pb(B.pos[0], B.pos[1], B.pos[2]),
            pc(C.pos[0], C.pos[1], C.pos[2]);
        const V3<float> n = normalize(cross(pb - pa, pc - pa));
        if (std::isnan(n.x)) continue;
        for (kf_vertex* q : {&A, &B, &C}) {
            q->normal[0] += n.x;
            q->normal[1] += n.y;
            q->normal[2] += n.z;
        }
    }
    for (size_t i = 0; i < P.size(); ++i) {
        V3<float> n(v[i].normal[0], v[i].normal[1], v[i].normal[2]);
        if (n.x == 0.0f && n.y == 0.0f && n.z == 0.0f) continue;
        n = normalize(n);
        v[i].normal[0] = n.x; v[i].normal[1] = n.y; v[i].normal[2] = n.z;
    }
    std::memcpy(idx, F.data(), F.size() * sizeof(uint32_t));
    return 0;
}

int kf_oracle_instance_rows(const float m[16], float rows[12]) {
    double A[3][3], t[3];
    for (int r = 0; r < 3; ++r) {
        for (int c = 0; c < 3; ++c) A[r][c] = m[c * 4 + r];
        t[r] = m[12 + r];
    }
    // adjugate / determinant of the linear part, then -A^-1 t for the translation
    const double c00 = A[1][1] * A[2][2] - A[1][2] * A[2][1];
    const double c01 = A[1][2] * A[2][0] - A[1][0] * A[2][2];
    const double c02 = A[1][0] * A[2][1] - A[1][1] * A[2][0];
    const double det = A[0][0] * c00 + A[0][1] * c01 + A[0][2] * c02;
    if (det == 0.0 || !std::isfinite(det)) return 1;
    double I[3][3];
    I[0][0] = c00 / det;
    I[0][1] = (A[0][2] * A[2][1] - A[0][1] * A[2][2]) / det;
    I[0][2] = (A[0][1] * A[1][2] - A[0][2] * A[1][1]) / det;
    I[1][0] = c01 / det;
    I[1][1] = (A[0][0] * A[2][2] - A[0][2] * A[2][0]) / det;
    I[1][2] = (A[0][2] * A[1][0] - A[0][0] * A[1][2]) / det;
    I[2][0] = c02 / det;
    I[2][1] = (A[0][1] * A[2][0] - A[0][0] * A[2][1]) / det;
    I[2][2] = (A[0][0] * A[1][1] - A[0][1] * A[1][0]) / det;
    for (int r = 0; r < 3; ++r) {
        rows[r * 4 + 0] = (float)I[r][0];
        rows[r * 4 + 1] = (float)I[r][1];
        rows[r * 4 + 2] = (float)I[r][2];
        rows[r * 4 + 3] = (float)(-(I[r][0] * t[0] + I[r][1] * t[1] + I[r][2] * t[2]));
    }
    return 0;
}

void kf_oracle_light_ubos(const float* dir, const float* points, uint32_t num_points, const float* actives,
                          uint32_t num_actives, uint32_t num_textures, kf_dir_light_ubo* d, kf_point_lights_ubo* p,
                          kf_active_lights_ubo* a) {
    std::memset(d, 0, sizeof(*d));
    std::memset(p, 0, sizeof(*p));
    std::memset(a, 0, sizeof(*a));
    if (dir) {  // direction = {normalize(direction), softness}, rgbs = {color, strength}
        const V3<float> dv(dir[0], dir[1], dir[2]);
        const float inv = 1.0f / std::sqrt(dot(dv, dv));
        d->direction[0] = dv.x * inv; d->direction[1] = dv.y * inv; d->direction[2] = dv.z * inv;
        d->direction[3] = dir[7];
        d->rgbs[0] = dir[3]; d->rgbs[1] = dir[4]; d->rgbs[2] = dir[5]; d->rgbs[3] = dir[6];
    }
    for (uint32_t i = 0; i < KF_MAX_POINT_LIGHTS && i < num_points; ++i) {
        const float* l = points + (size_t)i * 8;
        p->posr[i][0] = l[0]; p->posr[i][1] = l[1]; p->posr[i][2] = l[2]; p->posr[i][3] = l[6];
        p->rgbs[i][0] = l[3]; p->rgbs[i][1] = l[4]; p->rgbs[i][2] = l[5]; p->rgbs[i][3] = l[7];
    }
    for (uint32_t i = 0; i < KF_MAX_ACTIVE_LIGHTS && i < num_actives; ++i) {
        const float* l = actives + (size_t)i * 24;
        double vd[16], vi[16];
        for (int k = 0; k < 16; ++k) vd[k] = l[k];
        inverse4(vd, vi);  // glm::inverse(viewMat), in double rounded to float
        float inv[16];
        for (int k = 0; k < 16; ++k) inv[k] = (float)vi[k];
        std::memcpy(a->view[i], l, sizeof(float) * 16);
        // glm::perspective(fov, 1, 0.01, 1000): right-handed, clip depth [-1, 1]
        const float fov = l[19], zn = 0.01f, zf = 1000.0f, aspect = 1.0f;
        const float th = std::tan(fov / 2.0f);
        float* P = a->proj[i];
        P[0] = 1.0f / (aspect * th);
        P[5] = 1.0f / th;
        P[10] = -(zf + zn) / (zf - zn);
        P[11] = -1.0f;
        P[14] = -(2.0f * zf * zn) / (zf - zn);
        a->front[i][0] = -inv[8]; a->front[i][1] = -inv[9]; a->front[i][2] = -inv[10]; a->front[i][3] = 1.0f;
        a->rgbs[i][0] = l[16]; a->rgbs[i][1] = l[17]; a->rgbs[i][2] = l[18]; a->rgbs[i][3] = l[20];
        a->position[i][0] = inv[12]; a->position[i][1] = inv[13]; a->position[i][2] = inv[14];
        const int tex = (int)l[22];
        a->sftp[i][0] = l[21];
        a->sftp[i][1] = fov;
        a->sftp[i][2] = (tex >= 0 && (uint32_t)tex < num_textures) ? (float)tex : -1.0f;
    }
}

} // extern "C"
