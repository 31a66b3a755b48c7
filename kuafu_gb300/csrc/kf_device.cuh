// kf_device.cuh — device-side building blocks of the GB300 path tracer:
// vector math with GLSL semantics, Philox4x32-10 random streams, deterministic
// sin/cos/exp2, the watertight ray/triangle test and the wide-BVH node layout.
//
// Every translation unit that includes this header is compiled with
// -fmad=false: a*b+c rounds twice unless written as an explicit fmaf(), so the
// arithmetic is the one the shaders (resources/shaders/*) spell out.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/kf_types.h"

#define KF_DEV __device__ __forceinline__

namespace kf {

// 32-byte aligned double quadruple (FP64 accumulation targets).
struct alignas(32) dbl4 {
    double x, y, z, w;
};
__host__ __device__ __forceinline__ dbl4 make_dbl4(double x, double y, double z, double w) { return dbl4{x, y, z, w}; }

// ---------------------------------------------------------------------------
// vec3 with GLSL semantics (component-wise, left-to-right).
// ---------------------------------------------------------------------------
struct v3 {
    float x, y, z;
};
KF_DEV v3 mk(float a, float b, float c) { return v3{a, b, c}; }
KF_DEV v3 splat(float a) { return v3{a, a, a}; }
KF_DEV v3 operator+(v3 a, v3 b) { return v3{a.x + b.x, a.y + b.y, a.z + b.z}; }
KF_DEV v3 operator-(v3 a, v3 b) { return v3{a.x - b.x, a.y - b.y, a.z - b.z}; }
KF_DEV v3 operator-(v3 a) { return v3{-a.x, -a.y, -a.z}; }
KF_DEV v3 operator*(v3 a, v3 b) { return v3{a.x * b.x, a.y * b.y, a.z * b.z}; }
KF_DEV v3 operator*(v3 a, float s) { return v3{a.x * s, a.y * s, a.z * s}; }
KF_DEV v3 operator*(float s, v3 a) { return v3{s * a.x, s * a.y, s * a.z}; }
KF_DEV v3 operator/(v3 a, float s) { return v3{a.x / s, a.y / s, a.z / s}; }
KF_DEV bool operator==(v3 a, v3 b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
KF_DEV bool operator!=(v3 a, v3 b) { return !(a == b); }
KF_DEV float dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
KF_DEV v3 cross(v3 a, v3 b) { return v3{a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y}; }
KF_DEV float length(v3 a) { return sqrtf(dot(a, a)); }
KF_DEV v3 normalize(v3 a) {
    float inv = 1.0f / length(a);
    return a * inv;
}
KF_DEV float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }
KF_DEV v3 reflect(v3 I, v3 N) { return I - (2.0f * dot(N, I)) * N; }
KF_DEV v3 refract(v3 I, v3 N, float eta) {
    float d = dot(N, I);
    float k = 1.0f - eta * eta * (1.0f - d * d);
    if (k < 0.0f) return splat(0.0f);
    return eta * I - (eta * d + sqrtf(k)) * N;
}
KF_DEV v3 ld3(const float* p) { return v3{p[0], p[1], p[2]}; }
KF_DEV v3 xyz(float4 a) { return v3{a.x, a.y, a.z}; }

// GLSL clamp uses min(max(x, lo), hi): NaN inputs resolve like fmaxf/fminf.
// (std::min/max on the CPU oracle agree for the finite values the shaders produce.)

// ---------------------------------------------------------------------------
// Deterministic transcendentals: Cody-Waite reduction by pi/2 in three float
// parts, then Taylor series on [-pi/4, pi/4]; exp2 as 2^k * e^(f ln 2) with
// |f| <= 1/2 and a degree-7 Taylor polynomial. Constants are exact values
// rounded to float. The CPU oracle evaluates the same method, so results are
// bit-identical on both sides (<= 2 ulp from the true value).
// ---------------------------------------------------------------------------
KF_DEV float poly_sin(float r) {
    float r2 = r * r;
    float p = fmaf(r2, 0x1.71de3ap-19f, -0x1.a01a02p-13f);
    p = fmaf(r2, p, 0x1.111112p-7f);
    p = fmaf(r2, p, -0x1.555556p-3f);
    return fmaf(r * r2, p, r);
}
KF_DEV float poly_cos(float r) {
    float r2 = r * r;
    float p = fmaf(r2, -0x1.27e4fcp-22f, 0x1.a01a02p-16f);
    p = fmaf(r2, p, -0x1.6c16c2p-10f);
    p = fmaf(r2, p, 0x1.555556p-5f);
    p = fmaf(r2, p, -0.5f);
    return fmaf(r2, p, 1.0f);
}
KF_DEV float reduce_pio2(float x, int& q) {
    float k = rintf(x * 0x1.45f306p-1f);
    float r = fmaf(-k, 0x1.921fb6p+0f, x);
    r = fmaf(-k, -0x1.777a5cp-25f, r);
    r = fmaf(-k, -0x1.ee59dap-50f, r);
    q = ((int)k) & 3;
    return r;
}
KF_DEV float ksin(float x) {
    int q;
    float r = reduce_pio2(x, q);
    float s = (q & 1) ? poly_cos(r) : poly_sin(r);
    return (q & 2) ? -s : s;
}
KF_DEV float kcos(float x) {
    int q;
    float r = reduce_pio2(x, q);
    float c = (q & 1) ? poly_sin(r) : poly_cos(r);
    return ((q + 1) & 2) ? -c : c;
}
KF_DEV void ksincos(float x, float& s, float& c) {
    int q;
    float r = reduce_pio2(x, q);
    float ps = poly_sin(r), pc = poly_cos(r);
    float ss = (q & 1) ? pc : ps;
    float cc = (q & 1) ? ps : pc;
    s = (q & 2) ? -ss : ss;
    c = ((q + 1) & 2) ? -cc : cc;
}
KF_DEV float kexp2(float x) {
    if (!(x > -126.0f)) return (x != x) ? x : 0.0f;
    if (x > 127.0f) return __int_as_float(0x7f800000);
    float k = rintf(x);
    float f = x - k;
    float p = 0x1.ffcbfcp-17f;
    p = fmaf(p, f, 0x1.430912p-13f);
    p = fmaf(p, f, 0x1.5d87fep-10f);
    p = fmaf(p, f, 0x1.3b2ab6p-7f);
    p = fmaf(p, f, 0x1.c6b08ep-5f);
    p = fmaf(p, f, 0x1.ebfbe0p-3f);
    p = fmaf(p, f, 0x1.62e430p-1f);
    p = fmaf(p, f, 1.0f);
    return p * __int_as_float((int)(((int)k + 127) << 23));
}
KF_DEV float kpow5(float x) {
    float x2 = x * x;
    return (x2 * x2) * x;
}

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon et al., SC'11) and the per-path sub-streams.
// ---------------------------------------------------------------------------
// Not inlined: the shading kernel draws from a dozen call sites, and one shared copy of
// the ten rounds keeps its code (and register count) smaller.
static __device__ __noinline__ uint4 philox(uint4 c, uint2 k) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r) {
            k.x += 0x9E3779B9u;
            k.y += 0xBB67AE85u;
        }
        const uint32_t lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
        const uint32_t lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
        c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
    }
    return c;
}
KF_DEV float u24(uint32_t x) { return (float)(x >> 8) * (1.0f / 16777216.0f); }

// Identity of one path: its Philox key and the fixed counter words.
struct PathKey {
    uint2 key;       // {seed ^ pixel_index, camera_index}
    uint32_t sample; // ctr.x
    uint32_t frame;  // ctr.y
};

// One sequential sub-stream (a purpose at a bounce depth); caches one Philox block.
struct Stream {
    uint32_t tag; // (depth << 8) | purpose
    uint32_t idx;
    uint32_t blk;
    uint4 cache;
    KF_DEV void init(uint32_t depth, uint32_t purpose) {
        tag = (depth << 8) | purpose;
        idx = 0;
        blk = 0xFFFFFFFFu;
    }
    KF_DEV float next(const PathKey& pk) {
        const uint32_t b = idx >> 2;
        if (b != blk) {
            cache = philox(make_uint4(pk.sample, pk.frame, tag, b), pk.key);
            blk = b;
        }
        const uint32_t s = idx & 3;
        ++idx;
        const uint32_t w = s == 0 ? cache.x : (s == 1 ? cache.y : (s == 2 ? cache.z : cache.w));
        return u24(w);
    }
};

// ---------------------------------------------------------------------------
// Acceleration-structure layouts (replacing the driver's BLAS/TLAS of
// src/core/rt/rt.cpp:142-495).
// ---------------------------------------------------------------------------

// 4-wide node, 128 B = 8 x 16-B loads. Child c of the node is described by
// lane c of every field.  cnt[c] == 0: inner child, child[c] = node index;
// cnt[c] > 0: leaf with cnt[c] primitives starting at primitive f, child[c] =
// leaf_child(f, cnt[c]) (the traversal's stack entry for it); cnt[c] < 0: empty
// (inverted box, never hit).
struct alignas(16) Node4 {
    float4 lox, hix, loy, hiy, loz, hiz;
    int4 child;
    int4 cnt;
};
static_assert(sizeof(Node4) == 128, "Node4 must be 128 bytes");

// Leaf child link: bit 30 set, count - 1 (<= 15) in bits 26..29, first primitive in bits
// 0..25, so that the traversal pushes the link as it is. Rebasing a leaf by a primitive
// offset is a plain addition (the sum stays below 2^26).
constexpr uint32_t kLeafChildTag = 0x40000000u, kLeafFirstMask = 0x03FFFFFFu;
// A TLAS leaf of one instance links the instance itself: bit 31 set, instance index below.
constexpr uint32_t kInstChildTag = 0x80000000u;
__host__ __device__ __forceinline__ int leaf_child(int first, int count) {
    return (int)(kLeafChildTag | ((uint32_t)(count - 1) << 26) | (uint32_t)first);
}
__host__ __device__ __forceinline__ int leaf_first(int child) { return (int)((uint32_t)child & kLeafFirstMask); }

// TLAS instance record, 64 B: world->object rows + BLAS addressing.
struct alignas(16) InstanceRec {
    float4 w2o0, w2o1, w2o2;
    uint32_t blas_root; // node index in the BLAS node pool
    uint32_t geometry;  // geometry index
    uint32_t flags;     // bit0: opaque, bit1: hidden
    uint32_t pad;
};
static_assert(sizeof(InstanceRec) == 64, "InstanceRec must be 64 bytes");

// Precomputed triangle, 48 B: the three object-space vertices; w of the first
// float4 carries the primitive index within its geometry.
struct alignas(16) Tri {
    float4 v0, v1, v2;
};

// Ray prepared for the watertight test (Woop, Benthin, Wald, JCGT 2013) and
// for the slab test.
struct PRay {
    float ox, oy, oz;
    float dx, dy, dz;
    float ix, iy, iz; // 1 / d
    float Sx, Sy, Sz;
    int kx, ky, kz;
};

KF_DEV float comp(float x, float y, float z, int i) { return i == 0 ? x : (i == 1 ? y : z); }

KF_DEV void prep_ray(PRay& r) {
    int kz = 0;
    if (fabsf(r.dy) > fabsf(comp(r.dx, r.dy, r.dz, kz))) kz = 1;
    if (fabsf(r.dz) > fabsf(comp(r.dx, r.dy, r.dz, kz))) kz = 2;
    int kx = kz + 1;
    if (kx == 3) kx = 0;
    int ky = kx + 1;
    if (ky == 3) ky = 0;
    const float dkz = comp(r.dx, r.dy, r.dz, kz);
    if (dkz < 0.0f) {
        int t = kx;
        kx = ky;
        ky = t;
    }
    r.kx = kx;
    r.ky = ky;
    r.kz = kz;
    r.Sx = comp(r.dx, r.dy, r.dz, kx) / dkz;
    r.Sy = comp(r.dx, r.dy, r.dz, ky) / dkz;
    r.ix = 1.0f / r.dx;
    r.iy = 1.0f / r.dy;
    r.iz = 1.0f / r.dz;
    r.Sz = comp(r.ix, r.iy, r.iz, kz); // = 1 / dkz, the same correctly rounded quotient
}

// World -> object transform of a ray: o' = W2O (o, 1), d' = W2O (d, 0).
KF_DEV void to_object(const InstanceRec& in, float ox, float oy, float oz, float dx, float dy, float dz, PRay& r) {
    r.ox = in.w2o0.x * ox + in.w2o0.y * oy + in.w2o0.z * oz + in.w2o0.w;
    r.oy = in.w2o1.x * ox + in.w2o1.y * oy + in.w2o1.z * oz + in.w2o1.w;
    r.oz = in.w2o2.x * ox + in.w2o2.y * oy + in.w2o2.z * oz + in.w2o2.w;
    r.dx = in.w2o0.x * dx + in.w2o0.y * dy + in.w2o0.z * dz;
    r.dy = in.w2o1.x * dx + in.w2o1.y * dy + in.w2o1.z * dz;
    r.dz = in.w2o2.x * dx + in.w2o2.y * dy + in.w2o2.z * dz;
    prep_ray(r);
}

// Watertight ray/triangle test; both facings accepted (TRIANGLE_FACING_CULL_DISABLE,
// rt.cpp:134). Returns true with t in [tmin, tmax].
KF_DEV bool intersect_tri(const PRay& r, float4 a, float4 b, float4 c, float tmin, float tmax, float& t_out,
                          float& u_out, float& v_out) {
    const float Ax0 = a.x - r.ox, Ay0 = a.y - r.oy, Az0 = a.z - r.oz;
    const float Bx0 = b.x - r.ox, By0 = b.y - r.oy, Bz0 = b.z - r.oz;
    const float Cx0 = c.x - r.ox, Cy0 = c.y - r.oy, Cz0 = c.z - r.oz;
    const float Akx = comp(Ax0, Ay0, Az0, r.kx), Aky = comp(Ax0, Ay0, Az0, r.ky), Akz = comp(Ax0, Ay0, Az0, r.kz);
    const float Bkx = comp(Bx0, By0, Bz0, r.kx), Bky = comp(Bx0, By0, Bz0, r.ky), Bkz = comp(Bx0, By0, Bz0, r.kz);
    const float Ckx = comp(Cx0, Cy0, Cz0, r.kx), Cky = comp(Cx0, Cy0, Cz0, r.ky), Ckz = comp(Cx0, Cy0, Cz0, r.kz);
    const float Ax = Akx - r.Sx * Akz;
    const float Ay = Aky - r.Sy * Akz;
    const float Bx = Bkx - r.Sx * Bkz;
    const float By = Bky - r.Sy * Bkz;
    const float Cx = Ckx - r.Sx * Ckz;
    const float Cy = Cky - r.Sy * Ckz;
    float U = Cx * By - Cy * Bx;
    float V = Ax * Cy - Ay * Cx;
    float W = Bx * Ay - By * Ax;
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        const double CxBy = (double)Cx * (double)By, CyBx = (double)Cy * (double)Bx;
        U = (float)(CxBy - CyBx);
        const double AxCy = (double)Ax * (double)Cy, AyCx = (double)Ay * (double)Cx;
        V = (float)(AxCy - AyCx);
        const double BxAy = (double)Bx * (double)Ay, ByAx = (double)By * (double)Ax;
        W = (float)(BxAy - ByAx);
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    const float det = U + V + W;
    if (det == 0.0f) return false;
    const float Az = r.Sz * Akz;
    const float Bz = r.Sz * Bkz;
    const float Cz = r.Sz * Ckz;
    const float T = U * Az + V * Bz + W * Cz;
    const float t = T / det;
    if (!(t >= tmin && t <= tmax)) return false;
    t_out = t;
    u_out = V / det;
    v_out = W / det;
    return true;
}

// Conservative slab test against the four children of a node: far distances
// widened by 1 + 2*gamma(3) (Ize, JCGT 2013) so no box is culled by rounding.
// Returns a 4-bit mask of children hit and their entry distances.
#define KF_BOX_WIDEN (1.0f + 2.0f * (3.0f * 0x1.0p-24f) / (1.0f - 3.0f * 0x1.0p-24f))
// The current closest hit is widened too before a box is culled against it: a triangle
// whose computed t ties the closest hit (two walls meeting at a corner) may sit in a box
// whose computed entry distance lies a few ulp beyond that t; the tie rule needs it tested.
#define KF_TMAX_WIDEN (1.0f + 0x1.0p-19f)

KF_DEV float lane(float4 v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : (i == 2 ? v.z : v.w)); }
KF_DEV int lanei(int4 v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : (i == 2 ? v.z : v.w)); }

KF_DEV float slab1(float nearp, float farp, float o, float inv, float& tf) {
    tf = (farp - o) * inv;
    return (nearp - o) * inv;
}

KF_DEV int box4(const PRay& r, const Node4& n, float tmin, float tmax, float tn_out[4]) {
    int mask = 0;
    const bool px = r.ix >= 0.0f, py = r.iy >= 0.0f, pz = r.iz >= 0.0f;
    const float4 nx = px ? n.lox : n.hix, fx = px ? n.hix : n.lox;
    const float4 ny = py ? n.loy : n.hiy, fy = py ? n.hiy : n.loy;
    const float4 nz = pz ? n.loz : n.hiz, fz = pz ? n.hiz : n.loz;
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

// Closest-hit ordering with a deterministic tie rule (smallest t, then instance, then primitive).
KF_DEV bool closer(float t, uint32_t inst, uint32_t prim, float bt, uint32_t binst, uint32_t bprim) {
    if (binst == 0xFFFFFFFFu) return true;
    if (t < bt) return true;
    if (t == bt) return inst < binst || (inst == binst && prim < bprim);
    return false;
}

KF_DEV float4 ldg4(const float4* p) { return __ldg(p); }

KF_DEV Node4 load_node(const Node4* nodes, uint32_t i) {
    const float4* p = reinterpret_cast<const float4*>(nodes + i);
    Node4 n;
    n.lox = __ldg(p + 0);
    n.hix = __ldg(p + 1);
    n.loy = __ldg(p + 2);
    n.hiy = __ldg(p + 3);
    n.loz = __ldg(p + 4);
    n.hiz = __ldg(p + 5);
    const int4* q = reinterpret_cast<const int4*>(p + 6);
    n.child = __ldg(q);
    n.cnt = __ldg(q + 1);
    return n;
}

} // namespace kf
