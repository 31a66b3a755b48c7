"""Compiles kuafu's GLSL ray-tracing shaders as C++ (golden-vector generation only).

kuafu's render path is GLSL run by a Vulkan ray-tracing driver; neither exists
here. Its shaders are plain arithmetic over a few GLSL built-ins, so this module
turns them into one C++ translation unit:

  * the shader files are read where they lie (the reference checkout given by
    the caller; nothing of them is copied into the repository);
  * a mechanical rewrite: ``#version`` / ``#extension`` / ``#include`` lines go,
    resource declarations (``layout(...) uniform`` / ``buffer`` blocks, payload
    and hit-attribute declarations) go (this file declares them as C++ globals
    with the same member names), GLSL parameter qualifiers become C++
    (``inout T x`` -> ``T& x``, ``in T x`` -> ``T x``), swizzles ``.xyz`` /
    ``.rgb`` / ``.xy`` become accessor calls, and each shader's ``main`` is
    renamed after its stage;
  * COMPAT supplies vec2/vec3/vec4/mat4/mat4x3, the GLSL built-ins the shaders
    call, and brace-initialised constructors so constructor arguments are
    evaluated left to right as GLSL evaluates them (``vec3(rnd(s), rnd(s),
    rnd(s))`` draws in order);
  * g++ compiles with ``-fsingle-precision-constant`` (GLSL literals are float)
    and ``-ffp-contract=off``; sin / cos / pow(2, x) / pow(x, 5) come from the
    oracle's deterministic functions (GLSL leaves their rounding to the
    implementation), and the implementation-defined orders (dot products,
    matrix-vector sums) are the left-to-right ones the oracle states.

What stays the driver's (and so is supplied by the oracle): BVH traversal and
the watertight triangle test behind ``traceRayEXT``, the facing rule behind
``gl_HitKindEXT``, and texture filtering.
"""
from __future__ import annotations

import os
import re
from pathlib import Path


def reference_root(argv_path: str | None = None) -> Path:
    """The kuafu checkout: the command-line argument, else $KF_REFERENCE. No default."""
    p = argv_path or os.environ.get("KF_REFERENCE")
    if not p:
        raise SystemExit("give the kuafu checkout as the first argument or in $KF_REFERENCE")
    root = Path(p)
    if not (root / "resources" / "shaders" / "base" / "Random.glsl").exists():
        raise SystemExit(f"kuafu shaders not found under {root}/resources/shaders")
    return root


COMPAT = r"""
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#undef M_PI
typedef uint32_t uint;
extern "C" float kf_oracle_sin(float);
extern "C" float kf_oracle_cos(float);
extern "C" float kf_oracle_exp2(float);
namespace glsl {
struct uvec2_t { uint x, y; };
struct uvec3_t { uint x, y, z; uvec2_t xy() const { return uvec2_t{x, y}; } };
struct ivec2_t { int x, y;
  ivec2_t(int a, int b) : x(a), y(b) {}
  explicit ivec2_t(uvec2_t u) : x((int)u.x), y((int)u.y) {} };
struct ivec3_t { int x, y, z; ivec3_t(int a, int b, int c) : x(a), y(b), z(c) {} };
struct vec2_t { float x, y;
  vec2_t() : x(0), y(0) {}
  explicit vec2_t(float a) : x(a), y(a) {}
  vec2_t(float a, float b) : x(a), y(b) {}
  explicit vec2_t(uvec2_t u) : x((float)u.x), y((float)u.y) {} };
struct vec4_t;
struct vec3_t { float x, y, z;
  vec3_t() : x(0), y(0), z(0) {}
  explicit vec3_t(float a) : x(a), y(a), z(a) {}
  vec3_t(float a, float b, float c) : x(a), y(b), z(c) {}
  vec3_t(vec2_t a, float b) : x(a.x), y(a.y), z(b) {}
  explicit vec3_t(const vec4_t& v);
  vec2_t xy() const { return vec2_t(x, y); } };
struct vec4_t { float x, y, z, w;
  vec4_t() : x(0), y(0), z(0), w(0) {}
  explicit vec4_t(float a) : x(a), y(a), z(a), w(a) {}
  vec4_t(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
  vec4_t(vec3_t a, float b) : x(a.x), y(a.y), z(a.z), w(b) {}
  vec4_t(vec2_t a, float b, float c) : x(a.x), y(a.y), z(b), w(c) {}
  vec3_t xyz() const { return vec3_t(x, y, z); }
  vec2_t xy() const { return vec2_t(x, y); }
  vec4_t& operator/=(float s) { x /= s; y /= s; z /= s; w /= s; return *this; } };
inline vec3_t::vec3_t(const vec4_t& v) : x(v.x), y(v.y), z(v.z) {}
// column-major like GLSL: m[c * 4 + r]
struct mat4_t { float m[16]; };
// gl_WorldToObjectEXT: 4 columns of 3 rows
struct mat4x3_t { vec3_t c[4]; };

inline vec2_t operator+(vec2_t a, vec2_t b) { return vec2_t(a.x + b.x, a.y + b.y); }
inline vec2_t operator-(vec2_t a, float s) { return vec2_t(a.x - s, a.y - s); }
inline vec2_t operator+(vec2_t a, float s) { return vec2_t(a.x + s, a.y + s); }
inline vec2_t operator*(vec2_t a, float s) { return vec2_t(a.x * s, a.y * s); }
inline vec2_t operator*(float s, vec2_t v) { return vec2_t(s * v.x, s * v.y); }
inline vec2_t operator/(vec2_t a, vec2_t b) { return vec2_t(a.x / b.x, a.y / b.y); }

inline vec3_t operator+(vec3_t a, vec3_t b) { return vec3_t(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3_t operator-(vec3_t a, vec3_t b) { return vec3_t(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3_t operator-(vec3_t a) { return vec3_t(-a.x, -a.y, -a.z); }
inline vec3_t operator*(vec3_t a, vec3_t b) { return vec3_t(a.x * b.x, a.y * b.y, a.z * b.z); }
inline vec3_t operator*(vec3_t a, float s) { return vec3_t(a.x * s, a.y * s, a.z * s); }
inline vec3_t operator*(float s, vec3_t a) { return vec3_t(s * a.x, s * a.y, s * a.z); }
inline vec3_t operator/(vec3_t a, float s) { return vec3_t(a.x / s, a.y / s, a.z / s); }
inline vec3_t operator-(vec3_t a, float s) { return vec3_t(a.x - s, a.y - s, a.z - s); }
inline vec3_t& operator+=(vec3_t& a, vec3_t b) { a = a + b; return a; }
inline vec3_t& operator*=(vec3_t& a, vec3_t b) { a = a * b; return a; }
inline vec3_t& operator*=(vec3_t& a, float s) { a = a * s; return a; }
inline vec3_t& operator/=(vec3_t& a, float s) { a = a / s; return a; }
inline bool operator==(vec3_t a, vec3_t b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
inline bool operator!=(vec3_t a, vec3_t b) { return !(a == b); }

inline vec4_t operator*(const mat4_t& a, vec4_t v) {
  vec4_t o; float* p = &o.x;
  for (int r = 0; r < 4; ++r)
    p[r] = a.m[0 * 4 + r] * v.x + a.m[1 * 4 + r] * v.y + a.m[2 * 4 + r] * v.z + a.m[3 * 4 + r] * v.w;
  return o; }
inline mat4_t operator*(const mat4_t& a, const mat4_t& b) {
  mat4_t o;
  for (int c = 0; c < 4; ++c)
    for (int r = 0; r < 4; ++r)
      o.m[c * 4 + r] = a.m[0 * 4 + r] * b.m[c * 4 + 0] + a.m[1 * 4 + r] * b.m[c * 4 + 1] +
                       a.m[2 * 4 + r] * b.m[c * 4 + 2] + a.m[3 * 4 + r] * b.m[c * 4 + 3];
  return o; }

inline float dot(vec2_t a, vec2_t b) { return a.x * b.x + a.y * b.y; }
inline float dot(vec3_t a, vec3_t b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline vec4_t operator*(vec3_t v, const mat4x3_t& m) {
  return vec4_t(dot(v, m.c[0]), dot(v, m.c[1]), dot(v, m.c[2]), dot(v, m.c[3])); }
inline vec3_t cross(vec3_t a, vec3_t b) {
  return vec3_t(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y); }
inline float abs(float x) { return std::fabs(x); }
inline vec3_t abs(vec3_t v) { return vec3_t(std::fabs(v.x), std::fabs(v.y), std::fabs(v.z)); }
inline float sqrt(float x) { return std::sqrt(x); }
// GLSL: max(x, y) = x < y ? y : x; min(x, y) = y < x ? y : x; clamp = min(max(x, lo), hi)
inline float max(float a, float b) { return a < b ? b : a; }
inline float min(float a, float b) { return b < a ? b : a; }
inline float clamp(float x, float lo, float hi) { return min(max(x, lo), hi); }
inline float sin(float x) { return kf_oracle_sin(x); }
inline float cos(float x) { return kf_oracle_cos(x); }
inline float pow(float x, float y) {
  if (x == 2.0f) return kf_oracle_exp2(y);
  if (y == 5.0f) { float x2 = x * x; return (x2 * x2) * x; }
  return std::pow(x, y); }
inline float length(vec3_t v) { return sqrt(dot(v, v)); }
inline vec3_t normalize(vec3_t v) { float inv = 1.0f / length(v); return v * inv; }
inline vec3_t mix(vec3_t x, vec3_t y, float a) { return x * (1.0f - a) + y * a; }
inline vec3_t reflect(vec3_t I, vec3_t N) { return I - (2.0f * dot(N, I)) * N; }
inline vec3_t refract(vec3_t I, vec3_t N, float eta) {
  float d = dot(N, I);
  float k = 1.0f - eta * eta * (1.0f - d * d);
  if (k < 0.0f) return vec3_t(0.0f);
  return eta * I - (eta * d + sqrt(k)) * N; }
}
using namespace glsl;
#define nonuniformEXT(x) (x)
#define vec2(...) (glsl::vec2_t{__VA_ARGS__})
#define vec3(...) (glsl::vec3_t{__VA_ARGS__})
#define vec4(...) (glsl::vec4_t{__VA_ARGS__})
#define ivec2(...) (glsl::ivec2_t{__VA_ARGS__})
#define ivec3(...) (glsl::ivec3_t{__VA_ARGS__})
typedef glsl::vec2_t vec2;
typedef glsl::vec3_t vec3;
typedef glsl::vec4_t vec4;
typedef glsl::ivec2_t ivec2;
typedef glsl::ivec3_t ivec3;
typedef glsl::mat4_t mat4;
"""


def glsl_to_cpp(text: str, main_name: str | None = None) -> str:
    """Mechanical GLSL -> C++ rewrite of one shader source (see the module docstring)."""
    text = re.sub(r"^\s*#\s*(version|extension|include)\b.*$", "", text, flags=re.M)
    # resource blocks: layout(...) [readonly] uniform|buffer Name { ... } instance[];
    text = re.sub(r"layout\s*\([^)]*\)\s*(readonly\s+)?(uniform|buffer)\s+\w+\s*\{[^}]*\}\s*\w*\s*(\[\s*\])?\s*;",
                  "", text, flags=re.S)
    # opaque resources: acceleration structure, images, samplers
    text = re.sub(r"layout\s*\([^)]*\)\s*uniform\s+\w+\s+\w+\s*(\[\s*\])?\s*;", "", text)
    # payloads and hit attributes
    text = re.sub(r"layout\s*\([^)]*\)\s*rayPayload(In)?EXT\s+\w+\s+\w+\s*;", "", text)
    text = re.sub(r"hitAttributeEXT\s+\w+\s+\w+\s*;", "", text)
    # specialisation constants keep their default
    text = re.sub(r"layout\s*\(\s*constant_id\s*=\s*\d+\s*\)\s*const", "const", text)
    text = re.sub(r"\binout\s+(\w+)\s+(\w+)", r"\1 &\2", text)
    text = re.sub(r"([(,]\s*)in\s+(\w+)\s+(\w+)", r"\1\2 \3", text)
    text = re.sub(r"\.(xyz|rgb)\b(?!\s*\()", ".xyz()", text)
    text = re.sub(r"\.xy\b(?!\s*\()", ".xy()", text)
    if main_name:
        text = re.sub(r"\bvoid\s+main\s*\(\s*\)", f"void {main_name}()", text)
    return text
