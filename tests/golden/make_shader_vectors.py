"""Generates tests/golden/shader_vectors.json from kuafu's own shader library.

kuafu's render path is GLSL (resources/shaders/base/Random.glsl and
Sampling.glsl hold its RNG, BRDF and sampling helpers). There is no GLSL
toolchain or graphics stack here, but these two files are plain arithmetic, so
this script compiles them *as C++*:

  * the files are read where they lie (REFERENCE/resources/shaders/base);
  * a mechanical rewrite turns GLSL parameter qualifiers into C++
    (``inout T x`` -> ``T& x``, ``in T x`` -> ``T x``) and drops ``#include``;
  * a small compatibility header supplies vec2/vec3, the GLSL built-ins they
    call and brace-initialised constructors, so constructor arguments are
    evaluated left to right as GLSL evaluates them;
  * g++ compiles with ``-fsingle-precision-constant`` (GLSL literals are float)
    and ``-ffp-contract=off``; sin / cos / pow(2, x) / pow(x, 5) come from the
    oracle's deterministic functions (the GLSL spec leaves their rounding to the
    implementation).

The program evaluates each helper on seeded inputs (drawing its uniforms with
the shaders' own tea / lcg / rnd) and prints JSON, written next to this script.
The result is committed; tests/test_oracle.py compares the oracle against it.
Run from the repository root:  python tests/golden/make_shader_vectors.py
"""
from __future__ import annotations

import json
import os
import re
import subprocess
import sys
import tempfile
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
REFERENCE = Path(os.environ.get("KF_REFERENCE", "/root/reference"))
SHADERS = REFERENCE / "resources" / "shaders" / "base"

COMPAT = r"""
#include <cmath>
#include <cstdint>
#include <cstdio>
#undef M_PI
typedef uint32_t uint;
extern "C" float kf_oracle_sin(float);
extern "C" float kf_oracle_cos(float);
extern "C" float kf_oracle_exp2(float);
namespace glsl {
struct vec2_t { float x, y;
  vec2_t() : x(0), y(0) {}
  vec2_t(float a) : x(a), y(a) {}
  vec2_t(float a, float b) : x(a), y(b) {} };
struct vec3_t { float x, y, z;
  vec3_t() : x(0), y(0), z(0) {}
  vec3_t(float a) : x(a), y(a), z(a) {}
  vec3_t(float a, float b, float c) : x(a), y(b), z(c) {} };
inline vec2_t operator*(float s, vec2_t v) { return vec2_t(s * v.x, s * v.y); }
inline vec2_t operator-(vec2_t v, float s) { return vec2_t(v.x - s, v.y - s); }
inline vec3_t operator+(vec3_t a, vec3_t b) { return vec3_t(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3_t operator-(vec3_t a, vec3_t b) { return vec3_t(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3_t operator-(vec3_t a) { return vec3_t(-a.x, -a.y, -a.z); }
inline vec3_t operator*(vec3_t a, vec3_t b) { return vec3_t(a.x * b.x, a.y * b.y, a.z * b.z); }
inline vec3_t operator*(vec3_t a, float s) { return vec3_t(a.x * s, a.y * s, a.z * s); }
inline vec3_t operator*(float s, vec3_t a) { return vec3_t(s * a.x, s * a.y, s * a.z); }
inline vec3_t operator/(vec3_t a, float s) { return vec3_t(a.x / s, a.y / s, a.z / s); }
inline vec3_t operator-(vec3_t a, float s) { return vec3_t(a.x - s, a.y - s, a.z - s); }
inline float dot(vec2_t a, vec2_t b) { return a.x * b.x + a.y * b.y; }
inline float dot(vec3_t a, vec3_t b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline vec3_t cross(vec3_t a, vec3_t b) { return vec3_t(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y); }
inline float abs(float x) { return std::fabs(x); }
inline vec3_t abs(vec3_t v) { return vec3_t(std::fabs(v.x), std::fabs(v.y), std::fabs(v.z)); }
inline float sqrt(float x) { return std::sqrt(x); }
inline float max(float a, float b) { return std::fmax(a, b); }
inline float min(float a, float b) { return std::fmin(a, b); }
inline float clamp(float x, float lo, float hi) { return min(max(x, lo), hi); }
inline float sin(float x) { return kf_oracle_sin(x); }
inline float cos(float x) { return kf_oracle_cos(x); }
inline float pow(float x, float y) {
  if (x == 2.0f) return kf_oracle_exp2(y);
  if (y == 5.0f) { float x2 = x * x; return (x2 * x2) * x; }
  return std::pow(x, y); }
inline float length(vec3_t v) { return sqrt(dot(v, v)); }
inline vec3_t normalize(vec3_t v) { float inv = 1.0f / length(v); return v * inv; }
}
using namespace glsl;
#define vec2(...) (glsl::vec2_t{__VA_ARGS__})
#define vec3(...) (glsl::vec3_t{__VA_ARGS__})
typedef glsl::vec2_t vec2;
typedef glsl::vec3_t vec3;
"""

DRIVER = r"""
static void pv(const char* k, vec3 v) { std::printf("\"%s\": [%.9g, %.9g, %.9g]", k, v.x, v.y, v.z); }
int main() {
  std::printf("{\n\"tea\": [");
  for (uint i = 0; i < 64; ++i) {
    uint a = i * 2654435761u, b = i * 40503u + 17u;
    std::printf("%s{\"v0\": %u, \"v1\": %u, \"out\": %u}", i ? ", " : "", a, b, tea(a, b));
  }
  std::printf("],\n\"schlick\": [");
  uint s = 1u;
  for (int i = 0; i < 64; ++i) {
    float c = rnd(s), ior = 1.0f + 1.5f * rnd(s);
    std::printf("%s{\"cos\": %.9g, \"ior\": %.9g, \"out\": %.9g}", i ? ", " : "", c, ior, Schlick(c, ior));
  }
  std::printf("],\n\"ggx_d\": [");
  for (int i = 0; i < 64; ++i) {
    float n = 2.0f * rnd(s) - 1.0f, a2 = rnd(s);
    std::printf("%s{\"ndoth\": %.9g, \"a2\": %.9g, \"out\": %.9g}", i ? ", " : "", n, a2, ggxNormalDistribution(n, a2));
  }
  std::printf("],\n\"g1\": [");
  for (int i = 0; i < 64; ++i) {
    float d = rnd(s), a2 = rnd(s);
    std::printf("%s{\"d\": %.9g, \"a2\": %.9g, \"out\": %.9g}", i ? ", " : "", d, a2, G1(d, a2));
  }
  std::printf("],\n\"sample_ggx\": [");
  for (int i = 0; i < 64; ++i) {
    vec3 n = normalize(vec3(2.0f * rnd(s) - 1.0f, 2.0f * rnd(s) - 1.0f, 2.0f * rnd(s) - 1.0f));
    float a2 = rnd(s);
    uint t = s; float u0 = rnd(t), u1 = rnd(t);
    vec3 h = sampleGGX(s, a2, n);
    std::printf("%s{\"u0\": %.9g, \"u1\": %.9g, \"a2\": %.9g, ", i ? ", " : "", u0, u1, a2);
    pv("n", n); std::printf(", "); pv("out", h); std::printf("}");
  }
  std::printf("],\n\"cosine\": [");
  for (int i = 0; i < 64; ++i) {
    vec3 n = normalize(vec3(2.0f * rnd(s) - 1.0f, 2.0f * rnd(s) - 1.0f, 2.0f * rnd(s) - 1.0f));
    uint t = s; float u0 = rnd(t), u1 = rnd(t);
    vec3 d = cosineHemisphereSampling(s, n);
    std::printf("%s{\"u0\": %.9g, \"u1\": %.9g, ", i ? ", " : "", u0, u1);
    pv("n", n); std::printf(", "); pv("out", d); std::printf("}");
  }
  std::printf("]\n}\n");
  return 0;
}
"""


def glsl_to_cpp(text: str) -> str:
    text = re.sub(r'^\s*#\s*include\s+"[^"]*"\s*$', "", text, flags=re.M)
    text = re.sub(r"\binout\s+(\w+)\s+(\w+)", r"\1 &\2", text)
    text = re.sub(r"([(,]\s*)in\s+(\w+)\s+(\w+)", r"\1\2 \3", text)
    return text


def main() -> int:
    rnd = SHADERS / "Random.glsl"
    smp = SHADERS / "Sampling.glsl"
    if not rnd.exists():
        print(f"kuafu shaders not found under {SHADERS}", file=sys.stderr)
        return 1
    src = COMPAT + glsl_to_cpp(rnd.read_text()) + glsl_to_cpp(smp.read_text()) + DRIVER
    oracle_lib = ROOT / "oracle" / "liboracle.so"
    if not oracle_lib.exists():
        sys.path.insert(0, str(ROOT))
        from kuafu_gb300 import build

        build.build_oracle()
    with tempfile.TemporaryDirectory() as td:
        cpp = Path(td) / "shaders.cpp"
        exe = Path(td) / "shaders"
        cpp.write_text(src)
        subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fsingle-precision-constant",
                        "-Wno-narrowing", "-o", str(exe), str(cpp), str(oracle_lib),
                        f"-Wl,-rpath,{oracle_lib.parent}"], check=True)
        out = subprocess.run([str(exe)], check=True, stdout=subprocess.PIPE, text=True).stdout
    data = json.loads(out)
    data["_source"] = "kuafu resources/shaders/base/Random.glsl + Sampling.glsl compiled as C++"
    (HERE / "shader_vectors.json").write_text(json.dumps(data, indent=1) + "\n")
    print(f"wrote {HERE / 'shader_vectors.json'}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
