"""Generates tests/golden/shader_vectors.json from kuafu's own shader library.

kuafu's render path is GLSL (resources/shaders/base/Random.glsl and
Sampling.glsl hold its RNG, BRDF and sampling helpers). There is no GLSL
toolchain or graphics stack here, but these two files are plain arithmetic, so
this script compiles them *as C++*:

  * the files are read where they lie (<kuafu>/resources/shaders/base);
  * the mechanical rewrite and compatibility header of tests/golden/glsl_cpp.py
    (GLSL qualifiers to C++, vec2/vec3 and the built-ins, brace-initialised
    constructors evaluating their arguments left to right as GLSL does);
  * g++ compiles with ``-fsingle-precision-constant`` (GLSL literals are float)
    and ``-ffp-contract=off``; sin / cos / pow(2, x) / pow(x, 5) come from the
    oracle's deterministic functions (the GLSL spec leaves their rounding to the
    implementation).

The program evaluates each helper on seeded inputs (drawing its uniforms with
the shaders' own tea / lcg / rnd) and prints JSON, written next to this script.
The result is committed; tests/test_oracle.py compares the oracle against it.
Run from the repository root with the kuafu checkout:
  python tests/golden/make_shader_vectors.py <path-to-kuafu>   (or $KF_REFERENCE)
"""
from __future__ import annotations

import json
import subprocess
import sys
import tempfile
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(HERE))

import glsl_cpp  # noqa: E402

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
  std::printf("],\n\"schlick_fresnel\": [");
  for (int i = 0; i < 64; ++i) {
    vec3 f0 = vec3(rnd(s), rnd(s), rnd(s));
    float ldoth = rnd(s);
    std::printf("%s{\"ldoth\": %.9g, ", i ? ", " : "", ldoth);
    pv("f0", f0); std::printf(", "); pv("out", schlickFresnel(f0, ldoth)); std::printf("}");
  }
  std::printf("],\n\"perpendicular\": [");
  for (int i = 0; i < 64; ++i) {
    vec3 u = vec3(2.0f * rnd(s) - 1.0f, 2.0f * rnd(s) - 1.0f, 2.0f * rnd(s) - 1.0f);
    if (i % 8 == 1) u.y = u.x;        // ties between components
    if (i % 8 == 2) u.z = -u.x;
    std::printf("%s{", i ? ", " : "");
    pv("u", u); std::printf(", "); pv("out", getPerpendicularVector(u)); std::printf("}");
  }
  std::printf("],\n\"uniform_sphere\": [");
  for (int i = 0; i < 64; ++i) {
    uint st = s * 747796405u + (uint)i, before = st;
    vec3 p = uniformSphereSampling(st);
    std::printf("%s{\"state\": %u, \"state_after\": %u, ", i ? ", " : "", before, st);
    pv("out", p); std::printf("}");
  }
  std::printf("],\n\"disk\": [");
  for (int i = 0; i < 64; ++i) {
    uint st = s * 2891336453u + (uint)i, before = st;
    vec2 p = diskSampling(st);
    std::printf("%s{\"state\": %u, \"state_after\": %u, \"out\": [%.9g, %.9g]}", i ? ", " : "", before, st,
                p.x, p.y);
  }
  std::printf("],\n\"lcg\": [");
  for (int i = 0; i < 64; ++i) {
    uint st = (uint)i * 2246822519u + 3266489917u, before = st;
    uint a = lcg(st);
    float r = rnd(st);
    std::printf("%s{\"state\": %u, \"lcg\": %u, \"rnd\": %.9g, \"state_after\": %u}", i ? ", " : "", before,
                a, r, st);
  }
  std::printf("]\n}\n");
  return 0;
}
"""


def main(argv) -> int:
    shaders = glsl_cpp.reference_root(argv[1] if len(argv) > 1 else None) / "resources" / "shaders" / "base"
    src = (glsl_cpp.COMPAT + glsl_cpp.glsl_to_cpp((shaders / "Random.glsl").read_text()) +
           glsl_cpp.glsl_to_cpp((shaders / "Sampling.glsl").read_text()) + DRIVER)
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
    sys.exit(main(sys.argv))
