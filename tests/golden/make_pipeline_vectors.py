"""Generates tests/golden/pipeline_vectors.npz: per-path radiance of kuafu's own shader
pipeline, compiled as C++.

kuafu's PathTrace.rgen, PathTrace.rchit, PathTrace.rmiss and PathTraceShadow.rmiss
(with base/Random.glsl, Sampling.glsl, Ray.glsl, Geometry.glsl, Light.glsl,
Camera.glsl, PushConstants.glsl) are rewritten mechanically into one C++ translation
unit (tests/golden/glsl_cpp.py) and linked with a small runtime that plays the Vulkan
ray-tracing pipeline:

  * traceRayEXT: the closest hit (or, for the shadow rays' terminate-on-first-hit,
    any hit) from the oracle's traversal; a hit sets gl_InstanceID, gl_PrimitiveID,
    gl_HitTEXT, the barycentric hit attributes, gl_WorldRayOrigin/DirectionEXT,
    gl_WorldToObjectEXT and gl_HitKindEXT (back-facing when the object-space ray
    direction has a positive dot product with (v1 - v0) x (v2 - v0)) and runs the
    closest-hit shader, a miss runs the miss shader of the call's miss index;
  * clockARB(): pinned, returning TEA_CLOCK + the call index within the pixel, so
    kuafu's tea/lcg streams are reproducible;
  * one launch per pixel; the rgen sample loop is instrumented to record each
    sample's `color` (one added line before `colors += color;`);
  * the closest-hit shader's sum of its three light loops, which draw from the
    payload's random stream, is evaluated left to right (glslang's order; GLSL
    and C++ leave it open).

Output: for every scene of tests/golden/pipeline_scenes.py, the per-path radiance,
the pixel colour (imageStore of finalColor), albedo and normal. The result is
committed; tests/test_oracle_pipeline.py renders the same scenes with the oracle in
its TEA/LCG mode and compares.

Run from the repository root with the kuafu checkout:
  python tests/golden/make_pipeline_vectors.py <path-to-kuafu>   (or $KF_REFERENCE)
"""
from __future__ import annotations

import ctypes as C
import re
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(HERE))

import glsl_cpp  # noqa: E402
import pipeline_scenes  # noqa: E402

RUNTIME_DECLS = r"""
#include "kf_types.h"
// ---- the pipeline's resources, as the descriptor sets and push constants hold them ----
struct CameraBlock { mat4 view, proj, viewInverse, projInverse; vec4 position, viewingDirection, padding1, padding2; };
static CameraBlock cam;
static vec4 clearColor;
static int frameCount;
static uint sampleRatePerPixel, maxPathDepth;
static bool useEnvironmentMap, russianRoulette;
static uint russianRouletteMinBounces;
static bool isNextEventEstimation;
static uint nextEventEstimationMinBounces;
struct DirLightBlock { vec4 direction, rgbs; };
static DirLightBlock dlight;
struct PointLightsBlock { vec4 posr[MAX_POINT_LIGHTS]; vec4 rgbs[MAX_POINT_LIGHTS]; };
static PointLightsBlock plights;
struct ActiveLightsBlock { mat4 viewMat[MAX_ACTIVE_LIGHTS]; mat4 projMat[MAX_ACTIVE_LIGHTS];
  vec4 front[MAX_ACTIVE_LIGHTS], rgbs[MAX_ACTIVE_LIGHTS], position[MAX_ACTIVE_LIGHTS], sftp[MAX_ACTIVE_LIGHTS]; };
static ActiveLightsBlock alights;
struct GeometryInstancesBlock { GeometryInstance* i; };
static GeometryInstancesBlock geometryInstances;
struct VerticesBlock { const vec4* v; };
struct UintBlock { const uint* i; };
static VerticesBlock vertices[1024];
static UintBlock indices[1024];
static UintBlock matIndices[1024];
struct MaterialsBlock { const Material* m; };
static MaterialsBlock materials;
struct sampler2D { int id; };
struct samplerCube { int id; };
static sampler2D textures[64];
static samplerCube environmentMap;
struct image2D { float* data; };
static image2D image, albedoImage, normalImage;
static int topLevelAS;
// ---- ray-tracing built-ins ----
static uvec3_t gl_LaunchIDEXT, gl_LaunchSizeEXT;
static vec3 attribs;
static uint gl_InstanceID, gl_PrimitiveID, gl_HitKindEXT;
static float gl_HitTEXT;
static vec3 gl_WorldRayOriginEXT, gl_WorldRayDirectionEXT;
static mat4x3_t gl_WorldToObjectEXT;
static const uint gl_HitKindFrontFacingTriangleEXT = 0xFEu, gl_HitKindBackFacingTriangleEXT = 0xFFu;
static const uint gl_RayFlagsNoneEXT = 0u, gl_RayFlagsOpaqueEXT = 1u, gl_RayFlagsTerminateOnFirstHitEXT = 4u,
                  gl_RayFlagsSkipClosestHitShaderEXT = 8u;
static RayPayLoad ray;        // location 0: the rgen's payload, seen by the hit and miss shaders
static RayPayLoad shadowRay;  // location 2 of the rgen (unused by kuafu)
static bool isShadowed;       // location 1: the shadow rays' payload
static uint64_t g_clock;
static int g_texture_calls;
inline uint64_t clockARB() { return g_clock++; }
void traceRayEXT(int as, uint flags, uint mask, uint sbt_offset, uint sbt_stride, uint miss_index, vec3 origin,
                 float tmin, vec3 direction, float tmax, int payload);
inline vec4 texture(sampler2D, vec2) { ++g_texture_calls; return vec4(1.0f); }
inline vec4 texture(samplerCube, vec3) { ++g_texture_calls; return vec4(1.0f); }
static uint g_width;
inline void imageStore(image2D& img, ivec2 p, vec4 v) {
  float* d = img.data + ((size_t)p.y * g_width + (size_t)p.x) * 3; d[0] = v.x; d[1] = v.y; d[2] = v.z; }
inline vec4 imageLoad(image2D& img, ivec2 p) {
  const float* d = img.data + ((size_t)p.y * g_width + (size_t)p.x) * 3; return vec4(d[0], d[1], d[2], 1.0f); }
static float* g_paths;
static size_t g_npix;
inline void kf_sample_hook(uint i, vec3 c) {
  float* d = g_paths + ((size_t)i * g_npix + (size_t)gl_LaunchIDEXT.y * g_width + gl_LaunchIDEXT.x) * 3;
  d[0] = c.x; d[1] = c.y; d[2] = c.z; }
"""

RUNTIME_IMPL = r"""
extern "C" int kf_oracle_trace(const kf_flat_scene* scene, const float* rays, uint32_t n, uint32_t use_bvh,
                               kf_hit* out);
static const kf_flat_scene* g_scene;

void traceRayEXT(int, uint flags, uint, uint, uint, uint miss_index, vec3 origin, float tmin, vec3 direction,
                 float tmax, int) {
  const float r[8] = {origin.x, origin.y, origin.z, tmin, direction.x, direction.y, direction.z, tmax};
  kf_hit h;
  kf_oracle_trace(g_scene, r, 1, 0, &h);
  const bool hit = h.instance != 0xFFFFFFFFu;
  if (!hit) {
    if (miss_index == 1) shadow_rmiss_main(); else rmiss_main();
    return;
  }
  if (flags & gl_RayFlagsSkipClosestHitShaderEXT) return;
  const kf_flat_instance& in = g_scene->instances[h.instance];
  const kf_flat_geometry& g = g_scene->geometries[in.geometry_index];
  const float* m = in.world_to_object;
  gl_InstanceID = h.instance;
  gl_PrimitiveID = h.prim;
  gl_HitTEXT = h.t;
  attribs = vec3(h.u, h.v, 0.0f);
  gl_WorldRayOriginEXT = origin;
  gl_WorldRayDirectionEXT = direction;
  for (int j = 0; j < 4; ++j) gl_WorldToObjectEXT.c[j] = vec3(m[0 * 4 + j], m[1 * 4 + j], m[2 * 4 + j]);
  const float od[3] = {m[0] * direction.x + m[1] * direction.y + m[2] * direction.z,
                       m[4] * direction.x + m[5] * direction.y + m[6] * direction.z,
                       m[8] * direction.x + m[9] * direction.y + m[10] * direction.z};
  const float* p0 = g.vertices[g.indices[3 * h.prim + 0]].pos;
  const float* p1 = g.vertices[g.indices[3 * h.prim + 1]].pos;
  const float* p2 = g.vertices[g.indices[3 * h.prim + 2]].pos;
  const vec3 ng = cross(vec3(p1[0], p1[1], p1[2]) - vec3(p0[0], p0[1], p0[2]),
                        vec3(p2[0], p2[1], p2[2]) - vec3(p0[0], p0[1], p0[2]));
  gl_HitKindEXT = dot(vec3(od[0], od[1], od[2]), ng) > 0.0f ? gl_HitKindBackFacingTriangleEXT
                                                            : gl_HitKindFrontFacingTriangleEXT;
  rchit_main();
}

extern "C" int kf_kuafu_render(const kf_flat_scene* scene, const kf_camera_ubo* camera, const kf_push_constants* pc,
                               uint32_t width, uint32_t height, uint32_t tea_clock, float* paths, float* pixel,
                               float* albedo, float* normal) {
  static_assert(sizeof(Material) == sizeof(kf_material_gpu), "material layout");
  static_assert(sizeof(CameraBlock) == sizeof(kf_camera_ubo), "camera layout");
  static_assert(sizeof(ActiveLightsBlock) == sizeof(kf_active_lights_ubo), "active light layout");
  if (scene->num_geometries > 1024 || scene->num_textures > 0 || scene->env_size) return 1;
  g_scene = scene;
  std::memcpy(&cam, camera, sizeof(cam));
  std::memcpy(&dlight, &scene->dlight, sizeof(dlight));
  std::memcpy(&plights, &scene->plights, sizeof(plights));
  std::memcpy(&alights, &scene->alights, sizeof(alights));
  clearColor = vec4(pc->clear_color[0], pc->clear_color[1], pc->clear_color[2], pc->clear_color[3]);
  frameCount = pc->frame_count;
  sampleRatePerPixel = pc->spp;
  maxPathDepth = pc->max_path_depth;
  useEnvironmentMap = pc->use_env_map != 0;
  russianRoulette = pc->russian_roulette != 0;
  russianRouletteMinBounces = pc->rr_min_bounces;
  isNextEventEstimation = pc->nee != 0;
  nextEventEstimationMinBounces = pc->nee_min;
  static GeometryInstance inst[4096];
  if (scene->num_instances > 4096) return 1;
  for (uint32_t k = 0; k < scene->num_instances; ++k) {
    std::memset(&inst[k], 0, sizeof(inst[k]));
    std::memcpy(inst[k].transform.m, scene->instances[k].transform, sizeof(float) * 16);
    inst[k].geometryIndex = scene->instances[k].geometry_index;
  }
  geometryInstances.i = inst;
  for (uint32_t gi = 0; gi < scene->num_geometries; ++gi) {
    vertices[gi].v = reinterpret_cast<const vec4*>(scene->geometries[gi].vertices);
    indices[gi].i = scene->geometries[gi].indices;
    matIndices[gi].i = scene->geometries[gi].mat_index;
  }
  materials.m = reinterpret_cast<const Material*>(scene->materials);
  image.data = pixel;
  albedoImage.data = albedo;
  normalImage.data = normal;
  g_paths = paths;
  g_width = width;
  g_npix = (size_t)width * height;
  gl_LaunchSizeEXT = uvec3_t{width, height, 1u};
  g_texture_calls = 0;
  for (uint32_t y = 0; y < height; ++y)
    for (uint32_t x = 0; x < width; ++x) {
      gl_LaunchIDEXT = uvec3_t{x, y, 0u};
      g_clock = tea_clock;
      rgen_main();
    }
  return g_texture_calls ? 2 : 0;
}
"""


def translation_unit(shaders: Path) -> str:
    base = shaders / "base"
    rd = lambda p: p.read_text()
    rgen = rd(shaders / "PathTrace.rgen")
    hook = "colors += color;"
    if rgen.count(hook) != 1:
        raise SystemExit("PathTrace.rgen: the per-sample accumulation line was not found exactly once")
    rgen = rgen.replace(hook, "kf_sample_hook(i, color); " + hook)
    rchit = rd(shaders / "PathTrace.rchit")
    # The three light loops consume the payload's random stream, so their order matters;
    # GLSL leaves the evaluation order of `+` operands open (C++ does too). glslang emits
    # them left to right; state that order explicitly.
    rchit, n = re.subn(r"ray\.shadow_color\s*=\s*(traceDirectionalLight\([^;()]*\))\s*\+\s*"
                       r"(tracePointLights\([^;()]*\))\s*\+\s*(traceActiveLights\([^;()]*\))\s*;",
                       r"{ vec3 kf_dir = \1; vec3 kf_pts = \2; vec3 kf_act = \3; "
                       r"ray.shadow_color = kf_dir + kf_pts + kf_act; }", rchit)
    if n != 1:
        raise SystemExit("PathTrace.rchit: the light-sum statement was not found exactly once")
    parts = [glsl_cpp.COMPAT]
    for name in ("Random.glsl", "Sampling.glsl", "Ray.glsl", "Geometry.glsl", "Light.glsl", "Camera.glsl",
                 "PushConstants.glsl"):
        parts.append(f"// ---- base/{name} ----\n" + glsl_cpp.glsl_to_cpp(rd(base / name)))
    parts.append(RUNTIME_DECLS)
    parts.append("void rmiss_main(); void shadow_rmiss_main(); void rchit_main();")
    parts.append("// ---- PathTrace.rmiss ----\n" + glsl_cpp.glsl_to_cpp(rd(shaders / "PathTrace.rmiss"), "rmiss_main"))
    parts.append("// ---- PathTraceShadow.rmiss ----\n" +
                 glsl_cpp.glsl_to_cpp(rd(shaders / "PathTraceShadow.rmiss"), "shadow_rmiss_main"))
    parts.append("// ---- PathTrace.rchit ----\n" + glsl_cpp.glsl_to_cpp(rchit, "rchit_main"))
    parts.append("// ---- PathTrace.rgen ----\n" + glsl_cpp.glsl_to_cpp(rgen, "rgen_main"))
    parts.append(RUNTIME_IMPL)
    return "\n".join(parts)


def build_library(reference: Path, workdir: Path) -> Path:
    from kuafu_gb300 import build

    oracle_lib = build.build_oracle()
    cpp = workdir / "kuafu_pipeline.cpp"
    so = workdir / "libkuafu_pipeline.so"
    cpp.write_text(translation_unit(reference / "resources" / "shaders"))
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fsingle-precision-constant", "-Wno-narrowing",
                    "-fPIC", "-shared", "-I", str(ROOT / "include"), "-o", str(so), str(cpp), str(oracle_lib),
                    f"-Wl,-rpath,{oracle_lib.parent}"], check=True)
    return so


def render(lib, name: str):
    from oracle import oracle as O

    r, cam, pcargs = pipeline_scenes.build(name)
    flat = r.getScene().export()
    ubo = cam.ubo()
    w, h = cam._size()
    pc = O.push_constants(**pcargs)
    spp = pc.spp
    paths = np.zeros((spp, h, w, 3), np.float32)
    pixel = np.zeros((h, w, 3), np.float32)
    albedo = np.zeros((h, w, 3), np.float32)
    normal = np.zeros((h, w, 3), np.float32)
    rc = lib.kf_kuafu_render(C.byref(flat), C.byref(ubo), C.byref(pc), w, h, pipeline_scenes.TEA_CLOCK,
                             paths.ctypes.data, pixel.ctypes.data, albedo.ctypes.data, normal.ctypes.data)
    r.close()
    if rc != 0:
        raise RuntimeError(f"kf_kuafu_render({name}) failed: {rc}")
    return {"paths": paths, "pixel": pixel, "albedo": albedo, "normal": normal}


def main(argv) -> int:
    reference = glsl_cpp.reference_root(argv[1] if len(argv) > 1 else None)
    with tempfile.TemporaryDirectory() as td:
        lib = C.CDLL(str(build_library(reference, Path(td))))
        lib.kf_kuafu_render.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32,
                                        C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        out = {}
        for name in pipeline_scenes.NAMES:
            res = render(lib, name)
            for k, v in res.items():
                out[f"{name}/{k}"] = v
            print(f"{name}: {res['paths'].shape[0]} x {res['paths'].shape[1]} x {res['paths'].shape[2]} paths, "
                  f"mean radiance {res['paths'].mean():.4f}")
    np.savez_compressed(HERE / "pipeline_vectors.npz", **out)
    print(f"wrote {HERE / 'pipeline_vectors.npz'}")
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv))
