"""ctypes front-end of the CPU oracle (oracle/kf_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, by the smoke check and by the
CPU-baseline leg of bench.py, always as the checker. The product (libkf and the
kuafu_gb300 package) never imports it.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from kuafu_gb300 import _native as N

_LIB = Path(__file__).resolve().parent / "liboracle.so"

RNG_PHILOX, RNG_TEA_LCG = 0, 1
FP32, FP64 = 0, 1


class kf_oracle_view(C.Structure):
    _fields_ = [("camera", C.POINTER(N.kf_camera_ubo)), ("width", C.c_uint32), ("height", C.c_uint32),
                ("x0", C.c_uint32), ("y0", C.c_uint32), ("crop_w", C.c_uint32), ("crop_h", C.c_uint32),
                ("pc", N.kf_push_constants), ("seed", C.c_uint32), ("frame", C.c_uint32),
                ("camera_index", C.c_uint32), ("rng_mode", C.c_uint32), ("tea_clock", C.c_uint32),
                ("precision", C.c_uint32), ("threads", C.c_uint32), ("use_bvh", C.c_uint32)]


class kf_oracle_out(C.Structure):
    _fields_ = [("path_radiance", C.c_void_p), ("pixel_color", C.c_void_p), ("pixel_color64", C.c_void_p),
                ("albedo", C.c_void_p), ("normal", C.c_void_p), ("primary_hits", C.c_void_p),
                ("path_depths", C.c_void_p), ("rays_primary", C.c_uint64), ("rays_extension", C.c_uint64),
                ("rays_shadow", C.c_uint64)]


HIT_DTYPE = np.dtype([("t", "<f4"), ("u", "<f4"), ("v", "<f4"), ("instance", "<u4"), ("prim", "<u4"),
                      ("pad", "<u4", 3)])

_lib = None


def load():
    global _lib
    if _lib is None:
        if not _LIB.exists():
            raise ImportError(f"{_LIB} missing: build with `python -m kuafu_gb300.build`")
        L = C.CDLL(str(_LIB))
        L.kf_oracle_render.argtypes = [C.POINTER(N.kf_flat_scene), C.POINTER(kf_oracle_view),
                                       C.POINTER(kf_oracle_out)]
        L.kf_oracle_trace.argtypes = [C.POINTER(N.kf_flat_scene), C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p]
        L.kf_oracle_philox4x32_10.argtypes = [C.POINTER(C.c_uint32 * 4), C.POINTER(C.c_uint32 * 2),
                                              C.POINTER(C.c_uint32 * 4)]
        L.kf_oracle_tea.restype = C.c_uint32
        L.kf_oracle_tea.argtypes = [C.c_uint32, C.c_uint32]
        L.kf_oracle_rnd_lcg.restype = C.c_float
        L.kf_oracle_rnd_lcg.argtypes = [C.POINTER(C.c_uint32)]
        L.kf_oracle_uniform.restype = C.c_float
        L.kf_oracle_uniform.argtypes = [C.c_uint32] * 8
        for f in ("kf_oracle_sin", "kf_oracle_cos", "kf_oracle_exp2"):
            getattr(L, f).restype = C.c_float
            getattr(L, f).argtypes = [C.c_float]
        L.kf_oracle_intersect.argtypes = [C.POINTER(C.c_float * 3)] * 5 + [C.c_float, C.c_float] + \
            [C.POINTER(C.c_float)] * 3
        L.kf_oracle_sample_ggx.argtypes = [C.c_float, C.c_float, C.c_float, C.POINTER(C.c_float * 3),
                                           C.POINTER(C.c_float * 3)]
        L.kf_oracle_cosine_hemisphere.argtypes = [C.c_float, C.c_float, C.POINTER(C.c_float * 3),
                                                  C.POINTER(C.c_float * 3)]
        L.kf_oracle_schlick.restype = C.c_float
        L.kf_oracle_schlick.argtypes = [C.c_float, C.c_float]
        L.kf_oracle_ggx_d.restype = C.c_float
        L.kf_oracle_ggx_d.argtypes = [C.c_float, C.c_float]
        L.kf_oracle_g1.restype = C.c_float
        L.kf_oracle_g1.argtypes = [C.c_float, C.c_float]
        L.kf_oracle_schlick_fresnel.argtypes = [C.POINTER(C.c_float * 3), C.c_float, C.POINTER(C.c_float * 3)]
        L.kf_oracle_camera_ubo.argtypes = [C.POINTER(C.c_float * 3)] * 3 + [C.c_float] * 7 + \
            [C.POINTER(N.kf_camera_ubo)]
        L.kf_oracle_srgb8.restype = C.c_uint8
        L.kf_oracle_srgb8.argtypes = [C.c_float]
        L.kf_oracle_perpendicular.argtypes = [C.POINTER(C.c_float * 3), C.POINTER(C.c_float * 3)]
        L.kf_oracle_uniform_sphere_lcg.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_float * 3)]
        L.kf_oracle_disk_lcg.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_float * 2)]
        L.kf_oracle_icosphere.argtypes = [C.c_int, C.c_void_p, C.c_uint32, C.POINTER(C.c_uint32), C.c_uint32,
                                          C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
        L.kf_oracle_instance_rows.argtypes = [C.POINTER(C.c_float), C.POINTER(C.c_float)]
        L.kf_oracle_light_ubos.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_uint32,
                                           C.POINTER(N.kf_dir_light_ubo), C.POINTER(N.kf_point_lights_ubo),
                                           C.POINTER(N.kf_active_lights_ubo)]
        _lib = L
    return _lib


def push_constants(spp, depth, clear=(0, 0, 0, 1), rr=False, rr_min=4, frame_count=0,
                   env=False) -> N.kf_push_constants:
    pc = N.kf_push_constants()
    pc.clear_color[:] = [float(x) for x in clear]
    pc.frame_count = frame_count
    pc.spp = spp
    pc.max_path_depth = depth
    pc.use_env_map = int(bool(env))
    pc.russian_roulette = int(rr)
    pc.rr_min_bounces = rr_min
    pc.nee = 1
    pc.nee_min = 0
    return pc


def render(flat: N.kf_flat_scene, cam: N.kf_camera_ubo, width: int, height: int, pc: N.kf_push_constants, *,
           seed=0, frame=0, camera_index=0, rng=RNG_PHILOX, tea_clock=0, precision=FP32, threads=0, use_bvh=False,
           crop=None, want_paths=True, want_hits=True):
    """Runs the oracle on a crop (x0, y0, w, h) of the image; returns a dict of numpy arrays."""
    L = load()
    x0, y0, cw, ch = crop if crop else (0, 0, width, height)
    npx = cw * ch
    spp = pc.spp
    res = {
        "pixel": np.zeros((ch, cw, 3), np.float32),
        "pixel64": np.zeros((ch, cw, 3), np.float64),
        "albedo": np.zeros((ch, cw, 3), np.float32),
        "normal": np.zeros((ch, cw, 3), np.float32),
    }
    if want_paths:
        res["paths"] = np.zeros((spp, ch, cw, 3), np.float32)
        res["depths"] = np.zeros((spp, ch, cw), np.uint32)
    if want_hits:
        res["hits"] = np.zeros((spp, ch, cw), HIT_DTYPE)
    v = kf_oracle_view()
    v.camera = C.pointer(cam)
    v.width, v.height, v.x0, v.y0, v.crop_w, v.crop_h = width, height, x0, y0, cw, ch
    v.pc = pc
    v.seed, v.frame, v.camera_index, v.rng_mode, v.tea_clock = seed, frame, camera_index, rng, tea_clock
    v.precision, v.threads, v.use_bvh = precision, threads, int(use_bvh)
    o = kf_oracle_out()
    o.pixel_color = res["pixel"].ctypes.data
    o.pixel_color64 = res["pixel64"].ctypes.data
    o.albedo = res["albedo"].ctypes.data
    o.normal = res["normal"].ctypes.data
    if want_paths:
        o.path_radiance = res["paths"].ctypes.data
        o.path_depths = res["depths"].ctypes.data
    if want_hits:
        o.primary_hits = res["hits"].ctypes.data
    rc = L.kf_oracle_render(C.byref(flat), C.byref(v), C.byref(o))
    if rc != 0:
        raise RuntimeError(f"kf_oracle_render failed: {rc}")
    res["rays"] = (o.rays_primary, o.rays_extension, o.rays_shadow)
    return res


def trace(flat: N.kf_flat_scene, rays: np.ndarray, use_bvh=False) -> np.ndarray:
    r = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
    out = np.zeros(len(r), HIT_DTYPE)
    rc = load().kf_oracle_trace(C.byref(flat), r.ctypes.data, len(r), int(use_bvh), out.ctypes.data)
    if rc != 0:
        raise RuntimeError("kf_oracle_trace failed")
    return out


def philox(ctr, key):
    out = (C.c_uint32 * 4)()
    load().kf_oracle_philox4x32_10(C.byref((C.c_uint32 * 4)(*ctr)), C.byref((C.c_uint32 * 2)(*key)), C.byref(out))
    return tuple(out)


def camera_ubo(position, front, up, width, height, fx, fy, cx, cy, skew=0.0) -> N.kf_camera_ubo:
    u = N.kf_camera_ubo()
    f3 = lambda v: C.byref((C.c_float * 3)(*[float(x) for x in v]))
    load().kf_oracle_camera_ubo(f3(position), f3(front), f3(up), float(width), float(height), float(fx), float(fy),
                                float(cx), float(cy), float(skew), C.byref(u))
    return u
