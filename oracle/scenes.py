"""Benchmark scenes flattened on the oracle side, without the product library.

TEST INFRASTRUCTURE ONLY: used by tests/ and by the CPU legs of bench.py (the
reference arm and the CPU baseline), which must render the benchmark workload
without mapping libkf. It restates the workload generator (seeded splitmix64
draws, transforms, materials, lights, camera) and kuafu's host-side scene
upload (materials flattened as Scene::uploadMaterials lays them out, instance
world-to-object rows, Scene::uploadLightBuffers at scene.cpp:252-292, the camera
UBO of scene.cpp:236-250) through liboracle, and produces the same
kf_flat_scene bytes that kf_scene_export hands the oracle (a CPU test checks
that byte for byte against the product's export).
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from kuafu_gb300 import _native as N  # struct layouts only: loads no shared library

from . import oracle as O


class SplitMix64:
    """splitmix64 (Steele, Lea, Flood 2014) -> uniform doubles in [0, 1)."""

    def __init__(self, seed: int):
        self.s = seed & 0xFFFFFFFFFFFFFFFF

    def next_u64(self) -> int:
        self.s = (self.s + 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF
        z = self.s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & 0xFFFFFFFFFFFFFFFF
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & 0xFFFFFFFFFFFFFFFF
        return z ^ (z >> 31)

    def uniform(self, lo=0.0, hi=1.0) -> float:
        return lo + (hi - lo) * ((self.next_u64() >> 11) * (1.0 / 9007199254740992.0))


def _translate(x, y, z):
    m = np.eye(4)
    m[:3, 3] = (x, y, z)
    return m


def _scale(s):
    return np.diag([s, s, s, 1.0])


def _rotation(u1, u2, u3):
    """Uniform random rotation from three uniforms (Shoemake, Graphics Gems III)."""
    x, y, z, w = (math.sqrt(1 - u1) * math.sin(2 * math.pi * u2), math.sqrt(1 - u1) * math.cos(2 * math.pi * u2),
                  math.sqrt(u1) * math.sin(2 * math.pi * u3), math.sqrt(u1) * math.cos(2 * math.pi * u3))
    m = np.eye(4)
    m[:3, :3] = [[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                 [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                 [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]]
    return m


def _look_at(eye, target, up):
    """glm::lookAt as a row-major matrix (the view matrix of an active light)."""
    eye, target, up = (np.asarray(v, np.float64) for v in (eye, target, up))
    f = target - eye
    f /= np.linalg.norm(f)
    s = np.cross(f, up)
    s /= np.linalg.norm(s)
    u = np.cross(s, f)
    m = np.eye(4)
    m[0, :3], m[1, :3], m[2, :3] = s, u, -f
    m[0, 3], m[1, 3], m[2, 3] = -s @ eye, -u @ eye, f @ eye
    return m


def _col_major(m) -> np.ndarray:
    """A row-major numpy matrix rounded to float and laid out as glm's column-major mat4."""
    return np.ascontiguousarray(np.asarray(m, np.float32).reshape(4, 4).T.reshape(-1))


def icosphere_mesh(level: int):
    L = O.load()
    nv, ni = C.c_uint32(), C.c_uint32()
    if L.kf_oracle_icosphere(level, None, 0, None, 0, C.byref(nv), C.byref(ni)) != 0:
        raise ValueError("icosphere level must be in [0, 8]")
    v = (N.kf_vertex * nv.value)()
    idx = np.zeros(ni.value, np.uint32)
    rc = L.kf_oracle_icosphere(level, v, nv.value, idx.ctypes.data_as(C.POINTER(C.c_uint32)), ni.value,
                               C.byref(nv), C.byref(ni))
    if rc != 0:
        raise RuntimeError("kf_oracle_icosphere failed")
    return v, idx


class FlatScene:
    """A kf_flat_scene plus the buffers it points into, and the view's camera UBO."""

    def __init__(self):
        self.keep = []
        self.flat = N.kf_flat_scene()
        self.camera = None
        self.width = self.height = 0
        self.clear = (0.0, 0.0, 0.0, 1.0)


def icospheres(width=1920, height=1080, count=256, level=4, seed=0) -> FlatScene:
    """The icosphere workload (the generator of the Mrays/s benchmark): `count` level-`level`
    icospheres, one geometry and one PrincipledBSDF material each (base colour U[0,1]^3,
    roughness U[0.05, 1], metallic Bernoulli(0.3), transmission Bernoulli(0.2), IOR 1.45),
    placed at U[-20, 20]^3 with scale log-U[0.2, 3] and a uniform random rotation; one
    directional, four point and two spot lights; background 0.1; a 60 degree pinhole camera
    at (-30, 0, 0) looking along +x. Same draws, in the same order, as the product's scene
    generator, so both describe one scene."""
    L = O.load()
    out = FlatScene()
    rng = SplitMix64(seed)
    verts, idx = icosphere_mesh(level)
    ntri = len(idx) // 3
    mats = (N.kf_material_gpu * count)()
    geoms = (N.kf_flat_geometry * count)()
    insts = (N.kf_flat_instance * count)()
    mat_index = []
    for k in range(count):
        m = mats[k]
        m.diffuse[:] = [rng.uniform(), rng.uniform(), rng.uniform(), 0.0]
        m.roughness = rng.uniform(0.05, 1.0)
        m.metallic = 1.0 if rng.uniform() < 0.3 else 0.0
        m.transmission = 1.0 if rng.uniform() < 0.2 else 0.0
        m.ior = 1.45
        m.alpha, m.specular = 1.0, 0.5
        m.emission[:] = [1.0, 1.0, 1.0, 0.0]
        m.diffuse_tex = m.metallic_tex = m.roughness_tex = m.transmission_tex = -1
        # createX gives every index slot the geometry's material (one entry per index)
        mi = np.full(len(idx), k, np.uint32)
        mat_index.append(mi)
        g = geoms[k]
        g.vertices = C.cast(verts, C.POINTER(N.kf_vertex))
        g.num_vertices = len(verts)
        g.num_triangles = ntri
        g.indices = idx.ctypes.data_as(C.POINTER(C.c_uint32))
        g.mat_index = mi.ctypes.data_as(C.POINTER(C.c_uint32))
        g.opaque, g.hide_render = 1, 0
        pos = (rng.uniform(-20, 20), rng.uniform(-20, 20), rng.uniform(-20, 20))
        sc = math.exp(rng.uniform(math.log(0.2), math.log(3.0)))
        rot = _rotation(rng.uniform(), rng.uniform(), rng.uniform())
        t = _col_major(_translate(*pos) @ rot @ _scale(sc))
        inst = insts[k]
        inst.transform[:] = t.tolist()
        rows = (C.c_float * 12)()
        if L.kf_oracle_instance_rows((C.c_float * 16)(*t.tolist()), C.cast(rows, C.POINTER(C.c_float))) != 0:
            raise RuntimeError("singular instance transform")
        inst.world_to_object[:] = list(rows)
        inst.geometry_index = k
    dir_light = (C.c_float * 8)(-1.0, -0.5, -2.0, 1.0, 0.95, 0.9, 2.0, 0.05)
    points = np.zeros((4, 8), np.float32)
    for k in range(4):
        points[k, :3] = (rng.uniform(-20, 20), rng.uniform(-20, 20), rng.uniform(-20, 20))
        points[k, 3:6] = (rng.uniform(0.5, 1), rng.uniform(0.5, 1), rng.uniform(0.5, 1))
        points[k, 6:8] = (0.5, 300.0)
    actives = np.zeros((2, 24), np.float32)
    for k in range(2):
        eye = (rng.uniform(-25, 25), rng.uniform(-25, 25), 25.0)
        actives[k, :16] = _col_major(_look_at(eye, (0, 0, 0), (0, 1, 0)))
        actives[k, 16:19] = (1.0, 1.0, 1.0)
        actives[k, 19:24] = (math.radians(60.0), 2000.0, 0.0, -1.0, 0.0)
    f = out.flat
    L.kf_oracle_light_ubos(C.cast(dir_light, C.c_void_p), points.ctypes.data, 4, actives.ctypes.data, 2, 0,
                           C.byref(f.dlight), C.byref(f.plights), C.byref(f.alights))
    f.geometries = geoms
    f.num_geometries = count
    f.instances = insts
    f.num_instances = count
    f.materials = mats
    f.num_materials = count
    f.num_textures = 0
    f.env_size = 0
    out.keep += [verts, idx, mats, geoms, insts, mat_index, points, actives]
    fy = (height / 2.0) / math.tan(math.radians(60.0) / 2.0)
    out.camera = O.camera_ubo((-30.0, 0.0, 0.0), (1.0, 0.0, 0.0), (0.0, 0.0, 1.0), width, height, fy, fy,
                              width / 2.0, height / 2.0)
    out.width, out.height = width, height
    out.clear = (0.1, 0.1, 0.1, 1.0)
    return out
