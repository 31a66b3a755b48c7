"""Python mirror of kuafu's public C++ API over libkf's C-ABI.

Class and method names follow include/kuafu.hpp and include/core/*.hpp
(camelCase kept where kuafu uses it) so code written against kuafu reads the
same: ``Kuafu(config)``, ``renderer.getScene()``, ``scene.submitGeometry(g)``,
``scene.submitGeometryInstance(instance(g, m))``, ``renderer.run()``,
``renderer.downloadLatestFrame(camera)``. Errors raise ``KfError`` (kuafu
throws std::runtime_error).
"""
from __future__ import annotations

import ctypes as C
import os
import weakref
from dataclasses import dataclass, field

import numpy as np

from . import _native as N


def _lib():
    return N.load()


def _f16(m) -> C.Array:
    a = np.asarray(m, dtype=np.float32).reshape(4, 4)
    # numpy matrices are row-major [row][col]; kuafu's glm::mat4 is column-major.
    return (C.c_float * 16)(*a.T.reshape(-1).tolist())


def _f3(v) -> C.Array:
    return (C.c_float * 3)(*[float(x) for x in v])


class Config:
    """kuafu::Config (include/core/config.hpp:35-177)."""

    def __init__(self):
        self._c = N.kf_config()
        _lib().kf_config_init(C.byref(self._c))

    def setInitialWidth(self, w): self._c.initial_width = int(w)
    def setInitialHeight(self, h): self._c.initial_height = int(h)
    def setPerPixelSampleRate(self, spp): self._c.spp = int(spp)
    def getPerPixelSampleRate(self): return self._c.spp
    def setPathDepth(self, d): self._c.path_depth = int(d)
    def getPathDepth(self): return self._c.path_depth
    def getMaxPathDepth(self): return self._c.max_path_depth
    def setRussianRoulette(self, flag): self._c.russian_roulette = int(bool(flag))
    def getRussianRoulette(self): return bool(self._c.russian_roulette)
    def setRussianRouletteMinBounces(self, n): self._c.rr_min_bounces = int(n)
    def setNextEventEstimation(self, flag): self._c.nee = int(bool(flag))
    def setNextEventEstimationMinBounces(self, n): self._c.nee_min_bounces = int(n)
    def setAccumulatingFrames(self, flag): self._c.accumulate_frames = int(bool(flag))
    def isAccumulatingFrames(self): return bool(self._c.accumulate_frames)
    def setUseDenoiser(self, flag=True): self._c.use_denoiser = int(bool(flag))
    def isUsingDenoiser(self): return bool(self._c.use_denoiser)
    def setPresent(self, flag): self._c.present = int(bool(flag))
    def getPresent(self): return bool(self._c.present)
    def setGeometryLimit(self, n): self._c.max_geometries = int(n)
    def setGeometryInstanceLimit(self, n): self._c.max_instances = int(n)
    def setTextureLimit(self, n): self._c.max_textures = int(n)
    def setMaterialLimit(self, n): self._c.max_materials = int(n)
    def setAssetsPath(self, path): self.assets_path = str(path)
    # GB300 additions
    def setSeed(self, seed): self._c.seed = int(seed) & 0xFFFFFFFF
    def setDebugOutputs(self, flag): self._c.debug_outputs = int(bool(flag))
    def setProfile(self, flag): self._c.profile = int(bool(flag))
    def setUseGraph(self, flag): self._c.use_graph = int(bool(flag))
    def setBlasLeafSize(self, n): self._c.blas_leaf_size = int(n)
    def setTlasLeafSize(self, n): self._c.tlas_leaf_size = int(n)
    def setMaxPathsInFlight(self, n): self._c.max_paths_in_flight = int(n)
    def setHostOnly(self, flag): self._c.host_only = int(bool(flag))
    def setTraversal(self, mode): self._c.traversal = int(mode)
    def setBvhBuilder(self, mode): self._c.bvh_builder = int(mode)

    def setBlasShare(self, on): self._c.blas_share = int(bool(on))
    def setDynamicFetch(self, refill_below=16, steps=32):
        self._c.dyn_refill_below, self._c.dyn_steps = int(refill_below), int(steps)


@dataclass
class NiceMaterial:
    """kuafu::NiceMaterial (include/core/geometry.hpp:11-30)."""
    diffuseColor: tuple = (1.0, 1.0, 1.0)
    alpha: float = 1.0
    metallic: float = 0.0
    specular: float = 0.5
    roughness: float = 0.5
    ior: float = 1.4
    transmission: float = 0.0
    emission: tuple = (1.0, 1.0, 1.0)
    emissionStrength: float = 0.0
    diffuseTex: int = -1
    metallicTex: int = -1
    roughnessTex: int = -1
    transmissionTex: int = -1

    def _c(self) -> N.kf_material:
        m = N.kf_material()
        m.diffuse_color[:] = [float(x) for x in self.diffuseColor]
        m.alpha, m.metallic, m.specular = float(self.alpha), float(self.metallic), float(self.specular)
        m.roughness, m.ior, m.transmission = float(self.roughness), float(self.ior), float(self.transmission)
        m.emission[:] = [float(x) for x in self.emission]
        m.emission_strength = float(self.emissionStrength)
        m.diffuse_tex, m.metallic_tex = int(self.diffuseTex), int(self.metallicTex)
        m.roughness_tex, m.transmission_tex = int(self.roughnessTex), int(self.transmissionTex)
        return m


class Geometry:
    """kuafu::Geometry (geometry.hpp:32-46): vertices, indices, matIndex."""

    def __init__(self, handle):
        self._h = C.c_void_p(handle)

    @classmethod
    def from_arrays(cls, positions, indices, normals=None, uvs=None, mat_index=None):
        pos = np.asarray(positions, dtype=np.float32).reshape(-1, 3)
        idx = np.ascontiguousarray(np.asarray(indices, dtype=np.uint32).reshape(-1))
        v = np.zeros((len(pos), 12), dtype=np.float32)
        v[:, 0:3] = pos
        if normals is not None:
            v[:, 3:6] = np.asarray(normals, dtype=np.float32).reshape(-1, 3)
        if uvs is not None:
            v[:, 9:11] = np.asarray(uvs, dtype=np.float32).reshape(-1, 2)
        mi = np.zeros(len(idx) // 3, dtype=np.uint32) if mat_index is None else np.asarray(mat_index, np.uint32)
        mi = np.ascontiguousarray(mi)
        h = C.c_void_p()
        N.check(_lib().kf_geometry_create(v.ctypes.data, len(pos), idx.ctypes.data, len(idx), mi.ctypes.data,
                                          len(mi), C.byref(h)))
        return cls(h.value)

    def setMaterial(self, mat: NiceMaterial):
        m = mat._c()
        N.check(_lib().kf_geometry_set_material(self._h, C.byref(m)))

    def recalculateNormals(self):
        N.check(_lib().kf_geometry_recalculate_normals(self._h))

    def setFlags(self, opaque=True, hide_render=False, dynamic=False):
        N.check(_lib().kf_geometry_set_flags(self._h, int(opaque), int(hide_render), int(dynamic)))

    def arrays(self):
        nv, ni = C.c_uint32(), C.c_uint32()
        N.check(_lib().kf_geometry_get_info(self._h, C.byref(nv), C.byref(ni)))
        v = np.zeros((nv.value, 12), np.float32)
        i = np.zeros(ni.value, np.uint32)
        m = np.zeros(max(ni.value // 3, 1), np.uint32)
        N.check(_lib().kf_geometry_get_data(self._h, v.ctypes.data, i.ctypes.data, m.ctypes.data))
        return v, i, m[: ni.value // 3]

    def __del__(self):
        try:
            if self._h and N._lib is not None:
                N._lib.kf_geometry_release(self._h)
        except Exception:
            pass


def _builtin(kind, mat, p0=0.0, p1=0.0) -> Geometry:
    m = (mat or NiceMaterial())._c()
    h = C.c_void_p()
    N.check(_lib().kf_geometry_create_builtin(kind, float(p0), float(p1), C.byref(m), C.byref(h)))
    return Geometry(h.value)


def createYZPlane(dynamic=True, mat: NiceMaterial | None = None) -> Geometry:
    return _builtin(N.KF_MESH_YZ_PLANE, mat)


def createCube(dynamic=True, mat: NiceMaterial | None = None) -> Geometry:
    return _builtin(N.KF_MESH_CUBE, mat)


def createSphere(dynamic=True, mat: NiceMaterial | None = None) -> Geometry:
    return _builtin(N.KF_MESH_SPHERE, mat)


def createCapsule(halfHeight=1.0, radius=1.0, dynamic=True, mat: NiceMaterial | None = None) -> Geometry:
    return _builtin(N.KF_MESH_CAPSULE, mat, halfHeight, radius)


def createIcosphere(level=4, mat: NiceMaterial | None = None) -> Geometry:
    return _builtin(N.KF_MESH_ICOSPHERE, mat, level)


def loadScene(path, dynamic=False) -> list[Geometry]:
    """kuafu::loadScene (geometry.hpp:56): Wavefront OBJ + MTL, one geometry per material."""
    p = os.fsencode(path)
    n = C.c_uint32()
    N.check(_lib().kf_load_scene(p, int(dynamic), None, 0, C.byref(n)))
    arr = (C.c_void_p * max(n.value, 1))()
    N.check(_lib().kf_load_scene(p, int(dynamic), arr, n.value, C.byref(n)))
    return [Geometry(arr[i]) for i in range(n.value)]


def loadObj(path, dynamic=False) -> Geometry:
    """kuafu::loadObj (geometry.hpp:57): a file holding exactly one geometry."""
    scene = loadScene(path, dynamic)
    if len(scene) != 1:
        raise N.KfError(1, "complex scene! use loadScene")
    return scene[0]


@dataclass
class GeometryInstance:
    """kuafu::GeometryInstance (geometry.hpp:48-54)."""
    geometry: Geometry
    transform: np.ndarray = field(default_factory=lambda: np.eye(4, dtype=np.float32))
    _h: C.c_void_p = None

    def setTransform(self, m):
        self.transform = np.asarray(m, dtype=np.float32).reshape(4, 4)
        if self._h:
            N.check(_lib().kf_instance_set_transform(self._h, _f16(self.transform)))


def instance(geometry: Geometry, transform=None) -> GeometryInstance:
    """kuafu::instance (geometry.hpp:65-66, geometry.cpp:251-261)."""
    t = np.eye(4, dtype=np.float32) if transform is None else np.asarray(transform, np.float32).reshape(4, 4)
    return GeometryInstance(geometry, t)


@dataclass
class DirectionalLight:
    direction: tuple = (0.0, 0.0, -1.0)
    color: tuple = (1.0, 1.0, 1.0)
    strength: float = 0.0
    softness: float = 0.0


@dataclass
class PointLight:
    position: tuple = (0.0, 0.0, 0.0)
    color: tuple = (1.0, 1.0, 1.0)
    radius: float = 1.0
    strength: float = 0.0


@dataclass
class ActiveLight:
    viewMat: np.ndarray = field(default_factory=lambda: np.eye(4, dtype=np.float32))
    color: tuple = (1.0, 1.0, 1.0)
    fov: float = 0.0
    strength: float = 0.0
    softness: float = 0.0
    texID: int = -1


class Camera:
    """kuafu::Camera (include/core/camera.hpp:40-174)."""

    def __init__(self, handle):
        self._h = C.c_void_p(handle)

    def setPosition(self, p): N.check(_lib().kf_camera_set_position(self._h, _f3(p)))
    def setFront(self, f): N.check(_lib().kf_camera_set_front(self._h, _f3(f)))
    def setUp(self, u): N.check(_lib().kf_camera_set_up(self._h, _f3(u)))
    def setPose(self, m): N.check(_lib().kf_camera_set_pose(self._h, _f16(m)))
    def resetView(self): N.check(_lib().kf_camera_reset_view(self._h))

    def getPose(self):
        a = (C.c_float * 16)()
        N.check(_lib().kf_camera_get_pose(self._h, a))
        return np.array(a[:], np.float32).reshape(4, 4).T

    def setFullPerspective(self, width, height, fx, fy, cx, cy, skew=0.0):
        N.check(_lib().kf_camera_set_full_perspective(self._h, float(width), float(height), float(fx), float(fy),
                                                      float(cx), float(cy), float(skew)))

    def setSize(self, w, h): N.check(_lib().kf_camera_set_size(self._h, int(w), int(h)))

    def getWidth(self): return self._size()[0]
    def getHeight(self): return self._size()[1]

    def _size(self):
        w, h = C.c_int(), C.c_int()
        N.check(_lib().kf_camera_get_size(self._h, C.byref(w), C.byref(h)))
        return w.value, h.value

    def ubo(self) -> N.kf_camera_ubo:
        u = N.kf_camera_ubo()
        N.check(_lib().kf_camera_get_ubo(self._h, C.byref(u)))
        return u


class Scene:
    """kuafu::Scene (include/core/scene.hpp:40-295)."""

    def __init__(self, renderer, handle):
        self._r = renderer
        self._h = C.c_void_p(handle)
        self._geoms = []
        self._instances = []
        self._lights = {}  # light object -> handle (the object is kept alive with its handle)

    def submitGeometry(self, g: Geometry):
        N.check(_lib().kf_scene_submit_geometry(self._h, g._h))
        self._geoms.append(g)

    def setGeometries(self, gs):
        self.clearGeometries()
        for g in gs:
            self.submitGeometry(g)

    def clearGeometries(self):
        N.check(_lib().kf_scene_clear_geometries(self._h))
        self._geoms.clear()
        self._instances.clear()

    def removeGeometry(self, g):
        N.check(_lib().kf_scene_remove_geometry(self._h, g._h))

    def submitGeometryInstance(self, inst: GeometryInstance):
        h = C.c_void_p()
        N.check(_lib().kf_scene_submit_instance(self._h, inst.geometry._h, _f16(inst.transform), C.byref(h)))
        inst._h = h
        self._instances.append(inst)

    def setGeometryInstances(self, insts):
        self.clearGeometryInstances()
        for i in insts:
            self.submitGeometryInstance(i)

    def removeGeometryInstance(self, inst: GeometryInstance):
        N.check(_lib().kf_scene_remove_instance(self._h, inst._h))
        self._instances = [i for i in self._instances if i is not inst]

    def clearGeometryInstances(self):
        N.check(_lib().kf_scene_clear_instances(self._h))
        self._instances.clear()

    def getGeometryInstances(self):
        return list(self._instances)

    def setClearColor(self, rgba):
        N.check(_lib().kf_scene_set_clear_color(self._h, (C.c_float * 4)(*[float(x) for x in rgba])))

    def getClearColor(self):
        a = (C.c_float * 4)()
        N.check(_lib().kf_scene_get_clear_color(self._h, a))
        return tuple(a)

    def setEnvironmentMap(self, faces):
        """Scene::setEnvironmentMap: a KTX 1.1 cube map path, or a [6, n, n, 4] array
        (faces +X, -X, +Y, -Y, +Z, -Z; float32 linear or uint8 sRGB)."""
        if isinstance(faces, (str, bytes, os.PathLike)):
            N.check(_lib().kf_scene_set_environment_map_file(self._h, os.fsencode(faces)))
            return
        a = np.asarray(faces)
        assert a.ndim == 4 and a.shape[0] == 6 and a.shape[1] == a.shape[2] and a.shape[3] == 4
        if a.dtype == np.uint8:
            a = np.ascontiguousarray(a)
            N.check(_lib().kf_scene_set_environment_map_rgba8(self._h, a.ctypes.data, a.shape[1], 1))
        else:
            a = np.ascontiguousarray(a, np.float32)
            N.check(_lib().kf_scene_set_environment_map(self._h, a.ctypes.data, a.shape[1]))
        self._env = a

    def removeEnvironmentMap(self):
        N.check(_lib().kf_scene_remove_environment_map(self._h))

    def setDirectionalLight(self, l: DirectionalLight):
        c = N.kf_directional_light(_f3(l.direction), _f3(l.color), float(l.strength), float(l.softness))
        N.check(_lib().kf_scene_set_directional_light(self._h, C.byref(c)))

    def removeDirectionalLight(self):
        N.check(_lib().kf_scene_remove_directional_light(self._h))

    def addPointLight(self, l: PointLight):
        c = N.kf_point_light(_f3(l.position), _f3(l.color), float(l.radius), float(l.strength))
        h = C.c_void_p()
        N.check(_lib().kf_scene_add_point_light(self._h, C.byref(c), C.byref(h)))
        self._lights[id(l)] = (l, h)

    def addActiveLight(self, l: ActiveLight):
        c = N.kf_active_light(_f16(l.viewMat), _f3(l.color), float(l.fov), float(l.strength), float(l.softness),
                              int(l.texID))
        h = C.c_void_p()
        N.check(_lib().kf_scene_add_active_light(self._h, C.byref(c), C.byref(h)))
        self._lights[id(l)] = (l, h)

    def removePointLight(self, l):
        N.check(_lib().kf_scene_remove_light(self._h, self._lights.pop(id(l))[1]))

    removeActiveLight = removePointLight

    def removeLights(self):
        """Removes the directional light and every point / active light added through this object."""
        self.removeDirectionalLight()
        for _, h in list(self._lights.values()):
            N.check(_lib().kf_scene_remove_light(self._h, h))
        self._lights.clear()

    def createCamera(self, width, height) -> Camera:
        h = C.c_void_p()
        N.check(_lib().kf_scene_create_camera(self._h, int(width), int(height), C.byref(h)))
        return Camera(h.value)

    def removeCamera(self, cam: Camera):
        N.check(_lib().kf_scene_remove_camera(self._h, cam._h))

    def setCamera(self, cam: Camera):
        N.check(_lib().kf_scene_set_camera(self._h, cam._h))

    def getCamera(self) -> Camera:
        h = C.c_void_p()
        N.check(_lib().kf_scene_get_camera(self._h, C.byref(h)))
        return Camera(h.value) if h.value else None

    def export(self) -> N.kf_flat_scene:
        fs = N.kf_flat_scene()
        N.check(_lib().kf_scene_export(self._h, C.byref(fs)))
        return fs


class Kuafu:
    """kuafu::Kuafu (include/kuafu.hpp:31-93)."""

    def __init__(self, config: Config | None = None):
        self.config = config or Config()
        h = C.c_void_p()
        N.check(_lib().kf_renderer_create(C.byref(self.config._c), C.byref(h)))
        self._h = h
        s = C.c_void_p()
        N.check(_lib().kf_renderer_get_scene(self._h, C.byref(s)))
        self._scenes = {s.value: Scene(self, s.value)}
        self._current = s.value

    def close(self):
        if self._h:
            # the renderer frees the denoisers it still owns: their handles die with it
            for d in list(getattr(self, "_denoisers", ())):
                d._h = None
            N.check(_lib().kf_renderer_destroy(self._h))
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def getConfig(self) -> Config:
        return self.config

    def applyConfig(self):
        N.check(_lib().kf_renderer_set_config(self._h, C.byref(self.config._c)))

    def getScene(self) -> Scene:
        return self._scenes[self._current]

    def createScene(self) -> Scene:
        s = C.c_void_p()
        N.check(_lib().kf_renderer_create_scene(self._h, C.byref(s)))
        self._scenes[s.value] = Scene(self, s.value)
        return self._scenes[s.value]

    def setScene(self, scene: Scene):
        N.check(_lib().kf_renderer_set_scene(self._h, scene._h))
        self._current = scene._h.value

    def removeScene(self, scene: Scene):
        N.check(_lib().kf_renderer_remove_scene(self._h, scene._h))
        self._scenes.pop(scene._h.value, None)

    def isRunning(self) -> bool:
        v = C.c_int()
        N.check(_lib().kf_renderer_is_running(self._h, C.byref(v)))
        return bool(v.value)

    def run(self):
        N.check(_lib().kf_renderer_run(self._h))

    def measureL2Read(self, bytes=32 << 20, passes=64, reps=5) -> float:
        """Achievable L2 read bandwidth of this renderer's GPU, GB/s (kf_renderer_measure_l2_read)."""
        out = C.c_double()
        N.check(_lib().kf_renderer_measure_l2_read(self._h, int(bytes), int(passes), int(reps), C.byref(out)))
        return out.value

    def synchronize(self):
        N.check(_lib().kf_renderer_synchronize(self._h))

    def stream(self) -> int:
        """cudaStream_t (as an integer) that all of this renderer's kernels run on."""
        p = C.c_void_p()
        N.check(_lib().kf_renderer_get_stream(self._h, C.byref(p)))
        return p.value or 0

    def downloadLatestFrame(self, cam: Camera) -> np.ndarray:
        w, h = cam._size()
        out = np.empty((h, w, 4), np.uint8)
        N.check(_lib().kf_renderer_download_latest_frame(self._h, cam._h, out.ctypes.data, out.nbytes))
        return out

    def downloadAov(self, cam: Camera, kind: int, spp: int | None = None) -> np.ndarray:
        w, h = cam._size()
        if kind in (N.KF_AOV_RADIANCE_F32, N.KF_AOV_ALBEDO_F32, N.KF_AOV_NORMAL_F32, N.KF_AOV_DENOISED_F32):
            out = np.empty((h, w, 4), np.float32)
        elif kind == N.KF_AOV_DEPTH_F32:
            out = np.empty((h, w), np.float32)
        elif kind == N.KF_AOV_SUM_F64:
            out = np.empty((h, w, 4), np.float64)
        elif kind == N.KF_AOV_SEGMENTATION:
            out = np.empty((h, w, 4), np.uint32)  # instance, geometry, material, primitive
        elif kind == N.KF_AOV_PATH_RADIANCE:
            out = np.empty((spp or self.stats().last_spp, h, w, 4), np.float32)
        elif kind == N.KF_AOV_PRIMARY_HITS:
            out = np.empty((spp or self.stats().last_spp, h, w), dtype=np.dtype(
                [("t", "<f4"), ("u", "<f4"), ("v", "<f4"), ("instance", "<u4"), ("prim", "<u4"), ("pad", "<u4", 3)]))
        else:
            raise ValueError(kind)
        N.check(_lib().kf_renderer_download_aov(self._h, cam._h, int(kind), out.ctypes.data, out.nbytes))
        return out

    def stats(self) -> N.kf_stats:
        s = N.kf_stats()
        N.check(_lib().kf_renderer_get_stats(self._h, C.byref(s)))
        return s

    def resetFrame(self):
        """Restart accumulation (the next run() stores instead of blending)."""
        N.check(_lib().kf_renderer_reset_frame(self._h))

    def resetStats(self):
        N.check(_lib().kf_renderer_reset_stats(self._h))

    def countTraversal(self, enable: bool):
        N.check(_lib().kf_renderer_count_traversal(self._h, int(bool(enable))))

    @staticmethod
    def _batch(items):
        arr = (N.kf_batch_item * len(items))()
        for i, (scene, cam, spp) in enumerate(items):
            arr[i].scene = scene._h.value
            arr[i].camera = cam._h.value
            arr[i].spp = int(spp)
        return arr

    def runBatch(self, items):
        """One frame of every (scene, camera, spp) in one wavefront (kf_renderer_run_batch)."""
        N.check(_lib().kf_renderer_run_batch(self._h, self._batch(items), len(items)))

    def autotune(self, items, reps: int = 2) -> N.kf_autotune_result:
        """Measures launch configurations on this batch and keeps the fastest."""
        res = N.kf_autotune_result()
        N.check(_lib().kf_renderer_autotune(self._h, self._batch(items), len(items), int(reps), C.byref(res)))
        N.check(_lib().kf_renderer_get_config(self._h, C.byref(self.config._c)))
        return res

    def setDenoiser(self, denoiser: "Denoiser | None"):
        """Denoiser that run() applies when the config's use_denoiser is set."""
        N.check(_lib().kf_renderer_set_denoiser(self._h, denoiser._h if denoiser else None))


class Denoiser:
    """Learned U-Net denoiser: stands in for kuafu's OptiX pass (Config::setUseDenoiser,
    src/core/config.cpp:142; src/core/context/context.cpp:651-670), trained on this
    renderer's own low-spp / high-spp pairs. All work runs on the renderer's stream."""

    def __init__(self, renderer: Kuafu, seed: int = 0):
        h = C.c_void_p()
        N.check(_lib().kf_denoiser_create(renderer._h, int(seed), C.byref(h)))
        self._h = h
        self.renderer = renderer
        if not hasattr(renderer, "_denoisers"):
            renderer._denoisers = weakref.WeakSet()
        renderer._denoisers.add(self)

    def close(self):
        if self._h:
            N.check(_lib().kf_denoiser_destroy(self._h))
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def numParams(self) -> int:
        n = C.c_uint64()
        N.check(_lib().kf_denoiser_num_params(self._h, C.byref(n)))
        return n.value

    def getParams(self) -> np.ndarray:
        out = np.empty(self.numParams(), np.float32)
        N.check(_lib().kf_denoiser_get_params(self._h, out.ctypes.data, out.size))
        return out

    def setParams(self, p: np.ndarray):
        a = np.ascontiguousarray(p, dtype=np.float32)
        N.check(_lib().kf_denoiser_set_params(self._h, a.ctypes.data, a.size))

    def save(self, path):
        N.check(_lib().kf_denoiser_save(self._h, os.fsencode(path)))

    def load(self, path):
        N.check(_lib().kf_denoiser_load(self._h, os.fsencode(path)))

    def addView(self, scene: Scene, cam: Camera, low_spp: int, high_spp: int, high_frames: int = 1):
        N.check(_lib().kf_denoiser_add_view(self._h, scene._h, cam._h, int(low_spp), int(high_spp),
                                            int(high_frames)))

    def addViewInputs(self, scene: Scene, cam: Camera, low_spps, high_spp: int, high_frames: int = 1):
        """Several inputs (one frame of each low spp) paired with one shared target."""
        arr = (C.c_uint32 * len(low_spps))(*[int(k) for k in low_spps])
        N.check(_lib().kf_denoiser_add_view_inputs(self._h, scene._h, cam._h, arr, len(low_spps), int(high_spp),
                                                   int(high_frames)))

    def numViews(self) -> int:
        n = C.c_uint32()
        N.check(_lib().kf_denoiser_num_views(self._h, C.byref(n)))
        return n.value

    def train(self, iters: int, batch: int = 8, crop: int = 128, lr: float = 1e-3) -> float:
        loss = C.c_float()
        N.check(_lib().kf_denoiser_train(self._h, int(iters), int(batch), int(crop), float(lr), C.byref(loss)))
        return loss.value

    def apply(self, cam: Camera):
        N.check(_lib().kf_denoiser_apply(self._h, cam._h))

    def forward(self, feat_ptr: int, n: int, h: int, w: int, out_ptr: int, base_ptr: int | None = None):
        N.check(_lib().kf_denoiser_forward(self._h, feat_ptr, base_ptr, n, h, w, out_ptr))

    def cameraFeatures(self, cam: Camera):
        """The network input of cam's current frame: (BF16 features [hp, wp, 32], FP32 base
        [hp, wp, 4]) as torch CUDA tensors."""
        import torch

        hp, wp = C.c_int(), C.c_int()
        N.check(_lib().kf_denoiser_camera_features(self._h, cam._h, None, None, C.byref(hp), C.byref(wp)))
        feat = torch.empty((hp.value, wp.value, 32), dtype=torch.bfloat16, device="cuda")
        base = torch.empty((hp.value, wp.value, 4), dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        N.check(_lib().kf_denoiser_camera_features(self._h, cam._h, feat.data_ptr(), base.data_ptr(), C.byref(hp),
                                                   C.byref(wp)))
        return feat, base

    def trainStep(self, feat_ptr: int, target_ptr: int, n: int, h: int, w: int, lr: float = 0.0,
                  grads_ptr: int | None = None, apply: bool = False, base_ptr: int | None = None) -> float:
        loss = C.c_float()
        N.check(_lib().kf_denoiser_train_step(self._h, feat_ptr, base_ptr, target_ptr, n, h, w, float(lr),
                                              grads_ptr, int(bool(apply)), C.byref(loss)))
        return loss.value


def materialCount() -> int:
    return _lib().kf_material_count()


def createTexture(rgba8: np.ndarray, srgb=True) -> int:
    a = np.ascontiguousarray(rgba8, dtype=np.uint8)
    assert a.ndim == 3 and a.shape[2] == 4
    tid = C.c_int32()
    N.check(_lib().kf_texture_create(a.ctypes.data, a.shape[1], a.shape[0], int(srgb), C.byref(tid)))
    return tid.value
