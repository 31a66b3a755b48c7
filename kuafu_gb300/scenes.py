"""Synthetic workloads, built through the kuafu-shaped API.

* ``cornell``: the procedural Cornell box (kuafu's CornellBox.obj asset is not
  shipped): five wall quads (white 0.73 / red (0.63, 0.065, 0.05) / green
  (0.14, 0.45, 0.09)), two white diffuse boxes of roughness 1 rotated +-17
  degrees, a ceiling emitter quad of 0.25 x 0.2 room widths with emission 15,
  pinhole camera with a 40 degree vertical field of view. 34 non-emissive
  triangles plus the 2-triangle emitter (36 in total).
* ``icospheres``: 256 level-4 icospheres (5120 triangles each, 1.31 M total)
  with random translation U[-20, 20]^3, scale log-U[0.2, 3] and uniform random
  rotation, one PrincipledBSDF material each (base colour U[0,1]^3, roughness
  U[0.05, 1], metallic Bernoulli(0.3), transmission Bernoulli(0.2), IOR 1.45),
  one directional light, four point lights, two spot lights (active lights
  without a pattern) and a constant background of 0.1.

Random numbers come from splitmix64, so scenes are identical on every machine.
"""
from __future__ import annotations

import math

import numpy as np

from . import api


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


def translate(x, y, z):
    m = np.eye(4)
    m[:3, 3] = (x, y, z)
    return m


def scale(x, y, z):
    return np.diag([x, y, z, 1.0])


def rot_axis(axis: str, deg: float):
    a = math.radians(deg)
    c, s = math.cos(a), math.sin(a)
    m = np.eye(4)
    i, j = {"x": (1, 2), "y": (2, 0), "z": (0, 1)}[axis]
    m[i, i], m[i, j], m[j, i], m[j, j] = c, -s, s, c
    return m


def quat_matrix(u1, u2, u3):
    """Uniform random rotation from three uniforms (Shoemake, Graphics Gems III)."""
    q = (math.sqrt(1 - u1) * math.sin(2 * math.pi * u2), math.sqrt(1 - u1) * math.cos(2 * math.pi * u2),
         math.sqrt(u1) * math.sin(2 * math.pi * u3), math.sqrt(u1) * math.cos(2 * math.pi * u3))
    x, y, z, w = q
    m = np.eye(4)
    m[:3, :3] = [[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                 [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                 [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]]
    return m


def pinhole(cam: api.Camera, width: int, height: int, fov_deg: float = 40.0):
    fy = (height / 2.0) / math.tan(math.radians(fov_deg) / 2.0)
    cam.setFullPerspective(width, height, fy, fy, width / 2.0, height / 2.0, 0.0)


def cornell(renderer: api.Kuafu, width=256, height=256, scene: api.Scene | None = None, variation: int | None = None):
    """Builds the Cornell box into `scene` (default: the current scene) and returns its camera.

    `variation` (optional) perturbs box placement, wall colours and light size
    with a seeded generator, for the denoiser's training set."""
    s = scene or renderer.getScene()
    rng = SplitMix64(variation) if variation is not None else None

    def jit(v, amp):
        return v if rng is None else v + amp * (2.0 * rng.uniform() - 1.0)

    white = (0.73, 0.73, 0.73)
    red = (0.63, 0.065, 0.05)
    green = (0.14, 0.45, 0.09)
    if rng is not None:
        red = tuple(min(1.0, max(0.0, jit(c, 0.1))) for c in red)
        green = tuple(min(1.0, max(0.0, jit(c, 0.1))) for c in green)
    wall = lambda c: api.NiceMaterial(diffuseColor=c)
    geoms = []
    # walls: the YZ plane (normal +x) moved onto each face of [-1, 1]^3, facing inward
    walls = [
        (wall(white), translate(1, 0, 0) @ rot_axis("z", 180)),   # back
        (wall(white), translate(0, 0, -1) @ rot_axis("y", -90)),  # floor
        (wall(white), translate(0, 0, 1) @ rot_axis("y", 90)),    # ceiling
        (wall(red), translate(0, 1, 0) @ rot_axis("z", -90)),     # left (+y)
        (wall(green), translate(0, -1, 0) @ rot_axis("z", 90)),   # right (-y)
    ]
    box = api.NiceMaterial(diffuseColor=white, roughness=1.0)
    lw, ld = jit(0.25, 0.05), jit(0.2, 0.05)
    light = api.NiceMaterial(diffuseColor=(0.0, 0.0, 0.0), emission=(1.0, 1.0, 1.0), emissionStrength=15.0)
    items = []
    for mat, m in walls:
        g = api.createYZPlane(True, mat)
        items.append((g, m))
    short = api.createCube(True, box)
    tall = api.createCube(True, box)
    items.append((short, translate(jit(-0.25, 0.15), jit(-0.35, 0.1), -0.7) @ rot_axis("z", jit(-17, 10)) @
                  scale(0.3, 0.3, 0.3)))
    items.append((tall, translate(jit(0.35, 0.1), jit(0.35, 0.1), -0.4) @ rot_axis("z", jit(17, 10)) @
                  scale(0.3, 0.3, 0.6)))
    lamp = api.createYZPlane(True, light)
    items.append((lamp, translate(0, 0, 0.999) @ rot_axis("y", 90) @ scale(1.0, lw, ld)))
    for g, _ in items:
        if g not in geoms:
            s.submitGeometry(g)
            geoms.append(g)
    for g, m in items:
        s.submitGeometryInstance(api.instance(g, m))
    s.setClearColor((0.0, 0.0, 0.0, 1.0))
    cam = s.createCamera(width, height)
    s.setCamera(cam)
    cam.setPosition((-1.0 - 1.0 / math.tan(math.radians(20.0)) - 0.02, 0.0, 0.0))
    cam.setFront((1.0, 0.0, 0.0))
    cam.setUp((0.0, 0.0, 1.0))
    pinhole(cam, width, height, 40.0)
    return cam


def cornell_config(spp=64, depth=5, seed=0, debug=False) -> api.Config:
    cfg = api.Config()
    cfg.setPerPixelSampleRate(spp)
    cfg.setPathDepth(depth)
    cfg.setRussianRoulette(False)
    cfg.setPresent(False)
    cfg.setAccumulatingFrames(True)
    cfg.setSeed(seed)
    cfg.setDebugOutputs(debug)
    return cfg


def look_at_view(eye, target, up):
    """glm::lookAt as a row-major numpy matrix (the view matrix of an active light)."""
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


def icospheres(renderer: api.Kuafu, width=1920, height=1080, count=256, level=4, seed=0,
               scene: api.Scene | None = None):
    """The 256-icosphere scene; returns its camera."""
    s = scene or renderer.getScene()
    rng = SplitMix64(seed)
    for k in range(count):
        mat = api.NiceMaterial(
            diffuseColor=(rng.uniform(), rng.uniform(), rng.uniform()),
            roughness=rng.uniform(0.05, 1.0),
            metallic=1.0 if rng.uniform() < 0.3 else 0.0,
            transmission=1.0 if rng.uniform() < 0.2 else 0.0,
            ior=1.45)
        g = api.createIcosphere(level, mat)
        s.submitGeometry(g)
        pos = (rng.uniform(-20, 20), rng.uniform(-20, 20), rng.uniform(-20, 20))
        sc = math.exp(rng.uniform(math.log(0.2), math.log(3.0)))
        rot = quat_matrix(rng.uniform(), rng.uniform(), rng.uniform())
        s.submitGeometryInstance(api.instance(g, translate(*pos) @ rot @ scale(sc, sc, sc)))
    s.setDirectionalLight(api.DirectionalLight(direction=(-1.0, -0.5, -2.0), color=(1.0, 0.95, 0.9), strength=2.0,
                                               softness=0.05))
    for k in range(4):
        p = (rng.uniform(-20, 20), rng.uniform(-20, 20), rng.uniform(-20, 20))
        s.addPointLight(api.PointLight(position=p, color=(rng.uniform(0.5, 1), rng.uniform(0.5, 1),
                                                          rng.uniform(0.5, 1)), radius=0.5, strength=300.0))
    for k in range(2):
        eye = (rng.uniform(-25, 25), rng.uniform(-25, 25), 25.0)
        s.addActiveLight(api.ActiveLight(viewMat=look_at_view(eye, (0, 0, 0), (0, 1, 0)), color=(1.0, 1.0, 1.0),
                                         fov=math.radians(60.0), strength=2000.0, softness=0.0, texID=-1))
    s.setClearColor((0.1, 0.1, 0.1, 1.0))
    cam = s.createCamera(width, height)
    s.setCamera(cam)
    # framing the [-20, 20]^3 cloud: about 46 % of primary rays hit a sphere
    cam.setPosition((-30.0, 0.0, 0.0))
    cam.setFront((1.0, 0.0, 0.0))
    cam.setUp((0.0, 0.0, 1.0))
    pinhole(cam, width, height, 60.0)
    return cam


def batch_views(renderer: api.Kuafu, n_scenes=64, cams_per_scene=2, seed=0, min_side=128, max_side=1024,
                spp_range=(1, 32), inst_range=(2, 400), level=4, variants=8):
    """The batched workload: n_scenes Cornell rooms (seeded variations), each holding N
    level-`level` icospheres (N log-uniform in inst_range; `variants` material variants,
    one geometry each, shared by the instances), seen by cams_per_scene cameras of square
    resolution log-uniform in [min_side, max_side] (multiples of 16) with spp uniform in
    spp_range. Returns [(scene, camera, spp)]."""
    rng = SplitMix64(seed ^ 0x5EED)
    items = []
    for k in range(n_scenes):
        s = renderer.getScene() if k == 0 else renderer.createScene()
        side = lambda: max(16, int(round(math.exp(rng.uniform(math.log(min_side), math.log(max_side))) / 16)) * 16)
        w0 = side()
        cam0 = cornell(renderer, w0, w0, scene=s, variation=seed * 1000 + k)
        geoms = []
        for v in range(variants):
            mat = api.NiceMaterial(diffuseColor=(rng.uniform(), rng.uniform(), rng.uniform()),
                                   roughness=rng.uniform(0.05, 1.0), metallic=1.0 if rng.uniform() < 0.3 else 0.0,
                                   transmission=1.0 if rng.uniform() < 0.2 else 0.0, ior=1.45)
            g = api.createIcosphere(level, mat)
            s.submitGeometry(g)
            geoms.append(g)
        n = int(round(math.exp(rng.uniform(math.log(inst_range[0]), math.log(inst_range[1])))))
        for i in range(n):
            g = geoms[int(rng.uniform() * variants) % variants]
            pos = (rng.uniform(-0.85, 0.85), rng.uniform(-0.85, 0.85), rng.uniform(-0.85, 0.85))
            sc = math.exp(rng.uniform(math.log(0.02), math.log(0.12)))
            s.submitGeometryInstance(api.instance(g, translate(*pos) @ quat_matrix(rng.uniform(), rng.uniform(),
                                                                                   rng.uniform()) @
                                                  scale(sc, sc, sc)))
        cams = [cam0]
        for c in range(1, cams_per_scene):
            wc = side()
            cam = s.createCamera(wc, wc)
            cam.setPosition((-3.0 + rng.uniform(-0.3, 0.3), rng.uniform(-0.6, 0.6), rng.uniform(-0.4, 0.4)))
            cam.setFront((1.0, rng.uniform(-0.15, 0.15), rng.uniform(-0.1, 0.1)))
            cam.setUp((0.0, 0.0, 1.0))
            pinhole(cam, wc, wc, 45.0)
            cams.append(cam)
        for cam in cams:
            spp = spp_range[0] + int(rng.uniform() * (spp_range[1] - spp_range[0] + 1))
            items.append((s, cam, min(spp, spp_range[1])))
    return items


def dot_pattern(width, height, density=0.05, seed=0) -> np.ndarray:
    """Seeded binary dot pattern (RGBA8, white dots on black) for a structured-light projector."""
    rng = np.random.default_rng(seed)
    img = np.zeros((height, width, 4), np.uint8)
    img[..., 3] = 255
    img[..., :3][rng.random((height, width)) < density] = 255
    return img


def active_light_rig(renderer: api.Kuafu, count=64, seed=0, pattern=(1280, 720), ir=(848, 480), rgb=(1280, 720),
                     density=0.05, baseline=0.055, level=4):
    """Active light sensing: the icosphere scene trimmed to `count` instances, seen by an RGB
    camera (the scene's own lights) and by two IR cameras `baseline` apart (scene units are
    metres) that see only a structured-light projector: an active light whose texture is a
    seeded binary dot pattern (kuafu's ActiveLight with texPath, rchit:262-316; the pattern
    is stretched to the square frustum kuafu builds, scene.cpp:277-278). The IR response is
    one channel of the IR views' radiance. Returns {"rgb": (scene, cam), "ir": [(scene, left),
    (scene, right)], "pattern": texture id}."""
    rgb_scene = renderer.getScene()
    cam_rgb = icospheres(renderer, rgb[0], rgb[1], count=count, level=level, seed=seed, scene=rgb_scene)
    ir_scene = renderer.createScene()
    # the same objects, without the visible-light sources
    ir_probe = icospheres(renderer, ir[0], ir[1], count=count, level=level, seed=seed, scene=ir_scene)
    ir_scene.removeLights()
    ir_scene.setClearColor((0.0, 0.0, 0.0, 1.0))
    tex = api.createTexture(dot_pattern(pattern[0], pattern[1], density, seed), srgb=False)
    eye = np.array([-30.0, 0.0, 0.0])
    ir_scene.addActiveLight(api.ActiveLight(viewMat=look_at_view(eye, (0.0, 0.0, 0.0), (0.0, 0.0, 1.0)),
                                            color=(1.0, 1.0, 1.0), fov=math.radians(60.0), strength=3000.0,
                                            softness=0.0, texID=tex))
    cams = []
    for side in (-0.5, 0.5):
        cam = ir_probe if side < 0 else ir_scene.createCamera(ir[0], ir[1])
        cam.setPosition((-30.0, side * baseline, 0.0))
        cam.setFront((1.0, 0.0, 0.0))
        cam.setUp((0.0, 0.0, 1.0))
        pinhole(cam, ir[0], ir[1], 50.0)
        cams.append((ir_scene, cam))
    return {"rgb": (rgb_scene, cam_rgb), "ir": cams, "pattern": tex}


def batch_config(depth=5, seed=0) -> api.Config:
    cfg = cornell_config(spp=1, depth=depth, seed=seed)
    cfg.setGeometryInstanceLimit(512)
    return cfg


def icosphere_config(spp=8, depth=8, seed=0, count=256) -> api.Config:
    cfg = api.Config()
    cfg.setPerPixelSampleRate(spp)
    cfg.setPathDepth(depth)
    cfg.setPresent(False)
    cfg.setSeed(seed)
    cfg.setGeometryLimit(max(count + 8, 128))
    cfg.setGeometryInstanceLimit(max(count + 8, 256))
    return cfg
