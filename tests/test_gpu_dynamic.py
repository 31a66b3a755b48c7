"""Dynamic scenes: per-frame instance transforms (GeometryInstance::setTransform) refit the
TLAS and reuse every BLAS (kuafu: RayTracer::updateTlas every frame, context.cpp:334-341);
instance-set changes rebuild. A refitted TLAS finds exactly the hits of a fresh build."""
import math

import numpy as np
import pytest

from kuafu_gb300 import _native as N
from kuafu_gb300 import api, scenes
from oracle import oracle as O

pytestmark = pytest.mark.gpu

SPP, DEPTH = 2, 3


def _transforms(n, seed):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        pos = rng.uniform(-6, 6, 3)
        sc = math.exp(rng.uniform(math.log(0.5), math.log(2.0)))
        rot = scenes.quat_matrix(*rng.uniform(0, 1, 3))
        out.append(scenes.translate(*pos) @ rot @ scenes.scale(sc, sc, sc))
    return out


def _scene(r, transforms):
    s = r.getScene()
    mats = [api.NiceMaterial(diffuseColor=(0.8, 0.3, 0.2), roughness=0.4),
            api.NiceMaterial(diffuseColor=(0.2, 0.7, 0.9), metallic=1.0, roughness=0.2)]
    geoms = [api.createIcosphere(2, m) for m in mats]
    for g in geoms:
        s.submitGeometry(g)
    insts = []
    for k, m in enumerate(transforms):
        inst = api.instance(geoms[k % 2], m)
        s.submitGeometryInstance(inst)
        insts.append(inst)
    s.setDirectionalLight(api.DirectionalLight(direction=(-1.0, -0.5, -2.0), strength=2.0))
    s.addPointLight(api.PointLight(position=(0.0, 0.0, 8.0), color=(1, 1, 1), radius=0.2, strength=40.0))
    s.setClearColor((0.1, 0.1, 0.1, 1.0))
    cam = s.createCamera(64, 48)
    s.setCamera(cam)
    cam.setPosition((-16.0, 0.0, 0.0))
    cam.setFront((1.0, 0.0, 0.0))
    cam.setUp((0.0, 0.0, 1.0))
    scenes.pinhole(cam, 64, 48, 60.0)
    return s, cam, insts


def _cfg():
    cfg = scenes.icosphere_config(spp=SPP, depth=DEPTH, count=32)
    cfg.setDebugOutputs(True)
    cfg.setAccumulatingFrames(False)
    return cfg


def test_refit_equals_rebuild_and_oracle():
    before, after = _transforms(20, 1), _transforms(20, 2)
    with api.Kuafu(_cfg()) as a:
        s, cam, insts = _scene(a, before)
        a.run()
        assert a.stats().tlas_refits == 0
        for inst, m in zip(insts, after):
            inst.setTransform(m)
        a.run()  # frame word 1, refitted TLAS
        assert a.stats().tlas_refits == 1
        paths_a = a.downloadAov(cam, N.KF_AOV_PATH_RADIANCE, SPP).copy()
        hits_a = a.downloadAov(cam, N.KF_AOV_PRIMARY_HITS, SPP).copy()
        ref = O.render(s.export(), cam.ubo(), 64, 48, O.push_constants(SPP, DEPTH, clear=(0.1, 0.1, 0.1, 1.0)),
                       seed=0, frame=1, camera_index=1, use_bvh=True)
    with api.Kuafu(_cfg()) as b:
        _, cam_b, _ = _scene(b, after)
        b.run()
        b.run()  # frame word 1, freshly built TLAS
        assert b.stats().tlas_refits == 0
        paths_b = b.downloadAov(cam_b, N.KF_AOV_PATH_RADIANCE, SPP)
        hits_b = b.downloadAov(cam_b, N.KF_AOV_PRIMARY_HITS, SPP)
    assert np.array_equal(hits_a, hits_b)
    assert np.array_equal(paths_a, paths_b)
    assert np.array_equal(hits_a["instance"], ref["hits"]["instance"])
    moved = (hits_a["instance"] != 0xFFFFFFFF).mean()
    assert moved > 0.05
    g = paths_a[..., :3].astype(np.float64)
    c = ref["paths"].astype(np.float64)
    assert ((np.abs(g - c) / np.maximum(np.abs(c), 1e-6)).max(axis=-1) <= 1e-4).mean() >= 0.999


def test_many_refits_then_set_change():
    """Animate for several frames (refits only), then add an instance (rebuild)."""
    with api.Kuafu(_cfg()) as r:
        s, cam, insts = _scene(r, _transforms(12, 3))
        r.run()
        for f in range(5):
            for inst, m in zip(insts, _transforms(12, 10 + f)):
                inst.setTransform(m)
            r.run()
        assert r.stats().tlas_refits == 5
        extra = api.instance(api.createIcosphere(1, api.NiceMaterial()), scenes.translate(0, 0, 0))
        s.submitGeometry(extra.geometry)
        s.submitGeometryInstance(extra)
        r.run()
        hits = r.downloadAov(cam, N.KF_AOV_PRIMARY_HITS, SPP)
        ref = O.render(s.export(), cam.ubo(), 64, 48, O.push_constants(SPP, DEPTH, clear=(0.1, 0.1, 0.1, 1.0)),
                       seed=0, frame=6, camera_index=1, use_bvh=True, want_paths=False)
        assert np.array_equal(hits["instance"], ref["hits"]["instance"])


def test_light_swap_under_graph_replay_matches_direct_launch():
    """The light-slot map (which UBO entry each shadow-ray slot samples) is rebuilt every
    frame. Swapping the directional light for a point light keeps one slot but changes
    what it samples: a replayed graph must not keep the old map. Graph replay and direct
    launches give the same bytes, and both equal the oracle after the swap."""
    outs = []
    for use_graph in (False, True):
        cfg = _cfg()
        cfg.setUseGraph(use_graph)
        with api.Kuafu(cfg) as r:
            s, cam, _ = _scene(r, _transforms(12, 4))
            s.removeLights()
            s.setDirectionalLight(api.DirectionalLight(direction=(-1.0, -0.5, -2.0), strength=2.0))
            r.run()
            first = r.downloadAov(cam, N.KF_AOV_PATH_RADIANCE, SPP)
            s.removeDirectionalLight()
            s.addPointLight(api.PointLight(position=(0.0, 3.0, 8.0), color=(1, 1, 1), radius=0.2, strength=40.0))
            r.run()
            paths = r.downloadAov(cam, N.KF_AOV_PATH_RADIANCE, SPP)
            flat = s.export()
            ref = O.render(flat, cam.ubo(), 64, 48, O.push_constants(SPP, DEPTH, clear=(0.1, 0.1, 0.1, 1.0)),
                           seed=0, frame=1, camera_index=1, use_bvh=True, want_hits=False)
            g = paths[..., :3].astype(np.float64)
            c = ref["paths"].astype(np.float64)
            assert ((np.abs(g - c) / np.maximum(np.abs(c), 1e-6)).max(axis=-1) <= 1e-4).mean() >= 0.999
            assert not np.array_equal(first, paths)
            outs.append(paths)
    assert np.array_equal(outs[0], outs[1])


def _matches_oracle(r, s, cam, frame):
    paths = r.downloadAov(cam, N.KF_AOV_PATH_RADIANCE, SPP).copy()
    hits = r.downloadAov(cam, N.KF_AOV_PRIMARY_HITS, SPP).copy()
    ref = O.render(s.export(), cam.ubo(), 64, 48, O.push_constants(SPP, DEPTH, clear=(0.1, 0.1, 0.1, 1.0)),
                   seed=0, frame=frame, camera_index=1, use_bvh=True)
    assert np.array_equal(hits["instance"], ref["hits"]["instance"])
    hit = ref["hits"]["instance"] != 0xFFFFFFFF
    assert np.array_equal(hits["prim"][hit], ref["hits"]["prim"][hit])
    g = paths[..., :3].astype(np.float64)
    c = ref["paths"].astype(np.float64)
    assert ((np.abs(g - c) / np.maximum(np.abs(c), 1e-6)).max(axis=-1) <= 1e-4).mean() >= 0.999
    return paths, hits


def test_material_and_visibility_changes_between_frames():
    """Geometry::setMaterial, hideRender and isOpaque changed between frames reach the next
    frame (kuafu reads a geometry's hideRender and opacity when it rebuilds the TLAS every
    frame, rt.cpp:156, context.cpp:328-341): each frame equals the oracle's render of the
    scene as it then is, under graph replay."""
    with api.Kuafu(_cfg()) as r:
        s, cam, insts = _scene(r, _transforms(16, 5))
        red, blue = insts[0].geometry, insts[1].geometry
        r.run()
        first, hits0 = _matches_oracle(r, s, cam, 0)
        blue_ids = {i for i in range(1, 16, 2)}
        assert np.isin(hits0["instance"], list(blue_ids)).any()
        red.setMaterial(api.NiceMaterial(diffuseColor=(0.1, 0.9, 0.1), metallic=1.0, roughness=0.3))
        r.run()
        second, _ = _matches_oracle(r, s, cam, 1)
        assert not np.array_equal(first, second)
        blue.setFlags(opaque=True, hide_render=True)
        r.run()
        _, hits2 = _matches_oracle(r, s, cam, 2)
        assert not np.isin(hits2["instance"], list(blue_ids)).any()
        blue.setFlags(opaque=True, hide_render=False)
        r.run()
        _, hits3 = _matches_oracle(r, s, cam, 3)
        assert np.isin(hits3["instance"], list(blue_ids)).any()
