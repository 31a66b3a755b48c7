"""Batched rendering (kf_renderer_run_batch): views of several scenes, of uneven sizes and
sample counts, traced in one wavefront. Each view must be exactly what the oracle renders
for it alone (same frame word, its own camera index), as for kf_renderer_run."""
import numpy as np
import pytest

from kuafu_gb300 import _native as N
from kuafu_gb300 import api, scenes
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _check(r, scene, cam, cam_index, spp, depth, clear, use_bvh, env=False):
    paths = r.downloadAov(cam, N.KF_AOV_PATH_RADIANCE, spp)
    hits = r.downloadAov(cam, N.KF_AOV_PRIMARY_HITS, spp)
    w, h = cam._size()
    ref = O.render(scene.export(), cam.ubo(), w, h, O.push_constants(spp, depth, clear=clear, env=env), seed=0,
                   frame=0, camera_index=cam_index, use_bvh=use_bvh)
    assert np.array_equal(hits["instance"], ref["hits"]["instance"])
    hit = ref["hits"]["instance"] != 0xFFFFFFFF
    assert np.array_equal(hits["prim"][hit], ref["hits"]["prim"][hit])
    g = paths[..., :3].astype(np.float64)
    c = ref["paths"].astype(np.float64)
    within = ((np.abs(g - c) / np.maximum(np.abs(c), 1e-6)).max(axis=-1) <= 1e-4).mean()
    assert within >= 0.999, within
    # the resolved frame: finalColor = colors / spp, stored (independent single frame)
    rgba = r.downloadAov(cam, N.KF_AOV_RADIANCE_F32)
    assert np.allclose(rgba[..., :3], ref["pixel"], rtol=1e-6, atol=1e-7)
    # segmentation ids are scene-local in a batch too
    from test_gpu_parity import check_segmentation
    check_segmentation(r, scene, cam, spp)
    return paths


@pytest.mark.parametrize("traversal,chunk", [(0, 0), (1, 0), (1, 3000)])
def test_batch_of_uneven_views_matches_oracle(traversal, chunk):
    """chunk 3000: views split across chunks (camera rays queued per sample, or unpermuted
    where a sample straddles two chunks)."""
    depth = 4
    cfg = scenes.cornell_config(spp=1, depth=depth, debug=True)
    cfg.setTraversal(traversal)
    if chunk:
        cfg._c.max_paths_in_flight = chunk
    with api.Kuafu(cfg) as r:
        s0 = r.getScene()
        c0 = scenes.cornell(r, 40, 32, scene=s0, variation=1)
        c0b = s0.createCamera(24, 24)
        c0b.setPosition((-2.5, 0.3, 0.2))
        c0b.setFront((1.0, -0.1, -0.05))
        c0b.setUp((0.0, 0.0, 1.0))
        scenes.pinhole(c0b, 24, 24, 50.0)
        s1 = r.createScene()
        c1 = scenes.icospheres(r, 48, 32, count=12, level=2, scene=s1)
        s2 = r.createScene()
        c2 = scenes.cornell(r, 16, 40, scene=s2, variation=2)
        s2.setEnvironmentMap(np.full((6, 4, 4, 4), 0.25, np.float32))
        items = [(s0, c0, 3), (s1, c1, 2), (s2, c2, 1), (s0, c0b, 4)]
        r.runBatch(items)
        st = r.stats()
        assert st.rays_primary == 40 * 32 * 3 + 48 * 32 * 2 + 16 * 40 * 1 + 24 * 24 * 4
        _check(r, s0, c0, 1, 3, depth, (0, 0, 0, 1), False)
        _check(r, s1, c1, 1, 2, depth, s1.getClearColor(), True)
        _check(r, s2, c2, 1, 1, depth, (0, 0, 0, 1), False, env=True)
        _check(r, s0, c0b, 2, 4, depth, (0, 0, 0, 1), False)


def test_batch_view_equals_single_run():
    """One view through run() and through a one-item batch of a fresh renderer: same bytes."""
    outs = []
    for batched in (False, True):
        cfg = scenes.icosphere_config(spp=2, depth=4, count=12)
        with api.Kuafu(cfg) as r:
            cam = scenes.icospheres(r, 64, 40, count=12, level=2)
            if batched:
                r.runBatch([(r.getScene(), cam, 2)])
            else:
                r.run()
            outs.append((r.downloadAov(cam, N.KF_AOV_RADIANCE_F32), r.downloadLatestFrame(cam)))
    assert np.array_equal(outs[0][0], outs[1][0])
    assert np.array_equal(outs[0][1], outs[1][1])


def test_autotune_changes_speed_not_results():
    """kf_renderer_autotune tries traversal kernels, chunk sizes, grids and BLAS leaf sizes;
    whatever it keeps, the next batch is still exactly the oracle's render. The frame word of
    that batch is the number of batches the tuner ran: (1 + reps) per candidate + 1."""
    depth = 3
    cfg = scenes.batch_config(depth=depth)
    cfg.setDebugOutputs(True)
    with api.Kuafu(cfg) as r:
        items = scenes.batch_views(r, n_scenes=2, cams_per_scene=2, seed=3, min_side=32, max_side=64,
                                   spp_range=(1, 3), inst_range=(3, 12), level=2, variants=2)
        reps = 1
        res = r.autotune(items, reps=reps)
        assert res.candidates >= 8 and res.best_ms > 0 and res.best_ms <= res.start_ms
        assert r.config._c.traversal == res.traversal and r.config._c.blas_leaf_size == res.blas_leaf_size
        frame = res.candidates * (1 + reps) + 1
        r.runBatch(items)
        cams_seen = {}
        for s, cam, spp in items:
            idx = cams_seen.setdefault(id(s), 0) + 1
            cams_seen[id(s)] = idx
            paths = r.downloadAov(cam, N.KF_AOV_PATH_RADIANCE, spp)
            w, h = cam._size()
            ref = O.render(s.export(), cam.ubo(), w, h, O.push_constants(spp, depth), seed=0, frame=frame,
                           camera_index=idx, use_bvh=True, want_hits=False)
            g = paths[..., :3].astype(np.float64)
            c = ref["paths"].astype(np.float64)
            within = ((np.abs(g - c) / np.maximum(np.abs(c), 1e-6)).max(axis=-1) <= 1e-4).mean()
            assert within >= 0.999, within


def test_batch_replay_and_scene_change():
    """The captured batch graph replays; editing one scene rebuilds the batch pools."""
    cfg = scenes.cornell_config(spp=1, depth=3)
    with api.Kuafu(cfg) as r:
        s0 = r.getScene()
        c0 = scenes.cornell(r, 32, 32, scene=s0)
        s1 = r.createScene()
        c1 = scenes.cornell(r, 32, 32, scene=s1, variation=5)
        items = [(s0, c0, 2), (s1, c1, 2)]
        r.runBatch(items)
        a = r.downloadAov(c1, N.KF_AOV_RADIANCE_F32).copy()
        r.runBatch(items)  # replay: next frame word, same layout
        b = r.downloadAov(c1, N.KF_AOV_RADIANCE_F32).copy()
        assert not np.array_equal(a, b) and np.isfinite(b).all()
        # move a box of scene 1: its view changes, scene 0's view stays a valid render
        box = api.createCube(True, api.NiceMaterial(diffuseColor=(0.9, 0.1, 0.1)))
        s1.submitGeometry(box)
        s1.submitGeometryInstance(api.instance(box, scenes.translate(0, 0, 0) @ scenes.scale(0.4, 0.4, 0.4)))
        r.runBatch(items)
        hits = r.downloadAov(c1, N.KF_AOV_DEPTH_F32)
        assert np.isfinite(hits).all()
        with pytest.raises(N.KfError):
            r.runBatch([(s0, c0, 1), (s0, c0, 1)])  # a camera twice
