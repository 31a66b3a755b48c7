"""GPU parity: the CUDA path tracer against the CPU oracle on identical bytes.

Bar (from the shaders' semantics): primary-hit instance / triangle ids and hit
distances bit-exact; per-path radiance within 1e-4 relative in FP32 (the
kernels and the oracle evaluate the same operations in the same order with the
same deterministic transcendentals, so bit-exact is expected and reported).
"""
import numpy as np
import pytest

from kuafu_gb300 import _native as N
from kuafu_gb300 import api, scenes
from oracle import oracle as O

pytestmark = pytest.mark.gpu

REL_TOL = 1e-4  # per-path radiance, FP32


def _camera_index(scene_cams_before):
    return scene_cams_before


def _render_pair(r, cam, spp, depth, rr=False, rr_min=4, clear=(0, 0, 0, 1), cam_index=1, use_bvh=False, frame=0,
                 env=False):
    r.run()
    paths = r.downloadAov(cam, N.KF_AOV_PATH_RADIANCE, spp)
    hits = r.downloadAov(cam, N.KF_AOV_PRIMARY_HITS, spp)
    rgba = r.downloadAov(cam, N.KF_AOV_RADIANCE_F32)
    w, h = cam._size()
    flat = r.getScene().export()
    pc = O.push_constants(spp, depth, clear=clear, rr=rr, rr_min=rr_min, env=env)
    ref = O.render(flat, cam.ubo(), w, h, pc, seed=r.config._c.seed, frame=frame, camera_index=cam_index,
                   use_bvh=use_bvh)
    return paths, hits, rgba, ref


def _check_paths(paths, ref_paths, min_exact=0.999):
    g = paths[..., :3].astype(np.float64)
    c = ref_paths.astype(np.float64)
    err = np.abs(g - c) / np.maximum(np.abs(c), 1e-6)
    per_path = err.max(axis=-1)
    within = (per_path <= REL_TOL).mean()
    exact = (paths[..., :3] == ref_paths).all(axis=-1).mean()
    print(f"paths within 1e-4: {within:.6f}, bit-exact: {exact:.6f}")
    assert within >= min_exact, f"only {within:.5f} of paths within {REL_TOL}"
    return exact


def test_cornell_primary_hits_and_path_radiance():
    cfg = scenes.cornell_config(spp=8, depth=5, debug=True)
    with api.Kuafu(cfg) as r:
        cam = scenes.cornell(r, 64, 48)
        paths, hits, rgba, ref = _render_pair(r, cam, 8, 5)
        rh = ref["hits"]
        assert np.array_equal(hits["instance"], rh["instance"])
        hit = rh["instance"] != 0xFFFFFFFF
        assert hit.mean() > 0.5  # a 4:3 frame at 40 deg vertical FOV also sees past the open box
        assert np.array_equal(hits["prim"][hit], rh["prim"][hit])
        assert np.array_equal(hits["t"][hit], rh["t"][hit])
        assert np.array_equal(hits["u"][hit], rh["u"][hit]) and np.array_equal(hits["v"][hit], rh["v"][hit])
        exact = _check_paths(paths, ref["paths"])
        assert exact > 0.999
        # first frame: rgba = finalColor = colors / spp (PathTrace.rgen:144,155)
        assert np.allclose(rgba[..., :3], ref["pixel"], rtol=1e-6, atol=1e-7)
        assert (rgba[..., 3] == 1.0).all()
        alb = r.downloadAov(cam, N.KF_AOV_ALBEDO_F32)
        nrm = r.downloadAov(cam, N.KF_AOV_NORMAL_F32)
        assert np.array_equal(alb[..., :3], ref["albedo"])
        assert np.array_equal(nrm[..., :3], ref["normal"])


def check_segmentation(r, scene, cam, spp):
    """KF_AOV_SEGMENTATION = {instance, geometry, material, primitive} of sample 0's first hit."""
    seg = r.downloadAov(cam, N.KF_AOV_SEGMENTATION)
    hits0 = r.downloadAov(cam, N.KF_AOV_PRIMARY_HITS, spp)[0]
    flat = scene.export()
    assert np.array_equal(seg[..., 0], hits0["instance"])
    miss = hits0["instance"] == 0xFFFFFFFF
    assert (seg[..., 1][miss] == 0xFFFFFFFF).all() and (seg[..., 3][miss] == 0).all()
    for y, x in zip(*np.nonzero(~miss)):
        inst = int(seg[y, x, 0])
        gi = flat.instances[inst].geometry_index
        assert seg[y, x, 1] == gi
        assert seg[y, x, 3] == hits0["prim"][y, x]
        assert seg[y, x, 2] == flat.geometries[gi].mat_index[int(seg[y, x, 3])]
    return seg


def test_segmentation_aov():
    cfg = scenes.cornell_config(spp=2, depth=2, debug=True)
    with api.Kuafu(cfg) as r:
        cam = scenes.cornell(r, 40, 32)
        r.run()
        seg = check_segmentation(r, r.getScene(), cam, 2)
        assert len(np.unique(seg[..., 0])) >= 6  # walls, boxes, light, background


def test_frame_accumulation_and_srgb_frame():
    """frameCount running mean (rgen:151-163) and the B8G8R8A8_SRGB frame (config.hpp:144)."""
    spp = 2
    cfg = scenes.cornell_config(spp=spp, depth=5, debug=True)
    with api.Kuafu(cfg) as r:
        cam = scenes.cornell(r, 40, 40)
        flat = None
        acc = None
        for frame in range(3):
            r.run()
            flat = r.getScene().export()
            ref = O.render(flat, cam.ubo(), 40, 40, O.push_constants(spp, 5), seed=0, frame=frame, camera_index=1,
                           want_paths=False, want_hits=False)
            fin = ref["pixel"].astype(np.float32)
            if frame == 0:
                acc = fin.copy()
            else:
                a = np.float32(1.0) / np.float32(frame + 1)
                acc = (acc * (np.float32(1) - a) + fin * a).astype(np.float32)
        rgba = r.downloadAov(cam, N.KF_AOV_RADIANCE_F32)
        assert np.array_equal(rgba[..., :3], acc)
        assert r.stats().frame_count == 2
        bgra = r.downloadLatestFrame(cam)
        L = O.load()
        enc = np.vectorize(lambda x: L.kf_oracle_srgb8(float(x)))(acc)
        assert np.array_equal(bgra[..., 0], enc[..., 2])
        assert np.array_equal(bgra[..., 1], enc[..., 1])
        assert np.array_equal(bgra[..., 2], enc[..., 0])
        assert (bgra[..., 3] == 255).all()
        s64 = r.downloadAov(cam, N.KF_AOV_SUM_F64)
        assert (s64[..., 3] == 3.0).all()


@pytest.mark.parametrize("traversal", [0, 1])
def test_icospheres_with_lights_bvh_parity(traversal):
    """Two-level traversal over many BLAS, PrincipledBSDF lobes incl. transmission, NEE over
    directional / point / spot lights, Russian roulette; both traversal kernels."""
    spp, depth = 2, 4
    cfg = scenes.icosphere_config(spp=spp, depth=depth, count=24)
    cfg.setDebugOutputs(True)
    cfg.setRussianRouletteMinBounces(1)
    cfg.setTraversal(traversal)
    with api.Kuafu(cfg) as r:
        cam = scenes.icospheres(r, 96, 64, count=24, level=2)
        paths, hits, rgba, ref = _render_pair(r, cam, spp, depth, rr=True, rr_min=1, clear=(0.1, 0.1, 0.1, 1.0),
                                              use_bvh=True)
        rh = ref["hits"]
        assert np.array_equal(hits["instance"], rh["instance"])
        hit = rh["instance"] != 0xFFFFFFFF
        assert hit.mean() > 0.02  # 24 spheres in a 40^3 box: a sparse view
        assert np.array_equal(hits["prim"][hit], rh["prim"][hit])
        assert np.array_equal(hits["t"][hit], rh["t"][hit])
        _check_paths(paths, ref["paths"])
        st = r.stats()
        assert st.rays_shadow > 0 and st.rays_extension > 0
        assert st.rays_primary == 96 * 64 * spp


def test_loaded_obj_renders_like_the_oracle(tmp_path):
    """A quad-faced OBJ box without normals (fan triangulation, flat normals, MTL material
    with Ns -> roughness) loaded by kf_load_scene, inside the Cornell box."""
    verts = [(x, y, z) for x in (-0.3, 0.3) for y in (-0.3, 0.3) for z in (-0.9, -0.3)]
    quads = [(1, 2, 4, 3), (5, 7, 8, 6), (1, 5, 6, 2), (3, 4, 8, 7), (1, 3, 7, 5), (2, 6, 8, 4)]
    obj = ["mtllib box.mtl"] + [f"v {x} {y} {z}" for x, y, z in verts] + ["usemtl gold"] + \
          [f"f {a} {b} {c} {d}" for a, b, c, d in quads]
    (tmp_path / "box.obj").write_text("\n".join(obj) + "\n")
    (tmp_path / "box.mtl").write_text("newmtl gold\nKd 0.9 0.7 0.2\nNs 400\n")
    spp, depth = 4, 4
    cfg = scenes.cornell_config(spp=spp, depth=depth, debug=True)
    with api.Kuafu(cfg) as r:
        cam = scenes.cornell(r, 48, 48)
        s = r.getScene()
        (g,) = api.loadScene(tmp_path / "box.obj")
        s.submitGeometry(g)
        s.submitGeometryInstance(api.instance(g, scenes.rot_axis("z", 25)))
        paths, hits, rgba, ref = _render_pair(r, cam, spp, depth)
        assert np.array_equal(hits["instance"], ref["hits"]["instance"])
        assert (hits["instance"] == 8).any()  # the loaded box is seen
        _check_paths(paths, ref["paths"])


def _smooth_env(n, seed):
    """Six n x n faces of smooth positive radiance (float32 RGBA)."""
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:n, 0:n] / max(n - 1, 1)
    faces = np.ones((6, n, n, 4), np.float32)
    for f in range(6):
        for c in range(3):
            a, b, ph = rng.uniform(0.5, 3.0, 3)
            faces[f, :, :, c] = 0.3 + 0.25 * np.sin(a * x * 6.28 + ph) * np.cos(b * y * 6.28) + 0.1 * f
    return faces


@pytest.mark.parametrize("traversal", [0, 1])
def test_environment_map_parity(traversal):
    """PathTrace.rmiss with useEnvironmentMap: misses return the cube-map lookup of (-d.y, d.z, -d.x)."""
    spp, depth = 2, 4
    cfg = scenes.icosphere_config(spp=spp, depth=depth, count=24)
    cfg.setDebugOutputs(True)
    cfg.setTraversal(traversal)
    with api.Kuafu(cfg) as r:
        cam = scenes.icospheres(r, 96, 64, count=24, level=2)
        r.getScene().setEnvironmentMap(_smooth_env(16, 3))
        paths, hits, rgba, ref = _render_pair(r, cam, spp, depth, clear=(0.1, 0.1, 0.1, 1.0), use_bvh=True,
                                              env=True)
        assert np.array_equal(hits["instance"], ref["hits"]["instance"])
        _check_paths(paths, ref["paths"])
        miss = hits["instance"] == 0xFFFFFFFF
        assert miss.mean() > 0.5
        # escaped camera rays see the map, not the clear colour
        assert not np.allclose(paths[..., :3][miss], 0.1)


def test_textured_materials_and_projector_parity():
    """Diffuse / roughness textures (rchit:338-360) and a textured active light, i.e. a
    projector (rchit:262-316, texture(tex, uv) of proj * view * worldPos), against the oracle."""
    spp, depth = 4, 3
    cfg = scenes.cornell_config(spp=spp, depth=depth, debug=True)
    with api.Kuafu(cfg) as r:
        cam = scenes.cornell(r, 64, 48)
        s = r.getScene()
        rng = np.random.default_rng(5)
        checker = np.zeros((16, 16, 4), np.uint8)
        checker[..., 3] = 255
        checker[::2, ::2, :3] = 220
        checker[1::2, 1::2, :3] = 220
        checker[..., 0] |= rng.integers(0, 30, (16, 16), dtype=np.uint8)
        tex = api.createTexture(checker, srgb=True)
        rough = api.createTexture(rng.integers(0, 255, (8, 8, 4), dtype=np.uint8), srgb=False)
        mat = api.NiceMaterial(diffuseColor=(0.8, 0.8, 0.8), roughness=0.5, diffuseTex=tex, roughnessTex=rough)
        panel = api.createYZPlane(True, mat)
        s.submitGeometry(panel)
        s.submitGeometryInstance(api.instance(panel, scenes.translate(0.95, 0, 0) @ scenes.rot_axis("z", 180) @
                                              scenes.scale(1, 0.8, 0.8)))
        # a dot-pattern projector (5 % density, seeded) aimed at the back wall
        dots = np.zeros((64, 64, 4), np.uint8)
        dots[..., 3] = 255
        dots[..., :3][rng.random((64, 64)) < 0.05] = 255
        pat = api.createTexture(dots, srgb=False)
        view = scenes.look_at_view((-0.5, 0.0, 0.2), (1.0, 0.0, 0.0), (0.0, 0.0, 1.0))
        s.addActiveLight(api.ActiveLight(viewMat=view, fov=np.radians(50), strength=5, softness=0,
                                         texID=pat))
        paths, hits, rgba, ref = _render_pair(r, cam, spp, depth)
        assert np.array_equal(hits["instance"], ref["hits"]["instance"])
        _check_paths(paths, ref["paths"])


def test_traversal_counters():
    cfg = scenes.icosphere_config(spp=1, depth=2, count=16)
    with api.Kuafu(cfg) as r:
        scenes.icospheres(r, 64, 64, count=16, level=3)
        r.countTraversal(True)
        r.resetStats()
        r.run()
        st = r.stats()
        assert st.node_visits > st.rays_primary
        assert st.tri_tests > 0 and st.inst_visits > 0
        r.countTraversal(False)


def test_transparent_geometry_is_skipped_by_closest_hit():
    """alpha == 0 geometry is ignored by the any-hit shader (rahit:40-43)."""
    cfg = scenes.cornell_config(spp=1, depth=1, debug=True)
    with api.Kuafu(cfg) as r:
        cam = scenes.cornell(r, 32, 32)
        s = r.getScene()
        glass = api.createYZPlane(True, api.NiceMaterial(alpha=0.0))
        s.submitGeometry(glass)
        s.submitGeometryInstance(api.instance(glass, scenes.translate(-0.9, 0, 0) @ scenes.scale(1, 2, 2)))
        r.run()
        hits = r.downloadAov(cam, N.KF_AOV_PRIMARY_HITS, 1)
        assert not (hits["instance"] == 8).any()  # the invisible plane (instance 8) is never the closest hit


def test_graph_replay_matches_direct_launch():
    outs = []
    for use_graph in (False, True):
        cfg = scenes.cornell_config(spp=2, depth=5)
        cfg.setUseGraph(use_graph)
        with api.Kuafu(cfg) as r:
            cam = scenes.cornell(r, 48, 32)
            r.run()
            r.run()
            outs.append(r.downloadAov(cam, N.KF_AOV_RADIANCE_F32))
    assert np.array_equal(outs[0], outs[1])


def test_two_stream_schedule_matches_sequential():
    """The default schedule runs each bounce's shadow traversal and gather on a second
    stream beside the next bounce's closest-hit traversal; the profiling schedule runs every
    kernel in order on one stream. Same bytes, with several chunks of paths."""
    outs = []
    for profile in (False, True):
        cfg = scenes.icosphere_config(spp=3, depth=6, count=12)
        cfg.setProfile(profile)
        cfg._c.max_paths_in_flight = 4096  # several chunks, views split across them
        with api.Kuafu(cfg) as r:
            cam = scenes.icospheres(r, 64, 40, count=12, level=2)
            r.run()
            r.run()
            outs.append((r.downloadAov(cam, N.KF_AOV_RADIANCE_F32), r.downloadLatestFrame(cam)))
    assert np.array_equal(outs[0][0], outs[1][0])
    assert np.array_equal(outs[0][1], outs[1][1])
