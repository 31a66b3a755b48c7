"""Parity at the benchmark configurations themselves, not only at small stand-ins.

* Cornell box, 256x256, 64 spp, path depth 5, Russian roulette off (kuafu's example
  settings, example/main.cpp:20): every path of the full frame against the oracle.
* 256 level-4 icospheres (1.31 M triangles), 1920x1080, 8 spp, depth 8, Russian roulette
  from bounce 4, 1 directional + 4 point + 2 spot lights, background 0.1 (the Mrays/s
  workload): the GPU renders the whole frame, the oracle traverses its own CPU BVH for
  fixed crops of it (deep BLAS, long traversal stacks, 9-trace paths).
* All three BVH builders (GPU LBVH, host SAH, GPU PLOC) give the same hits and paths.
* Converged FP64 accumulation: the GPU's FP64 sum of 1024 spp against the oracle's FP64
  render, on the same sample streams (agreement far below the noise) and on independent
  streams (agreement within the noise floor of 1024 spp).

Bar: primary-hit instance / primitive ids and hit distances bit-exact, per-path radiance
within 1e-4 relative (FP32) for at least 99.9 % of the paths.
"""
import numpy as np
import pytest

from kuafu_gb300 import _native as N
from kuafu_gb300 import api, scenes
from oracle import oracle as O

pytestmark = pytest.mark.gpu

REL_TOL = 1e-4  # per-path radiance, FP32
MIN_WITHIN = 0.999


def _within(gpu_paths, ref_paths):
    g = gpu_paths[..., :3].astype(np.float64)
    c = ref_paths.astype(np.float64)
    per_path = (np.abs(g - c) / np.maximum(np.abs(c), 1e-6)).max(axis=-1)
    return (per_path <= REL_TOL).mean(), (gpu_paths[..., :3] == ref_paths).all(axis=-1).mean()


def _relmse(x, ref, eps=1e-2):
    x = np.asarray(x, np.float64)
    ref = np.asarray(ref, np.float64)
    return float(((x - ref) ** 2 / (ref ** 2 + eps)).mean())


def test_cornell_full_config_256x256_64spp_depth5():
    spp, depth, w, h = 64, 5, 256, 256
    cfg = scenes.cornell_config(spp=spp, depth=depth, debug=True)
    with api.Kuafu(cfg) as r:
        cam = scenes.cornell(r, w, h)
        r.run()
        paths = r.downloadAov(cam, N.KF_AOV_PATH_RADIANCE, spp)
        hits = r.downloadAov(cam, N.KF_AOV_PRIMARY_HITS, spp)
        rgba = r.downloadAov(cam, N.KF_AOV_RADIANCE_F32)
        flat = r.getScene().export()
        ref = O.render(flat, cam.ubo(), w, h, O.push_constants(spp, depth), seed=0, frame=0, camera_index=1)
    rh = ref["hits"]
    hit = rh["instance"] != 0xFFFFFFFF
    within, exact = _within(paths, ref["paths"])
    px_close = np.isclose(rgba[..., :3], ref["pixel"], rtol=1e-5, atol=1e-6).all(axis=-1)
    print(f"C1 full: {paths.shape[0] * w * h} paths, hit {hit.mean():.4f}, ids equal "
          f"{(hits['instance'] == rh['instance']).mean():.6f}, within 1e-4 {within:.6f}, bit-exact {exact:.6f}, "
          f"pixels close {px_close.mean():.6f}")
    assert np.array_equal(hits["instance"], rh["instance"])
    assert hit.mean() > 0.9  # a square 40 degree view sees the inside of the box
    assert np.array_equal(hits["prim"][hit], rh["prim"][hit])
    assert np.array_equal(hits["t"][hit], rh["t"][hit])
    assert within >= MIN_WITHIN
    # the pixel mean of 64 paths: close wherever its paths agree
    assert px_close.mean() >= MIN_WITHIN


# Crops of the 1920x1080 frame: mostly spheres, a sparse region and the frame centre.
C2_CROPS = [(1200, 700, 96, 96), (600, 300, 96, 96), (912, 492, 96, 96)]


@pytest.fixture(scope="module")
def c2_frame():
    spp, depth, w, h = 8, 8, 1920, 1080
    cfg = scenes.icosphere_config(spp=spp, depth=depth, count=256)
    cfg.setDebugOutputs(True)
    with api.Kuafu(cfg) as r:
        cam = scenes.icospheres(r, w, h, count=256, level=4, seed=0)
        r.run()
        st = r.stats()
        out = {
            "paths": r.downloadAov(cam, N.KF_AOV_PATH_RADIANCE, spp),
            "hits": r.downloadAov(cam, N.KF_AOV_PRIMARY_HITS, spp),
            "flat_ubo": (r.getScene().export(), cam.ubo()),
            "rays": (st.rays_primary, st.rays_extension, st.rays_shadow),
        }
        yield out


@pytest.mark.parametrize("crop", C2_CROPS)
def test_icospheres_full_scene_1080p_crop(c2_frame, crop):
    spp, depth = 8, 8
    flat, ubo = c2_frame["flat_ubo"]
    pc = O.push_constants(spp, depth, clear=(0.1, 0.1, 0.1, 1.0), rr=True, rr_min=4)
    ref = O.render(flat, ubo, 1920, 1080, pc, seed=0, frame=0, camera_index=1, use_bvh=True, crop=crop)
    x0, y0, cw, ch = crop
    hits = c2_frame["hits"][:, y0:y0 + ch, x0:x0 + cw]
    paths = c2_frame["paths"][:, y0:y0 + ch, x0:x0 + cw]
    rh = ref["hits"]
    assert np.array_equal(hits["instance"], rh["instance"])
    hit = rh["instance"] != 0xFFFFFFFF
    assert hit.any()
    assert np.array_equal(hits["prim"][hit], rh["prim"][hit])
    assert np.array_equal(hits["t"][hit], rh["t"][hit])
    assert np.array_equal(hits["u"][hit], rh["u"][hit]) and np.array_equal(hits["v"][hit], rh["v"][hit])
    within, exact = _within(paths, ref["paths"])
    print(f"C2 crop {crop}: hit {hit.mean():.3f}, deepest path {ref['depths'].max()} traces, "
          f"within 1e-4 {within:.6f}, bit-exact {exact:.6f}")
    assert within >= MIN_WITHIN


def test_icospheres_full_scene_ray_count(c2_frame):
    """All 16.6 M camera rays are traced; the frame issues extension and shadow rays."""
    prim, ext, shadow = c2_frame["rays"]
    assert prim == 1920 * 1080 * 8
    assert ext > 0.3 * prim and shadow > prim


@pytest.mark.parametrize("builder", [0, 1, 2])
@pytest.mark.parametrize("leaf", [1, 4, 16])
def test_both_bvh_builders_find_the_same_hits(builder, leaf):
    """GPU LBVH (bvh_builder 0), host SAH (1) and GPU PLOC (2) change the tree, never
    the hits."""
    spp, depth = 2, 3
    cfg = scenes.icosphere_config(spp=spp, depth=depth, count=24)
    cfg.setDebugOutputs(True)
    cfg.setBvhBuilder(builder)
    cfg.setBlasLeafSize(leaf)
    with api.Kuafu(cfg) as r:
        cam = scenes.icospheres(r, 80, 48, count=24, level=2)
        r.run()
        paths = r.downloadAov(cam, N.KF_AOV_PATH_RADIANCE, spp)
        hits = r.downloadAov(cam, N.KF_AOV_PRIMARY_HITS, spp)
        st = r.stats()
        assert st.blas_nodes > 0
        ref = O.render(r.getScene().export(), cam.ubo(), 80, 48,
                       O.push_constants(spp, depth, clear=(0.1, 0.1, 0.1, 1.0)), seed=0, frame=0, camera_index=1,
                       use_bvh=True)
    rh = ref["hits"]
    assert np.array_equal(hits["instance"], rh["instance"])
    hit = rh["instance"] != 0xFFFFFFFF
    assert np.array_equal(hits["prim"][hit], rh["prim"][hit])
    assert np.array_equal(hits["t"][hit], rh["t"][hit])
    within, _ = _within(paths, ref["paths"])
    assert within >= MIN_WITHIN


@pytest.mark.parametrize("share", [1, 0])
def test_gpu_builders_on_the_full_icosphere_scene(share):
    """The GPU LBVH and PLOC builders build the 1.31 M-triangle scene (one shared BLAS, or
    256 separate builds); their hits equal the host SAH tree's over the whole 1080p frame."""
    res = []
    for builder in (0, 2, 1):
        cfg = scenes.icosphere_config(spp=1, depth=1, count=256)
        cfg.setDebugOutputs(True)
        cfg.setBvhBuilder(builder)
        cfg.setBlasShare(share)
        with api.Kuafu(cfg) as r:
            cam = scenes.icospheres(r, 1920, 1080, count=256, level=4, seed=0)
            r.run()
            res.append(r.downloadAov(cam, N.KF_AOV_PRIMARY_HITS, 1))
    ref = res[-1]
    hit = ref["instance"] != 0xFFFFFFFF
    assert hit.mean() > 0.2
    for got in res[:-1]:
        assert np.array_equal(got["instance"], ref["instance"])
        assert np.array_equal(got["prim"][hit], ref["prim"][hit])
        assert np.array_equal(got["t"][hit], ref["t"][hit])


def test_shared_blas_gives_the_same_frame():
    """blas_share: the 256 identical icosphere geometries (one material each) share one BLAS
    copy instead of 256; the frame's hits and per-path radiance are bit-identical, and the
    node pool holds one sphere's nodes."""
    spp, depth, w, h = 2, 6, 320, 180
    res, nodes = [], []
    for share in (0, 1):
        cfg = scenes.icosphere_config(spp=spp, depth=depth, count=256)
        cfg.setDebugOutputs(True)
        cfg.setBlasShare(share)
        with api.Kuafu(cfg) as r:
            cam = scenes.icospheres(r, w, h, count=256, level=4, seed=0)
            r.run()
            res.append((r.downloadAov(cam, N.KF_AOV_PRIMARY_HITS, spp),
                        r.downloadAov(cam, N.KF_AOV_PATH_RADIANCE, spp)))
            nodes.append(r.stats().blas_nodes)
    (h0, p0), (h1, p1) = res
    for f in ("instance", "prim", "t", "u", "v"):
        assert np.array_equal(h0[f], h1[f]), f
    assert (h0["instance"] != 0xFFFFFFFF).mean() > 0.2
    assert np.array_equal(p0, p1)
    assert nodes[1] * 200 < nodes[0]


def test_converged_fp64_accumulation_against_fp64_oracle():
    """The FP64 sum target (KF_AOV_SUM_F64) over 64 frames x 16 spp = 1024 spp of a 48x48
    Cornell view against the oracle's FP64 render of the same frames. Same sample streams:
    the images differ only by FP32-vs-FP64 rounding (relMSE far below the 1024-spp noise).
    Independent streams (seed 1): relMSE within twice the expected noise of two
    independent 1024-spp estimates, measured from the oracle's own half-split."""
    frames, spp, depth, w, h = 64, 16, 5, 48, 48
    cfg = scenes.cornell_config(spp=spp, depth=depth)
    with api.Kuafu(cfg) as r:
        cam = scenes.cornell(r, w, h)
        for _ in range(frames):
            r.run()
        s64 = r.downloadAov(cam, N.KF_AOV_SUM_F64)
        flat = r.getScene().export()  # points into the renderer's scene: used before it closes
        ubo = cam.ubo()

        def oracle_frames(seed):
            acc = []
            for f in range(frames):
                res = O.render(flat, ubo, w, h, O.push_constants(spp, depth), seed=seed, frame=f, camera_index=1,
                               precision=O.FP64, want_paths=False, want_hits=False)
                acc.append(res["pixel64"])
            return np.stack(acc)

        same = oracle_frames(0)
        indep = oracle_frames(1)
    assert s64.dtype == np.float64 and (s64[..., 3] == frames).all()
    gpu = s64[..., :3] / frames
    ref_same = same.mean(axis=0)
    ref_indep = indep.mean(axis=0)
    # noise of a 1024-spp estimate: relMSE(A, B) of two 512-spp halves is 4x it
    half = _relmse(indep[: frames // 2].mean(axis=0), indep[frames // 2:].mean(axis=0))
    floor_1024 = half / 4.0
    r_same = _relmse(gpu, ref_same)
    r_indep = _relmse(gpu, ref_indep)
    print(f"FP64 converged: relMSE same streams {r_same:.3e}, independent {r_indep:.3e}, "
          f"1024-spp floor {floor_1024:.3e}")
    assert floor_1024 > 0
    assert r_same < 1e-3 * floor_1024
    assert r_indep < 2.0 * (2.0 * floor_1024)


def test_1080p_reference_crop_against_fp64_oracle():
    """The time-to-relMSE reference image is the GPU's FP64 accumulation of the 1920x1080
    Cornell box. A 32x32 crop of a 2048-spp accumulation against the oracle's FP64 render of
    that crop at 1024 spp with independent streams: relMSE within twice the noise expected of
    the two estimates, the noise measured from the oracle's own two 512-spp halves."""
    frames, spp, depth, w, h = 8, 256, 5, 1920, 1080
    crop = (944, 524, 32, 32)
    cfg = scenes.cornell_config(spp=spp, depth=depth)
    with api.Kuafu(cfg) as r:
        cam = scenes.cornell(r, w, h)
        for _ in range(frames):
            r.run()
        s64 = r.downloadAov(cam, N.KF_AOV_SUM_F64)
        flat = r.getScene().export()  # points into the renderer's scene: used before it closes
        ubo = cam.ubo()
        halves = [O.render(flat, ubo, w, h, O.push_constants(512, depth), seed=77, frame=f, camera_index=1,
                           precision=O.FP64, crop=crop, want_paths=False, want_hits=False)["pixel64"]
                  for f in (0, 1)]
    x0, y0, cw, ch = crop
    gpu = s64[y0:y0 + ch, x0:x0 + cw, :3] / frames
    ora = 0.5 * (halves[0] + halves[1])
    c = _relmse(halves[0], halves[1]) * 512 / 2.0  # relMSE of an n-spp estimate ~ c / n
    expected = c * (1.0 / (frames * spp) + 1.0 / 1024)
    got = _relmse(gpu, ora)
    print(f"1080p reference crop: relMSE vs FP64 oracle {got:.3e}, expected noise {expected:.3e}")
    assert c > 0
    assert got < 2.0 * expected


@pytest.mark.parametrize("builder", [0, 1, 2])
def test_builders_with_coincident_triangles(builder):
    """Degenerate input for every builder: 200 copies of one triangle, 100 copies of another
    and a strip of distinct ones, in one geometry (equal Morton codes, equal split and merge
    costs). The hits equal the oracle's brute force, the lowest primitive winning a tie."""
    rng = np.random.default_rng(5)
    pos, idx = [], []

    def tri(a, b, c, copies):
        for _ in range(copies):
            base = len(pos)
            pos.extend([a, b, c])
            idx.extend([base, base + 1, base + 2])

    tri((1.0, -0.8, -0.8), (1.0, 0.8, -0.8), (1.0, 0.0, 0.8), 200)
    tri((0.5, -0.3, -0.3), (0.5, 0.3, -0.3), (0.5, 0.0, 0.3), 100)
    for k in range(64):
        y = -1.0 + k / 32.0
        z = rng.uniform(-0.5, 0.5)
        tri((1.5, y, z - 0.5), (1.5, y + 0.03, z - 0.5), (1.5, y, z + 0.5), 1)
    spp, depth, w, h = 1, 1, 48, 48
    cfg = scenes.cornell_config(spp=spp, depth=depth)
    cfg.setDebugOutputs(True)
    cfg.setBvhBuilder(builder)
    with api.Kuafu(cfg) as r:
        s = r.getScene()
        g = api.Geometry.from_arrays(pos, idx)
        g.setMaterial(api.NiceMaterial(diffuseColor=(0.7, 0.7, 0.7)))
        s.submitGeometry(g)
        s.submitGeometryInstance(api.instance(g, np.eye(4)))
        cam = s.createCamera(w, h)
        s.setCamera(cam)
        cam.setPosition((-2.0, 0.0, 0.0))
        cam.setFront((1.0, 0.0, 0.0))
        cam.setUp((0.0, 0.0, 1.0))
        scenes.pinhole(cam, w, h, 60.0)
        r.run()
        hits = r.downloadAov(cam, N.KF_AOV_PRIMARY_HITS, spp)
        ref = O.render(s.export(), cam.ubo(), w, h, O.push_constants(spp, depth), seed=0, frame=0, camera_index=1)
    rh = ref["hits"]
    assert np.array_equal(hits["instance"], rh["instance"])
    hit = rh["instance"] != 0xFFFFFFFF
    assert hit.mean() > 0.05
    assert np.array_equal(hits["prim"][hit], rh["prim"][hit])
    assert np.array_equal(hits["t"][hit], rh["t"][hit])
    # within each stack of copies the lowest primitive (0, 200) wins every tie
    p = hits["prim"][hit]
    assert (p == 200).any() and (p == 0).any()
    assert not ((p > 0) & (p < 200)).any() and not ((p > 200) & (p < 300)).any()


@pytest.mark.parametrize("builder", [0, 1, 2])
@pytest.mark.parametrize("instances", [1, 5])
def test_builders_on_tiny_geometries(builder, instances):
    """BLAS of 1, 2, 3 and 5 triangles (a one-leaf BLAS, and trees of one or two levels),
    a second geometry with the 3-triangle one's positions and indices (a shared BLAS), and a
    TLAS of one instance or of five: every builder gives the oracle's brute-force hits."""
    rng = np.random.default_rng(11)

    def geometry(n):
        # n roughly equilateral triangles of circumradius 0.3 facing the camera (-x), their
        # centres spread over [-0.3, 0.3] in y and z, depth jittered by 0.05
        pos = []
        for _ in range(n):
            c = np.array([rng.uniform(-0.05, 0.05), rng.uniform(-0.3, 0.3), rng.uniform(-0.3, 0.3)])
            a0 = rng.uniform(0.0, 2.0 * np.pi)
            for k in range(3):
                a = a0 + 2.0 * np.pi * k / 3.0
                pos.append(c + (rng.uniform(-0.05, 0.05), 0.3 * np.cos(a), 0.3 * np.sin(a)))
        return np.array(pos), np.arange(3 * n)

    shapes = [geometry(n) for n in (1, 2, 3, 5)]
    shapes.append(shapes[2])
    spp, depth, w, h = 1, 1, 48, 40
    cfg = scenes.cornell_config(spp=spp, depth=depth)
    cfg.setDebugOutputs(True)
    cfg.setBvhBuilder(builder)
    with api.Kuafu(cfg) as r:
        s = r.getScene()
        for k, (pos, idx) in enumerate(shapes[:instances]):
            g = api.Geometry.from_arrays(pos, idx)
            g.setMaterial(api.NiceMaterial(diffuseColor=(0.7, 0.7, 0.7)))
            s.submitGeometry(g)
            m = np.eye(4)
            m[:3, :3] *= 2.5 if instances == 1 else 1.0
            m[:3, 3] = (0.2 * k, -0.9 + 0.45 * k, 0.3 * (k % 2) - 0.15) if instances > 1 else (0.0, 0.0, 0.0)
            s.submitGeometryInstance(api.instance(g, m))
        cam = s.createCamera(w, h)
        s.setCamera(cam)
        cam.setPosition((-2.0, 0.0, 0.0))
        cam.setFront((1.0, 0.0, 0.0))
        cam.setUp((0.0, 0.0, 1.0))
        scenes.pinhole(cam, w, h, 60.0)
        r.run()
        hits = r.downloadAov(cam, N.KF_AOV_PRIMARY_HITS, spp)
        ref = O.render(s.export(), cam.ubo(), w, h, O.push_constants(spp, depth), seed=0, frame=0, camera_index=1)
    rh = ref["hits"]
    assert np.array_equal(hits["instance"], rh["instance"])
    hit = rh["instance"] != 0xFFFFFFFF
    assert hit.mean() > 0.05
    assert len(np.unique(rh["instance"][hit])) == instances
    assert np.array_equal(hits["prim"][hit], rh["prim"][hit])
    assert np.array_equal(hits["t"][hit], rh["t"][hit])
    assert np.array_equal(hits["u"][hit], rh["u"][hit]) and np.array_equal(hits["v"][hit], rh["v"][hit])


def test_out_of_range_material_index_is_refused():
    """A geometry whose matIndex names a material that does not exist is refused on the
    host, before any upload or launch, and the renderer stays usable."""
    cfg = scenes.cornell_config(spp=1, depth=1)
    with api.Kuafu(cfg) as r:
        s = r.getScene()
        g = api.Geometry.from_arrays([(1.0, -0.5, -0.5), (1.0, 0.5, -0.5), (1.0, 0.0, 0.5)], [0, 1, 2],
                                     mat_index=[1 << 30])
        s.submitGeometry(g)
        s.submitGeometryInstance(api.instance(g, np.eye(4)))
        cam = s.createCamera(16, 16)
        s.setCamera(cam)
        with pytest.raises(N.KfError, match="material"):
            r.run()
        g.setMaterial(api.NiceMaterial(diffuseColor=(0.5, 0.5, 0.5)))
        r.run()
        r.synchronize()
        assert r.downloadLatestFrame(cam).shape == (16, 16, 4)
