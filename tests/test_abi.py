"""CPU checks of the C-ABI library: it loads, exports every declared symbol, and
its host-side scene logic (kuafu's Scene / Camera / Geometry semantics) behaves
as kuafu's does. No kernel is launched here (host-only renderer)."""
import ctypes as C
import math
import re
from pathlib import Path

import numpy as np
import pytest

from kuafu_gb300 import _native as N
from kuafu_gb300 import api, scenes

ROOT = Path(__file__).resolve().parent.parent


def declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        for m in re.finditer(r"KF_API\s+[\w\s\*]+?\b(kf_\w+)\s*\(", h.read_text()):
            names.add(m.group(1))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    lib = N.load()
    names = declared_symbols()
    assert len(names) > 60
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # and the Python binding declares a prototype for each
    assert set(names) <= set(N.PROTOTYPES), sorted(set(names) - set(N.PROTOTYPES))


def test_struct_sizes_match_the_shader_layouts():
    assert C.sizeof(N.kf_vertex) == 48          # vertex.hpp:28-34
    assert C.sizeof(N.kf_material_gpu) == 80    # Geometry.glsl:1-19 (2 vec4 + 6 float + 4 int + 2 pad)
    assert C.sizeof(N.kf_dir_light_ubo) == 32
    assert C.sizeof(N.kf_point_lights_ubo) == 32 * 32
    assert C.sizeof(N.kf_camera_ubo) == 320     # camera.hpp:181-192
    assert C.sizeof(N.kf_push_constants) == 48


def host_renderer(**kw):
    cfg = scenes.cornell_config(**kw)
    cfg.setHostOnly(True)
    return api.Kuafu(cfg)


def test_host_only_renderer_refuses_to_render():
    r = host_renderer()
    with pytest.raises(N.KfError) as e:
        r.run()
    assert e.value.code == 7  # KF_ERR_NO_DEVICE: no CPU fallback


def test_host_only_renderer_has_no_denoiser_and_no_tensor_kernels():
    r = host_renderer()
    with pytest.raises(N.KfError) as e:
        api.Denoiser(r)
    assert e.value.code == 7
    # use_denoiser without an attached denoiser is a state error before anything renders
    r.config.setUseDenoiser(True)
    r.applyConfig()
    with pytest.raises(N.KfError):
        r.run()
    r.close()


def test_config_defaults_are_kuafus():
    c = api.Config()._c
    assert (c.spp, c.path_depth, c.max_path_depth, c.russian_roulette, c.rr_min_bounces) == (32, 8, 12, 1, 4)
    assert (c.accumulate_frames, c.use_denoiser, c.max_geometries, c.max_instances) == (1, 0, 128, 256)
    assert (c.max_textures, c.max_materials) == (128, 256)


def test_builtin_meshes():
    v, i, m = api.createCube().arrays()
    assert len(v) == 24 and len(i) == 36
    v, i, m = api.createYZPlane().arrays()
    assert len(v) == 4 and list(i) == [0, 1, 2, 0, 2, 3]
    # stored normal of the plane equals (v1 - v0) x (v2 - v0) direction
    p = v[:, 0:3]
    n = np.cross(p[1] - p[0], p[2] - p[0])
    assert np.allclose(n / np.linalg.norm(n), v[0, 3:6])
    v, i, m = api.createIcosphere(4).arrays()
    assert len(i) // 3 == 5120
    pos, nrm = v[:, 0:3], v[:, 3:6]
    assert np.allclose(np.linalg.norm(pos, axis=1), 1, atol=1e-6)
    assert (np.sum(pos * nrm, axis=1) > 0.99).all()
    t = i.reshape(-1, 3)
    fn = np.cross(pos[t[:, 1]] - pos[t[:, 0]], pos[t[:, 2]] - pos[t[:, 0]])
    assert (np.sum(fn * pos[t[:, 0]], axis=1) > 0).all()  # outward winding
    v, i, m = api.createSphere().arrays()
    assert len(i) // 3 == 2 * 48 * 50 + 2 * 50
    v, i, m = api.createCapsule(1.0, 0.5).arrays()
    assert len(i) % 3 == 0 and len(v) > 0


def test_material_table_is_global_and_set_material_appends():
    before = api.materialCount()
    g = api.createCube(True, api.NiceMaterial(diffuseColor=(0.1, 0.2, 0.3)))
    assert api.materialCount() == before + 1
    g.setMaterial(api.NiceMaterial(diffuseColor=(0.5, 0.5, 0.5), alpha=0.5))
    assert api.materialCount() == before + 2
    _, _, m = g.arrays()
    assert (m == before + 1).all()


def test_scene_limits_and_errors():
    cfg = scenes.cornell_config()
    cfg.setHostOnly(True)
    cfg.setGeometryLimit(16)
    cfg._c.max_geometries = 2
    r = api.Kuafu(cfg)
    s = r.getScene()
    a, b, c = api.createCube(), api.createCube(), api.createCube()
    s.submitGeometry(a)
    s.submitGeometry(b)
    with pytest.raises(N.KfError) as e:
        s.submitGeometry(c)
    assert e.value.code == 3
    with pytest.raises(N.KfError):
        s.submitGeometryInstance(api.instance(c))  # geometry not submitted
    with pytest.raises(N.KfError) as e:
        s.removeGeometry(a)
    assert e.value.code == 5  # "Not implemented!" as in kuafu
    with pytest.raises(N.KfError):
        s.submitGeometryInstance(api.instance(a, np.zeros((4, 4))))  # singular transform
    s.submitGeometryInstance(api.instance(a))
    h = C.c_void_p()
    assert N.load().kf_scene_get_instance(s._h, 5, C.byref(h)) == 2  # out of bound


def test_geometry_validation():
    with pytest.raises(N.KfError):
        api.Geometry.from_arrays([[0, 0, 0], [1, 0, 0], [0, 1, 0]], [0, 1, 3])
    with pytest.raises(N.KfError):
        api.Geometry.from_arrays([[0, 0, float("nan")], [1, 0, 0], [0, 1, 0]], [0, 1, 2])


def test_camera_ubo_matches_oracle_host_math():
    from oracle import oracle as O

    r = host_renderer()
    cam = r.getScene().createCamera(320, 200)
    cam.setPosition((1.0, -2.0, 0.5))
    cam.setFront((0.3, 0.9, -0.1))
    cam.setUp((0.0, 0.0, 1.0))
    cam.setFullPerspective(320, 200, 250.0, 260.0, 161.0, 99.0, 0.5)
    u = cam.ubo()
    o = O.camera_ubo((1.0, -2.0, 0.5), (0.3, 0.9, -0.1), (0, 0, 1), 320, 200, 250.0, 260.0, 161.0, 99.0, 0.5)
    for f in ("view", "proj", "view_inv", "proj_inv", "position"):
        assert np.array_equal(np.array(getattr(u, f)[:]), np.array(getattr(o, f)[:])), f


def test_set_pose_follows_kuafu():
    r = host_renderer()
    cam = r.getScene().createCamera(8, 8)
    pose = np.eye(4)
    pose[:3, 3] = (1, 2, 3)
    pose[:3, :3] = scenes.rot_axis("z", 30)[:3, :3]
    cam.setPose(pose)
    got = cam.getPose()
    # Camera::setPose reads position = pose[3], front = -pose[2], up = pose[1];
    # getPose returns columns (front, -right, up, position) with right untouched.
    assert np.allclose(got[:3, 3], (1, 2, 3))
    assert np.allclose(got[:3, 0], -pose[:3, 2])
    assert np.allclose(got[:3, 2], pose[:3, 1])
    assert np.allclose(got[:3, 1], (0, 1, 0))


def test_light_ubos_follow_upload_light_buffers():
    r = host_renderer()
    s = r.getScene()
    s.submitGeometry(g := api.createCube())
    s.submitGeometryInstance(api.instance(g))
    s.setDirectionalLight(api.DirectionalLight(direction=(0, 0, -2), color=(1, 0.5, 0.25), strength=3, softness=0.1))
    s.addPointLight(api.PointLight(position=(1, 2, 3), color=(1, 1, 1), radius=0.2, strength=5))
    view = scenes.look_at_view((0, 0, 5), (0, 0, 0), (0, 1, 0))
    s.addActiveLight(api.ActiveLight(viewMat=view, fov=math.radians(60), strength=7, softness=0))
    f = s.export()
    assert list(f.dlight.direction) == [0.0, 0.0, -1.0, np.float32(0.1)]
    assert list(f.dlight.rgbs) == [1.0, 0.5, 0.25, 3.0]
    assert list(f.plights.posr[0]) == [1.0, 2.0, 3.0, np.float32(0.2)]
    assert f.plights.rgbs[1][3] == 0.0
    assert np.allclose(f.alights.position[0][:3], (0, 0, 5), atol=1e-6)
    assert np.allclose(f.alights.front[0][:3], (0, 0, -1), atol=1e-6) and f.alights.front[0][3] == 1.0
    assert f.alights.sftp[0][2] == -1.0 and f.alights.front[1][3] == 0.0
    # glm::perspective(fov, 1, 0.01, 1000)
    t = math.tan(math.radians(60) / 2)
    assert f.alights.proj[0][5] == pytest.approx(1 / t, rel=1e-6)


def test_cornell_export_shape():
    r = host_renderer()
    scenes.cornell(r, 32, 32)
    f = r.getScene().export()
    tris = sum(f.geometries[i].num_triangles for i in range(f.num_geometries))
    assert f.num_instances == 8 and tris == 36
    # world_to_object really inverts the instance transform
    for k in range(f.num_instances):
        inst = f.instances[k]
        m = np.array(inst.transform[:], np.float64).reshape(4, 4).T
        w2o = np.array(inst.world_to_object[:], np.float64).reshape(3, 4)
        prod = w2o @ m
        assert np.allclose(prod[:, :3], np.eye(3), atol=1e-5)


def test_relmse_entry_points_reject_zero_pixels():
    """kf_relmse and kf_relmse_noalloc agree: a mean over zero pixels is an invalid
    argument, refused before anything touches a device."""
    import ctypes as C

    lib = N.load()
    got = C.c_double()
    assert lib.kf_relmse_noalloc(C.c_void_p(16), C.c_void_p(16), 0, 1e-2, None, C.byref(got)) == 1
    r = host_renderer()
    assert lib.kf_relmse(r._h, C.c_void_p(16), C.c_void_p(16), 0, 1e-2, C.byref(got)) == 1
    assert b"zero pixels" in lib.kf_last_error()
    r.close()


def test_tensor_kernel_arguments_are_checked_before_any_launch():
    """kf_conv3x3_bf16, kf_gemm_bf16_tn and kf_relmse_noalloc refuse shapes and alignments
    their TMA loads and vector loads and stores cannot take, before touching the device (KF_ERR_INVALID_ARGUMENT); the
    pointer values below are never dereferenced."""
    lib = N.load()
    INVALID = 1  # KF_ERR_INVALID_ARGUMENT
    A = 1 << 20  # a 16-byte aligned stand-in address

    def conv(x=A, cin=32, w=A, rows=32, cout=32, y=A, cs=32, co=0, n=1, h=8, wd=8):
        return lib.kf_conv3x3_bf16(x, n, h, wd, cin, w, rows, None, cout, 1, y, cs, co, None)

    assert conv(y=A + 2) == INVALID          # output not 16-byte aligned
    assert conv(x=A + 8) == INVALID          # input not 16-byte aligned
    assert conv(cin=48) == INVALID           # channels neither 16 nor a multiple of 32
    assert conv(rows=24, cout=24) == INVALID  # weight rows not a multiple of 16
    assert conv(co=8, cs=32) == INVALID      # output slice past the channel stride
    assert conv(n=0) == INVALID
    assert conv(y=0) == INVALID
    assert lib.kf_gemm_bf16_tn(A, 128, A, 64, 64, A + 2, 64, 1, None) == INVALID   # output misaligned
    assert lib.kf_gemm_bf16_tn(A, 128, A, 64, 64, A, 32, 1, None) == INVALID       # ldd < n
    assert lib.kf_gemm_bf16_tn(A, 128, A, 64, 60, A, 64, 1, None) == INVALID       # k % 8 != 0
    assert lib.kf_gemm_bf16_tn(A + 8, 128, A, 64, 64, A, 64, 1, None) == INVALID   # operand misaligned
    assert lib.kf_tc_wait_probe(0, None) == INVALID                          # empty budget
    assert lib.kf_tc_wait_probe(3_000_000_000, None) == INVALID              # beyond the kernels' own
    got = C.c_double()
    assert lib.kf_relmse_noalloc(C.c_void_p(A + 4), C.c_void_p(A), 16, 1e-2, None, C.byref(got)) == INVALID
    assert b"16-byte aligned" in lib.kf_last_error()
