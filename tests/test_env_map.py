"""Environment cube map (Scene::setEnvironmentMap, scene.cpp:182-188; PathTrace.rmiss:14-29):
the KTX 1.1 reader, the RGBA8 / sRGB path, and the oracle's cube-face mapping. CPU only."""
import struct

import numpy as np
import pytest

from kuafu_gb300 import _native as N
from kuafu_gb300 import api, scenes
from oracle import oracle as O

KTX_ID = bytes([0xAB, 0x4B, 0x54, 0x58, 0x20, 0x31, 0x31, 0xBB, 0x0D, 0x0A, 0x1A, 0x0A])


def _ktx(path, faces, gl_type, gl_format, gl_internal, kv=b""):
    """Writes an uncompressed KTX 1.1 cube map (faces: [6, n, n, comps] of the texel dtype)."""
    n = faces.shape[1]
    comps = faces.shape[3]
    tsize = faces.dtype.itemsize
    row = n * comps * tsize
    row_pad = (row + 3) // 4 * 4
    hdr = struct.pack("<13I", 0x04030201, gl_type, tsize, gl_format, gl_internal, gl_format, n, n, 0, 0, 6, 1,
                      len(kv))
    face_bytes = row_pad * n
    body = struct.pack("<I", face_bytes)
    for f in range(6):
        for y in range(n):
            body += faces[f, y].tobytes() + b"\0" * (row_pad - row)
    with open(path, "wb") as fh:
        fh.write(KTX_ID + hdr + kv + body)


def _host_scene():
    cfg = api.Config()
    cfg.setHostOnly(True)
    r = api.Kuafu(cfg)
    return r, r.getScene()


def _env_of(scene):
    fs = scene.export()
    n = fs.env_size
    if n == 0:
        return None
    return np.ctypeslib.as_array(fs.env_rgba32f, shape=(6 * n * n * 4,)).reshape(6, n, n, 4).copy()


def test_ktx_float_half_and_srgb(tmp_path):
    r, s = _host_scene()
    rng = np.random.default_rng(0)
    f32 = rng.random((6, 5, 5, 4)).astype(np.float32)
    _ktx(tmp_path / "f.ktx", f32, 0x1406, 0x1908, 0x8814)  # GL_FLOAT, GL_RGBA, GL_RGBA32F
    s.setEnvironmentMap(str(tmp_path / "f.ktx"))
    assert np.array_equal(_env_of(s), f32)
    # RGB half floats (3 x 2 bytes per texel: rows padded to 4 bytes), alpha becomes 1
    h = (rng.random((6, 3, 3, 3)) * 4).astype(np.float16)
    _ktx(tmp_path / "h.ktx", h, 0x140B, 0x1907, 0x881B, kv=b"\x08\0\0\0abc\0def\0")
    s.setEnvironmentMap(str(tmp_path / "h.ktx"))
    e = _env_of(s)
    assert np.array_equal(e[..., :3], h.astype(np.float32)) and (e[..., 3] == 1).all()
    # sRGB 8-bit: decoded with the sRGB transfer function, alpha linear
    u8 = rng.integers(0, 256, (6, 4, 4, 4), dtype=np.uint8)
    _ktx(tmp_path / "s.ktx", u8, 0x1401, 0x1908, 0x8C43)  # GL_UNSIGNED_BYTE, GL_RGBA, GL_SRGB8_ALPHA8
    s.setEnvironmentMap(str(tmp_path / "s.ktx"))
    e = _env_of(s)
    c = u8[..., :3] / 255.0
    ref = np.where(c <= 0.04045, c / 12.92, ((c + 0.055) / 1.055) ** 2.4)
    assert np.allclose(e[..., :3], ref, atol=2e-7)
    assert np.allclose(e[..., 3], u8[..., 3] / 255.0)
    # the same bytes through the RGBA8 entry point
    s.setEnvironmentMap(u8)
    assert np.array_equal(_env_of(s), e)
    s.removeEnvironmentMap()
    assert _env_of(s) is None
    r.close()


def test_ktx_rejects_bad_files(tmp_path):
    r, s = _host_scene()
    (tmp_path / "x.ktx").write_bytes(b"not a ktx file at all" * 4)
    with pytest.raises(N.KfError):
        s.setEnvironmentMap(str(tmp_path / "x.ktx"))
    bad = np.zeros((6, 4, 4, 2), np.uint8)
    _ktx(tmp_path / "rg.ktx", bad, 0x1401, 0x8227, 0x8227)  # GL_RG: unsupported
    with pytest.raises(N.KfError):
        s.setEnvironmentMap(str(tmp_path / "rg.ktx"))
    with pytest.raises(N.KfError):
        s.setEnvironmentMap(str(tmp_path / "missing.ktx"))
    r.close()


@pytest.mark.parametrize("front,up,face", [
    ((1, 0, 0), (0, 0, 1), 5),    # d = +x -> (-d.y, d.z, -d.x) = (0, 0, -1): -Z
    ((-1, 0, 0), (0, 0, 1), 4),   # +Z
    ((0, 1, 0), (0, 0, 1), 1),    # (-1, 0, 0): -X
    ((0, -1, 0), (0, 0, 1), 0),   # +X
    ((0, 0, 1), (1, 0, 0), 2),    # +Y
    ((0, 0, -1), (1, 0, 0), 3),   # -Y
])
def test_oracle_cube_face_selection(front, up, face):
    """Camera rays that all miss: the centre pixel shows the face of rmiss's remapped direction."""
    r, s = _host_scene()
    colors = np.array([[1, 0, 0], [0, 1, 0], [0, 0, 1], [1, 1, 0], [0, 1, 1], [1, 0, 1]], np.float32)
    faces = np.ones((6, 4, 4, 4), np.float32)
    faces[..., :3] = colors[:, None, None, :]
    s.setEnvironmentMap(faces)
    cam = s.createCamera(9, 9)
    s.setCamera(cam)
    cam.setPosition((0.0, 0.0, 0.0))
    cam.setFront(front)
    cam.setUp(up)
    scenes.pinhole(cam, 9, 9, 20.0)
    flat = s.export()
    pc = O.push_constants(1, 1, env=True)
    ref = O.render(flat, cam.ubo(), 9, 9, pc, seed=0, camera_index=1, want_hits=False)
    centre = ref["paths"][0, 4, 4]
    assert np.array_equal(centre, colors[face]), (centre, face)
    # a narrow view stays on one face: every pixel shows it
    assert (ref["paths"][0] == colors[face]).all()
    r.close()
