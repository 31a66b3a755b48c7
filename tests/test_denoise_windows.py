"""Training windows of the denoiser (kuafu_gb300.denoise_eval.window_camera).

A size x size window camera must trace, through each of its pixels, the ray that the
full-size pinhole camera of the same pose traces through the corresponding pixel of the
full frame: the camera UBO's inverse projection and view matrices, applied as
PathTrace.rgen:35-56 applies them, give the same directions.
"""
import numpy as np

from kuafu_gb300 import api, denoise_eval, scenes


def _dirs(cam, px, py):
    """World-space ray directions through pixel positions (px, py) of cam (rgen:35-56)."""
    u = cam.ubo()
    w, h = cam.getWidth(), cam.getHeight()
    pinv = np.array(u.proj_inv[:], np.float64).reshape(4, 4).T  # GLSL mat4 is column-major
    vinv = np.array(u.view_inv[:], np.float64).reshape(4, 4).T
    d = np.stack([px / w * 2.0 - 1.0, py / h * 2.0 - 1.0, np.ones_like(px), np.ones_like(px)], axis=-1)
    t = d @ pinv.T
    t3 = t[:, :3] / np.linalg.norm(t[:, :3], axis=1, keepdims=True)
    out = np.concatenate([t3, np.zeros((len(px), 1))], axis=1) @ vinv.T
    return out[:, :3] / np.linalg.norm(out[:, :3], axis=1, keepdims=True)


def test_window_camera_at_the_icosphere_views_60_degrees():
    """The 60-degree icosphere camera (add_icosphere_views) windows the same way."""
    cfg = scenes.icosphere_config(spp=1, depth=1, count=4)
    cfg.setHostOnly(True)
    r = api.Kuafu(cfg)
    full = scenes.icospheres(r, 1920, 1080, count=4, level=1)
    s2 = r.createScene()
    win = scenes.icospheres(r, 256, 256, count=4, level=1, scene=s2)
    x0, y0 = 700, 90
    denoise_eval.window_camera(win, 256, 1920, 1080, x0, y0, fov_deg=60.0)
    rng = np.random.default_rng(4)
    i = rng.uniform(0, 256, 64)
    j = rng.uniform(0, 256, 64)
    assert np.abs(_dirs(win, i, j) - _dirs(full, x0 + i, y0 + j)).max() < 1e-5


def test_window_camera_traces_the_rays_of_its_crop():
    cfg = scenes.cornell_config()
    cfg.setHostOnly(True)
    r = api.Kuafu(cfg)
    full = scenes.cornell(r, 1920, 1080)
    win = r.getScene().createCamera(256, 256)
    win.setPosition((-1.0 - 1.0 / np.tan(np.radians(20.0)) - 0.02, 0.0, 0.0))
    win.setFront((1.0, 0.0, 0.0))
    win.setUp((0.0, 0.0, 1.0))
    x0, y0 = 1201, 377
    denoise_eval.window_camera(win, 256, 1920, 1080, x0, y0)
    rng = np.random.default_rng(3)
    i = rng.uniform(0, 256, 64)
    j = rng.uniform(0, 256, 64)
    a = _dirs(win, i, j)
    b = _dirs(full, x0 + i, y0 + j)
    assert np.abs(a - b).max() < 1e-5
    # and a window at the origin of a frame of its own size is the plain pinhole camera
    win2 = r.getScene().createCamera(256, 256)
    scenes.pinhole(win2, 256, 256, 40.0)
    ref = win2.ubo()
    denoise_eval.window_camera(win2, 256, 256, 256, 0, 0)
    assert np.array_equal(np.array(win2.ubo().proj[:]), np.array(ref.proj[:]))
