"""Active light sensing: a dot-pattern projector seen by two IR cameras (55 mm baseline)
plus an RGB camera, the three views traced in one batch. IR views are checked against the
oracle (no denoising); the learned denoiser runs on the RGB view only."""
import numpy as np
import pytest

from kuafu_gb300 import _native as N
from kuafu_gb300 import api, scenes
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _paths_match(r, scene, cam, cam_index, spp, depth, clear):
    paths = r.downloadAov(cam, N.KF_AOV_PATH_RADIANCE, spp)
    hits = r.downloadAov(cam, N.KF_AOV_PRIMARY_HITS, spp)
    w, h = cam._size()
    ref = O.render(scene.export(), cam.ubo(), w, h, O.push_constants(spp, depth, clear=clear), seed=0, frame=0,
                   camera_index=cam_index, use_bvh=True)
    assert np.array_equal(hits["instance"], ref["hits"]["instance"])
    g = paths[..., :3].astype(np.float64)
    c = ref["paths"].astype(np.float64)
    within = ((np.abs(g - c) / np.maximum(np.abs(c), 1e-6)).max(axis=-1) <= 1e-4).mean()
    assert within >= 0.999, within


def test_projector_rig_batch_ir_parity_and_rgb_denoise():
    spp, depth = 4, 6
    cfg = scenes.icosphere_config(spp=spp, depth=depth, count=16)
    cfg.setDebugOutputs(True)
    with api.Kuafu(cfg) as r:
        rig = scenes.active_light_rig(r, count=16, pattern=(128, 72), ir=(96, 56), rgb=(128, 72), level=2)
        (irs, left), (_, right) = rig["ir"]
        rgbs, rgb = rig["rgb"]
        r.runBatch([(irs, left, spp), (irs, right, spp), (rgbs, rgb, spp)])
        _paths_match(r, irs, left, 1, spp, depth, (0.0, 0.0, 0.0, 1.0))
        _paths_match(r, irs, right, 2, spp, depth, (0.0, 0.0, 0.0, 1.0))
        _paths_match(r, rgbs, rgb, 1, spp, depth, rgbs.getClearColor())
        # IR response: one channel; lit only where dots land on geometry
        ir_l = r.downloadAov(left, N.KF_AOV_RADIANCE_F32)[..., 0]
        lit = (ir_l > 0).mean()
        assert 0.0 < lit < 0.5, lit
        # the two IR views differ by the baseline: not the same image
        ir_r = r.downloadAov(right, N.KF_AOV_RADIANCE_F32)[..., 0]
        assert not np.array_equal(ir_l, ir_r)
        # denoiser on the RGB view only
        d = api.Denoiser(r, seed=1)
        d.apply(rgb)
        den = r.downloadAov(rgb, N.KF_AOV_DENOISED_F32)
        assert den.shape == (72, 128, 4) and np.isfinite(den).all()
        with pytest.raises(N.KfError):
            r.downloadAov(left, N.KF_AOV_DENOISED_F32)
        d.close()
