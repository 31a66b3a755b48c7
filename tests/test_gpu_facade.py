"""The kuafu-shaped C++ facade (include/kuafu_gb300/kuafu.hpp) renders the same
frame as the same scene built through the Python binding: both go through the
C-ABI, so the downloaded B8G8R8A8 frames must be byte-identical."""
import subprocess

import numpy as np
import pytest

from kuafu_gb300 import api, build, scenes

pytestmark = pytest.mark.gpu


def test_cpp_facade_frame_equals_python_api_frame(tmp_path):
    exe = build.build_example()
    w, h, spp, frames = 64, 48, 4, 2
    out = tmp_path / "frame.bgra"
    p = subprocess.run([str(exe), str(w), str(h), str(spp), str(frames), str(out)], capture_output=True, text=True,
                       timeout=300)
    assert p.returncode == 0, p.stderr
    cpp = np.fromfile(out, np.uint8).reshape(h, w, 4)
    cfg = scenes.cornell_config(spp=spp, depth=5)
    with api.Kuafu(cfg) as r:
        cam = scenes.cornell(r, w, h)
        for _ in range(frames):
            r.run()
        py = r.downloadLatestFrame(cam)
    assert np.array_equal(cpp, py)
    assert cpp[..., 3].min() == 255 and cpp[..., :3].max() > 0
