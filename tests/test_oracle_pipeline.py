"""The oracle's bounce loop against kuafu's own shaders.

tests/golden/pipeline_vectors.npz holds per-path radiance, pixel colours, albedo and
normals rendered by kuafu's PathTrace.rgen / PathTrace.rchit / PathTrace.rmiss /
PathTraceShadow.rmiss compiled as C++ (tests/golden/make_pipeline_vectors.py: GLSL
rewritten mechanically, traceRayEXT answered by the oracle's traversal, clockARB()
pinned). The oracle renders the same scenes in its TEA/LCG mode, which draws kuafu's
own tea/lcg sequence, and must give the same numbers: the camera ray, the material
lobes, the three light loops with their rejection samplers, Russian roulette and the
sample average, as kuafu's source computes them."""
import sys
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle as O

GOLDEN = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(GOLDEN))

import pipeline_scenes  # noqa: E402


@pytest.fixture(scope="module")
def vectors():
    path = GOLDEN / "pipeline_vectors.npz"
    if not path.exists():
        pytest.fail("tests/golden/pipeline_vectors.npz is missing: run tests/golden/make_pipeline_vectors.py")
    return np.load(path)


@pytest.mark.parametrize("name", pipeline_scenes.NAMES)
def test_oracle_tea_lcg_mode_equals_kuafus_compiled_shaders(vectors, name):
    r, cam, pcargs = pipeline_scenes.build(name)
    w, h = cam._size()
    res = O.render(r.getScene().export(), cam.ubo(), w, h, O.push_constants(**pcargs), rng=O.RNG_TEA_LCG,
                   tea_clock=pipeline_scenes.TEA_CLOCK, camera_index=1)
    r.close()
    want = vectors[f"{name}/paths"]
    got = res["paths"]
    exact = (got == want).all(axis=-1).mean()
    print(f"{name}: {want.shape[0] * h * w} paths, bit-exact {exact:.6f}")
    assert np.array_equal(got, want)
    assert np.array_equal(res["pixel"], vectors[f"{name}/pixel"])
    assert np.array_equal(res["albedo"], vectors[f"{name}/albedo"])
    assert np.array_equal(res["normal"], vectors[f"{name}/normal"])
    # not a dark scene: in the Cornell box only paths reaching its small emitter carry radiance
    assert (want.sum(axis=-1) > 0).mean() > 0.01
