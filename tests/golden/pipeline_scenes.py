"""Scenes of the compiled-shader golden vectors (tests/golden/make_pipeline_vectors.py) and of
the test that checks the oracle against them (tests/test_oracle_pipeline.py). Built through
the kuafu-shaped API on a host-only renderer (no device), so both sides rebuild the same
flattened scene bytes from this one description."""
from __future__ import annotations

import math

from kuafu_gb300 import api, scenes


def _lights(s):
    s.setDirectionalLight(api.DirectionalLight(direction=(0.3, -0.2, -1.0), color=(1.0, 0.9, 0.8), strength=1.5,
                                               softness=0.1))
    s.addPointLight(api.PointLight(position=(0.2, 0.3, 0.7), color=(0.9, 0.9, 1.0), radius=0.2, strength=1.0))
    s.addActiveLight(api.ActiveLight(viewMat=scenes.look_at_view((-0.8, 0.5, 0.6), (0.5, -0.2, -0.8), (0, 0, 1)),
                                     color=(1.0, 0.8, 0.6), fov=math.radians(50.0), strength=2.0, softness=0.3,
                                     texID=-1))


def build(name: str):
    """Returns (renderer, camera, push-constant kwargs for the oracle) of scene `name`."""
    if name == "cornell":
        cfg = scenes.cornell_config(spp=4, depth=5)
        cfg.setHostOnly(True)
        r = api.Kuafu(cfg)
        cam = scenes.cornell(r, 24, 24)
        return r, cam, dict(spp=4, depth=5)
    if name == "cornell_lit":
        cfg = scenes.cornell_config(spp=4, depth=6)
        cfg.setHostOnly(True)
        r = api.Kuafu(cfg)
        cam = scenes.cornell(r, 24, 24)
        s = r.getScene()
        gold = api.createIcosphere(1, api.NiceMaterial(diffuseColor=(0.9, 0.7, 0.3), metallic=1.0, roughness=0.3))
        glass = api.createIcosphere(1, api.NiceMaterial(diffuseColor=(0.9, 0.95, 1.0), transmission=1.0, ior=1.5,
                                                        roughness=0.1))
        plastic = api.createIcosphere(1, api.NiceMaterial(diffuseColor=(0.2, 0.4, 0.8), specular=0.8,
                                                          roughness=0.6))
        for g in (gold, glass, plastic):
            s.submitGeometry(g)
        s.submitGeometryInstance(api.instance(gold, scenes.translate(0.1, -0.45, -0.75) @ scenes.scale(0.22, 0.22,
                                                                                                      0.22)))
        s.submitGeometryInstance(api.instance(glass, scenes.translate(-0.35, 0.35, -0.3) @ scenes.scale(0.25, 0.25,
                                                                                                       0.25)))
        s.submitGeometryInstance(api.instance(plastic, scenes.translate(0.4, 0.5, 0.4) @ scenes.scale(0.2, 0.2, 0.2)))
        _lights(s)
        return r, cam, dict(spp=4, depth=6, rr=True, rr_min=2)
    if name == "icospheres":
        cfg = scenes.icosphere_config(spp=2, depth=4, count=24)
        cfg.setHostOnly(True)
        r = api.Kuafu(cfg)
        cam = scenes.icospheres(r, 32, 24, count=24, level=2)
        return r, cam, dict(spp=2, depth=4, rr=True, rr_min=1, clear=(0.1, 0.1, 0.1, 1.0))
    raise KeyError(name)


NAMES = ("cornell", "cornell_lit", "icospheres")
TEA_CLOCK = 12345
