"""Wavefront OBJ / MTL loading (kuafu's loadScene over assimp, geometry.cpp:46-265), CPU."""
import math

import numpy as np
import pytest

from kuafu_gb300 import _native as N
from kuafu_gb300 import api

OBJ = """# test scene
mtllib scene.mtl
v 0 0 0
v 1 0 0
v 1 1 0
v 0 1 0
v 0 0 1 0.5 0.25 0.125
vt 0 0
vt 1 0
vt 1 1
vt 0 1
vn 0 0 1
usemtl red
f 1/1/1 2/2/1 3/3/1 4/4/1
usemtl green
f 1 2 5
usemtl red
f -5/-4/-1 -3/-2/-1 -2/-1/-1
o nomat
usemtl missing
f 2 3 5
"""

MTL = """newmtl red
Kd 1 0 0
Ke 0.5 0.5 0
Ns 100
Ni 1.5
d 0.5
newmtl green
Kd 0 1 0
Ns 3
Tr 0.25
"""


@pytest.fixture
def obj_path(tmp_path):
    (tmp_path / "scene.mtl").write_text(MTL)
    p = tmp_path / "scene.obj"
    p.write_text(OBJ)
    return p


def _material(i):
    m = N.kf_material()
    N.check(N.load().kf_material_get(int(i), m))
    return m


def test_geometries_per_material_and_vertices(obj_path):
    geoms = api.loadScene(obj_path)
    assert len(geoms) == 3  # red (quad + triangle), green, "missing" (defaults)
    v, i, m = geoms[0].arrays()
    # red: the quad's 4 corners (fan 0-1-2, 0-2-3) then the triangle's 3 corners
    assert len(v) == 7 and list(i) == [0, 1, 2, 0, 2, 3, 4, 5, 6]
    assert np.allclose(v[:4, 0:3], [[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0]])
    assert np.allclose(v[:4, 3:6], [0, 0, 1])                         # given normals
    assert np.allclose(v[:4, 9:11], [[0, 1], [1, 1], [1, 0], [0, 0]])  # V flipped
    assert len(set(m)) == 1
    # green: no normals in the file -> the face's flat normal; vertex colour from "v x y z r g b"
    v2, i2, _ = geoms[1].arrays()
    n = np.cross(v2[1, 0:3] - v2[0, 0:3], v2[2, 0:3] - v2[0, 0:3])
    n /= np.linalg.norm(n)
    assert np.allclose(v2[:, 3:6], n)
    assert np.allclose(v2[2, 6:9], [0.5, 0.25, 0.125])


def test_material_mapping(obj_path):
    geoms = api.loadScene(obj_path)
    red = _material(geoms[0].arrays()[2][0])
    assert list(red.diffuse_color) == [1, 0, 0] and list(red.emission) == [0.5, 0.5, 0]
    assert red.alpha == 0.5 and math.isclose(red.ior, 1.5, rel_tol=1e-6)
    assert math.isclose(red.roughness, 1 - math.sqrt(95) * 0.025, rel_tol=1e-6)  # Ns > 5
    assert (red.metallic, red.specular, red.transmission, red.emission_strength) == (0, 0.5, 0, 1)
    green = _material(geoms[1].arrays()[2][0])
    assert green.roughness == 1.0 and math.isclose(green.alpha, 0.75)  # Ns <= 5; Tr
    dflt = _material(geoms[2].arrays()[2][0])
    assert [round(x, 6) for x in dflt.diffuse_color] == [0.6, 0.6, 0.6]
    assert dflt.roughness == 1.0 and dflt.ior == 1.0 and dflt.alpha == 1.0


def test_materials_are_deduplicated(obj_path):
    api.loadScene(obj_path)
    n = api.materialCount()
    again = api.loadScene(obj_path)
    assert api.materialCount() == n
    assert again[0].arrays()[2][0] == api.loadScene(obj_path)[0].arrays()[2][0]


def test_load_obj_single_and_errors(tmp_path, obj_path):
    with pytest.raises(N.KfError):
        api.loadObj(obj_path)  # three geometries: "complex scene! use loadScene"
    one = tmp_path / "tri.obj"
    one.write_text("v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\n")
    g = api.loadObj(one)
    assert len(g.arrays()[0]) == 3
    bad = tmp_path / "bad.obj"
    bad.write_text("v 0 0 0\nf 1 2 7\n")
    with pytest.raises(N.KfError):
        api.loadScene(bad)
    with pytest.raises(N.KfError):
        api.loadScene(tmp_path / "missing.obj")
