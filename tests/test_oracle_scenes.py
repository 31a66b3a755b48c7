"""The oracle-side flattening of the benchmark scene (oracle/scenes.py), which the CPU legs
of the benchmark render without mapping the product library, equals the product's own
kf_scene_export of the same workload byte for byte: vertices, indices, materials, instance
transforms and world-to-object rows, the three light UBOs and the camera UBO."""
import ctypes as C

import numpy as np

from kuafu_gb300 import api, scenes
from oracle import scenes as OS


def _bytes(ptr, n):
    return C.string_at(ptr, n)


def test_oracle_flattened_icosphere_scene_equals_the_product_export():
    count, level = 64, 3
    fs = OS.icospheres(640, 360, count=count, level=level, seed=5)
    cfg = scenes.icosphere_config(spp=1, depth=1, count=count)
    cfg.setHostOnly(True)
    with api.Kuafu(cfg) as r:
        cam = scenes.icospheres(r, 640, 360, count=count, level=level, seed=5)
        a = r.getScene().export()
        b = fs.flat
        assert a.num_geometries == b.num_geometries == count
        assert a.num_instances == b.num_instances == count
        for g in range(count):
            ga, gb = a.geometries[g], b.geometries[g]
            assert (ga.num_vertices, ga.num_triangles, ga.opaque) == (gb.num_vertices, gb.num_triangles, gb.opaque)
            assert _bytes(ga.vertices, ga.num_vertices * 48) == _bytes(gb.vertices, gb.num_vertices * 48)
            assert _bytes(ga.indices, ga.num_triangles * 12) == _bytes(gb.indices, gb.num_triangles * 12)
            ma = np.ctypeslib.as_array(ga.mat_index, (ga.num_triangles,))
            mb = np.ctypeslib.as_array(gb.mat_index, (gb.num_triangles,))
            # the material table is process-global: compare the entries the geometries name
            for i, j in {(int(x), int(y)) for x, y in zip(ma, mb)}:
                assert bytes(a.materials[i]) == bytes(b.materials[j])
            ia, ib = a.instances[g], b.instances[g]
            assert list(ia.transform) == list(ib.transform)
            assert list(ia.world_to_object) == list(ib.world_to_object)
            assert ia.geometry_index == ib.geometry_index == g
        assert bytes(a.dlight) == bytes(b.dlight)
        assert bytes(a.plights) == bytes(b.plights)
        assert bytes(a.alights) == bytes(b.alights)
        assert bytes(cam.ubo()) == bytes(fs.camera)
