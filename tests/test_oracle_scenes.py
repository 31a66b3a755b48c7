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


def test_oracle_refuses_out_of_range_references():
    """A flat scene whose material, vertex or geometry index points past its arrays is
    refused by both oracle entry points (return code 3) instead of being read out of bounds;
    the product refuses such a scene before its upload. The mistakes are planted in copies
    of the exported scene's records."""
    import pytest

    from kuafu_gb300 import _native as N
    from oracle import oracle as O

    cfg = scenes.cornell_config(spp=1, depth=1)
    cfg.setHostOnly(True)
    with api.Kuafu(cfg) as r:
        s = r.getScene()
        g = api.Geometry.from_arrays([(1.0, -0.5, -0.5), (1.0, 0.5, -0.5), (1.0, 0.0, 0.5)], [0, 1, 2])
        g.setMaterial(api.NiceMaterial(diffuseColor=(0.5, 0.5, 0.5)))
        s.submitGeometry(g)
        s.submitGeometryInstance(api.instance(g, np.eye(4)))
        cam = s.createCamera(8, 8)
        s.setCamera(cam)
        cam.setPosition((-2.0, 0.0, 0.0))
        cam.setFront((1.0, 0.0, 0.0))
        cam.setUp((0.0, 0.0, 1.0))
        flat = s.export()
        ubo = cam.ubo()
        rays = np.array([[-2.0, 0.0, 0.0, 1e-3, 1.0, 0.0, 0.0, 1e6]], np.float32)
        assert O.trace(flat, rays)["instance"][0] == 0
        O.render(flat, ubo, 8, 8, O.push_constants(1, 1))

        def planted(field, value, where="geometry"):
            f2 = N.kf_flat_scene.from_buffer_copy(flat)
            keep = []
            if where == "geometry":
                g2 = N.kf_flat_geometry.from_buffer_copy(flat.geometries[0])
                n = 3 * g2.num_triangles if field == "indices" else g2.num_triangles
                arr = np.ctypeslib.as_array(getattr(g2, field), (n,)).copy()
                arr[0] = value(g2)
                setattr(g2, field, arr.ctypes.data_as(type(getattr(g2, field))))
                geoms = (N.kf_flat_geometry * 1)(g2)
                f2.geometries = C.cast(geoms, C.POINTER(N.kf_flat_geometry))
                keep += [arr, geoms]
            else:
                i2 = N.kf_flat_instance.from_buffer_copy(flat.instances[0])
                i2.geometry_index = flat.num_geometries
                insts = (N.kf_flat_instance * 1)(i2)
                f2.instances = C.cast(insts, C.POINTER(N.kf_flat_instance))
                keep.append(insts)
            return f2, keep

        for f2, keep in (planted("mat_index", lambda g2: flat.num_materials),
                         planted("indices", lambda g2: g2.num_vertices),
                         planted(None, None, where="instance")):
            with pytest.raises(RuntimeError, match="failed: 3"):
                O.render(f2, ubo, 8, 8, O.push_constants(1, 1))
            with pytest.raises(RuntimeError):
                O.trace(f2, rays)
