"""CPU checks of the oracle itself: known answers, accuracy bounds and invariants.

kuafu ships no tests or golden vectors for its render path; the oracle is pinned
by (1) the Philox4x32-10 known-answer vectors of Random123 (Salmon et al.,
SC'11), (2) golden vectors in tests/golden/ generated by compiling kuafu's own
GLSL shader library as C++ (tests/golden/make_shader_vectors.py), matched
exactly, (3) closed-form checks of every shader helper against float64 formulas,
and (4) watertightness / BVH-equivalence properties of the traversal. The whole
bounce loop is checked against kuafu's compiled ray-tracing shaders in
tests/test_oracle_pipeline.py.
"""
import json
import math
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle as O

GOLDEN = Path(__file__).resolve().parent / "golden"


def f32(x):
    return float(np.float32(x))


# Random123 kat_vectors for philox4x32-10
PHILOX_KAT = [
    ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
]


@pytest.mark.parametrize("ctr,key,expect", PHILOX_KAT)
def test_philox_known_answers(ctr, key, expect):
    assert O.philox(ctr, key) == expect


def _py_tea(v0, v1):
    m = 0xFFFFFFFF
    s0 = 0
    for _ in range(16):
        s0 = (s0 + 0x9E3779B9) & m
        v0 = (v0 + ((((v1 << 4) & m) + 0xA341316C) ^ ((v1 + s0) & m) ^ ((v1 >> 5) + 0xC8013EA4))) & m
        v1 = (v1 + ((((v0 << 4) & m) + 0xAD90777D) ^ ((v0 + s0) & m) ^ ((v0 >> 5) + 0x7E95761E))) & m
    return v0


def test_tea_lcg_match_glsl_semantics():
    L = O.load()
    for a, b in [(0, 0), (1, 2), (123456, 99), (0xFFFFFFFF, 7), (65535, 0xDEADBEEF)]:
        assert L.kf_oracle_tea(a, b) == _py_tea(a, b)
    import ctypes as C

    st = C.c_uint32(12345)
    prev = 12345
    for _ in range(100):
        got = L.kf_oracle_rnd_lcg(C.byref(st))
        prev = (1664525 * prev + 1013904223) & 0xFFFFFFFF
        assert got == f32((prev & 0xFFFFFF) / float(1 << 24))
        assert 0.0 <= got < 1.0


def test_uniform_stream_layout():
    """u = (philox(ctr, key)[draw & 3] >> 8) * 2^-24 with ctr/key as documented in kf_types.h."""
    L = O.load()
    seed, pix, cam, s, fr, depth, purpose = 7, 1234, 2, 5, 9, 3, 16 + 4
    for draw in range(9):
        out = O.philox((s, fr, (depth << 8) | purpose, draw >> 2), (seed ^ pix, cam))
        expect = f32((out[draw & 3] >> 8) * 2.0 ** -24)
        assert L.kf_oracle_uniform(seed, pix, cam, s, fr, depth, purpose, draw) == expect


def _ulps(got, ref):
    got = np.asarray(got, np.float32)
    ref = np.asarray(ref, np.float64)
    return np.abs(got.astype(np.float64) - ref) / np.spacing(np.abs(ref).astype(np.float32)).astype(np.float64)


def test_deterministic_sin_cos_exp2_accuracy():
    L = O.load()
    xs = np.float32(np.linspace(0.0, 2 * 3.141592 * 1.0001, 20001))
    s = np.array([L.kf_oracle_sin(float(x)) for x in xs], np.float32)
    c = np.array([L.kf_oracle_cos(float(x)) for x in xs], np.float32)
    big = np.abs(np.sin(xs.astype(np.float64))) > 1e-3
    assert _ulps(s, np.sin(xs.astype(np.float64)))[big].max() <= 2.0
    big = np.abs(np.cos(xs.astype(np.float64))) > 1e-3
    assert _ulps(c, np.cos(xs.astype(np.float64)))[big].max() <= 2.0
    assert np.abs(s - np.sin(xs.astype(np.float64))).max() < 2e-7
    es = np.float32(np.linspace(-14.0, 1.0, 20001))
    e = np.array([L.kf_oracle_exp2(float(x)) for x in es], np.float32)
    assert _ulps(e, np.exp2(es.astype(np.float64))).max() <= 1.0


def test_shader_helpers_closed_form():
    """Random.glsl helpers against float64 evaluations of the same formulas."""
    import ctypes as C

    L = O.load()
    rng = np.random.default_rng(1)
    for _ in range(200):
        a2 = f32(rng.uniform(0.0, 1.0))
        nd = f32(rng.uniform(-1, 1))
        d = max(nd * nd * (a2 - 1) + 1, 1e-6)
        assert L.kf_oracle_ggx_d(nd, a2) == pytest.approx(a2 / (d * d * 3.141592), rel=1e-5)
        x = f32(rng.uniform(0.0, 1.0))
        assert L.kf_oracle_g1(x, a2) == pytest.approx(2 * x / (x + math.sqrt(a2 + (1 - a2) * x * x)), rel=1e-5)
        cosv, ior = f32(rng.uniform(0, 1)), f32(rng.uniform(1.0, 2.5))
        r0 = ((1 - ior) / (1 + ior)) ** 2
        assert L.kf_oracle_schlick(cosv, ior) == pytest.approx(r0 + (1 - r0) * (1 - cosv) ** 5, rel=1e-5, abs=1e-7)
        f0 = (C.c_float * 3)(*rng.uniform(0, 1, 3).astype(np.float32).tolist())
        out = (C.c_float * 3)()
        L.kf_oracle_schlick_fresnel(C.byref(f0), x, C.byref(out))
        p = 2.0 ** ((-5.55473 * x - 6.98316) * x)
        for k in range(3):
            assert out[k] == pytest.approx(f0[k] + (1 - f0[k]) * p, rel=1e-5)


def test_sampling_directions_are_unit_and_in_hemisphere():
    import ctypes as C

    L = O.load()
    rng = np.random.default_rng(2)
    for _ in range(500):
        n = rng.normal(size=3)
        n /= np.linalg.norm(n)
        nn = (C.c_float * 3)(*n.astype(np.float32).tolist())
        out = (C.c_float * 3)()
        u0, u1 = f32(rng.uniform()), f32(rng.uniform())
        L.kf_oracle_cosine_hemisphere(u0, u1, C.byref(nn), C.byref(out))
        v = np.array(out[:])
        assert abs(np.linalg.norm(v) - 1) < 1e-5
        assert v @ n >= -1e-6
        # cos(theta) of the sample is sqrt(u1) (Sampling.glsl:32)
        assert v @ n == pytest.approx(math.sqrt(u1), abs=2e-5)
        a2 = f32(rng.uniform(0.01, 1))
        L.kf_oracle_sample_ggx(u0, u1, a2, C.byref(nn), C.byref(out))
        h = np.array(out[:])
        # Random.glsl:88-100 builds T and B from an unnormalised cross product, so H is
        # not unit length in kuafu either; its component along N is exactly cos(theta_h).
        ct = math.sqrt(min(max((1 - u0) / ((a2 - 1) * u0 + 1), 0), 1))
        assert h @ n == pytest.approx(ct, abs=2e-5)


def _isect(o, d, v0, v1, v2, tmin=0.0, tmax=1e30):
    import ctypes as C

    L = O.load()
    a = [(C.c_float * 3)(*map(float, x)) for x in (o, d, v0, v1, v2)]
    t, u, v = C.c_float(), C.c_float(), C.c_float()
    hit = L.kf_oracle_intersect(*[C.byref(x) for x in a], tmin, tmax, C.byref(t), C.byref(u), C.byref(v))
    return bool(hit), t.value, u.value, v.value


def test_watertight_shared_edge_and_vertex():
    """A ray through a shared edge or vertex of a fan hits at least one triangle (Woop et al. 2013)."""
    # quad split along its diagonal (0,0)-(1,1) in the z = 0 plane
    v = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0)]
    tris = [(v[0], v[1], v[2]), (v[0], v[2], v[3])]
    rng = np.random.default_rng(3)
    for _ in range(2000):
        s = f32(rng.uniform(0, 1))
        o = (s, s, 5.0)           # exactly on the diagonal edge
        d = (0.0, 0.0, -1.0)
        hits = [_isect(o, d, *tr)[0] for tr in tris]
        assert any(hits)
    # slanted rays through the shared edge
    for _ in range(2000):
        s = rng.uniform(0.01, 0.99)
        dx, dy = rng.uniform(-0.3, 0.3, 2)
        o = (f32(s + 3 * dx), f32(s + 3 * dy), 3.0)
        d = (f32(-dx), f32(-dy), -1.0)
        hits = [_isect(o, d, *tr)[0] for tr in tris]
        t = [_isect(o, d, *tr) for tr in tris]
        if not any(hits):
            # the ray may miss the edge by rounding of its own origin: then it must also miss the quad interior
            p = np.array(o, np.float64) + 3.0 * np.array(d, np.float64)
            assert not (0.001 < p[0] < 0.999 and 0.001 < p[1] < 0.999 and abs(p[0] - p[1]) > 1e-5)
    # vertex of a 6-triangle fan
    c = (0.0, 0.0, 0.0)
    ring = [(math.cos(k * math.pi / 3), math.sin(k * math.pi / 3), 0.0) for k in range(6)]
    fan = [(c, ring[k], ring[(k + 1) % 6]) for k in range(6)]
    assert any(_isect((0.0, 0.0, 1.0), (0.0, 0.0, -1.0), *tr)[0] for tr in fan)


def test_intersection_barycentrics_and_facing_independence():
    ok, t, u, v = _isect((0.25, 0.25, 2.0), (0, 0, -1), (0, 0, 0), (1, 0, 0), (0, 1, 0))
    assert ok and t == pytest.approx(2.0) and u == pytest.approx(0.25) and v == pytest.approx(0.25)
    # same triangle, reversed winding: still hit (culling disabled), barycentrics swap
    ok2, t2, u2, v2 = _isect((0.25, 0.25, 2.0), (0, 0, -1), (0, 0, 0), (0, 1, 0), (1, 0, 0))
    assert ok2 and t2 == pytest.approx(2.0) and u2 == pytest.approx(0.25)
    # tmin / tmax are honoured
    assert not _isect((0.25, 0.25, 2.0), (0, 0, -1), (0, 0, 0), (1, 0, 0), (0, 1, 0), 0.0, 1.5)[0]
    assert not _isect((0.25, 0.25, 2.0), (0, 0, -1), (0, 0, 0), (1, 0, 0), (0, 1, 0), 2.5, 10.0)[0]


def test_srgb_encode_matches_formula():
    L = O.load()
    xs = np.concatenate([np.linspace(0, 1, 5001), [-1.0, 0.0, 1e-9, 0.5, 1.0, 2.0]]).astype(np.float32)
    for x in xs:
        xd = float(x)
        ref = 0 if xd <= 0 else 255 if xd >= 1 else int(
            math.floor(255 * (12.92 * xd if xd <= 0.0031308 else 1.055 * xd ** (1 / 2.4) - 0.055) + 0.5))
        got = L.kf_oracle_srgb8(xd)
        assert abs(got - ref) <= 1
        if abs(255 * (12.92 * xd if xd <= 0.0031308 else 1.055 * xd ** (1 / 2.4) - 0.055) % 1 - 0.5) > 1e-3:
            assert got == ref


def test_golden_shader_vectors():
    """Outputs of kuafu's own GLSL helpers (Random.glsl / Sampling.glsl compiled as C++, the
    same operations in the same order): the oracle must reproduce every one exactly. JSON
    holds each float32 result with 9 significant digits, which round-trips to the float."""
    path = GOLDEN / "shader_vectors.json"
    if not path.exists():
        pytest.fail("tests/golden/shader_vectors.json is missing: run tests/golden/make_shader_vectors.py")
    import ctypes as C

    L = O.load()
    g = json.loads(path.read_text())
    F = np.float32
    v3 = lambda out: [F(x) for x in out[:]]
    want3 = lambda xs: [F(x) for x in xs]
    for case in g["tea"]:
        assert L.kf_oracle_tea(case["v0"], case["v1"]) == case["out"]
    for case in g["schlick"]:
        assert F(L.kf_oracle_schlick(case["cos"], case["ior"])) == F(case["out"])
    for case in g["ggx_d"]:
        assert F(L.kf_oracle_ggx_d(case["ndoth"], case["a2"])) == F(case["out"])
    for case in g["g1"]:
        assert F(L.kf_oracle_g1(case["d"], case["a2"])) == F(case["out"])
    for case in g["sample_ggx"]:
        nn = (C.c_float * 3)(*case["n"])
        out = (C.c_float * 3)()
        L.kf_oracle_sample_ggx(case["u0"], case["u1"], case["a2"], C.byref(nn), C.byref(out))
        assert v3(out) == want3(case["out"])
    for case in g["cosine"]:
        nn = (C.c_float * 3)(*case["n"])
        out = (C.c_float * 3)()
        L.kf_oracle_cosine_hemisphere(case["u0"], case["u1"], C.byref(nn), C.byref(out))
        assert v3(out) == want3(case["out"])
    for case in g["schlick_fresnel"]:
        f0 = (C.c_float * 3)(*case["f0"])
        out = (C.c_float * 3)()
        L.kf_oracle_schlick_fresnel(C.byref(f0), case["ldoth"], C.byref(out))
        assert v3(out) == want3(case["out"])
    for case in g["perpendicular"]:
        u = (C.c_float * 3)(*case["u"])
        out = (C.c_float * 3)()
        L.kf_oracle_perpendicular(C.byref(u), C.byref(out))
        assert v3(out) == want3(case["out"])
    for case in g["uniform_sphere"]:
        st = C.c_uint32(case["state"])
        out = (C.c_float * 3)()
        L.kf_oracle_uniform_sphere_lcg(C.byref(st), C.byref(out))
        assert v3(out) == want3(case["out"]) and st.value == case["state_after"]
    for case in g["disk"]:
        st = C.c_uint32(case["state"])
        out = (C.c_float * 2)()
        L.kf_oracle_disk_lcg(C.byref(st), C.byref(out))
        assert [F(x) for x in out[:]] == want3(case["out"]) and st.value == case["state_after"]
    for case in g["lcg"]:
        st = C.c_uint32(case["state"])
        got = L.kf_oracle_rnd_lcg(C.byref(st))  # one lcg step, as rnd
        assert F(got) == F((case["lcg"] & 0xFFFFFF) / float(1 << 24))
        assert F(L.kf_oracle_rnd_lcg(C.byref(st))) == F(case["rnd"]) and st.value == case["state_after"]
