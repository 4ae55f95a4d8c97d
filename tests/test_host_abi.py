"""Host-side checks (no GPU): the C ABI library loads and exports what include/grisrt.h
declares; layouts; alias table vs the reference's AliasTable.h; cameras; scenes."""
import ctypes
import os
import re

import numpy as np
import pytest

import grisrt as G

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    src = open(os.path.join(REPO, "include", "grisrt.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(gris[A-Z]\w*)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(G.LIB_PATH)
    names = header_functions()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(names) == set(G.EXPORTS)


def test_layout_sizes_match_reference_std430():
    lib = G.load()
    assert [lib.grisSizeof(i) for i in range(10)] == [352, 96, 32, 32, 224, 64, 8, 64, 64, 16]
    assert G.DI_RESERVOIR.itemsize == 64 and ctypes.sizeof(G.DISettings) == 16
    assert ctypes.sizeof(G.PostSettings) == 16 and ctypes.sizeof(G.GuideConfig) == 40
    from oracle import pyoracle
    ora = pyoracle.oracle()
    assert [ora.sizeof(i) for i in range(7)] == [352, 96, 32, 32, 224, 64, 8]


def _alias_ref(dist):
    from oracle import pyoracle
    path = os.path.join(os.path.dirname(pyoracle.REF_LIB), "libaliasref.so")
    if not os.path.exists(path):
        pytest.skip("reference AliasTable.h build absent (oracle/_ref)")
    lib = ctypes.CDLL(path)
    d = np.ascontiguousarray(dist, np.float32)
    prob = np.zeros(len(d) + 1, np.float32)
    fail = np.zeros(len(d) + 1, np.uint32)
    lib.aliasref_build(ctypes.c_void_p(d.ctypes.data), ctypes.c_uint32(len(d)), ctypes.c_void_p(prob.ctypes.data),
                       ctypes.c_void_p(fail.ctypes.data))
    return prob, fail


@pytest.mark.parametrize("n,seed", [(1, 0), (2, 1), (7, 2), (64, 3), (1000, 4), (5, 5)])
def test_light_table_matches_reference_alias_table(n, seed):
    rng = np.random.default_rng(seed)
    dist = rng.uniform(0.0, 10.0, n).astype(np.float32)
    if seed == 5:
        dist[:] = 2.0   # all equal
    t = G.build_light_table(dist)
    prob, fail = _alias_ref(dist)
    assert t["prob"].tobytes() == prob.tobytes()
    assert np.array_equal(t["failId"], fail)


def test_light_table_is_a_valid_alias_table():
    rng = np.random.default_rng(9)
    dist = rng.uniform(0.1, 5.0, 33).astype(np.float64)
    t = G.build_light_table(dist.astype(np.float32))
    n = len(dist)
    assert t[0]["failId"] == n and abs(t[0]["prob"] - dist.sum()) < 1e-3
    # probability of index i under the table (r.x uniform over slots, r.y over [0,1))
    p = np.zeros(n)
    for i in range(n):
        keep = min(max(float(t[i + 1]["prob"]), 0.0), 1.0)
        p[i] += keep / n
        p[int(t[i + 1]["failId"]) - 1] += (1.0 - keep) / n
    assert np.allclose(p, dist / dist.sum(), atol=1e-5)


def test_camera_setup_orthonormal_basis():
    c = G.camera_setup([0, -0.92, 0.05], [0.0, -4.0, 0.0], 70.0, 64, 48)
    f, r, u = np.array(c.front), np.array(c.right), np.array(c.up)
    assert abs(np.dot(f, r)) < 1e-6 and abs(np.dot(f, u)) < 1e-6 and abs(np.dot(r, u)) < 1e-6
    assert np.allclose([np.linalg.norm(f), np.linalg.norm(r), np.linalg.norm(u)], 1.0, atol=1e-6)
    assert tuple(c.filmSize) == (64, 48) and c.frameIndex == 0
    # projView maps a point in front of the camera into the unit cube
    pv = np.array(c.projView, np.float64).reshape(4, 4).T
    p = np.array(c.pos) + 2.0 * f
    q = pv @ np.append(p, 1.0)
    assert abs(q[0] / q[3]) < 1e-5 and abs(q[1] / q[3]) < 1e-5 and 0 < q[2] / q[3] < 1


@pytest.mark.parametrize("kind", [0, 1, 2])
def test_host_scene_deterministic_and_well_formed(kind):
    a = G.HostScene(kind, seed=5, grid=24, spheres=16)
    b = G.HostScene(kind, seed=5, grid=24, spheres=16)
    for x, y in zip(a.arrays(), b.arrays()):
        assert x.tobytes() == y.tobytes()
    c = G.HostScene(kind, seed=6, grid=24, spheres=16)
    assert any(x.tobytes() != y.tobytes() for x, y in zip(a.arrays(), c.arrays()))
    for inst in a.instances:
        off, cnt = int(inst["indexOffset"]), int(inst["indexCount"])
        assert cnt % 3 == 0 and off + cnt <= len(a.indices) and off % 3 == 0
        assert len(a.material_indices) >= off // 3 + cnt // 3
    assert a.indices.max() < len(a.vertices)
    assert a.material_indices.max() < len(a.materials)
    assert len(a.light_table) == len(a.lights) + 1
    assert np.all(a.lights["area"] > 0)


def test_box_scene_matches_config():
    s = G.HostScene(0, seed=1)
    assert s.triangle_count() == 26   # 12 quads (24 triangles) + a 2-triangle quad light
    assert np.all(s.materials["type"] == 1)
    assert np.all((s.materials["baseColor"] >= 0.2) & (s.materials["baseColor"] <= 0.8))
    assert np.allclose(s.lights["radiance"], 15.0)
    assert abs(s.lights["area"].sum() - 4.0 / 16.0) < 1e-6


def test_terrain_scene_sizes():
    s = G.HostScene(1, seed=1, grid=512, spheres=2000)
    n = s.triangle_count()
    assert n == 2 * 511 * 511 + 2000 * 320 + 8
    m = s.materials[1:]
    assert np.all((m["roughness"] >= 0.05) & (m["roughness"] <= 1.0))
    assert set(np.unique(m["metallic"]).tolist()) <= {0.0, 1.0}


def test_f16_conversion_matches_ieee():
    from oracle import pyoracle
    ora = pyoracle.oracle()
    ora.lib.oracle_f16.restype = ctypes.c_uint16
    ora.lib.oracle_f16.argtypes = [ctypes.c_float]
    rng = np.random.default_rng(0)
    vals = np.concatenate([rng.normal(0, 0.01, 2000), rng.normal(0, 100, 500), [0.0, -0.0, 65504.0, 65520.0, 1e-8, -6e-8,
                           5.96e-8, 2.98e-8, 1e5, np.inf, -np.inf]]).astype(np.float32)
    got = np.array([ora.lib.oracle_f16(float(v)) for v in vals], np.uint16)
    want = vals.astype(np.float16).view(np.uint16)
    assert np.array_equal(got, want)
