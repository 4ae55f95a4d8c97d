"""Seeded workload definitions (batched views) and the oracle's resident scene slots."""
import numpy as np
import pytest

import grisrt as G
from grisrt import workloads
from oracle import pyoracle as O


def test_batched_views_are_seeded_and_in_range():
    a = workloads.batched_views(64, seed=7)
    b = workloads.batched_views(64, seed=7)
    assert a == b
    assert len(a) == 64
    assert {v["width"] for v in a} <= set(workloads.RESOLUTIONS)
    assert all(v["width"] == v["height"] for v in a)
    assert all(2 <= v["maxDepth"] <= 10 for v in a)
    assert {v["kind"] for v in a} == {1, 3}
    assert workloads.batched_views(64, seed=8) != a


def test_batched_view_scenes_hit_their_triangle_range():
    for v in workloads.batched_views(12, seed=3):
        hs = G.HostScene(v["kind"], seed=v["seed"], grid=v["grid"], spheres=v["spheres"])
        t = hs.triangle_count()
        assert 0.8 * 10_000 <= t <= 1.1 * 200_000, (v, t)
        assert abs(t - v["target_tris"]) <= 0.2 * v["target_tris"] + 400


def test_box_with_spheres_scene():
    hs = G.HostScene(3, seed=5, spheres=40)
    assert hs.triangle_count() == 12 * 2 + 40 * 320 + 2   # room + block + spheres + light
    assert len(hs.instances) == 2 + 40
    # every sphere sits inside the room
    t = hs.instances["transform"].reshape(-1, 4, 4)[2:]
    assert np.all(np.abs(t[:, :3, 3]) < 1.0)


def test_oracle_scene_slots_keep_scenes_resident():
    ora = O.oracle()
    ora.set_traversal(True)
    scenes = [G.HostScene(0, seed=4), G.HostScene(3, seed=6, spheres=10)]
    W, H = 16, 12
    runs = []
    for i, hs in enumerate(scenes):
        ora.select_scene(i)
        ora.set_scene(hs)
    st = G.Settings.make(maxDepth=3)
    for i, hs in enumerate(scenes):
        cams, prevs = G.sequence_cameras(hs, 1, W, H, seed=2)
        runs.append((cams, prevs))
    got = []
    for i in (0, 1, 0):
        ora.select_scene(i)
        got.append(O.run_sequence(ora, runs[i][0], runs[i][1], st, W, H, record=("resv", "out"))[0])
    assert got[0]["resv"].tobytes() == got[2]["resv"].tobytes()
    assert got[0]["out"].tobytes() == got[2]["out"].tobytes()
    # a fresh single-scene oracle agrees with the slot
    ora.select_scene(7)
    ora.set_scene(scenes[1])
    ref = O.run_sequence(ora, runs[1][0], runs[1][1], st, W, H, record=("resv",))[0]
    assert ref["resv"].tobytes() == got[1]["resv"].tobytes()
    ora.select_scene(0)


@pytest.mark.parametrize("kind,grid,spheres", [(0, 0, 0), (1, 48, 30), (2, 40, 20)])
def test_oracle_side_generator_builds_the_same_inputs(kind, grid, spheres):
    """The benchmark's CPU reference arm builds its inputs with oracle/_build/libscenegen.so (the
    same generator compiled on the oracle side, so that arm loads no part of libgrisrt): every scene
    array and every camera of a sequence are byte-identical to libgrisrt's."""
    from oracle import build_oracle
    lib = G.scene_library(build_oracle.build_scenegen())
    a = G.HostScene(kind, seed=5, grid=grid, spheres=spheres)
    b = G.HostScene(kind, seed=5, grid=grid, spheres=spheres, lib=lib)
    for x, y in zip(a.arrays(), b.arrays()):
        assert x.tobytes() == y.tobytes()
    ca, pa = G.sequence_cameras(a, 5, 64, 48, seed=3, orbit_frames=60)
    cb, pb = G.sequence_cameras(b, 5, 64, 48, seed=3, orbit_frames=60)
    for u, v in zip(ca + pa, cb + pb):
        assert bytes(memoryview(u)) == bytes(memoryview(v))
