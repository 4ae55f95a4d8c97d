"""Scene files in the reference's XML format (src/Scene.cpp:131-303) with OBJ meshes: the loaded
arrays against values computed here (model matrices as src/Model.cpp:11-21, light radiance as
power over world-space area, material overrides, MTL colours, triangulation, generated
normals), error reporting, and a GPU render of a loaded scene against the oracle."""
import numpy as np
import pytest

import grisrt as G

CUBE_OBJ = """# unit cube, two materials, no normals
mtllib cube.mtl
v -0.5 -0.5 -0.5
v 0.5 -0.5 -0.5
v 0.5 0.5 -0.5
v -0.5 0.5 -0.5
v -0.5 -0.5 0.5
v 0.5 -0.5 0.5
v 0.5 0.5 0.5
v -0.5 0.5 0.5
vt 0 0
vt 1 0
vt 1 1
vt 0 1
usemtl red
f 1/1 4/4 3/3 2/2
f 5/1 6/2 7/3 8/4
f 1/1 2/2 6/3 5/4
usemtl white
f 2 3 7 6
f 3 4 8 7
f 4 1 5 8
"""
CUBE_MTL = """newmtl red
Kd 0.8 0.1 0.1
newmtl white
Kd 0.7 0.7 0.7
"""
ROOM_OBJ = """v -2 -2 0
v 2 -2 0
v 2 2 0
v -2 2 0
vn 0 0 1
f 1//1 2//1 3//1 4//1
"""
LIGHT_OBJ = """v -0.5 -0.5 0
v 0.5 -0.5 0
v 0.5 0.5 0
v -0.5 0.5 0
f 1 2 3 4
"""
SCENE_XML = """<?xml version="1.0" encoding="utf-8"?>
<!-- a test scene -->
<scene version="0.1">
  <integrator type="restir">
    <size width="40" height="30"/>
  </integrator>
  <camera type="pinhole">
    <position value="0 -6 2"/>
    <lookAt value="0 0 0.5"/>
    <fov value="50"/>
  </camera>
  <modelInstances>
    <modelInstance name="cube" path="meshes/cube.obj">
      <transform translate="0.3 0.2 0.5" scale="1 1.5 0.5" rotate="30 -90 10"/>
      <material type="metalWorkflow">
        <metallic value="1"/>
        <roughness value="0.3"/>
        <baseColor value="0.9 0.8 0.2"/>
      </material>
    </modelInstance>
    <modelInstance name="cube2" path="meshes/cube.obj">
      <transform translate="-1 0.5 0.5" scale="0.6 0.6 0.6" rotate="0 -90 0"/>
      <material type="default"/>
    </modelInstance>
    <modelInstance name="floor" path="meshes/room.obj">
      <transform translate="0 0 0" scale="1 1 1" rotate="0 -90 0"/>
      <material type="lambertian">
        <baseColor value="0.5 0.5 0.5"/>
      </material>
    </modelInstance>
    <modelInstance type="light" path="meshes/light.obj" flip="true">
      <transform translate="0 0 3" scale="1 1 1" rotate="0 -90 0"/>
      <radiance value="12 10 8"/>
    </modelInstance>
  </modelInstances>
</scene>
"""


def _write_scene(tmp_path, xml=SCENE_XML):
    (tmp_path / "meshes").mkdir(exist_ok=True)
    (tmp_path / "meshes" / "cube.obj").write_text(CUBE_OBJ)
    (tmp_path / "meshes" / "cube.mtl").write_text(CUBE_MTL)
    (tmp_path / "meshes" / "room.obj").write_text(ROOM_OBJ)
    (tmp_path / "meshes" / "light.obj").write_text(LIGHT_OBJ)
    p = tmp_path / "scene.xml"
    p.write_text(xml)
    return str(p)


def _rot(deg, axis):
    a = np.radians(deg)
    c, s = np.cos(a), np.sin(a)
    r = np.eye(4)
    i, j = (axis + 1) % 3, (axis + 2) % 3
    r[i, i], r[i, j], r[j, i], r[j, j] = c, -s, s, c
    return r


def _model(pos, scale, rot):
    t = np.eye(4)
    t[:3, 3] = pos
    s = np.diag([scale[0], scale[2], scale[1], 1.0])
    return t @ _rot(rot[0], 2) @ _rot(rot[1] + 90, 0) @ _rot(rot[2], 1) @ s


def test_scene_file_arrays(tmp_path):
    hs = G.HostScene.load(_write_scene(tmp_path))
    assert hs.film_size() == (40, 30)
    # 3 object instances; the cube's 6 quads -> 12 triangles, the floor quad -> 2
    assert len(hs.instances) == 3
    assert [int(i["indexCount"]) // 3 for i in hs.instances] == [12, 12, 2]
    assert len(hs.lights) == 2
    # model matrices (column-major in the arrays)
    for inst, (pos, scale, rot) in zip(hs.instances, [((0.3, 0.2, 0.5), (1, 1.5, 0.5), (30, -90, 10)),
                                                      ((-1, 0.5, 0.5), (0.6, 0.6, 0.6), (0, -90, 0)),
                                                      ((0, 0, 0), (1, 1, 1), (0, -90, 0))]):
        M = inst["transform"].reshape(4, 4).T
        assert np.allclose(M, _model(pos, scale, rot), atol=2e-6)
        Minv = inst["transformInv"].reshape(4, 4).T
        assert np.allclose(Minv @ M, np.eye(4), atol=1e-5)
    # light: radiance = power / world area (1 x 1 quad), normal flipped from +z to -z
    L = hs.lights
    assert np.allclose(L["area"].sum(), 1.0, atol=1e-6)
    assert np.allclose(L["radiance"], np.array([12, 10, 8]) / L["area"].sum(), rtol=1e-6)
    assert np.allclose(L["nz"], -1.0)
    assert np.allclose(L["v0"][:, 2], 3.0)
    # materials: [0] default magenta, cube overridden (metalWorkflow), cube2 from the MTL file, floor lambertian
    mats = hs.materials
    assert np.allclose(mats["baseColor"][0], [1, 0, 1])
    mi = hs.material_indices
    cube = mats[mi[0:12]]
    assert np.all(cube["type"] == 2) and np.allclose(cube["metallic"], 1.0) and np.allclose(cube["roughness"], 0.3)
    assert np.allclose(cube["baseColor"], [0.9, 0.8, 0.2])
    cube2 = mats[mi[12:24]]
    assert np.all(cube2["type"] == 1)
    assert np.allclose(cube2["baseColor"][:6], [0.8, 0.1, 0.1]) and np.allclose(cube2["baseColor"][6:], [0.7, 0.7, 0.7])
    floor = mats[mi[24:26]]
    assert np.all(floor["type"] == 1) and np.allclose(floor["baseColor"], [0.5, 0.5, 0.5])
    # generated smooth normals of the cube: per material group (18 corners each), the normalised
    # mean of the unit face normals at each position
    v = hs.vertices
    cube_v = v[:36]
    n = cube_v["norm"].astype(np.float64)
    assert np.allclose(np.linalg.norm(n, axis=1), 1.0, atol=1e-6)
    p = cube_v["pos"].astype(np.float64)
    for g in (slice(0, 18), slice(18, 36)):
        pg, ng = p[g], n[g]
        tri = pg.reshape(-1, 3, 3)
        fn = np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0])
        fn /= np.linalg.norm(fn, axis=1, keepdims=True)
        fn = np.repeat(fn, 3, axis=0)
        for k in range(len(pg)):
            same = np.all(pg == pg[k], axis=1)
            m = fn[same].sum(axis=0)
            assert np.allclose(ng[k], m / np.linalg.norm(m), atol=1e-6)
            assert np.dot(ng[k], np.sign(pg[k])) > 0.5   # outward
    # texture v flipped
    assert set(np.round(cube_v["uvy"], 6)) <= {0.0, 1.0}
    # the file's normals are kept
    assert np.allclose(v[72:]["norm"], [0, 0, 1])
    # camera from position + lookAt
    cam = hs.camera(0, 1, 40, 30)
    assert np.allclose(np.array(cam.pos)[:3], [0, -6, 2])


def test_scene_file_errors(tmp_path):
    with pytest.raises(G.GrisError, match="cannot read"):
        G.HostScene.load(str(tmp_path / "missing.xml"))
    bad = _write_scene(tmp_path, SCENE_XML.replace("</scene>", ""))
    with pytest.raises(G.GrisError, match="unterminated"):
        G.HostScene.load(bad)
    tex = _write_scene(tmp_path, SCENE_XML.replace('<baseColor value="0.9 0.8 0.2"/>', '<baseColor image="a.png"/>'))
    with pytest.raises(G.GrisError, match="textures"):
        G.HostScene.load(tex)
    nolight = _write_scene(tmp_path, SCENE_XML.replace('type="light" ', ''))
    with pytest.raises(G.GrisError, match="no light"):
        G.HostScene.load(nolight)


@pytest.mark.gpu
def test_scene_file_renders_like_the_oracle(tmp_path):
    from oracle import pyoracle as O
    hs = G.HostScene.load(_write_scene(tmp_path))
    W, H = hs.film_size()
    cams, prevs = G.sequence_cameras(hs, 3, W, H, seed=3)
    st = G.Settings.make(maxDepth=5, spatialRadius=10.0)
    ora = O.oracle()
    ora.set_scene(hs)
    want = O.run_sequence(ora, cams, prevs, st, W, H, record=("resv", "out"))
    ctx = G.Context(0)
    scene = G.Scene(ctx, hs)
    fr = G.Frame(ctx, W, H)
    for f in range(3):
        fr.render(scene, cams[f], prevs[f], st)
        assert fr.download(G.BUF_RESERVOIR).tobytes() == want[f]["resv"].tobytes()
        assert fr.download(G.BUF_OUTPUT).tobytes() == want[f]["out"].tobytes()
    out = want[-1]["out"][:, :3]
    assert out.max() > 0.0
    fr.close()
    scene.close()
    ctx.close()
