"""The oracle's pairwise MIS weights (GrisSettings.misWeights = 1, an extension of the reference's
merge): well-formed reservoirs (finite, non-negative weights, M within the cap), the same G-buffer
and candidate pass as the reference merge, different reuse results; and on the Lambertian box a
single spatial pass keeps the image energy of the canonical samples (the weights are unbiased)."""
import numpy as np

import grisrt as G
from oracle import pyoracle as O


def test_pairwise_oracle_reservoirs_are_well_formed():
    ora = O.oracle()
    hs = G.HostScene(1, seed=3, grid=32, spheres=20)
    W, H = 40, 32
    cams, prevs = G.sequence_cameras(hs, 4, W, H, seed=9)
    ora.set_scene(hs)
    ref = O.run_sequence(ora, cams, prevs, G.Settings.make(maxDepth=6), W, H)
    pw = O.run_sequence(ora, cams, prevs, G.Settings.make(maxDepth=6, misWeights=1), W, H)
    for f in range(4):
        r = pw[f]["resv"]
        assert np.all(np.isfinite(r["resampleWeight"])) and np.all(r["resampleWeight"] >= 0)
        assert r["sampleCount"].max() <= 20
        assert np.isfinite(pw[f]["out"]).all()
        assert pw[f]["dn"].tobytes() == ref[f]["dn"].tobytes()
    assert pw[-1]["resv"].tobytes() != ref[-1]["resv"].tobytes()


def test_pairwise_single_spatial_pass_keeps_energy():
    ora = O.oracle()
    hs = G.HostScene(0, seed=2)
    W, H, F = 32, 32, 24
    c0 = hs.camera(0, 1, W, H)
    import ctypes
    cams, prevs = [], []
    for f in range(F):
        c = c0.copy()
        c.seed = G.frame_seed(5, f)
        ctypes.memmove(c.lastProjView, c0.projView, 64)
        c.frameIndex = f   # accumulate
        cams.append(c)
        prevs.append(c0.copy())
    ora.set_scene(hs)
    base = O.run_sequence(ora, cams, prevs, G.Settings.make(maxDepth=3, temporalReuse=False, spatialReuse=False), W, H,
                          record=("out",))
    pw = O.run_sequence(ora, cams, prevs, G.Settings.make(maxDepth=3, temporalReuse=False, misWeights=1), W, H,
                        record=("out",))
    e0 = base[-1]["out"][:, :3].sum()
    e1 = pw[-1]["out"][:, :3].sum()
    assert e0 > 0 and abs(e1 / e0 - 1.0) < 0.05, (e0, e1)
