"""Batches (grisBatch*): many views with their own scene, size, depth and reuse settings rendered
with one launch per pass, by the megakernel and by the wavefront path tracer (per-bounce
compacted queues). Every buffer of every view must equal the oracle's, bit for bit."""
import numpy as np
import pytest

import grisrt as G
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu

VIEWS = [   # kind, grid, spheres, W, H, settings
    (0, 0, 0, 40, 32, dict(maxDepth=3, spatialRadius=30.0)),
    (1, 40, 30, 64, 48, dict(maxDepth=8)),
    (2, 32, 24, 24, 24, dict(maxDepth=10, rrScale=0.5)),
    (0, 0, 0, 16, 16, dict(maxDepth=2, temporalReuse=False)),
    (1, 24, 10, 33, 17, dict(maxDepth=5, spatialNeighbors=5, cap=7)),
    (2, 40, 40, 48, 40, dict(maxDepth=6, shiftType=0)),
]
FRAMES = 3


@pytest.fixture(scope="module")
def setup():
    ctx = G.Context(0)
    hss = [G.HostScene(k, seed=10 + i, grid=g, spheres=sp) for i, (k, g, sp, W, H, kw) in enumerate(VIEWS)]
    scenes = [G.Scene(ctx, hs) for hs in hss]
    seqs = [G.sequence_cameras(hs, FRAMES, W, H, seed=30 + i) for i, (hs, (k, g, sp, W, H, kw)) in enumerate(zip(hss, VIEWS))]
    settings = [G.Settings.make(**kw) for (k, g, sp, W, H, kw) in VIEWS]
    ora = O.oracle()
    want = []
    for i, (k, g, sp, W, H, kw) in enumerate(VIEWS):
        ora.set_scene(hss[i])
        want.append(O.run_sequence(ora, seqs[i][0], seqs[i][1], settings[i], W, H))
    yield ctx, hss, scenes, seqs, settings, want
    for sc in scenes:
        sc.close()
    ctx.close()


@pytest.mark.parametrize("form,graphs,wave,refill", [
    (G.PATH_WAVEFRONT, True, (16, 8), False), (G.PATH_WAVEFRONT, False, (16, 8), False),
    (G.PATH_WAVEFRONT, True, (8, 4), False), (G.PATH_WAVEFRONT, True, (32, 16), False),
    (G.PATH_WAVEFRONT, True, (8, 16), True), (G.PATH_WAVEFRONT, False, (2, 8), True),
    (G.PATH_MEGAKERNEL, True, (16, 8), False), (G.PATH_MEGAKERNEL, False, (16, 8), False)],
    ids=["wavefront-graph", "wavefront-eager", "wavefront-small-grids", "wavefront-large-grids", "wavefront-refill",
         "wavefront-refill-eager-tiny-grid", "megakernel-graph", "megakernel-eager"])
def test_batch_views_match_oracle(setup, form, graphs, wave, refill):
    ctx, hss, scenes, seqs, settings, want = setup
    ctx.set_path_form(form)
    ctx.set_graphs(graphs)
    ctx.set_wave_launch(*wave)
    ctx.set_wave_refill(refill)
    batch = G.Batch(ctx, scenes, [(W, H) for (k, g, sp, W, H, kw) in VIEWS])
    ctx.counters(reset=True)
    keys = {"resv": G.BUF_RESERVOIR, "temp": G.BUF_TEMP, "out": G.BUF_OUTPUT, "dn": G.BUF_DEPTH_NORMAL,
            "am": G.BUF_ALBEDO_MATID, "mv": G.BUF_MOTION}
    for f in range(FRAMES):
        batch.render([seqs[v][0][f] for v in range(len(VIEWS))], [seqs[v][1][f] for v in range(len(VIEWS))], settings)
        for v in range(len(VIEWS)):
            for k, which in keys.items():
                got = batch.download(v, which)
                w = want[v][f][k]
                assert got.tobytes() == w.tobytes(), "form %d frame %d view %d buffer %s differs" % (form, f, v, k)
    ctx.sync()
    assert ctx.counters()[3] == 0
    batch.close()
    ctx.set_path_form(G.PATH_WAVEFRONT)
    ctx.set_graphs(True)
    ctx.set_wave_launch(16, 8)
    ctx.set_wave_refill(False)


def test_autotune_picks_a_candidate_and_results_stay_exact(setup):
    """The autotuner renders frames with every candidate configuration and keeps the fastest;
    a fresh batch rendered with the chosen configuration still matches the oracle."""
    ctx, hss, scenes, seqs, settings, want = setup
    sizes = [(W, H) for (k, g, sp, W, H, kw) in VIEWS]
    n = len(VIEWS)
    tb = G.Batch(ctx, scenes, sizes)
    r = tb.autotune([seqs[v][0][1] for v in range(n)], [seqs[v][1][1] for v in range(n)], settings, frames=2)
    tb.close()
    assert r.candidates == 13
    ms = list(r.candidateMs)[:r.candidates]
    assert all(m > 0 for m in ms)
    assert r.msPerFrame == min(ms)
    assert r.pathForm in (G.PATH_MEGAKERNEL, G.PATH_WAVEFRONT)
    batch = G.Batch(ctx, scenes, sizes)
    for f in range(FRAMES):
        batch.render([seqs[v][0][f] for v in range(n)], [seqs[v][1][f] for v in range(n)], settings)
        for v in range(n):
            assert batch.download(v, G.BUF_RESERVOIR).tobytes() == want[v][f]["resv"].tobytes()
            assert batch.download(v, G.BUF_OUTPUT).tobytes() == want[v][f]["out"].tobytes()
    batch.close()
    ctx.set_path_form(G.PATH_WAVEFRONT)
    ctx.set_wave_launch(16, 8)
    ctx.set_wave_refill(False)


def test_single_view_batch_equals_frame_api(setup):
    ctx, hss, scenes, seqs, settings, want = setup
    k, g, sp, W, H, kw = VIEWS[1]
    batch = G.Batch(ctx, [scenes[1]], [(W, H)])
    fr = G.Frame(ctx, W, H)
    for f in range(FRAMES):
        batch.render([seqs[1][0][f]], [seqs[1][1][f]], [settings[1]])
        fr.render(scenes[1], seqs[1][0][f], seqs[1][1][f], settings[1])
        assert batch.download(0, G.BUF_RESERVOIR).tobytes() == fr.download(G.BUF_RESERVOIR).tobytes()
        assert batch.download(0, G.BUF_OUTPUT).tobytes() == fr.download(G.BUF_OUTPUT).tobytes()
    fr.close()
    batch.close()


def test_batched_workload_views_match_oracle():
    """Views drawn by the batched-views workload generator (box-with-spheres and terrain scenes of
    10k-200k triangles, uneven depths), at small resolutions, through graphs and the wavefront."""
    from grisrt import workloads
    specs = workloads.batched_views(5, seed=11, resolutions=(16, 24, 40))
    ctx = G.Context(0)
    ctx.set_path_form(G.PATH_WAVEFRONT)
    hss = [G.HostScene(s["kind"], seed=s["seed"], grid=s["grid"], spheres=s["spheres"]) for s in specs]
    assert {s["kind"] for s in specs} == {1, 3}
    scenes = [G.Scene(ctx, hs) for hs in hss]
    sets = [G.Settings.make(maxDepth=s["maxDepth"], spatialRadius=20.0) for s in specs]
    seqs = [G.sequence_cameras(hs, 2, s["width"], s["height"], seed=60 + i) for i, (hs, s) in enumerate(zip(hss, specs))]
    ora = O.oracle()
    batch = G.Batch(ctx, scenes, [(s["width"], s["height"]) for s in specs])
    want = []
    for i, s in enumerate(specs):
        ora.set_scene(hss[i])
        want.append(O.run_sequence(ora, seqs[i][0], seqs[i][1], sets[i], s["width"], s["height"], record=("resv", "out")))
    for f in range(2):
        batch.render([q[0][f] for q in seqs], [q[1][f] for q in seqs], sets)
        for v in range(len(specs)):
            assert batch.download(v, G.BUF_RESERVOIR).tobytes() == want[v][f]["resv"].tobytes(), (f, v)
            assert batch.download(v, G.BUF_OUTPUT).tobytes() == want[v][f]["out"].tobytes(), (f, v)
    batch.close()
    for sc in scenes:
        sc.close()
    ctx.close()


def test_batch_graph_follows_the_mis_weights_setting():
    """One batch (graphs on) renders a sequence with the reference merge and then one with the
    pairwise weights: the second must not replay the first's captured graph. Closed box: every
    pixel has geometry, so no buffer keeps data from the first sequence."""
    ctx = G.Context(0)
    ctx.set_graphs(True)
    hs = G.HostScene(0, seed=7)
    scene = G.Scene(ctx, hs)
    W, H = 32, 24
    batch = G.Batch(ctx, [scene], [(W, H)])
    ora = O.oracle()
    ora.set_scene(hs)
    for seed, mis in ((3, 0), (4, 1), (5, 0)):
        cams, prevs = G.sequence_cameras(hs, 3, W, H, seed=seed)
        st = G.Settings.make(maxDepth=4, misWeights=mis)
        want = O.run_sequence(ora, cams, prevs, st, W, H, record=("resv", "out"))
        for f in range(3):
            batch.render([cams[f]], [prevs[f]], [st])
            assert batch.download(0, G.BUF_RESERVOIR).tobytes() == want[f]["resv"].tobytes(), (mis, f)
            assert batch.download(0, G.BUF_OUTPUT).tobytes() == want[f]["out"].tobytes(), (mis, f)
    batch.close()
    scene.close()
    ctx.close()


@pytest.mark.parametrize("guided", [False, True], ids=["plain", "guided"])
def test_overlapped_frame_equals_the_frame_in_order(guided):
    """A wavefront frame forks onto side streams (a bounce's closest hits beside the previous
    bounce's shadow queries and post(); the temporal pass's shifts and visibility walk beside the
    path tracer; the spatial pass in two halves of the batch's tiles, from 2,048 tiles). With the
    kernel timer on everything runs in order on one stream. Both must give the same buffers bit
    for bit, through captured graphs and eager launches, on frames whose bounce levels are full
    (the resident walks) with temporal history, and raise no error bit (bit 3: post() disagreeing
    with the next ray queued ahead of it). Two views of 1,425 and 1,024 tiles: the halves meet
    inside the first view."""
    hs = G.HostScene(2, seed=21, grid=48, spheres=60)
    sizes = [(400, 450), (512, 256)]
    seq = [G.sequence_cameras(hs, 4, W, H, seed=5 + i) for i, (W, H) in enumerate(sizes)]
    st = G.Settings.make(maxDepth=8, spatialRadius=20.0)
    keys = {"resv": G.BUF_RESERVOIR, "temp": G.BUF_TEMP, "out": G.BUF_OUTPUT}
    runs = []
    for graphs, profiling in ((True, False), (False, False), (False, True)):
        ctx = G.Context(0)
        ctx.set_path_form(G.PATH_WAVEFRONT)
        ctx.set_wave_refill(True)
        ctx.set_graphs(graphs)
        ctx.set_profiling(profiling)
        scene = G.Scene(ctx, hs)
        batch = G.Batch(ctx, [scene, scene], sizes)
        guide = None
        if guided:   # untrained (training folds gradients with float atomics: not bit-reproducible)
            guide = G.Guide(ctx, G.GuideConfig.make(seed=3, train=False))
            batch.set_guide(guide)
        ctx.counters(reset=True)
        got = []
        for f in range(4):
            batch.render([s[0][f] for s in seq], [s[1][f] for s in seq], [st, st])
            got.append({(v, k): batch.download(v, b).tobytes() for v in range(2) for k, b in keys.items()})
        ctx.sync()
        assert ctx.counters()[3] == 0
        runs.append(got)
        batch.close()
        if guide is not None:
            guide.close()
        scene.close()
        ctx.close()
    for f in range(4):
        for k in runs[0][f]:
            assert runs[0][f][k] == runs[2][f][k], ("graphs vs in order", f, k)
            assert runs[1][f][k] == runs[2][f][k], ("eager vs in order", f, k)


def test_pipelined_downloads_equal_the_waiting_ones():
    """grisFrameDownloadAsync / grisBatchDownloadAsync: each frame's buffers staged after the frame
    and copied to the host beside the next one equal what the waiting download reads after that
    frame, for a frame and for a two-view batch, with several downloads queued between waits (the
    staging area reused from its start and grown) and the next frames queued behind them."""
    torch = pytest.importorskip("torch")
    hs = G.HostScene(1, seed=3, grid=24, spheres=12)
    W, H = 160, 120
    cams, prevs = G.sequence_cameras(hs, 4, W, H, seed=9)
    st = G.Settings.make(maxDepth=4, spatialRadius=20.0)
    ctx = G.Context(0)
    scene = G.Scene(ctx, hs)
    keys = (G.BUF_OUTPUT, G.BUF_RESERVOIR)
    # frame API: per frame the output (307 KB) and the reservoirs (1.8 MB) into pinned buffers,
    # two frames' copies queued between waits (the 2-MB staging area is reused from its start)
    frame = G.Frame(ctx, W, H)
    want = []
    for f in range(4):
        frame.render(scene, cams[f], prevs[f], st)
        want.append([frame.download(k).tobytes() for k in keys])
    frame.close()
    frame = G.Frame(ctx, W, H)
    hosts = []
    for f in range(4):
        frame.render(scene, cams[f], prevs[f], st)
        if f > 0 and f % 2 == 0:
            ctx.download_wait()
        bufs = []
        for k in keys:
            n = len(want[f][keys.index(k)])
            b = torch.zeros(n, dtype=torch.uint8, pin_memory=True)
            frame.download_async(k, (b.data_ptr(), n))
            bufs.append(b)
        hosts.append(bufs)
    ctx.download_wait()
    for f in range(4):
        assert [b.numpy().tobytes() for b in hosts[f]] == want[f], ("frame", f)
    frame.close()
    # batch API: two views, their downloads of a frame queued before the next frame; the second
    # view's reservoirs (3.9 MB) make the staging area grow once the copies in flight are done
    sizes = [(W, H), (256, 160)]
    seqs = [G.sequence_cameras(hs, 3, w, h, seed=11 + i) for i, (w, h) in enumerate(sizes)]
    runs = []
    for pipelined in (False, True):
        batch = G.Batch(ctx, [scene, scene], sizes)
        got = []
        for f in range(3):
            batch.render([s[0][f] for s in seqs], [s[1][f] for s in seqs], [st, st])
            if pipelined:
                bufs = []
                for v, (w, h) in enumerate(sizes):
                    for k, per in ((G.BUF_OUTPUT, 16), (G.BUF_RESERVOIR, 96)):
                        b = torch.zeros(w * h * per, dtype=torch.uint8, pin_memory=True)
                        batch.download_async(v, k, (b.data_ptr(), w * h * per))
                        bufs.append(b)
                got.append(bufs)
            else:
                got.append([batch.download(v, k).tobytes() for v in range(2) for k in keys])
        # every view's output at once (GRIS_BATCH_ALL_VIEWS), pipelined and waiting
        total = sum(w * h for (w, h) in sizes) * 16
        allv = torch.zeros(total, dtype=torch.uint8, pin_memory=True)
        batch.download_async(G.BATCH_ALL_VIEWS, G.BUF_OUTPUT, (allv.data_ptr(), total))
        ctx.download_wait()
        ctx.sync()
        assert allv.numpy().tobytes() == batch.download(G.BATCH_ALL_VIEWS, G.BUF_OUTPUT).tobytes()
        assert allv.numpy().tobytes() == b"".join(batch.download(v, G.BUF_OUTPUT).tobytes() for v in range(2))
        if pipelined:
            got = [[b.numpy().tobytes() for b in bufs] for bufs in got]
        runs.append(got)
        batch.close()
    assert runs[0] == runs[1]
    scene.close()
    ctx.close()
