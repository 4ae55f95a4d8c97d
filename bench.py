#!/usr/bin/env python3
"""bench.py — ReSTIR PT (GRIS) frames/s and Mrays/s on one GB300.

Workloads (--workload):
  c2  (default) 1920x1080, the ~1.16M-triangle synthetic scene (512x512 fBm heightfield + 2000
      instanced icospheres, GGX materials, 4 quad lights), max depth 8, temporal + spatial
      reuse (hybrid shift), camera orbit (60 frames per quarter turn);
  c3  64 independent views in one batch: resolutions from {64,128,256,512}^2, each with its own
      box-or-terrain scene of 10k-200k triangles, max depth uniform in [2, 10];
  c4  guided vs plain ReSTIR PT on the glossy variant (run_guided);
  di  the ReSTIR DI pass (TestReSTIR::render) on the c2 scene at 1920x1080: G-buffer, candidates,
      temporal and spatial reuse, direct output (run_di).

One step = one frame of every view: G-buffer + path trace + temporal reuse + spatial reuse /
final shading, rendered through grisBatchRender (a captured CUDA graph replayed per frame; the
launch configuration picked by grisBatchAutotune first).

  value   frames/s timed on the device with CUDA events on the library's stream, scenes and
          frame buffers resident in HBM, L2 flushed (256 MiB write) between frames outside the
          timed events;
  e2e     frames/s through the C ABI from the host: the per-frame cameras and settings come
          from host memory and every view's RGBA32F radiance is read back into pinned host
          memory each frame, wall-clock timed with the same L2 flush before every frame (on the
          library's stream, its time included); the readback is pipelined
          (grisFrameDownloadAsync / grisBatchDownloadAsync: staged on the device after the frame,
          copied to the host beside the next frame, waited for before the next readback and
          after the last frame);
  roofline  the kernel with the largest share of the frame: its algorithmic bytes per launch
          (BVH nodes x 80 B + triangles x 48 B + per-ray / per-pixel record bytes, counted on the
          same frames) over its average CUDA-event launch time (a separate profiled pass, eager
          launches), against the measured HBM copy bandwidth;
  cpu_baseline  the oracle restatement (C++, OpenMP, binary BVH) on this host's cores on a
          band of rows of every view, scaled to frames/s.

--impl reference times that CPU implementation alone (rank 0), the reference's own GLSL
path being unavailable on this machine (no graphics stack).
Multi-GPU: replicas (each rank renders the same workload; no collective in the path).
"""
import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

REPO = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(REPO, "vulkan-restir-pt_gb300")
for p in (PKG, REPO):
    if p not in sys.path:
        sys.path.insert(0, p)

METRICS = {
    "c1": "ReSTIR PT frames/s at 256x256 (box scene, 24 triangles + light, depth 3, temporal+spatial reuse)",
    "c2": "ReSTIR PT frames/s at 1080p (1.16M-tri synthetic scene, depth 8, temporal+spatial reuse)",
    "c3": "Batched ReSTIR PT frames/s (64 views of {64..512}^2, 10k-200k tris each, depth 2-10)",
    "c4": "Guided / plain ReSTIR PT time to equal relMSE (1080p glossy scene, depth 8, accumulating frames)",
    "di": "ReSTIR DI frames/s at 1080p (1.16M-tri synthetic scene, candidates + temporal + spatial reuse)",
}
UNIT = "frames/s"
NODE_BYTES, TRI_BYTES = 80, 48
SURFACE_BYTES = 264   # per closest hit shaded: 3 vertices (96) + transform and inverse-transpose (128) + offsets (8) + material (32)
WAVE_STATE = 248      # one path's wavefront record, the mean of the 240 B the plain tracer reads (15 x 16 B)
                      # and the 256 B it writes (16 x 16 B: whole 32-byte sectors)
NEE_STATE = 96        # one shadow query's record (6 x 16 B)


def alg_bytes(slot, w, px):
    """Algorithmic bytes of one frame of kernel `slot` (work `w` per frame, `px` pixels):
      gbuffer      traversal + 28 B G-buffer texel + a surface fetch per primary hit
      path_trace   (megakernel) traversal + 24 B G-buffer read + 96 B reservoir write + surface fetches
      temporal     traversal + 24+4+24 B G-buffer + 2 x 96 B reservoir reads + 96 B write + surface fetches
      spatial      traversal + 4 x 24 B G-buffer + 4 x 96 B reservoir reads + 96 B write + 32 B output r/w
                   + surface fetches
      wave_begin   24 B G-buffer read + a path record write + its 32 B next ray + a 4 B queue
                   entry per pixel
      wave_extend  per ray: 32 B ray + 16 B hit + 4 B queue entry, plus traversal
      wave_shade   per path: record read and write + 16 B hit + a surface fetch + 32 B next ray +
                   4 B queue entry; per shadow query: its 96 B record + 4 B queue entry
      wave_shadow  per shadow ray: 48 B query + 1 B verdict + 4 B queue entry, plus traversal
      wave_post    per shadow query: record read and write + query read + verdict + queue entry
    The reuse passes in three launches (prepare, visibility walk, finish; w["split"] true):
      temporal     (prepare + finish) the per-pixel figure + a 37 B merge record written and read
                   + the 96 B reservoir read again by the finish + a 32 B queue entry per query
      spatial      (prepare + finish) the per-pixel figure + 37 B written and read per neighbour
                   slot + the pixel's G-buffer and reservoir read again by the finish (120 B)
                   + a 32 B queue entry per query
      reuse_vis_*  per query: 32 B queue entry + 1 B verdict read and written, plus traversal"""
    trav = w["nodes"] * NODE_BYTES + w["tris"] * TRI_BYTES
    r = w["rays"]
    per_px = {"gbuffer": 28, "path_trace": 120, "temporal": 340, "spatial": 608, "wave_begin": 24 + WAVE_STATE + 32 + 4}
    if slot in ("temporal", "spatial") and w.get("split"):
        extra = 2 * 37 + 96 if slot == "temporal" else 2 * 37 * w["neighbours"] + 120
        return trav + (per_px[slot] + extra) * px + SURFACE_BYTES * r + 32 * w["queries"]
    if slot in ("gbuffer", "path_trace", "temporal", "spatial"):
        return trav + per_px[slot] * px + SURFACE_BYTES * r
    if slot in ("reuse_vis_temporal", "reuse_vis_spatial"):
        return trav + 34 * r
    if slot == "wave_begin":
        return per_px[slot] * px
    if slot == "wave_extend":
        return trav + 52 * r
    if slot == "wave_shade":
        return w["paths"] * (2 * WAVE_STATE + 16 + SURFACE_BYTES + 32 + 4) + w["shadow_paths"] * (NEE_STATE + 4)
    if slot == "wave_shadow":
        return trav + 53 * r
    if slot == "wave_post":
        return w["shadow_paths"] * (2 * WAVE_STATE + NEE_STATE + 1 + 4)
    return 0


def kernel_launches_per_frame(prof, slots, frames, wavefront, refill):
    """The library's kernel launches per frame from the per-slot launch counts of the profiled
    pass. With the refilling wavefront each timed extension / shadow level launches two kernels
    (the refilling walk of a full level and the one-ray-per-warp walk of a sparse level; one of
    them returns at once) inside one timed slot."""
    n = sum(prof[s]["launches"] for s in slots) / frames
    if wavefront and refill:
        n += (prof["wave_extend"]["launches"] + prof["wave_shadow"]["launches"]) / frames
    return n


def max_over_ranks(x, device):
    """The maximum of a per-rank scalar over the process group (x itself on one rank)."""
    import torch
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_rate(units_per_rank, seconds_max, world):
    """Whole-job rate of replicas: every rank processed `units_per_rank` in at most `seconds_max`."""
    return world * units_per_rank / seconds_max


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="grisrt", choices=["grisrt", "reference"])
    ap.add_argument("--workload", default="c2", choices=["c1", "c2", "c3", "c4", "di"])
    ap.add_argument("--di-shift", default="reconnection", choices=["reconnection", "replay", "hybrid"],
                    help="di: the DI pass's shift")
    ap.add_argument("--di-sample", default="both", choices=["light", "bsdf", "both"], help="di: candidate types")
    ap.add_argument("--di-temporal", default="on", choices=["on", "off"], help="di: temporal reuse")
    ap.add_argument("--ref-spp", type=int, default=1024, help="c4: samples per pixel of the converged image")
    ap.add_argument("--mis", default="reference", choices=["reference", "pairwise"],
                    help="c4: the reuse passes' MIS weights (the reference's merge, or the pairwise extension)")
    ap.add_argument("--guide-tc", default="off", choices=["on", "off"],
                    help="c4: the guide's inference on tcgen05 (tensor memory) or mma.sync")
    ap.add_argument("--guide-train", default="tcgen05", choices=["tcgen05", "mma.sync"],
                    help="c4: the kernel of the guide's loss gradient")
    ap.add_argument("--ref-cache", default=None, help="c4: path prefix of a saved converged image to reuse")
    ap.add_argument("--guide-mix", type=float, default=0.5, help="c4: probability of drawing from the guide")
    ap.add_argument("--guide-lr", type=float, default=1e-3, help="c4: Adam learning rate")
    ap.add_argument("--guide-records", type=int, default=1 << 18, help="c4: training records per frame")
    ap.add_argument("--guide-steps", type=int, default=4, help="c4: Adam steps per frame")
    ap.add_argument("--c4-reuse", default="on", choices=["on", "off"],
                    help="c4: temporal + spatial reuse on (ReSTIR PT) or off (the canonical samples alone)")
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--grid", type=int, default=512)
    ap.add_argument("--spheres", type=int, default=2000)
    ap.add_argument("--depth", type=int, default=8)
    ap.add_argument("--views", type=int, default=64, help="views of the c3 workload")
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--wave", default=None,
                    help="with --no-autotune: the wavefront launch as TRACE,SHADE[,refill] blocks per SM (e.g. 16,16,refill), "
                         "the form the autotuner picks, so that a profiler run can skip the tuning frames")
    ap.add_argument("--no-graphs", action="store_true")
    ap.add_argument("--launch-mode", default="grid", choices=["persistent", "grid"])
    ap.add_argument("--api", default="batch", choices=["batch", "frame"],
                    help="grisBatchRender or grisFrameRender (c2 only)")
    ap.add_argument("--path-form", default="wavefront", choices=["wavefront", "megakernel"],
                    help="starting form (the autotuner may switch)")
    ap.add_argument("--cpu-seconds", type=float, default=20.0, help="target CPU work of the baseline sample")
    return ap.parse_args()


def load_peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax.append(float(parts[2]))
                except ValueError:
                    continue
                for n, v in zip(names, parts[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


class View:
    def __init__(self, hs, width, height, settings, frames, seed):
        import grisrt as G
        self.hs, self.w, self.h, self.settings = hs, width, height, settings
        self.cams, self.prevs = G.sequence_cameras(hs, frames, width, height, seed=seed, orbit_frames=60)


def make_views(args, frames, scene_lib=None):
    """The workload's views with `frames` cameras each, and its config dict (the workload alone:
    both arms print the same one). scene_lib: the generator library (grisrt.scene_library) —
    the reference arm's, which loads no part of libgrisrt; default libgrisrt's own."""
    import grisrt as G
    from grisrt import workloads

    def settings(depth):
        return G.Settings.make(shiftType=2, rrScale=1.0, temporalReuse=True, spatialReuse=True, cap=20,
                               maxDepth=depth, spatialNeighbors=3, spatialRadius=20.0)
    common = {"spatial_neighbors": 3, "spatial_radius_px": 20.0, "cap": 20, "shift": "hybrid",
              "l2": "flushed between frames (256 MiB write; outside the timed events, inside the e2e wall clock)"}
    if args.workload == "c1":
        hs = G.HostScene(0, seed=args.seed, lib=scene_lib)
        st = G.Settings.make(shiftType=2, rrScale=1.0, temporalReuse=True, spatialReuse=True, cap=20, maxDepth=3,
                             spatialNeighbors=3, spatialRadius=30.0)
        views = [View(hs, 256, 256, st, frames, args.seed)]
        config = {"workload": "C1: 256x256 box (%d tris), depth 3, static camera" % hs.triangle_count(),
                  "width": 256, "height": 256, "triangles": hs.triangle_count(), "max_depth": 3}
        config.update(common)
        config["spatial_radius_px"] = 30.0
        return views, config
    if args.workload in ("c2", "c4"):
        hs = G.HostScene(2 if args.workload == "c4" else 1, seed=args.seed, grid=args.grid, spheres=args.spheres,
                         lib=scene_lib)
        views = [View(hs, args.width, args.height, settings(args.depth), frames, args.seed)]
        config = {"workload": "C2: %dx%d, %d^2 fBm heightfield + %d icospheres (%d tris), depth %d, orbit" % (
            args.width, args.height, args.grid, args.spheres, hs.triangle_count(), args.depth),
            "width": args.width, "height": args.height, "triangles": hs.triangle_count(), "max_depth": args.depth}
    else:
        specs = workloads.batched_views(args.views, seed=args.seed + 6)
        views = []
        for i, s in enumerate(specs):
            hs = G.HostScene(s["kind"], seed=s["seed"], grid=s["grid"], spheres=s["spheres"], lib=scene_lib)
            views.append(View(hs, s["width"], s["height"], settings(s["maxDepth"]), frames, args.seed + i))
        tris = [v.hs.triangle_count() for v in views]
        px = sum(v.w * v.h for v in views)
        config = {"workload": "C3: %d views, {64,128,256,512}^2 (%d px), box-or-terrain scenes %d-%d tris (%d total), "
                              "depth 2-10" % (len(views), px, min(tris), max(tris), sum(tris)),
                  "views": len(views), "pixels": px, "triangles": sum(tris),
                  "max_depth": [v.settings.maxDepth for v in views]}
    config.update(common)
    return views, config


def cpu_oracle_run(views, target_seconds, frames=2, ora=None, plan=None):
    """Times the oracle on a band of rows of every view over `frames` frames; the band is
    calibrated so the sample takes about `target_seconds` (pass `plan` to repeat a calibrated
    sample). Returns (frames/s, threads, sample text, rays/s, plan)."""
    from oracle import pyoracle as O
    if ora is None:
        ora = O.oracle()
        ora.set_traversal(True)
        for i, v in enumerate(views):
            ora.select_scene(i)
            ora.set_scene(v.hs)
    threads = ora.threads()
    max_frames = min(len(v.cams) for v in views)

    def run(frac, nf):
        t_sample, t_full = 0.0, 0.0
        ora.read_counters(reset=True)
        for i, v in enumerate(views):
            rows = max(1, min(v.h, int(round(v.h * frac))))
            ora.select_scene(i)
            ora.set_rows(0, rows)
            t0 = time.perf_counter()
            O.run_sequence(ora, v.cams[:nf], v.prevs[:nf], v.settings, v.w, v.h, record=())
            dt = time.perf_counter() - t0
            t_sample += dt
            t_full += dt * v.h / rows
        cnt = ora.read_counters(reset=True)
        ora.set_rows(0, 1 << 30)
        return t_sample, t_full, cnt[0] + cnt[1] + cnt[2]

    if plan is None:
        frac, nf = 1.0 / 32.0, min(frames, max_frames)
        for _ in range(6):
            t_sample, t_full, rays = run(frac, nf)
            if t_sample >= 0.5 * target_seconds:
                break
            grow = max(2.0, min(16.0, target_seconds / max(t_sample, 1e-3)))
            if frac < 1.0:
                frac = min(1.0, frac * grow)
            elif nf < max_frames:
                nf = min(max_frames, int(math.ceil(nf * grow)))
            else:
                break
        plan = (frac, nf)
    else:
        t_sample, t_full, rays = run(*plan)
    frac, nf = plan
    fps = nf / t_full
    sample = "%d frame(s) x the first %.1f%% of the rows of each of %d view(s), %.2f s of CPU time" % (
        nf, 100.0 * min(1.0, frac), len(views), t_sample)
    return fps, threads, sample, rays / t_sample, plan, ora


def run_guided(args):
    """c4: plain and guided ReSTIR PT on the glossy scene, each accumulating frames (static camera)
    from a cold start; the relMSE of the running mean against a converged image (FP64 sums of
    independent paths, --ref-spp per pixel) after every frame, and each frame's device time. The
    value is the guided run's time to reach the plain run's final relMSE over the plain run's
    time (lower is better; the guide's training from scratch is inside the guided time)."""
    import torch
    import grisrt as G
    W, H, F = args.width, args.height, args.steps
    ctx = G.Context(0)
    ctx.set_path_form(G.PATH_WAVEFRONT)
    hs = G.HostScene(2, seed=args.seed, grid=args.grid, spheres=args.spheres)
    scene = G.Scene(ctx, hs)
    reuse = args.c4_reuse == "on"
    st = G.Settings.make(shiftType=2, rrScale=1.0, temporalReuse=reuse, spatialReuse=reuse, cap=20,
                         maxDepth=args.depth, spatialNeighbors=3, spatialRadius=20.0,
                         misWeights=1 if args.mis == "pairwise" else 0)
    stream = torch.cuda.ExternalStream(ctx.stream(), device=torch.device("cuda", 0))
    cam0 = hs.camera(0, 60, W, H)
    cams, prevs = [], []
    for f in range(F + 4):
        c = cam0.copy()
        c.seed = G.frame_seed(args.seed, f)
        ctypes.memmove(c.lastProjView, cam0.projView, 64)
        c.frameIndex = G.CLEAR_FLAG if f == 0 else f
        cams.append(c)
        prevs.append(cam0.copy())
    # converged image
    n = W * H
    dn = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    am = torch.zeros((n, 2), dtype=torch.int32, device="cuda")
    mv = torch.zeros((n, 2), dtype=torch.int16, device="cuda")
    gb = G.GBufferBindings(W, H, dn.data_ptr(), am.data_ptr(), mv.data_ptr())
    lib = G.load()
    ctx.check(lib.grisPassGBuffer(ctx.h, scene.h, ctypes.byref(gb), ctypes.byref(cam0)), "grisPassGBuffer")
    # the converged image as two independent halves (even / odd chunks of 32 samples): their
    # disagreement measures the converged image's own noise, stated beside every error it judges
    halves = [torch.zeros(n * 3, dtype=torch.float64, device="cuda") for _ in range(2)]
    t0 = time.perf_counter()
    cache = None
    if args.ref_cache:   # the same converged image for several runs (it depends on the scene, camera and depth only)
        cache = "%s_%dx%d_d%d_s%d_g%d_n%d_spp%d.npy" % (args.ref_cache, W, H, args.depth, args.seed, args.grid, args.spheres,
                                                          args.ref_spp)
    cached = bool(cache and os.path.exists(cache))
    if cached:
        import numpy as np
        both = np.load(cache)
        for j in (0, 1):
            halves[j].copy_(torch.from_numpy(both[j]))
    else:
        for i, k in enumerate(range(0, args.ref_spp, 32)):
            scene.converged(cam0, st, W, H, dn.data_ptr(), am.data_ptr(), halves[i & 1].data_ptr(), None, spp_begin=k,
                            spp=min(32, args.ref_spp - k), estimator=G.ESTIMATOR_CANDIDATES)
        ctx.sync()
        if cache:
            import numpy as np
            np.save(cache, np.stack([halves[0].cpu().numpy(), halves[1].cpu().numpy()]))
    ref_s = time.perf_counter() - t0
    ref = halves[0] + halves[1]
    scale = 1.0 / args.ref_spp
    import numpy as np
    ref_host = ref.cpu().numpy().reshape(-1, 3) * scale
    fg = ref_host.sum(axis=1) > 0
    nh = [sum(min(32, args.ref_spp - k) for i, k in enumerate(range(0, args.ref_spp, 32)) if (i & 1) == j) for j in (0, 1)]
    ha, hb = (halves[j].cpu().numpy().reshape(-1, 3) / max(1, nh[j]) for j in (0, 1))
    # relMSE of one half against the other = (var_a + var_b) / (ref^2 + eps), each half's variance
    # twice the full image's: a quarter of it estimates the converged image's own relMSE
    e_halves = (ha - hb) ** 2 / (ref_host ** 2 + 1e-2)
    ref_noise = {"relmse": float(np.mean(e_halves) / 4.0), "median": float(np.median(e_halves.mean(axis=1)[fg]) / 4.0),
                 "how": "relMSE / median per-pixel error between the two halves of the converged image's samples, / 4"}

    def run(guided):
        batch = G.Batch(ctx, [scene], [(W, H)])
        guide = None
        if guided:
            guide = G.Guide(ctx, G.GuideConfig.make(seed=args.seed, samplesPerFrame=args.guide_records,
                                                    stepsPerFrame=args.guide_steps, learningRate=args.guide_lr,
                                                    mix=args.guide_mix, tensorCores=args.guide_tc == "on",
                                                    trainKernel=1 if args.guide_train == "mma.sync" else 0))
            batch.set_guide(guide)
        out_ptr, _ = batch.device_ptr(0, G.BUF_OUTPUT)
        times, rel, med, energy = [], [], [], []
        with torch.cuda.stream(stream):
            for f in range(F):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                batch.render([cams[f]], [prevs[f]], [st])
                e1.record(stream)
                rel.append(ctx.relmse(out_ptr, ref.data_ptr(), scale, n)[0])
                times.append(e0.elapsed_time(e1))
                img = batch.download(0, G.BUF_OUTPUT)[:, :3].astype(np.float64)
                e = np.mean((img - ref_host) ** 2 / (ref_host ** 2 + 1e-2), axis=1)
                med.append(float(np.median(e[fg])))
                energy.append(float(img.sum() / max(ref_host.sum(), 1e-30)))
        # one profiled frame: the network's share of a frame
        ctx.set_profiling(True)
        ctx.kernel_profile(reset=True)
        batch.render([cams[F]], [prevs[F]], [st])
        ctx.sync()
        prof = ctx.kernel_profile(reset=True)
        ctx.set_profiling(False)
        batch.close()
        if guide is not None:
            guide.close()
        total = sum(prof[k]["ms"] for k in ("gbuffer", "path_trace", "temporal", "spatial")) + prof["guide_train"]["ms"]
        mlp = prof["guide_infer"]["ms"] + prof["guide_train"]["ms"]
        return np.array(times), np.array(rel), np.array(med), {"frame_ms": total, "mlp_ms": mlp,
                                                               "mlp_share": mlp / total if total > 0 else 0.0,
                                                               "energy_curve": energy,
                                                               "frame_ms_curve": [float(t) for t in times]}

    # warm-up outside the measured runs: the first launch of each kernel loads its code
    for guided in (False, True):
        wb = G.Batch(ctx, [scene], [(W, H)])
        wg = None
        if guided:
            wg = G.Guide(ctx, G.GuideConfig.make(seed=args.seed + 1, samplesPerFrame=1 << 16, stepsPerFrame=1,
                                                 tensorCores=args.guide_tc == "on",
                                                 trainKernel=1 if args.guide_train == "mma.sync" else 0))
            wb.set_guide(wg)
        for f in range(2):
            wb.render([cams[f]], [prevs[f]], [st])
        ctx.sync()
        wb.close()
        if wg is not None:
            wg.close()
    sampler = ClockSampler(0)
    sampler.start()
    tp, rp, mp, pp = run(False)
    tg, rg, mg, pg = run(True)
    clocks = sampler.stop()
    Tp = tp.sum()
    cg = np.cumsum(tg)

    def time_to(curve_g, target):
        """guided time (ms) to first reach `target` on its error curve (log-linear crossing)"""
        hit = np.nonzero(curve_g <= target)[0]
        if not len(hit):
            return None
        f = int(hit[0])
        if f > 0 and curve_g[f - 1] > target:
            a = (np.log(curve_g[f - 1]) - np.log(target)) / (np.log(curve_g[f - 1]) - np.log(curve_g[f]))
            return float(cg[f - 1] + a * (cg[f] - cg[f - 1]))
        return float(cg[f])

    Tg = time_to(rg, rp[-1])
    ratio = Tg / Tp if Tg is not None else None
    Tg_med = time_to(mg, mp[-1])
    ratio_med = Tg_med / Tp if Tg_med is not None else None
    # guided error at the plain run's total time
    k = min(int(np.searchsorted(cg, Tp)), F - 1)
    rel_equal_time = float(rg[k])
    line = {"metric": METRICS["c4"], "value": ratio, "unit": "x", "n_gpus": 1, "steps": F, "warmup": 0,
            "ms_per_step": float(tg.mean()), "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 paths, bf16 network", "data": "synthetic (seeded scene generator, no dataset)",
            "config": {"workload": "C4: %dx%d glossy variant (%d tris), depth %d, temporal+spatial reuse, static camera, "
                                   "frames accumulated" % (W, H, hs.triangle_count(), args.depth),
                       "guide": "MLP 80-64x4-48 BF16 (inference: %s; training: %s), 8 vMF lobes, mix %g, Adam %g, "
                                "%d records/frame, %d steps" % ("tcgen05" if args.guide_tc == "on" else "mma.sync",
                                                                "mma.sync" if args.guide_train == "mma.sync" else "tcgen05",
                                                                args.guide_mix, args.guide_lr, args.guide_records,
                                                                args.guide_steps)},
            "reference": {"spp": args.ref_spp, "seconds": ref_s, "estimator": "candidates", "noise_floor": ref_noise,
                          "loaded_from_cache": cached},
            "reuse": reuse, "mis": args.mis, "clocks": clocks,
            "median_error_time_ratio": ratio_med,
            "plain": {"fps": 1000.0 / float(tp.mean()), "total_ms": float(Tp), "relmse_final": float(rp[-1]),
                      "median_final": float(mp[-1]), "relmse_curve": [float(x) for x in rp],
                      "median_curve": [float(x) for x in mp], "profile": pp},
            "guided": {"fps": 1000.0 / float(tg.mean()), "total_ms": float(cg[-1]), "relmse_final": float(rg[-1]),
                       "median_final": float(mg[-1]), "relmse_at_plain_time": rel_equal_time,
                       "median_at_plain_time": float(mg[k]), "relmse_curve": [float(x) for x in rg],
                       "median_curve": [float(x) for x in mg], "profile": pg},
            "gpu_launches": None}
    print(json.dumps(line))
    scene.close()
    ctx.close()
    return 0


def di_alg_bytes(slot, w, px):
    """Algorithmic bytes of one frame of a DI kernel (work `w`, `px` pixels): traversal (nodes x 80 B
    + triangles x 48 B) plus
      di_candidates  24 B G-buffer read + 64 B reservoir write per pixel, a surface fetch per ray
      di_temporal    24+4 B G-buffer + motion, 24 B previous G-buffer, 2 x 64 B reservoir reads,
                     64 B write per pixel, a surface fetch per ray
      di_spatial     11 x 24 B G-buffer + 11 x 64 B reservoir reads, 64 B write, 32 B output r/w per
                     pixel, a surface fetch per ray."""
    trav = w["nodes"] * NODE_BYTES + w["tris"] * TRI_BYTES
    per_px = {"gbuffer": 28, "di_candidates": 88, "di_temporal": 244, "di_spatial": 11 * 24 + 11 * 64 + 64 + 32}
    return trav + per_px[slot] * px + (SURFACE_BYTES * w["rays"] if slot != "gbuffer" else SURFACE_BYTES * px)


def cpu_di_run(hs, cams, prevs, di, W, H, target_seconds, ora=None, plan=None):
    """The oracle's DI pass (G-buffer + TestReSTIR::render) on a band of rows, calibrated to about
    `target_seconds`; returns (frames/s, threads, sample text, plan, oracle)."""
    from oracle import pyoracle as O
    if ora is None:
        ora = O.oracle()
        ora.set_traversal(True)
        ora.set_scene(hs)

    def run(frac, nf):
        rows = max(1, min(H, int(round(H * frac))))
        ora.set_rows(0, rows)
        t0 = time.perf_counter()
        O.run_di_sequence(ora, ora, cams[:nf], prevs[:nf], di, W, H, record=())
        dt = time.perf_counter() - t0
        ora.set_rows(0, 1 << 30)
        return dt, dt * H / rows

    if plan is None:
        frac, nf = 1.0 / 16.0, 2
        for _ in range(6):
            t_sample, t_full = run(frac, nf)
            if t_sample >= 0.5 * target_seconds:
                break
            grow = max(2.0, min(16.0, target_seconds / max(t_sample, 1e-3)))
            if frac < 1.0:
                frac = min(1.0, frac * grow)
            elif nf < len(cams):
                nf = min(len(cams), int(math.ceil(nf * grow)))
            else:
                break
        plan = (frac, nf)
    else:
        t_sample, t_full = run(*plan)
    frac, nf = plan
    sample = "%d frame(s) x the first %.1f%% of the rows, %.2f s of CPU time" % (nf, 100.0 * min(1.0, frac), t_sample)
    return nf / t_full, ora.threads(), sample, plan, ora


def run_di(args, rank, world, local):
    """di: the ReSTIR DI pass through grisFrameRenderDI (G-buffer + candidates + temporal + spatial,
    no indirect pass) on the c2 scene, camera orbit. Timed like c2: CUDA events on the library's
    stream around every frame, L2 flushed between frames outside the events; e2e adds the direct
    output's read-back into pinned host memory each frame; roofline from a profiled pass and a
    work-counting pass of the same frames; the CPU baseline and the reference arm run the oracle's
    DI pass (bit-identical to the reference's DI shaders run as C++)."""
    import grisrt as G
    K, WU = args.steps, max(args.warmup, 0)
    shift = {"reconnection": G.DI_SHIFT_RECONNECTION, "replay": G.DI_SHIFT_REPLAY, "hybrid": G.DI_SHIFT_HYBRID}
    sample = {"light": G.DI_SAMPLE_LIGHT, "bsdf": G.DI_SAMPLE_BSDF, "both": G.DI_SAMPLE_BOTH}
    di = G.DISettings.make(shiftType=shift[args.di_shift], sampleType=sample[args.di_sample],
                           temporalReuse=args.di_temporal == "on", spatialReuse=True)
    scene_lib = None
    if args.impl == "reference":   # the reference arm builds its inputs without libgrisrt
        from oracle import build_oracle
        scene_lib = G.scene_library(build_oracle.build_scenegen())
    hs = G.HostScene(1, seed=args.seed, grid=args.grid, spheres=args.spheres, lib=scene_lib)
    W, H = args.width, args.height
    total = WU + 3 * K + 4
    cams, prevs = G.sequence_cameras(hs, total, W, H, seed=args.seed, orbit_frames=60)
    config = {"workload": "DI: %dx%d, %d^2 fBm heightfield + %d icospheres (%d tris), ReSTIR DI (%s shift, %s "
                          "candidates, temporal %s, spatial 10 neighbours / 20 px, cap 40), orbit" % (
                              W, H, args.grid, args.spheres, hs.triangle_count(), args.di_shift, args.di_sample,
                              args.di_temporal),
              "width": W, "height": H, "triangles": hs.triangle_count(), "di_shift": args.di_shift,
              "di_sample": args.di_sample, "di_temporal": args.di_temporal,
              "l2": "flushed between frames (256 MiB write; outside the timed events, inside the e2e wall clock)"}
    metric = METRICS["di"]
    if args.impl == "reference":
        if rank != 0:
            return 0
        budget = max(5.0, min(60.0, 150.0 / max(1, K + WU)))
        vals, plan, ora, threads, text = [], None, None, 0, ""
        for step in range(WU + K):
            fps, threads, text, plan, ora = cpu_di_run(hs, cams, prevs, di, W, H, budget, ora=ora, plan=plan)
            if step >= WU:
                vals.append(fps)
        value = statistics.median(vals) if vals else 0.0
        print(json.dumps({"metric": metric, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": K,
                          "warmup": WU, "ms_per_step": 1000.0 / value if value else None, "higher_is_better": True,
                          "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                          "data": "synthetic (seeded scene generator)", "config": config,
                          "run": {"parallelism": "host cores (OpenMP)"}, "impl": "reference",
                          "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                                           "sample": text},
                          "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))
        return 0
    import torch
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    run = {"parallelism": "replicas" if world > 1 else "1 GPU"}
    ctx = G.Context(local)
    scene = G.Scene(ctx, hs)
    frame = G.Frame(ctx, W, H)
    stream = torch.cuda.ExternalStream(ctx.stream(), device=torch.device("cuda", local))
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    fi = 0

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    for _ in range(WU):
        frame.render_di(scene, cams[fi], prevs[fi], di)
        fi += 1
    ctx.sync()
    ctx.counters(reset=True)
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    barrier()
    events = []
    with torch.cuda.stream(stream):
        for _ in range(K):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            frame.render_di(scene, cams[fi], prevs[fi], di)
            e1.record(stream)
            events.append((e0, e1))
            fi += 1
    barrier()
    clocks = sampler.stop()
    ms = sum(a.elapsed_time(b) for a, b in events)
    cnt = ctx.counters(reset=True)
    t_max = max_over_ranks(ms, "cuda")
    value = aggregate_rate(K, t_max / 1000.0, world)
    rays = cnt[0] + cnt[1] + cnt[2]
    # per-kernel profile and work counts of the same frames
    fi_p = fi - K
    ctx.set_profiling(True)
    with torch.cuda.stream(stream):   # one untimed eager frame: first-launch costs stay out of the profile
        frame.render_di(scene, cams[fi_p], prevs[fi_p], di)
    ctx.sync()
    ctx.kernel_profile(reset=True)
    with torch.cuda.stream(stream):
        for i in range(K):
            flush.zero_()
            frame.render_di(scene, cams[fi_p + i], prevs[fi_p + i], di)
    ctx.sync()
    prof = ctx.kernel_profile(reset=True)
    ctx.set_profiling(False)
    ctx.set_work_counting(True)
    ctx.kernel_profile(reset=True)
    for i in range(K):
        frame.render_di(scene, cams[fi_p + i], prevs[fi_p + i], di)
    ctx.sync()
    work = ctx.kernel_profile(reset=True)
    ctx.set_work_counting(False)
    slots = ["gbuffer", "di_candidates", "di_temporal", "di_spatial"]
    # the library's kernels per profiled pass: the candidates pass is four launches (prepare, the
    # two walks, finish) and the spatial pass with the reconnection shift three (prepare, walk,
    # finish); the G-buffer and the temporal pass one each
    per_pass = {"di_candidates": 4,
                "di_spatial": 3 if (di.spatialReuse and di.shiftType == G.DI_SHIFT_RECONNECTION) else 1}
    launches = sum(prof[s]["launches"] * per_pass.get(s, 1) for s in slots)
    # end to end: the direct output into pinned host memory every frame (pipelined as in the GRIS
    # workloads: a frame's copy to the host runs beside the next frame)
    out_host = torch.empty((W * H * 4,), dtype=torch.float32, pin_memory=True)
    barrier()
    t0 = time.perf_counter()
    for k in range(K):
        with torch.cuda.stream(stream):   # L2 flushed between frames here too, inside the wall clock
            flush.zero_()
        frame.render_di(scene, cams[fi], prevs[fi], di)
        if k > 0:
            ctx.download_wait()
        frame.download_async(G.BUF_DIRECT_OUTPUT, (out_host.data_ptr(), W * H * 16))
        fi += 1
    ctx.download_wait()
    ctx.sync()
    barrier()
    e2e_s = max_over_ranks(time.perf_counter() - t0, "cuda")
    e2e = {"value": aggregate_rate(K, e2e_s, world), "unit": UNIT, "h2d_bytes_per_step": 2 * 352 + 16,
           "d2h_bytes_per_step": W * H * 16}
    peak, peak_kind = load_peaks()
    l2_gbs = ctx.l2_bandwidth()
    per_kernel = {}
    for s_ in slots:
        L = max(1, prof[s_]["launches"])
        w = {k: work[s_][k] / K for k in ("nodes", "tris", "rays")}
        alg = di_alg_bytes(s_, w, W * H)
        avg_ms = prof[s_]["ms"] / L
        per_kernel[s_] = {"ms_per_frame": prof[s_]["ms"] / K, "avg_launch_ms": avg_ms,
                          "alg_bytes_per_launch": alg * K / L,
                          "gbs": (alg * K / L) / (avg_ms / 1000.0) / 1e9 if avg_ms > 0 else None,
                          "nodes_per_frame": w["nodes"], "tris_per_frame": w["tris"], "rays_per_frame": w["rays"]}
    top = max(slots, key=lambda s_: prof[s_]["ms"])
    pk = per_kernel[top]
    achieved = pk["gbs"] or 0.0
    traffic = None
    tfile = os.path.join(REPO, "profiles", "ncu_dram_traffic.json")
    if os.path.exists(tfile):
        try:
            e = json.load(open(tfile)).get("di", {}).get(top)
            if e:
                traffic = float(e["bytes_per_launch"]) * (W * H / float(e.get("pixels", W * H)))
        except Exception:
            traffic = None
    roofline = {"bound": "hbm", "kernel": top, "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "peak_source": peak_kind, "traffic": traffic,
                "l2_peak": round(l2_gbs, 1), "l2_frac": round(achieved / l2_gbs, 4) if l2_gbs else None,
                "l2_peak_source": "measured in this run (grisMeasureL2Bandwidth: 48 MiB read 20 times per launch, "
                                  "best of 5)",
                "algorithmic_bytes_per_launch": pk["alg_bytes_per_launch"], "avg_launch_ms": pk["avg_launch_ms"],
                "share_of_frame": round(prof[top]["ms"] / max(1e-9, sum(prof[s_]["ms"] for s_ in slots)), 3),
                "kernels": per_kernel}
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        try:
            fps, threads, text, _, _ = cpu_di_run(hs, cams, prevs, di, W, H, args.cpu_seconds)
            cpu = {"value": fps, "unit": UNIT, "cores": threads, "kind": "port", "sample": text}
        except Exception as ex:
            cpu = {"value": None, "unit": UNIT, "cores": 0, "kind": "port", "sample": "failed: %s" % ex}
    if rank == 0:
        print(json.dumps({"metric": metric, "value": value, "unit": UNIT, "n_gpus": world, "steps": K, "warmup": WU,
                          "ms_per_step": t_max / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                          "dtype": "f32", "data": "synthetic (seeded scene generator, no dataset)", "config": config,
                          "run": run, "mrays_per_s": world * rays / (t_max / 1000.0) / 1e6, "rays_per_frame": rays / K,
                          "clocks": clocks, "e2e": e2e, "gpu_launches": int(launches), "roofline": roofline,
                          "cpu_baseline": cpu}))
    frame.close()
    scene.close()
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def main():
    args = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    K, WU = args.steps, max(args.warmup, 0)
    if args.workload == "c3":
        args.api = "batch"
    if args.workload == "c4" and args.impl != "reference":
        return run_guided(args)
    if args.workload == "di":
        return run_di(args, rank, world, local)
    import grisrt as G
    metric = METRICS[args.workload]

    if args.impl == "reference":
        if rank != 0:
            return 0
        from oracle import build_oracle
        views, config = make_views(args, 16, scene_lib=G.scene_library(build_oracle.build_scenegen()))
        run = {"parallelism": "host cores (OpenMP)", "api": "oracle restatement (C++)"}
        budget = max(5.0, min(60.0, 150.0 / max(1, K + WU)))
        vals = []
        plan, ora = None, None
        threads, sample = 0, ""
        for step in range(WU + K):
            fps, threads, sample, rays, plan, ora = cpu_oracle_run(views, budget, ora=ora, plan=plan)
            if step >= WU:
                vals.append(fps)
        value = statistics.median(vals) if vals else 0.0
        line = {"metric": metric, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": K, "warmup": WU,
                "ms_per_step": 1000.0 / value if value else None, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scene generator)", "config": config,
                "run": run, "impl": "reference",
                "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
                "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                "note": "the reference's GLSL/Vulkan path is unavailable on this box (no graphics stack); this arm "
                        "times the oracle restatement of that path (C++/OpenMP, checked bit for bit against the "
                        "reference shaders compiled as C++)"}
        print(json.dumps(line))
        return 0

    import torch
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    total = WU + 3 * K + 8
    views, config = make_views(args, total)
    run = {"parallelism": "replicas" if world > 1 else "1 GPU"}   # how this arm ran the workload
    n = len(views)
    px = sum(v.w * v.h for v in views)
    ctx = G.Context(local)
    ctx.set_launch_mode(G.LAUNCH_PERSISTENT if args.launch_mode == "persistent" else G.LAUNCH_GRID)
    ctx.set_path_form(G.PATH_WAVEFRONT if args.path_form == "wavefront" else G.PATH_MEGAKERNEL)
    if args.wave:
        parts = args.wave.split(",")
        ctx.set_wave_launch(int(parts[0]), int(parts[1]))
        ctx.set_wave_refill(len(parts) > 2 and parts[2] == "refill")
    ctx.set_graphs(not args.no_graphs)
    scenes = [G.Scene(ctx, v.hs) for v in views]
    stats = [sc.stats() for sc in scenes]
    batch = G.Batch(ctx, scenes, [(v.w, v.h) for v in views]) if args.api == "batch" else None
    frame = G.Frame(ctx, views[0].w, views[0].h) if args.api == "frame" else None
    run["api"] = args.api
    stream = torch.cuda.ExternalStream(ctx.stream(), device=torch.device("cuda", local))
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    fi = 0

    def render(i):
        if batch is not None:
            batch.render([v.cams[i] for v in views], [v.prevs[i] for v in views], [v.settings for v in views])
        else:
            v = views[0]
            frame.render(scenes[0], v.cams[i], v.prevs[i], v.settings)

    for _ in range(WU):
        render(fi)
        fi += 1
    ctx.sync()
    tune = None
    if batch is not None and not args.no_autotune:
        r = batch.autotune([v.cams[fi] for v in views], [v.prevs[fi] for v in views], [v.settings for v in views],
                           frames=3)
        fi += 1
        names = (["megakernel"] + ["wavefront t%d s%d" % (t, s) for t in (8, 16, 32) for s in (4, 8, 16)] +
                 ["wavefront refill t%d s16" % t for t in (4, 8, 16)])
        tune = {"chosen": "megakernel" if r.pathForm == G.PATH_MEGAKERNEL else
                "wavefront%s t%d s%d" % (" refill" if r.refill else "", r.traceBlocksPerSM, r.shadeBlocksPerSM),
                "ms": {names[i]: round(r.candidateMs[i], 3) for i in range(r.candidates)}}
        form = r.pathForm
    else:
        form = G.PATH_WAVEFRONT if args.path_form == "wavefront" else G.PATH_MEGAKERNEL
    run["path_form"] = ("wavefront" if form == G.PATH_WAVEFRONT else "megakernel") if batch is not None else "megakernel"
    run["graphs"] = batch is not None and not args.no_graphs
    run["autotune"] = tune
    if args.wave and tune is None:
        run["wave"] = args.wave

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    # ---------------- device-timed frames (graph replays, no per-kernel events)
    ctx.counters(reset=True)
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    barrier()
    events = []
    with torch.cuda.stream(stream):
        for _ in range(K):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            render(fi)
            e1.record(stream)
            events.append((e0, e1))
            fi += 1
    barrier()
    clocks = sampler.stop()
    ms = sum(a.elapsed_time(b) for a, b in events)
    cnt = ctx.counters(reset=True)
    ctx.sync()
    t_max = max_over_ranks(ms, "cuda")
    value = aggregate_rate(K, t_max / 1000.0, world)
    rays = cnt[0] + cnt[1] + cnt[2]
    mrays = world * rays / (t_max / 1000.0) / 1e6

    # ---------------- per-kernel profile of the same frames (eager launches with events)
    fi_p = fi - K
    ctx.set_profiling(True)
    with torch.cuda.stream(stream):   # one untimed eager frame: first-launch costs stay out of the profile
        render(fi_p)
    ctx.sync()
    ctx.kernel_profile(reset=True)
    with torch.cuda.stream(stream):
        for i in range(K):
            flush.zero_()
            render(fi_p + i)
    ctx.sync()
    prof = ctx.kernel_profile(reset=True)
    ctx.set_profiling(False)
    # ---------------- work counting on the same frames (untimed)
    ctx.set_work_counting(True)
    ctx.kernel_profile(reset=True)
    for i in range(K):
        render(fi_p + i)
    ctx.sync()
    work = ctx.kernel_profile(reset=True)
    ctx.set_work_counting(False)

    wave = run["path_form"] == "wavefront"
    slots = (["gbuffer", "temporal", "spatial", "wave_begin", "wave_extend", "wave_shade", "wave_shadow", "wave_post"]
             if wave else ["gbuffer", "path_trace", "temporal", "spatial"])
    # batches run each reuse pass as prepare -> visibility walk -> finish: the pass's span (slot
    # "temporal" / "spatial") then holds its walk (slot "reuse_vis_*"), counted on its own here
    split = prof["reuse_vis_spatial"]["launches"] > 0 or prof["reuse_vis_temporal"]["launches"] > 0
    if split:
        for pas, vis in (("temporal", "reuse_vis_temporal"), ("spatial", "reuse_vis_spatial")):
            prof[pas] = dict(prof[pas])
            prof[pas]["ms"] = max(0.0, prof[pas]["ms"] - prof[vis]["ms"])
            prof[pas]["launches"] = 2 * prof[pas]["launches"]     # prepare + finish
            work[pas] = dict(work[pas])
            for k in ("nodes", "tris"):
                work[pas][k] = max(0, work[pas][k] - work[vis][k])
        slots += ["reuse_vis_temporal", "reuse_vis_spatial"]
    refill = (tune is not None and " refill" in tune["chosen"]) or (tune is None and bool(args.wave) and
                                                                    args.wave.endswith("refill"))
    launches_per_frame = kernel_launches_per_frame(prof, slots, K, wave, refill)

    # ---------------- end to end through the C ABI with host buffers
    out_host = torch.empty((px * 4,), dtype=torch.float32, pin_memory=True)
    lib = G.load()
    barrier()
    t0 = time.perf_counter()
    for k in range(K):
        with torch.cuda.stream(stream):   # L2 flushed between frames here too, inside the wall clock
            flush.zero_()
        render(fi)
        # every view's radiance into pinned host memory through the C ABI, pipelined: the previous
        # frame's copies are waited for once this frame is queued, then this frame's are queued
        # (staged on the device after the frame, copied to the host beside the next frame)
        if k > 0:
            ctx.download_wait()
        if batch is not None:   # the views' outputs are contiguous: one staged copy for all of them
            batch.download_async(G.BATCH_ALL_VIEWS, G.BUF_OUTPUT, (out_host.data_ptr(), px * 16))
        else:
            ctx.check(lib.grisFrameDownloadAsync(ctx.h, frame.handle, G.BUF_OUTPUT, 0, ctypes.c_void_p(out_host.data_ptr()),
                                                 px * 16), "grisFrameDownloadAsync")
        fi += 1
    ctx.download_wait()
    ctx.sync()
    barrier()
    e2e_s = max_over_ranks(time.perf_counter() - t0, "cuda")
    e2e = {"value": aggregate_rate(K, e2e_s, world), "unit": UNIT, "h2d_bytes_per_step": n * (2 * 352 + 64),
           "d2h_bytes_per_step": px * 16}

    # ---------------- roofline of the kernel with the largest share
    peak, peak_kind = load_peaks()
    # the second denominator: the BVH (tens of MB) and the queues stay in the 129-MB L2, so the
    # traversal and reuse kernels read most of their algorithmic bytes from L2
    l2_gbs = ctx.l2_bandwidth()
    per_kernel = {}
    for s in slots:
        L = max(1, prof[s]["launches"])
        w = {k: work[s][k] / K for k in ("nodes", "tris", "rays")}
        w["paths"] = work["wave_extend"]["rays"] / K
        w["shadow_paths"] = work["wave_shadow"]["rays"] / K
        w["split"] = split
        w["neighbours"] = max(v.settings.spatialNeighbors for v in views)
        w["queries"] = work["reuse_vis_" + s]["rays"] / K if s in ("temporal", "spatial") else 0
        alg_frame = alg_bytes(s, w, px)
        avg_ms = prof[s]["ms"] / L
        per_kernel[s] = {"ms_per_frame": prof[s]["ms"] / K, "launches_per_frame": prof[s]["launches"] / K,
                         "avg_launch_ms": avg_ms, "alg_bytes_per_launch": alg_frame * K / L,
                         "gbs": (alg_frame * K / L) / (avg_ms / 1000.0) / 1e9 if avg_ms > 0 else None,
                         "nodes_per_frame": w["nodes"], "tris_per_frame": w["tris"], "rays_per_frame": w["rays"]}
        g = per_kernel[s]["gbs"]
        per_kernel[s]["hbm_frac"] = round(g / peak, 4) if g else None
        per_kernel[s]["l2_frac"] = round(g / l2_gbs, 4) if g and l2_gbs else None
    top = max(slots, key=lambda s: prof[s]["ms"])
    pk = per_kernel[top]
    achieved = pk["gbs"] or 0.0
    traffic = None
    tfile = os.path.join(REPO, "profiles", "ncu_dram_traffic.json")
    if os.path.exists(tfile):
        try:
            tj = json.load(open(tfile)).get(args.workload, {})
            e = tj.get(top)
            if e:
                traffic = float(e["bytes_per_launch"]) * (px / float(e.get("pixels", px)))
        except Exception:
            traffic = None
    roofline = {"bound": "hbm", "kernel": top, "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "peak_source": peak_kind, "traffic": traffic,
                "l2_peak": round(l2_gbs, 1), "l2_frac": round(achieved / l2_gbs, 4) if l2_gbs else None,
                "l2_peak_source": "measured in this run (grisMeasureL2Bandwidth: 48 MiB read 20 times per launch, "
                                  "best of 5)",
                "algorithmic_bytes_per_launch": pk["alg_bytes_per_launch"], "avg_launch_ms": pk["avg_launch_ms"],
                "share_of_frame": round(prof[top]["ms"] / max(1e-9, sum(prof[s]["ms"] for s in slots)), 3),
                "kernels": per_kernel}

    # ---------------- CPU baseline (rank 0)
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        try:
            fps, threads, sample, rps, _, _ = cpu_oracle_run(views, args.cpu_seconds)
            cpu = {"value": fps, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample,
                   "mrays_per_s": rps / 1e6}
        except Exception as ex:   # the baseline is reported, never required
            cpu = {"value": None, "unit": UNIT, "cores": 0, "kind": "port", "sample": "failed: %s" % ex}

    if rank == 0:
        line = {"metric": metric, "value": value, "unit": UNIT, "n_gpus": world, "steps": K, "warmup": WU,
                "ms_per_step": t_max / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f32", "data": "synthetic (seeded scene generator, no dataset)", "config": config,
                "run": run, "mrays_per_s": mrays, "rays_per_frame": rays / K,
                "bvh": {"nodes": sum(s.nodeCount for s in stats), "node_mb": sum(s.nodeBytes for s in stats) / 1e6,
                        "tri_mb": sum(s.triangleBytes for s in stats) / 1e6, "depth": max(s.maxDepth for s in stats),
                        "build_s": sum(s.buildSeconds for s in stats)},
                "clocks": clocks, "e2e": e2e, "gpu_launches": int(round(launches_per_frame * K)),
                "roofline": roofline, "cpu_baseline": cpu}
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
