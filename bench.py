#!/usr/bin/env python3
"""bench.py — ReSTIR PT (GRIS) frames/s and Mrays/s at 1920x1080 on the ~1.16M-triangle
synthetic scene (512x512 fBm heightfield + 2000 instanced icospheres, GGX materials, 4 quad
lights), max depth 8, temporal + spatial reuse (hybrid shift), camera orbit (60 frames per
quarter turn).

One step = one frame: G-buffer + path trace + temporal reuse + spatial reuse / final shading.

  value   frames/s timed on the device with CUDA events on the library's stream, scene and
          frame buffers resident in HBM, L2 flushed (256 MiB write) between frames outside the
          timed events;
  e2e     frames/s through the C ABI from the host: the per-frame cameras and settings come
          from host memory (kernel parameters) and each frame's RGBA32F radiance is read back
          into pinned host memory, wall-clock timed;
  roofline  the dominant kernel's algorithmic bytes per launch (BVH nodes x 80 B + triangles
          x 48 B + surface fetches + the per-pixel G-buffer / reservoir bytes, counted on the
          same frames) over its average CUDA-event launch time, against the measured HBM copy
          bandwidth;
  cpu_baseline  the oracle restatement (C++, OpenMP, binary BVH) on this host's cores on a
          band of rows of the same frames, scaled to frames/s.

--impl reference times that CPU implementation alone (rank 0), the reference's own GLSL
path being unavailable on this machine (no graphics stack).
Multi-GPU: replicas (each rank renders the same workload; no collective in the path).
"""
import argparse
import ctypes
import json
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

METRIC = "ReSTIR PT frames/s at 1080p (1.16M-tri synthetic scene, depth 8, temporal+spatial reuse)"
UNIT = "frames/s"
KERNELS = ["k_gbuffer", "k_path_trace", "k_temporal", "k_spatial"]
# Fixed G-buffer / reservoir bytes per pixel and kernel (28 B G-buffer texel, 96 B reservoir):
#   G-buffer write 28; path trace 24 read + 96 write; temporal 24+4+24 G-buffer + 2 x 96 reservoir
#   read + 96 write; spatial 4 x 24 + 4 x 96 read + 96 write + 32 output read/write.
PIXEL_BYTES = [28, 120, 340, 608]
NODE_BYTES, TRI_BYTES = 80, 48
SURFACE_BYTES = 264   # per closest hit: 3 vertices (96) + transform and inverse-transpose (128) + offsets (8) + material (32)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="grisrt", choices=["grisrt", "reference"])
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--grid", type=int, default=512)
    ap.add_argument("--spheres", type=int, default=2000)
    ap.add_argument("--depth", type=int, default=8)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--launch-mode", default="grid", choices=["persistent", "grid"])
    ap.add_argument("--api", default="batch", choices=["batch", "frame"],
                    help="grisBatchRender (one-view batch) or grisFrameRender")
    ap.add_argument("--path-form", default="wavefront", choices=["wavefront", "megakernel"])
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


def cpu_oracle_run(hs, cams, prevs, settings, width, height, target_seconds, frames=2):
    """Times the oracle on a band of rows of `frames` frames; returns (frames/s, threads, sample, rays/s)."""
    import numpy as np
    from oracle import pyoracle as O
    ora = O.oracle()
    ora.set_scene(hs)
    ora.set_traversal(True)
    threads = ora.threads()
    n = width * height
    rows = max(8, height // 32)
    # calibrate the band: one frame of `rows` rows
    results = None
    for attempt in range(3):
        ora.set_rows(0, rows)
        ora.read_counters(reset=True)
        t0 = time.perf_counter()
        O.run_sequence(ora, cams[:frames], prevs[:frames], settings, width, height, record=())
        dt = time.perf_counter() - t0
        if dt * (height / rows) >= target_seconds * 0.5 or rows >= height or dt > target_seconds / 2:
            results = dt
            break
        rows = min(height, int(rows * max(2.0, min(8.0, target_seconds / 2 / max(dt, 1e-3)))))
    if results is None:
        results = dt
    cnt = ora.read_counters(reset=True)
    ora.set_rows(0, 1 << 30)
    frac = rows / height
    fps = frames * frac / results
    rays = (cnt[0] + cnt[1] + cnt[2]) / results
    sample = "%d frames x rows [0,%d) of %dx%d (%.1f%% of each frame), %.2f s" % (frames, rows, width, height, 100 * frac, results)
    return fps, threads, sample, rays


def main():
    args = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    W, H, K, WU = args.width, args.height, args.steps, max(args.warmup, 0)
    import grisrt as G
    settings = G.Settings.make(shiftType=2, rrScale=1.0, temporalReuse=True, spatialReuse=True, cap=20,
                               maxDepth=args.depth, spatialNeighbors=3, spatialRadius=20.0)
    config = {"workload": "C2: %dx%d, 512^2 fBm heightfield + %d icospheres (~1.16M tris), depth %d, orbit" % (
        W, H, args.spheres, args.depth), "width": W, "height": H, "triangles": None, "max_depth": args.depth,
        "spatial_neighbors": 3, "spatial_radius_px": 20.0, "cap": 20, "shift": "hybrid",
        "l2": "flushed between frames (256 MiB write outside the timed events)", "parallelism": "replicas" if world > 1 else "1 GPU"}

    if args.impl == "reference":
        if rank != 0:
            return 0
        hs = G.HostScene(1, seed=args.seed, grid=args.grid, spheres=args.spheres)
        config["triangles"] = hs.triangle_count()
        cams, prevs = G.sequence_cameras(hs, 2, W, H, seed=args.seed, orbit_frames=60)
        budget = max(5.0, min(60.0, 150.0 / max(1, K + WU)))
        vals = []
        threads, sample = 0, ""
        for step in range(WU + K):
            fps, threads, sample, rays = cpu_oracle_run(hs, cams, prevs, settings, W, H, budget)
            if step >= WU:
                vals.append(fps)
        value = statistics.median(vals) if vals else 0.0
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": K, "warmup": WU,
                "ms_per_step": 1000.0 / value if value else None, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scene generator)", "config": config,
                "impl": "reference",
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
    hs = G.HostScene(1, seed=args.seed, grid=args.grid, spheres=args.spheres)
    config["triangles"] = hs.triangle_count()
    ctx = G.Context(local)
    ctx.set_launch_mode(G.LAUNCH_PERSISTENT if args.launch_mode == "persistent" else G.LAUNCH_GRID)
    ctx.set_path_form(G.PATH_WAVEFRONT if args.path_form == "wavefront" else G.PATH_MEGAKERNEL)
    config["api"] = args.api
    config["launch"] = args.launch_mode if args.api == "frame" else "batch tiles"
    config["path_form"] = args.path_form if args.api == "batch" else "megakernel"
    scene = G.Scene(ctx, hs)
    stats = scene.stats()
    frame = G.Frame(ctx, W, H) if args.api == "frame" else None
    batch = G.Batch(ctx, [scene], [(W, H)]) if args.api == "batch" else None
    total = WU + 2 * K + 4
    cams, prevs = G.sequence_cameras(hs, total, W, H, seed=args.seed, orbit_frames=60)
    stream = torch.cuda.ExternalStream(ctx.stream(), device=torch.device("cuda", local))
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    fi = 0

    def render(i):
        if batch is not None:
            batch.render([cams[i]], [prevs[i]], [settings])
        else:
            frame.render(scene, cams[i], prevs[i], settings)

    for _ in range(WU):
        render(fi)
        fi += 1
    ctx.sync()

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    # ---------------- device-timed frames
    ctx.counters(reset=True)
    ctx.set_profiling(True)
    ctx.profile(reset=True)
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
    kms, klaunch = ctx.profile(reset=True)
    # kernels per frame: G-buffer, temporal, spatial + the path tracer (one kernel, or the
    # wavefront's begin + 4 stages for each further bounce)
    launches_per_frame = 4 if (args.api == "frame" or args.path_form == "megakernel") else 3 + 1 + 4 * (args.depth - 1)
    ctx.set_profiling(False)
    cnt = ctx.counters(reset=True)
    ctx.sync()
    t_max = ms
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        t_max = float(t.item())
    value = world * K / (t_max / 1000.0)
    rays = cnt[0] + cnt[1] + cnt[2]
    mrays = world * rays / (t_max / 1000.0) / 1e6

    # ---------------- work counting on the same frames (untimed)
    ctx.set_work_counting(True)
    ctx.work(reset=True)
    fi_c = fi - K
    for i in range(K):
        render(fi_c + i)
    ctx.sync()
    nodes, tris, kr = ctx.work(reset=True)
    ctx.set_work_counting(False)

    # ---------------- end to end through the C ABI with host buffers
    out_host = torch.empty((W * H * 4,), dtype=torch.float32, pin_memory=True)
    lib = G.load()
    barrier()
    t0 = time.perf_counter()
    for _ in range(K):
        render(fi)
        # the frame's radiance into pinned host memory through the C ABI (copy + wait)
        if batch is not None:
            batch.download(0, G.BUF_OUTPUT, out=(out_host.data_ptr(), W * H * 16))
        else:
            ctx.check(lib.grisFrameDownload(ctx.h, frame.handle, G.BUF_OUTPUT, 0, ctypes.c_void_p(out_host.data_ptr()),
                                            W * H * 16), "grisFrameDownload")
        fi += 1
    barrier()
    e2e_s = time.perf_counter() - t0
    if world > 1:
        t = torch.tensor([e2e_s], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e = {"value": world * K / e2e_s, "unit": UNIT, "h2d_bytes_per_step": 2 * 352 + 64,
           "d2h_bytes_per_step": W * H * 16}

    # ---------------- roofline of the dominant kernel
    peak, peak_kind = load_peaks()
    k = max(range(4), key=lambda i: kms[i])
    launches = max(1, klaunch[k])
    avg_s = kms[k] / launches / 1000.0
    px = W * H
    alg = (nodes[k] * NODE_BYTES + tris[k] * TRI_BYTES) / K + PIXEL_BYTES[k] * px
    # surface fetches: closest hits of the kernel (primary hits for the G-buffer)
    alg += SURFACE_BYTES * (kr[k] / K)
    achieved = alg / avg_s / 1e9
    traffic = None
    tfile = os.path.join(REPO, "profiles", "ncu_dram_traffic.json")
    if os.path.exists(tfile):
        try:
            tj = json.load(open(tfile))
            e = tj.get(KERNELS[k])
            if e:
                traffic = float(e["bytes_per_launch"]) * (px / float(e.get("pixels", px)))
        except Exception:
            traffic = None
    roofline = {"bound": "hbm", "kernel": KERNELS[k], "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "peak_source": peak_kind, "traffic": traffic,
                "algorithmic_bytes_per_launch": alg, "avg_launch_ms": avg_s * 1000.0,
                "per_kernel_ms_per_frame": {KERNELS[i]: kms[i] / max(1, klaunch[i]) for i in range(4)},
                "nodes_per_frame": [n / K for n in nodes], "tris_per_frame": [t / K for t in tris],
                "closest_rays_per_frame": [r / K for r in kr]}

    # ---------------- CPU baseline (rank 0)
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        try:
            fps, threads, sample, rps = cpu_oracle_run(hs, cams[:2], prevs[:2], settings, W, H, args.cpu_seconds)
            cpu = {"value": fps, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample,
                   "mrays_per_s": rps / 1e6}
        except Exception as ex:   # the baseline is reported, never required
            cpu = {"value": None, "unit": UNIT, "cores": 0, "kind": "port", "sample": "failed: %s" % ex}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K, "warmup": WU,
                "ms_per_step": t_max / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f32", "data": "synthetic (seeded scene generator, no dataset)", "config": config,
                "mrays_per_s": mrays, "rays_per_frame": rays / K,
                "bvh": {"nodes": stats.nodeCount, "node_mb": stats.nodeBytes / 1e6, "tri_mb": stats.triangleBytes / 1e6,
                        "depth": stats.maxDepth, "build_s": stats.buildSeconds},
                "clocks": clocks, "e2e": e2e, "gpu_launches": launches_per_frame * K, "roofline": roofline,
                "cpu_baseline": cpu}
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
