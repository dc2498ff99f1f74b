#!/usr/bin/env python
"""Benchmark of the ReSTIR direct-lighting hot path on one GB300 per rank.

One step = one frame of the reference's pass sequence at config 3
(1920x1080, 1,048,588 triangles, 1,048,576 point lights): RIS with 32
candidates + visibility reuse + temporal reuse, 3 unbiased spatial passes
(k=5, R=30), shading.  Inputs (scene, per-frame G-buffers, reservoirs) are
resident in HBM before timing; the working set (~1.3 GB) is far larger than
the 129 MB L2, so no flush is needed between steps.

Reported (one JSON line on rank 0):
  value     reservoir-samples/s over all ranks (RIS candidates + temporal merges
            + spatial neighbour merges), device-timed with CUDA events;
  e2e       the same metric through rg_render_frame_host: host G-buffer in,
            image out, copies inside the timed region;
  roofline  the dominant kernel's algorithmic bytes per launch over its mean
            event-timed duration, against the measured HBM copy bandwidth;
  cpu_baseline  the CPU oracle on a crop of the same frame (all host threads),
            scaled per pixel.
--impl reference times the CPU implementation of the path (the oracle port
of the reference's shaders) on the same workload instead.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "restir-vulkan_gb300"))

METRIC = "reservoir-samples/s & Mrays/s at 1080p/1M lights; GPU time to equal RMSE"
UNIT = "reservoir-samples/s"
# Compulsory HBM bytes per pixel per launch (reference formats; reservoir = 52
# useful bytes; neighbour re-reads are cache hits):
#   RIS+vis+temporal: cur G 32 + prev G 28 + prev reservoir 52 + out 52
#   unbiased spatial: G 32 + reservoir in 52 + out 52
#   biased spatial:   G 36 + in 52 + out 52;  shade: G 32 + reservoir 52 + RGBA32F 16
BYTES_PER_PX = {"initial_temporal": 164, "spatial_unbiased": 136, "spatial_biased": 140, "shade": 100}


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def measured_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


# ------------------------------------------------------------------ clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-i", str(self.gpu), "-lms", "200"], stdout=open(self.path, "w"),
                                         stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self) -> dict | None:
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for line in Path(self.path).read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# ------------------------------------------------------------------ workload
def make_scene(name: str, width: int | None, height: int | None, frames: int | None):
    from restir_gb300 import scenes
    kw = {}
    if width:
        kw["width"] = width
    if height:
        kw["height"] = height
    if frames:
        kw["frames"] = frames
    return scenes.CONFIGS[name](**kw)


def workload_desc(s) -> str:
    mode = (f"temporal + {s.spatial_passes} unbiased spatial pass(es) k={s.neighbors}" if s.unbiased else
            f"{s.spatial_passes} biased spatial iteration(s) k={s.neighbors}")
    return (f"{s.name}: {s.width}x{s.height}, {len(s.triangles):,} triangles, {len(s.point_lights):,} point lights, "
            f"RIS C={s.candidates} ({s.source_pdf} source pdf) + visibility reuse + {mode}, R={s.radius:g}, shading")


# ------------------------------------------------------------------ CPU oracle sample
def cpu_sample(s, gbufs: list, crop_size: int, threads: int | None = None) -> dict:
    """Times the oracle's pass sequence for frame 1 of `s` on a centred crop.

    Each pass runs on the region it must cover for the final crop to be exact
    (the crop grown by R+1 pixels per later spatial pass); frame 0 is run on
    the same regions first to supply temporal inputs.  The per-pixel cost of
    each pass is then applied to the full frame: samples/s of a full frame."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle_binding as ob
    from restir_gb300 import _lib

    if threads:
        ob.oracle().or_set_threads(threads)
    W, H = s.width, s.height
    n = W * H
    full = crop_size <= 0 or crop_size >= max(W, H)
    cw_, ch_ = (W, H) if full else (min(crop_size, W), min(crop_size, H))
    cx, cy = (W - cw_) // 2, (H - ch_) // 2
    halo = int(s.radius) + 1
    n_sp = s.spatial_passes if s.unbiased else 2 * s.spatial_passes

    def region(grow):
        x0, y0 = max(cx - grow, 0), max(cy - grow, 0)
        x1, y1 = min(cx + cw_ + grow, W), min(cy + ch_ + grow, H)
        return (x0, y0, x1 - x0, y1 - y0)

    regions = [region(halo * (n_sp - k)) for k in range(n_sp + 1)]  # [RIS, pass0, ..., pass n-1]
    times = {"initial_temporal": 0.0, "spatial": 0.0, "shade": 0.0}
    pix = {"initial_temporal": 0, "spatial": 0, "shade": 0}
    rays = 0
    prev = np.zeros(n, _lib.RESERVOIR_DTYPE)
    for f in range(2):
        u = s.uniforms(f)
        g = gbufs[f]
        st = ob.Stats()
        r = np.zeros(n, _lib.RESERVOIR_DTYPE)
        t0 = time.perf_counter()
        ob.initial_temporal(s, g, gbufs[f - 1] if f else None, prev if f else None, r, u, crop=regions[0], stats=st)
        t1 = time.perf_counter()
        ts = 0.0
        for k in range(n_sp):
            o = np.zeros(n, _lib.RESERVOIR_DTYPE)
            a = time.perf_counter()
            if s.unbiased:
                ob.spatial_unbiased(s, g, r, o, u, s.neighbors, k, crop=regions[k + 1], stats=st)
            else:
                ob.spatial_biased(s, g, r, o, u, k, crop=regions[k + 1])
            ts += time.perf_counter() - a
            r = o
        img = np.zeros((H, W, 4), np.float32)
        a = time.perf_counter()
        ob.shade(s, g, r, s.lighting_uniforms(f), img, crop=regions[-1])
        tsh = time.perf_counter() - a
        if f == 1:
            times["initial_temporal"] = t1 - t0
            times["spatial"] = ts
            times["shade"] = tsh
            area = lambda c: c[2] * c[3]
            pix["initial_temporal"] = area(regions[0])
            pix["spatial"] = sum(area(c) for c in regions[1:])
            pix["shade"] = area(regions[-1])
            rays = st.rays
        prev = r
    per_px = (times["initial_temporal"] / pix["initial_temporal"] + times["spatial"] / pix["spatial"] * n_sp
              + times["shade"] / pix["shade"])
    frame_s = per_px * n
    samples = s.samples_per_frame(1)
    return {"value": samples / frame_s, "frame_seconds_estimate": frame_s,
            "measured_seconds": sum(times.values()), "threads": ob.oracle().or_max_threads(),
            "sample": (f"oracle pass sequence of frame 1 over the whole {W}x{H} frame (frame 0 run first for the "
                       f"temporal input)" if full else
                       f"oracle pass sequence of frame 1 on a {cw_}x{ch_} crop centred in the {W}x{H} frame "
                       f"(RIS on the crop grown by {halo * n_sp}px, each spatial pass by {halo}px less), "
                       f"per-pixel cost of each pass scaled to the full frame"),
            "rays_in_sample": rays}


# ------------------------------------------------------------------ ranks
def aggregate_ranks(total_ms: float, samples: float, rays: float, dist, device: str = "cuda"):
    """Whole-job figures over replicas: the slowest rank's time and the sum
    of the samples and rays every rank processed (no data is exchanged)."""
    if dist is None:
        return float(total_ms), float(samples), float(rays)
    import torch
    t = torch.tensor([float(total_ms)], dtype=torch.float64, device=device)
    u = torch.tensor([float(samples), float(rays)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(t[0]), float(u[0]), float(u[1])


# ------------------------------------------------------------------ GPU arm
def gpu_arm(args, rank: int, world: int, dist) -> dict | None:
    import torch

    from restir_gb300.passes import Context, DeviceGBuffer, reservoirs

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    t_setup = time.perf_counter()
    s = make_scene(args.config, args.width, args.height, args.frames)
    ctx = Context(dev)
    ctx.upload_scene(s)
    n = s.width * s.height
    dgs = []
    for f in range(s.frames):
        d = DeviceGBuffer(s.width, s.height)
        ctx.trace_gbuffer(s.cameras[f], d)
        dgs.append(d)
    torch.cuda.synchronize()
    log(f"[rank {rank}] setup {time.perf_counter() - t_setup:.1f}s: {workload_desc(s)}")
    stream = torch.cuda.current_stream()
    res = [reservoirs(n), reservoirs(n)]
    tmp = reservoirs(n)
    image = torch.zeros((s.height, s.width, 4), dtype=torch.float32, device="cuda")
    kinds = ["initial_temporal"] + (["spatial_unbiased"] * s.spatial_passes if s.unbiased else
                                    ["spatial_biased"] * (2 * s.spatial_passes)) + ["shade"]

    def step(k: int, events=None):
        f = 1 + (k % (s.frames - 1)) if s.frames > 1 else 0
        slot = f % 2
        cur, prev = res[slot], res[1 - slot]
        u = s.uniforms(f)
        ev = iter(events) if events is not None else None
        if s.unbiased:
            passes = s.spatial_passes
            first = tmp if passes % 2 == 1 else cur
            ctx.initial_temporal(dgs[f], dgs[f - 1] if f else None, prev, first, u, stream)
            if ev:
                next(ev).record(stream)
            src = first
            for p in range(passes):
                dst = cur if src is tmp else tmp
                ctx.spatial_unbiased(dgs[f], src, dst, u, s.neighbors, p, stream)
                if ev:
                    next(ev).record(stream)
                src = dst
        else:
            ctx.initial_temporal(dgs[f], dgs[f - 1] if f else None, prev, cur, u, stream)
            if ev:
                next(ev).record(stream)
            for j in range(s.spatial_passes):
                ctx.spatial_biased(dgs[f], cur, prev, u, 2 * j, stream)
                if ev:
                    next(ev).record(stream)
                ctx.spatial_biased(dgs[f], prev, cur, u, 2 * j + 1, stream)
                if ev:
                    next(ev).record(stream)
        ctx.shade(dgs[f], cur, s.lighting_uniforms(f), image, stream)
        if ev:
            next(ev).record(stream)
        return f

    for k in range(args.warmup):
        step(k)
    torch.cuda.synchronize()
    ctx.stats(reset=True)
    samples = 0
    evs = [[torch.cuda.Event(enable_timing=True) for _ in kinds] for _ in range(args.steps)]
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler(dev)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    start.record(stream)
    for k in range(args.steps):
        f = step(args.warmup + k, evs[k])
        samples += s.samples_per_frame(f)
    end.record(stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clock_rec = clocks.stop()
    total_ms = start.elapsed_time(end)
    st = ctx.stats()
    per_kind = {}
    for k in range(args.steps):
        prev_ev = start if k == 0 else evs[k - 1][-1]
        for i, kind in enumerate(kinds):
            a = prev_ev if i == 0 else evs[k][i - 1]
            per_kind.setdefault(kind, []).append(a.elapsed_time(evs[k][i]))
    # first pass of step 0 starts at `start`; every later launch directly follows its predecessor
    max_ms, units, rays_total = aggregate_ranks(total_ms, samples, st.rays_traced, dist, "cuda")
    if rank != 0:
        return None
    value = units / (max_ms / 1000.0)
    mrays = rays_total / (max_ms / 1000.0) / 1e6

    # dominant kernel and its roofline
    tot = {k: sum(v) for k, v in per_kind.items()}
    dom = max(tot, key=tot.get)
    launches_dom = len(per_kind[dom])
    mean_ms = tot[dom] / launches_dom
    alg_bytes = BYTES_PER_PX[dom] * n
    peaks = measured_peaks()
    achieved = alg_bytes / (mean_ms / 1000.0) / 1e9
    traffic = None
    tp = ROOT / "profiles" / "traffic.json"
    if tp.exists():
        tr = json.loads(tp.read_text()).get(dom)
        if tr:
            traffic = float(tr["bytes_per_pixel"]) * n
    roofline = {"kernel": dom, "bound": "hbm", "achieved": round(achieved, 2), "peak": peaks["hbm_gbs"],
                "unit": "GB/s", "frac": round(achieved / peaks["hbm_gbs"], 5), "traffic": traffic,
                "peak_source": peaks["source"], "algorithmic_bytes_per_launch": alg_bytes,
                "mean_launch_ms": round(mean_ms, 4), "share_of_step": round(tot[dom] / sum(tot.values()), 4)}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": max_ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic: seeded procedural scene, lights and camera path (no dataset exists)",
        "config": {"workload": workload_desc(s), "frames_cycled": s.frames, "pixels": n,
                   "samples_per_frame": s.samples_per_frame(1), "nominal_rays_per_frame": s.nominal_rays_per_frame(),
                   "l2": "inputs larger than L2 (G-buffers, 3 reservoir buffers, tree and lights ~1.3 GB); no flush",
                   "parallelism": f"replicas x{world}"},
        "mrays_per_s": mrays,
        "rays_per_step": rays_total / args.steps / world,
        "traversal": {"node_visits_per_ray": round(st.node_visits / max(st.rays_traced, 1), 2),
                      "triangle_tests_per_ray": round(st.triangle_tests / max(st.rays_traced, 1), 2),
                      "tree_bytes_per_ray": round((64 * st.node_visits + 48 * st.triangle_tests)
                                                  / max(st.rays_traced, 1), 1),
                      "note": "a node visit fetches 64 B (both child boxes), a triangle test 48 B"},
        "passes_ms_mean": {k: round(sum(v) / len(v), 4) for k, v in per_kind.items()},
        "roofline": roofline,
        "gpu_launches": len(kinds) * args.steps,
        "clocks": clock_rec,
    }

    # e2e through the host-buffer C ABI call
    if not args.no_e2e:
        host_frames = []
        for f in range(s.frames):
            h = dgs[f].to_host()
            pinned = {}
            for k2, a in h.items():
                t = torch.empty(a.shape, dtype=torch.uint8 if a.dtype == np.uint8 else
                                (torch.int16 if a.dtype == np.uint16 else torch.float32), pin_memory=True)
                arr = t.numpy()
                if a.dtype == np.uint16:
                    arr = arr.view(np.uint16)
                arr[...] = a
                pinned[k2] = (t, arr)
            host_frames.append({k2: v[1] for k2, v in pinned.items()} | {"_keep": pinned})
        out_t = torch.empty((s.height, s.width, 4), dtype=torch.float32, pin_memory=True)
        out = out_t.numpy()
        for k in range(args.warmup):
            f = 1 + (k % (s.frames - 1))
            ctx.render_frame_host(host_frames[f], s.frame_params(f), out, stream)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        e_samples = 0
        for k in range(args.steps):
            f = 1 + ((args.warmup + k) % (s.frames - 1))
            ctx.render_frame_host(host_frames[f], s.frame_params(f), out, stream)
            e_samples += s.samples_per_frame(f)
        e1.record(stream)
        torch.cuda.synchronize()
        e_ms = e0.elapsed_time(e1)
        line["e2e"] = {"value": e_samples / (e_ms / 1000.0), "unit": UNIT, "h2d_bytes_per_step": n * (4 + 8 + 4 + 16 + 4),
                       "d2h_bytes_per_step": n * 16, "ms_per_step": e_ms / args.steps,
                       "api": "rg_render_frame_host (pinned host planes)"}

    # CPU baseline on the host cores (rank 0, N = 1 only)
    if world == 1 and not args.no_cpu:
        host_g = [dgs[0].to_host(), dgs[1].to_host()]
        cb = cpu_sample(s, host_g, args.cpu_crop)
        line["cpu_baseline"] = {"value": cb["value"], "unit": UNIT, "cores": cb["threads"], "kind": "port",
                                "sample": cb["sample"], "measured_seconds": round(cb["measured_seconds"], 2),
                                "full_frame_seconds_estimate": round(cb["frame_seconds_estimate"], 2)}
    ctx.close()
    return line


# ------------------------------------------------------------------ reference arm
def reference_arm(args, rank: int, world: int) -> dict | None:
    if rank != 0:
        return None
    s = make_scene(args.config, args.width, args.height, args.frames)
    from restir_gb300 import scenes
    gb = [scenes.trace_gbuffer_host(s, 0), scenes.trace_gbuffer_host(s, 1)]
    vals = []
    for k in range(args.warmup + args.steps):
        r = cpu_sample(s, gb, args.cpu_crop)
        if k >= args.warmup:
            vals.append(r)
    value = statistics.median(v["value"] for v in vals)
    ms = statistics.median(v["frame_seconds_estimate"] for v in vals) * 1000.0
    return {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic: seeded procedural scene, lights and camera path",
            "config": {"workload": workload_desc(s)},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": vals[0]["threads"], "kind": "port",
                             "sample": vals[0]["sample"]},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": ("the reference's passes are Vulkan GLSL (no graphics stack on this box); its CPU "
                     "implementation of the path is the oracle's restatement, pinned against the reference's "
                     "own BVH builder, BRDF/p-hat and traversal compiled from source")}


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--config", default="config3")
    ap.add_argument("--width", type=int, default=None)
    ap.add_argument("--height", type=int, default=None)
    ap.add_argument("--frames", type=int, default=None)
    ap.add_argument("--cpu-crop", type=int, default=0, help="0: the whole frame")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    args = ap.parse_args(argv)
    if args.warmup < 3:
        log("warmup raised to 3 (timing rule)")
        args.warmup = 3
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    dist = None
    if args.impl == "reference":
        line = reference_arm(args, rank, world)
    else:
        if world > 1:
            import torch
            import torch.distributed as tdist
            torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
            tdist.init_process_group("nccl")
            dist = tdist
        line = gpu_arm(args, rank, world, dist)
        if dist:
            dist.destroy_process_group()
    if line is not None:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
