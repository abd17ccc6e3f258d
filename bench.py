#!/usr/bin/env python3
"""Benchmark of the iVR hot path on one GB300 (one JSON line on stdout).

Default workload (sorted_brick_512): a 512^3 float32 volume of 64 seeded
Gaussian blobs plus 3-octave value noise (amplitude 0.1), split into 2x2x2
bricks with a one-voxel halo, rendered at 1024x1024 with sort-last
compositing of the 8 bricks on device in exact view order, 16^3 macrocell
empty-space skipping, step 0.5 voxel, front-to-back FP32 accumulation with
early termination at alpha >= 0.99, 8-bit RGBA output.  A step is one frame
of a new seeded view (camera at distance 5 in a seeded azimuth/elevation
direction, 30 degree field of view); the volume stays resident in HBM and is
larger than L2, so no L2 flush is needed between frames.

value: frames/s with the STATE already on the host side of the launch and
the RGBA8 frame left in device memory.  e2e: the same frames through
ivr_render_host (STATE from host memory in, RGBA8 frame copied to pinned
host memory out, inside the timed region).  Gsamples/s counts the plain
method's lattice points (no skipping, no termination), so skipping shows
as a higher rate.

--impl reference times the CPU restatement of the same path (the oracle,
all host threads) on a bounded sample of the same workload: each step
renders one band of 1/16 of the image rows, rotating through the frame.
Under torchrun (N>1) every rank renders its own stream of views (replicas;
the path has no exchange step), value = all frames / max time over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    "sorted_brick_512": dict(shape=(512, 512, 512), dtype="f32", n_blobs=64, noise=0.0, value_noise=0.1,
                             bricks=(2, 2, 2), image=(1024, 1024), step=0.5, term=0.99, fovy=30.0, seed=2),
    # same kernel and data type, smaller: the case ncu captures in full
    "prof_384": dict(shape=(384, 384, 384), dtype="f32", n_blobs=64, noise=0.0, value_noise=0.1,
                     bricks=(2, 2, 2), image=(1024, 1024), step=0.5, term=0.99, fovy=30.0, seed=2),
    "plain_128": dict(shape=(128, 128, 128), dtype="u8", n_blobs=8, noise=0.05, value_noise=0.0,
                      bricks=(1, 1, 1), image=(512, 512), step=0.5, term=0.99, fovy=30.0, seed=1),
}
# batched render: 64 views x 4 TFs on the sorted-brick volume, image sizes
# mixed from {256^2, 512^2, 1024^2, 1920x1080}, steps 0.25-1.0 voxel, one
# persistent launch per step (a CUDA-graph replay), kernel variant picked by
# the autotuner
BATCH = dict(base="sorted_brick_512", views=64, tfs=4, sizes=[(256, 256), (512, 512), (1024, 1024), (1920, 1080)],
             steps=(0.25, 1.0), seed=40)
# steering-server workload: 4 resident volumes, 32 Poisson clients at 10-60
# requests/s, a TF edit every 5th request, sizes 256^2 .. 1920x1080
SERVE = dict(volumes=[((256, 256, 256), "u8", 8, 0.05, 0.0, 0.0), ((512, 512, 512), "u16", 64, 0.0, 0.0, 0.0),
                      ((512, 512, 512), "f32", 64, 0.0, 0.1, 0.0), ((1024, 1024, 1024), "u16", 256, 0.0, 0.0, 0.7)],
             clients=32, rate=(10.0, 60.0), duration=10.0, warm=2.0, slots=4, batch=16, arena_mib=160,
             budget_gib=32)
# learned empty-space skipping: 1024^3 u16 of 256 blobs (sigmas scaled by
# (8/256)^(1/3) so they do not sum to saturation) with 70% of the
# macrocells exactly zero, 1920x1080, 50 random 16-knot TFs (the lowest
# fifteenth of the range transparent); the predictor is trained on the exact
# bounds of 8 of them (65^3 cells x 8 = 2.2M samples) and every TF is
# rendered plain (no skipping), with the exact grid and with the learned grid
LEARNED = dict(shape=(1024, 1024, 1024), dtype="u16", n_blobs=256, sigma_scale=(8 / 256) ** (1 / 3),
               zero_fraction=0.7, image=(1920, 1080),
               step=0.5, term=0.99, fovy=30.0, seed=3, tfs=50, train_tfs=8, epochs=30, batch_rows=8192, lr=2e-3,
               wneg=4.0, slack=0.02, judge_stride=16, frames=3)
# the same at 256^3 and 1280x720 with 10 TFs: the case ncu captures
LEARNED_SMALL = dict(LEARNED, shape=(256, 256, 256), n_blobs=32, sigma_scale=(8 / 32) ** (1 / 3), image=(1280, 720),
                     tfs=10, train_tfs=4, epochs=5)
METRIC = "frames/s & Gsamples/s, learned-skip vs plain GPU at <=1/255 err; p99 ms"
PROFILE_TRAFFIC = os.path.join(ROOT, "profiles", "march_cfg_sorted_brick_512.txt")


def views(seed, n, w, h, fovy):
    from ivr_gb300.state import orbit_state
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        az, el = float(rng.uniform(0, 360)), float(rng.uniform(-60, 60))
        out.append(orbit_state(az, el, w, h, fovy=fovy, alpha=1.0))
    return out


def make_volume(wl, device):
    from ivr_gb300 import synth
    return synth.blob_volume(wl["shape"], n_blobs=wl["n_blobs"], seed=wl["seed"], dtype=wl["dtype"],
                             noise=wl["noise"], value_noise=wl["value_noise"], device=device)


def lut_scale(wl):
    return 256.0 / 65536.0 if wl["dtype"] == "u16" else 1.0


class ClockSampler:
    """nvidia-smi clock/throttle samples every 200 ms while running."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.p = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        time.sleep(0.3)
        self.lines = []
        if self.p:
            self.p.terminate()
            out, _ = self.p.communicate(timeout=10)
            self.lines = [ln for ln in out.splitlines() if ln.strip()]

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx = max(mx, float(f[1]))
            except ValueError:
                continue
            for n, v in zip(names, f[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def profiled_traffic():
    """DRAM bytes per launch of the march kernel from the committed ncu
    summary (dram__bytes_read.sum + dram__bytes_write.sum), if present."""
    try:
        for ln in open(PROFILE_TRAFFIC):
            if ln.startswith("dram_bytes_per_launch:"):
                return float(ln.split(":")[1])
    except OSError:
        pass
    return None


def cpu_baseline(wl, vol, states, budget_s=20.0, threads=0):
    """The oracle on bands of image rows of the same workload, all threads."""
    from oracle import oracle
    from ivr_gb300 import synth
    lut = synth.ramp_tf(256)
    w, h = wl["image"]
    band = h // 16
    cores = os.cpu_count() or 1
    prep = oracle.Prepared(vol, wl["bricks"])  # volume load: outside the timing, as for the GPU
    t0 = time.perf_counter()
    rows = 0
    nb = 0
    while True:
        b = nb % 16
        st = states[nb % len(states)]
        oracle.render(vol, st, lut, 0, 6, preset=1, procdims=wl["bricks"], step=wl["step"], term_alpha=wl["term"],
                      lut_scale=lut_scale(wl), rows=(b * band, (b + 1) * band), threads=threads or cores,
                      prepared=prep)
        rows += band
        nb += 1
        el = time.perf_counter() - t0
        # at least one frame's worth of bands, then about half the budget
        if nb >= 16 and (el > budget_s / 2 or nb >= 16 * len(states)):
            break
    fps = (rows / h) / el
    return {"value": fps, "unit": "frames/s", "cores": threads or cores, "kind": "port",
            "sample": f"{nb} bands of {band} of {h} rows (oracle, CONFIG preset, same volume and views), "
                      f"{el:.1f} s"}


def run_reference(args, wl):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import oracle
    from ivr_gb300 import synth
    vol = make_volume(wl, None if wl["shape"][0] <= 160 else _gen_device())
    w, h = wl["image"]
    states = views(wl["seed"] + 100, max(args.steps + args.warmup, 1), w, h, wl["fovy"])
    lut = synth.ramp_tf(256)
    band = h // 16
    cores = os.cpu_count() or 1
    prep = oracle.Prepared(vol, wl["bricks"])  # volume load: outside the timing

    def step(k):
        b = k % 16
        oracle.render(vol, states[k % len(states)], lut, 0, 6, preset=1, procdims=wl["bricks"], step=wl["step"],
                      term_alpha=wl["term"], lut_scale=lut_scale(wl), rows=(b * band, (b + 1) * band),
                      threads=cores, prepared=prep)

    for k in range(args.warmup):
        step(k)
    t0 = time.perf_counter()
    for k in range(args.steps):
        step(args.warmup + k)
    el = time.perf_counter() - t0
    fps = (args.steps / 16.0) / el
    line = {"impl": "reference", "metric": METRIC, "value": fps, "unit": "frames/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * el / max(args.steps, 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded blobs; the reference's datasets are not available)",
            "config": {k: v for k, v in config_of(args, wl).items() if k != "layout"},
            "cpu_baseline": {"value": fps, "unit": "frames/s", "cores": cores, "kind": "port",
                             "sample": f"each step renders 1/16 of the rows ({band} of {h}); value = steps/16 "
                                       f"frames over the time"},
            "e2e": {"value": fps, "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def _gen_device():
    try:
        import torch
        return "cuda" if torch.cuda.is_available() else None
    except ImportError:
        return None


def tile_order(args):
    from ivr_gb300 import api
    return api.TILES_RASTER if getattr(args, "tiles", "cost") == "raster" else api.TILES_COST


def measure_cells(v, view, tf, params, states, args, o8, stream, cell):
    """frames/s and executed samples of the timed views with the volume's
    macrocell edge switched to `cell` (outside the headline's timed region),
    and whether the last frame is the headline's frame bit for bit."""
    import torch
    sp = stream.cuda_stream
    ref = o8.clone()
    v.macrocell(cell)
    with torch.cuda.stream(stream):
        for k in range(args.warmup):
            view.set(v, states[k], params)
            view.render(tf, None, o8.data_ptr(), sp)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for k in range(args.steps):
            view.set(v, states[args.warmup + k], params)
            view.render(tf, None, o8.data_ptr(), sp)
        e1.record(stream)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    same = bool(torch.equal(o8, ref))
    executed = 0
    for st in states[args.warmup:]:
        view.set(v, st, params)
        executed += view.census(tf, sp)["executed"]
    return {"fps": args.steps / (ms / 1000.0), "executed_per_frame": executed / args.steps,
            "last_frame_equal": same}


def config_of(args, wl):
    w, h = wl["image"]
    return {"workload": args.workload, "volume": "x".join(map(str, wl["shape"][::-1])) + " " + wl["dtype"],
            "bricks": "x".join(map(str, wl["bricks"])) + " + 1-voxel halo", "image": f"{w}x{h}",
            "step_voxels": wl["step"], "early_termination_alpha": wl["term"],
            "skip": f"macrocell grid of {getattr(args, 'cell', 16)}^3-voxel cells",
            "layout": "bricks" if args.linear else "bricks + corner-packed copies",
            "tile_order": "costliest first (estimated)" if getattr(args, "tiles", "cost") == "cost" else "row order",
            "tf": "256-entry RGBA FP32 ramp", "l2": "inputs larger than L2 (volume resident, > 129 MB)",
            "parallelism": f"replicas x{args.gpus}"}


def run_batch(args):
    """The batched workload: one batch of 64 views x 4 TFs per step."""
    import torch
    from ivr_gb300 import api, synth
    from ivr_gb300.state import orbit_state
    wl = WORKLOADS[BATCH["base"]]
    torch.cuda.set_device(0)
    vol = make_volume(wl, "cuda:0")
    torch.cuda.empty_cache()
    ctx = api.Context(0)
    v = ctx.load_volume(vol).bricks(*wl["bricks"], overlap=1)
    tfs = [ctx.transfer_function().set_lut(synth.knot_tf(BATCH["seed"] + t)[0], 0, lut_scale(wl), api.TF_F2B)
           for t in range(BATCH["tfs"])]
    rng = np.random.default_rng(BATCH["seed"])
    n = BATCH["views"] * BATCH["tfs"]
    frames = []
    for k in range(n):
        w, h = BATCH["sizes"][int(rng.integers(len(BATCH["sizes"])))]
        st = orbit_state(float(rng.uniform(0, 360)), float(rng.uniform(-60, 60)), w, h, fovy=wl["fovy"], alpha=1.0)
        step = float(rng.uniform(*BATCH["steps"]))
        view = ctx.view().set(v, st, api.config_params(step=step, term_alpha=wl["term"]))
        out = torch.empty((h, w, 4), dtype=torch.uint8, device="cuda")
        frames.append((view, tfs[k % BATCH["tfs"]], out, w * h))
    lattice = sum(view.census(tf)["lattice"] for view, tf, _, _ in frames)
    pixels = sum(p for *_, p in frames)
    b = ctx.batch(n)
    for view, tf, out, _ in frames:
        b.add(view, tf, None, out.data_ptr())
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream
    variant, tune_ms = b.autotune(sp)
    for _ in range(args.warmup):
        b.render(use_graph=True, stream=sp)
    torch.cuda.synchronize()
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(0) as clk:
        start.record(stream)
        for _ in range(args.steps):
            b.render(use_graph=True, stream=sp)
        stop.record(stream)
        torch.cuda.synchronize()
    t_ms = start.elapsed_time(stop)
    gsps = lattice * args.steps / (t_ms / 1000.0) / 1e9
    line = {
        "metric": METRIC, "value": gsps, "unit": "Gsamples/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded blobs + value noise, random 16-knot TFs)",
        "config": {"workload": "batch_64x4", "volume": "512x512x512 f32, 2x2x2 bricks + halo",
                   "frames_per_step": n, "sizes": "uniform from 256^2, 512^2, 1024^2, 1920x1080",
                   "step_voxels": "uniform 0.25-1.0", "launch": "one persistent launch per step, CUDA-graph replay",
                   "l2": "inputs larger than L2"},
        "frames_per_s": n * args.steps / (t_ms / 1000.0), "megapixels_per_step": pixels / 1e6,
        "lattice_per_step": lattice, "autotune": {"chosen": api.Batch.VARIANTS[variant],
                                                 "ms": dict(zip(api.Batch.VARIANTS, tune_ms))},
        "gpu_launches": args.steps, "clocks": clk.summary(),
    }
    print(json.dumps(line), flush=True)
    b.free()
    v.free()
    ctx.close()


def run_serve(args, quiet=False):
    """The serving workload: the steering server under Poisson load."""
    import torch
    from ivr_gb300 import api, serve, synth
    torch.cuda.set_device(0)
    ctx = api.Context(0, hbm_budget=SERVE["budget_gib"] << 30)
    vols, scales, names = [], [], []
    for k, (shape, dt, nb, noise, vn, zf) in enumerate(SERVE["volumes"]):
        vol = synth.blob_volume(shape, n_blobs=nb, seed=50 + k, dtype=dt, noise=noise, value_noise=vn,
                                zero_fraction=zf, device="cuda:0", sigma_scale=min(1.0, (8 / nb) ** (1 / 3)))
        torch.cuda.empty_cache()
        vols.append(ctx.load_volume(vol))
        del vol
        scales.append(256.0 / 65536.0 if dt == "u16" else 1.0)
        names.append("x".join(map(str, shape)) + " " + dt)
    resident = ctx.mem_used
    slots = args.serve_slots or SERVE["slots"]
    batch = args.serve_batch or SERVE["batch"]
    srv = api.Server(ctx, slots=slots, max_batch_frames=batch, arena_mib=SERVE["arena_mib"])
    ids = [srv.add_volume(v) for v in vols]
    rate = tuple(float(x) for x in args.serve_rate.split(",")) if args.serve_rate else SERVE["rate"]
    serve.run(srv, ids, scales, duration=SERVE["warm"], clients=SERVE["clients"], rate=rate, seed=1)
    with ClockSampler(0) as clk:
        res, wall = serve.run(srv, ids, scales, duration=SERVE["duration"], clients=SERVE["clients"],
                              rate=rate, seed=2)
    stats = srv.stats()
    srv.close()
    ok = [r for r in res if r["status"] == 0]
    lat = np.array([r["latency"] for r in ok]) * 1000.0
    px = sum(r["vw"] * r["vh"] for r in ok)
    line = {
        "metric": METRIC, "value": len(ok) / wall, "unit": "frames/s", "n_gpus": 1,
        "steps": len(res), "warmup": 0, "ms_per_step": 1000.0 * wall / max(len(res), 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8/u16/f32",
        "data": "synthetic (seeded blobs; Poisson arrivals)",
        "config": {"workload": "serve_32", "volumes": names, "clients": SERVE["clients"],
                   "rate_per_client": rate, "duration_s": SERVE["duration"],
                   "sizes": "uniform from 256^2, 512^2, 1024^2, 1280x720, 1920x1080",
                   "tf_edit": "every 5th request per client", "slots": slots,
                   "max_batch_frames": batch, "arena_mib": SERVE["arena_mib"],
                   "hbm_budget_gib": SERVE["budget_gib"], "resident_volume_bytes": resident},
        "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                       "max": float(lat.max()), "from": "scheduled arrival to RGBA8 frame in host memory"},
        "latency_parts_ms": {
            k: {"p50": float(np.percentile(a, 50)), "p99": float(np.percentile(a, 99))}
            for k, a in (("generator_late", np.array([r["late"] for r in ok]) * 1000.0),
                         ("queued", np.array([r["t_queue"] for r in ok]) * 1000.0),
                         ("batch_to_host", np.array([r["t_total"] - r["t_queue"] for r in ok]) * 1000.0))},
        "requests": len(res), "rejected": len(res) - len(ok),
        "rejected_status": sorted({r["status"] for r in res if r["status"] != 0}),
        "megapixels_per_s": px / wall / 1e6, "batches": stats["batches"],
        "server_seconds": {k: stats[k] for k in ("gpu_s", "dispatch_s", "finish_s")}, "wall_s": wall,
        "clocks": clk.summary(),
    }
    for v in vols:
        v.free()
    ctx.close()
    if not quiet:
        print(json.dumps(line), flush=True)
    return line


def run_learned(args, quiet=False):
    """The learned-skip workload: learned skipping against the plain march and the exact grid."""
    import torch
    from ivr_gb300 import api, synth
    from ivr_gb300.state import orbit_state
    L = LEARNED_SMALL if getattr(args, "workload", "") == "learned_256" else LEARNED
    torch.cuda.set_device(0)
    vol = synth.blob_volume(L["shape"], n_blobs=L["n_blobs"], seed=L["seed"], dtype=L["dtype"], noise=0.0,
                            zero_fraction=L["zero_fraction"], device="cuda:0", sigma_scale=L["sigma_scale"])
    torch.cuda.empty_cache()
    ctx = api.Context(0)
    # ingestion: the volume from a raw file (just written, so in the page
    # cache) through ivr_volume_load_file's streamed upload
    ingest = {"bytes": int(vol.nbytes), "source": "raw little-endian file in the page cache"}
    try:
        import tempfile
        fd, path = tempfile.mkstemp(suffix=".raw")
        os.close(fd)
        try:
            vol.tofile(path)
            t0 = time.perf_counter()
            v = ctx.load_volume_file(path, L["shape"][2], L["shape"][1], L["shape"][0], api.U16)
            ingest["seconds"] = time.perf_counter() - t0
            ingest["gb_per_s"] = vol.nbytes / ingest["seconds"] / 1e9
            ingest["note"] = "includes the macrocell grid and the corner-packed copy"
        finally:
            os.unlink(path)
    except OSError as e:
        ingest["error"] = str(e)
        v = ctx.load_volume(vol)
    del vol
    scale = 256.0 / 65536.0
    tfs = [ctx.transfer_function().set_lut(synth.knot_tf(1000 + t, zero_first=True)[0], 0, scale, api.TF_F2B)
           for t in range(L["tfs"])]
    w, h = L["image"]
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream

    # training on the device: exact bounds of train_tfs TFs, Adam, calibration
    mlp = ctx.mlp(L["seed"])
    t0 = time.perf_counter()
    n = 0
    for tf in tfs[:L["train_tfs"]]:
        n = mlp.add_samples(v, tf)
    t_feat = time.perf_counter() - t0
    t0 = time.perf_counter()
    losses = mlp.train(L["epochs"], batch_rows=L["batch_rows"], lr=L["lr"], wneg=L["wneg"])
    t_train = time.perf_counter() - t0
    margin, recall = mlp.calibrate(L["slack"])
    v.set_mlp(mlp, margin, certify=True)

    methods = {"plain": api.SKIP_NONE, "grid": api.SKIP_GRID, "learned": api.SKIP_LEARNED}
    vw = {m: ctx.view() for m in methods}
    rng = np.random.default_rng(L["seed"] + 77)
    states = [orbit_state(float(rng.uniform(0, 360)), float(rng.uniform(-60, 60)), w, h, fovy=L["fovy"])
              for _ in range(L["tfs"])]
    outs = {m: torch.empty((h, w, 4), dtype=torch.uint8, device="cuda") for m in methods}
    ms = {m: [] for m in methods}
    first_ms = {m: [] for m in methods}
    lattice, executed = 0, {m: 0 for m in methods}
    worst = 0
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(0) as clk:
        for t, (tf, st) in enumerate(zip(tfs, states)):
            for m, skip in methods.items():
                p = api.config_params(step=L["step"], term_alpha=L["term"], skip=skip,
                                      judge_stride=getattr(args, "judge_stride", 0) or L["judge_stride"],
                                      tiles=tile_order(args))
                view = vw[m].set(v, st, p)
                # first frame of a new TF: includes building its grid
                torch.cuda.synchronize()
                ev0.record(stream)
                view.render(tf, None, outs[m].data_ptr(), sp)
                ev1.record(stream)
                torch.cuda.synchronize()
                first_ms[m].append(ev0.elapsed_time(ev1))
                ev0.record(stream)
                for _ in range(L["frames"]):
                    view.render(tf, None, outs[m].data_ptr(), sp)
                ev1.record(stream)
                torch.cuda.synchronize()
                ms[m].append(ev0.elapsed_time(ev1) / L["frames"])
            d = (outs["learned"].int() - outs["plain"].int()).abs().max().item()
            worst = max(worst, d)
            if t < 10:  # census of a subset: lattice and executed samples
                for m in methods:
                    c = vw[m].census(tf, sp)
                    executed[m] += c["executed"]
                lattice += c["lattice"]
    judge = vw["learned"].judge_stats()
    tot = {m: sum(ms[m]) for m in methods}
    fps = {m: L["tfs"] / (tot[m] / 1000.0) for m in methods}
    held = slice(L["train_tfs"], None)
    fps_held = {m: len(ms[m][held]) / (sum(ms[m][held]) / 1000.0) for m in methods}
    ncensus = min(10, L["tfs"])
    lat_per_frame = lattice / ncensus
    ls = v.learned_stats()
    line = {
        "metric": METRIC, "value": fps["learned"], "unit": "frames/s", "n_gpus": 1,
        "steps": L["tfs"] * L["frames"], "warmup": L["tfs"], "ms_per_step": tot["learned"] / L["tfs"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u16",
        "data": "synthetic (seeded blobs, 70% zero macrocells, random 16-knot TFs)",
        "config": {"workload": "learned_256" if L is LEARNED_SMALL else "learned_1024",
                   "volume": "x".join(map(str, L["shape"])) + f" u16, one brick, {L['n_blobs']} blobs, "
                             "70% zero macrocells",
                   "image": f"{w}x{h}", "tfs": L["tfs"], "train_tfs": L["train_tfs"], "step_voxels": L["step"],
                   "early_termination_alpha": L["term"], "judge": f"1 in {L['judge_stride']} tiles, tol 1/255",
                   "l2": "inputs larger than L2 (2 GiB volume resident)"},
        "fps": fps, "fps_held_out_tfs": fps_held,
        "learned_grid": dict(ls, recall_of_exact=(ls["learned_transparent"] - ls["false_skips"]) /
                             max(ls["exact_transparent"], 1),
                             note="cells over the 50 learned grids; false skips kept opaque by certification"),
        "speedup": {"learned_vs_plain": fps["learned"] / fps["plain"], "learned_vs_grid": fps["learned"] / fps["grid"],
                    "grid_vs_plain": fps["grid"] / fps["plain"]},
        "gsamples_per_s": {m: lat_per_frame * fps[m] / 1e9 for m in methods},
        "executed_per_frame": {m: executed[m] / ncensus for m in methods}, "lattice_per_frame": lat_per_frame,
        "max_abs_diff_8bit_vs_plain": worst,
        "first_frame_ms_median": {m: float(np.median(first_ms[m])) for m in methods},
        "frame_ms_median": {m: float(np.median(ms[m])) for m in methods},
        "judge": judge,
        "ingest": ingest,
        "training": {"samples": n, "epochs": L["epochs"], "batch_rows": L["batch_rows"],
                     "loss_first": float(losses[0]), "loss_last": float(losses[-1]), "features_s": t_feat,
                     "train_s": t_train, "margin": margin, "recall_of_transparent_cells": recall},
        # per TF and frame: plain 1; grid 1; learned 3 (march, compare, gated
        # fallback); the cost order adds 2 to the grid and learned frames
        "gpu_launches": L["tfs"] * (L["frames"] + 1) * (9 if tile_order(args) == api.TILES_COST else 5),
        "clocks": clk.summary(),
    }
    for m in methods:
        vw[m].free()
    v.set_mlp(None)
    mlp.free()
    for tf in tfs:
        tf.free()
    v.free()
    ctx.close()
    if not quiet:
        print(json.dumps(line), flush=True)
    return line


def run_ref_preset(args, quiet=True):
    """The drop-in path with the reference's own semantics (REF preset:
    ray-parameter step 0.001, 256-sample cap, getlinearsample weights, the
    SEISMIC2 transfer function over the seismic colormap) on the
    CPU-runnable configuration (plain_128: 128^3 u8, one brick, 512x512):
    GPU frames/s, the CPU restatement on the same frames, and a bitwise check
    of one frame against it."""
    import torch
    from oracle import oracle
    from ivr_gb300 import api
    wl = WORKLOADS["plain_128"]
    vol = make_volume(wl, None)
    w, h = wl["image"]
    states = views(wl["seed"] + 300, 8, w, h, wl["fovy"])
    ctx = api.Context(0)
    v = ctx.load_volume(vol)
    tf = ctx.transfer_function().set_colormap(v, api.CM_SEISMIC, api.TF_SEISMIC2)
    view = ctx.view()
    params = api.ref_params()
    o32 = torch.empty((h, w, 4), dtype=torch.float32, device="cuda")
    for st in states[:2]:
        view.set(v, st, params)
        view.render(tf, o32.data_ptr())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    for st in states:
        view.set(v, st, params)
        view.render(tf, o32.data_ptr())
    e1.record()
    torch.cuda.synchronize()
    gpu_ms = e0.elapsed_time(e1) / len(states)
    view.set(v, states[-1], params)
    view.render(tf, o32.data_ptr())
    torch.cuda.synchronize()
    got = o32.cpu().numpy()
    lut, off = oracle.lut_for(vol, api.CM_SEISMIC)
    cores = os.cpu_count() or 1
    prep = oracle.Prepared(vol, (1, 1, 1))
    t0 = time.perf_counter()
    n = 0
    ref = None
    for st in states[-2:]:
        ref = oracle.render(vol, st, lut, off, api.TF_SEISMIC2, threads=cores, prepared=prep)
        n += 1
    cpu_s = (time.perf_counter() - t0) / n
    bitwise = bool(np.array_equal(got.view(np.uint32), ref["rgba32"].view(np.uint32)))
    view.free()
    tf.free()
    v.free()
    ctx.close()
    return {"workload": "plain_128 (128^3 u8, 512x512), REF preset, SEISMIC2 over the seismic colormap",
            "fps": 1000.0 / gpu_ms, "cpu_fps": 1.0 / cpu_s, "cpu_cores": cores,
            "cpu": "the CPU restatement (REF preset) on the same frames, all host threads",
            "bitwise_equal_to_cpu": bitwise}


def max_over_ranks(values, device):
    """Each value's maximum over the ranks of the process group (the values
    themselves without one): the job's time is its slowest rank's."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return [float(x) for x in values]
    t = torch.tensor([float(x) for x in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t.tolist()]


def whole_job_rate(steps_per_rank, world, t_ms):
    """Frames of all ranks per second of the slowest rank (weak scaling:
    every rank renders its own views)."""
    return steps_per_rank * world / (t_ms / 1000.0)


def _extra(fn, args, keys):
    """A workload's line reduced to `keys`, or the error it raised."""
    import torch
    try:
        full = fn(args, quiet=True)
        return {k: full[k] for k in keys if k in full}
    except Exception as e:  # reported in the line, not hidden
        return {"error": f"{type(e).__name__}: {e}"}
    finally:
        torch.cuda.empty_cache()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="sorted_brick_512",
                    choices=sorted(WORKLOADS) + ["batch_64x4", "serve_32", "learned_1024", "learned_256"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-budget", type=float, default=20.0)
    ap.add_argument("--serve-slots", type=int, default=0)
    ap.add_argument("--serve-batch", type=int, default=0)
    ap.add_argument("--serve-rate", default="", help="per-client request rate range lo,hi (req/s)")
    ap.add_argument("--judge-stride", type=int, default=0, help="learned skipping: judge 1 in this many tiles")
    ap.add_argument("--tiles", default="cost", choices=["cost", "raster"],
                    help="tile order of the skipping launches: costliest first, or row order")
    ap.add_argument("--cell", type=int, default=16,
                    help="macrocell edge of the skipping grid in voxels (a power of two, 4-32)")
    ap.add_argument("--linear", action="store_true",
                    help="render from the bricks themselves, without the corner-packed copies")
    ap.add_argument("--no-extras", action="store_true",
                    help="default workload only: skip the learned-skip and serving summaries")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.workload == "batch_64x4":
        return run_batch(args)
    if args.workload == "serve_32":
        return run_serve(args)
    if args.workload in ("learned_1024", "learned_256"):
        return run_learned(args)
    wl = WORKLOADS[args.workload]
    if args.impl == "reference":
        return run_reference(args, wl)

    import torch
    import torch.distributed as dist
    from ivr_gb300 import api, synth

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")

    vol = make_volume(wl, f"cuda:{local}")
    torch.cuda.empty_cache()  # release the generator's temporaries
    w, h = wl["image"]
    nviews = args.steps + args.warmup
    states = views(wl["seed"] + 100 + 7919 * rank, nviews, w, h, wl["fovy"])
    lut = synth.ramp_tf(256)

    ctx = api.Context(local)
    v = ctx.load_volume(vol).bricks(*wl["bricks"], overlap=1).quads(not args.linear).macrocell(args.cell)
    tf = ctx.transfer_function().set_lut(lut, 0, lut_scale(wl), api.TF_F2B)
    params = api.config_params(step=wl["step"], term_alpha=wl["term"], skip=True, tiles=tile_order(args))
    view = ctx.view()
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream
    o8 = torch.empty((h, w, 4), dtype=torch.uint8, device="cuda")

    # the plain march (no skipping) on the first views: its executed
    # samples/s against the sample-rate roofline (outside the timed region)
    plain_view = ctx.view()
    plain_params = api.config_params(step=wl["step"], term_alpha=wl["term"], skip=False)
    p_exec, p_ms = 0, 0.0
    for st in states[args.warmup:args.warmup + 3]:
        plain_view.set(v, st, plain_params)
        p_exec += plain_view.census(tf, sp)["executed"]
        plain_view.render(tf, None, o8.data_ptr(), sp)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        plain_view.render(tf, None, o8.data_ptr(), sp)
        e1.record(stream)
        torch.cuda.synchronize()
        p_ms += e0.elapsed_time(e1)
    plain_view.free()

    # work census of the timed views (diagnostic launches, outside timing)
    lattice = executed = touched = 0
    for st in states[args.warmup:]:
        view.set(v, st, params)
        c = view.census(tf, sp)
        lattice += c["lattice"]
        executed += c["executed"]
        touched += c["touched_bytes"]
    torch.cuda.synchronize()

    def frame(k):
        view.set(v, states[k], params)
        view.render(tf, None, o8.data_ptr(), sp)

    with torch.cuda.stream(stream):
        for k in range(args.warmup):
            frame(k)
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
        start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()
        with ClockSampler(local) as clk:
            start.record(stream)
            for k in range(args.steps):
                ev[k][0].record(stream)
                frame(args.warmup + k)
                ev[k][1].record(stream)
            stop.record(stream)
            torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
        t_ms = start.elapsed_time(stop)
        kern_ms = [a.elapsed_time(b) for a, b in ev]

        # end to end through ivr_render_host: pinned host output, same views
        host8 = torch.empty((h, w, 4), dtype=torch.uint8).pin_memory().numpy()
        for k in range(args.warmup):
            view.render_host(v, tf, states[k], params, host8, sp)
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
        t0 = time.perf_counter()
        for k in range(args.steps):
            view.render_host(v, tf, states[args.warmup + k], params, host8, sp)
        e2e_s = time.perf_counter() - t0

    t_ms, e2e_ms = max_over_ranks([t_ms, e2e_s * 1000.0], "cuda")
    fps = whole_job_rate(args.steps, world, t_ms)
    e2e_fps = whole_job_rate(args.steps, world, e2e_ms)
    frames = args.steps * world
    gsps = lattice * world / (t_ms / 1000.0) / 1e9

    if rank == 0:
        kavg = statistics.mean(kern_ms)
        peak, how = peaks()
        sample_peak = ctx.sample_peak(v.dtype, sp)
        layouts = {}
        for name, code in (("corner_packed", api.SAMPLER_QUADS), ("bricks", api.SAMPLER_BRICKS),
                           ("texture_point_x8", api.SAMPLER_TEX_POINT), ("texture_filtered", api.SAMPLER_TEX_LINEAR)):
            g, err = ctx.sample_peak_layout(v.dtype, code, sp)
            layouts[name] = {"gsamples_per_s": g, "max_abs_sample_err": err}
        other_cells = {}
        if world == 1 and not args.no_extras:
            # the same frames with another macrocell edge (same image)
            for cell in ((8,) if args.cell != 8 else (16,)):
                other_cells[f"{cell}^3"] = measure_cells(v, view, tf, params, states, args, o8, stream, cell)
            v.macrocell(args.cell)
        alg_bytes = touched / args.steps + w * h * 4  # compulsory volume bytes + RGBA8 out, per launch
        achieved = alg_bytes / (kavg / 1000.0) / 1e9
        traffic = profiled_traffic()
        line = {
            "metric": METRIC, "value": fps, "unit": "frames/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded blobs + value noise; the reference's datasets are not available)",
            "config": config_of(args, wl),
            "gsamples_per_s": gsps,
            "samples": {"lattice_per_frame": lattice / args.steps, "executed_per_frame": executed / args.steps,
                        "note": "lattice = plain method without skipping or termination"},
            "kernel_ms": {"mean": kavg, "p50": statistics.median(kern_ms), "max": max(kern_ms)},
            "e2e": {"value": e2e_fps, "unit": "frames/s", "h2d_bytes_per_step": 184,
                    "d2h_bytes_per_step": w * h * 4,
                    "path": "ivr_render_host: host STATE in, RGBA8 to pinned host memory"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "peak_source": how,
                         "algorithmic_bytes_per_launch": alg_bytes,
                         "note": "algorithmic bytes = macrocells an executed sample read + RGBA8 output"},
            "sample_roofline": {"bound": "sampler", "achieved": executed / args.steps / (kavg / 1000.0) / 1e9,
                                "peak": sample_peak, "unit": "Gsamples/s",
                                "frac": executed / args.steps / (kavg / 1000.0) / 1e9 / sample_peak,
                                "note": "executed samples/s of the render launch against ivr_sample_peak: the "
                                        "same sampler, LUT fetch and blend alone on a cache-resident brick"},
            "sampler_layouts": dict(layouts, note="the sampler roofline through each layout of a cache-resident "
                                    "64^3 brick: the march reads corner_packed; bricks (8 gathers) and 8 point "
                                    "texture fetches give the same samples; one filtered texture fetch has "
                                    "fixed-point weights (errors in volume units; values span 0-255)"),
            "plain_kernel": {"executed_gsamples_per_s": p_exec / (p_ms / 1000.0) / 1e9,
                             "frac_of_sample_roofline": p_exec / (p_ms / 1000.0) / 1e9 / sample_peak,
                             "ms_per_frame": p_ms / 3,
                             "note": "the march without skipping (the plain method) on 3 of the views"},
            "gpu_launches": args.steps * (3 if tile_order(args) == api.TILES_COST else 1),  # + cost and order kernels
            "clocks": clk.summary(),
        }
        if other_cells:
            line["other_macrocell_edges"] = dict(other_cells, note=(
                "the same views with the skipping grid's cells of another edge (ivr_volume_set_macrocell); "
                "the headline uses the configuration's 16^3-voxel cells; the images are the same"))
        if not args.no_cpu_baseline and world == 1:
            line["cpu_baseline"] = cpu_baseline(wl, vol, states[args.warmup:], budget_s=args.cpu_budget)
    v.free()
    ctx.close()
    if rank == 0 and world == 1 and args.workload == "sorted_brick_512" and not args.no_extras:
        # the metric's other two parts, each from its own workload
        line["learned_skip"] = _extra(run_learned, args, ["fps", "speedup", "max_abs_diff_8bit_vs_plain",
                                                          "gsamples_per_s", "learned_grid", "judge", "training", "ingest",
                                                          "first_frame_ms_median", "config", "clocks"])
        line["serving"] = _extra(run_serve, args, ["value", "unit", "latency_ms", "requests", "rejected",
                                                   "megapixels_per_s", "config", "clocks"])
        line["ref_preset"] = _extra(run_ref_preset, args, ["workload", "fps", "cpu_fps", "cpu_cores", "cpu",
                                                           "bitwise_equal_to_cpu"])
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
