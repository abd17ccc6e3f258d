#!/usr/bin/env python3
"""Benchmark of the iVR hot path on one GB300 (one JSON line on stdout).

Default workload (learned_1024): a 1024^3 uint16 volume (2 GiB) of 256
seeded Gaussian blobs with 70% of the 16^3-voxel macrocells exactly zero,
rendered at 1920x1080 with learned empty-space skipping: a 26-64-64-1 BF16
MLP, trained on the device on the exact per-macrocell opacity bounds of 8
of the workload's 50 random 16-knot transfer functions, predicts each TF's
skipping grid; every frame is judged on the device against the exact grid
(1 tile in 16) with fallback.  Step 0.5 voxel, front-to-back FP32
accumulation with early termination at alpha >= 0.99, 8-bit RGBA output.

A step is one frame of a new seeded view (camera at distance 5 in a seeded
azimuth/elevation direction, 30 degree field of view) under the next of the
50 TFs; the TFs' skipping grids were built when each TF was first rendered,
before the timed region (the first-frame latency after a TF edit is reported
beside).  The volume stays resident in HBM and is larger than L2 (2 GiB plus
its 8 GiB corner-packed copy), so no L2 flush is needed between frames.

value: frames/s with the STATE on the host side of the launch and the RGBA8
frame left in device memory.  e2e: the same frames through ivr_render_host
(STATE from host memory in, RGBA8 frame copied to pinned host memory out,
inside the timed region).  Gsamples/s counts the plain method's lattice
points (no skipping, no termination), so skipping shows as a higher rate.

Nested beside the headline: the plain march, the exact macrocell grid and
the learned grid over all 50 TFs (methods); the 512^3 f32 sorted-brick
workload (sorted_brick_512); the batched workload (batch_64x4); the
steering server with a saturation sweep (serving); the reference's own
semantics on the CPU-runnable workload (ref_preset).

--impl reference times the CPU restatement of the same path (the oracle, no
skipping, all host threads) on a bounded sample of the same workload: each
step renders one band of 1/16 of the image rows of the step's frame.
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
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from ivr_gb300 import workloads  # noqa: E402
from ivr_gb300.workloads import BATCH, LEARNED, LEARNED_CASES, LEARNED_SMALL, RENDER, SERVE  # noqa: E402

METRIC = "frames/s & Gsamples/s, learned-skip vs plain GPU at <=1/255 err; p99 ms"
PROFILES = os.path.join(ROOT, "profiles")
# committed ncu summaries carrying dram_bytes_per_launch of the dominant kernel
PROFILE_TRAFFIC = {"learned_1024": os.path.join(PROFILES, "march_judged_learned_1024.txt"),
                   "sorted_brick_512": os.path.join(PROFILES, "march_cfg_sorted_brick_512.txt")}
# kernel launches of one frame: learned skipping = tile cost + tile scatter
# + judged march + judge compare + gated exact re-march; the exact grid =
# tile cost + tile scatter + march
LAUNCHES_LEARNED = 5
LAUNCHES_GRID = 3


class ClockSampler:
    """nvidia-smi clock/throttle samples every 200 ms while running."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.p = None
        self.lines = []

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


def profiled_traffic(workload):
    """DRAM bytes per launch of the dominant kernel from the committed ncu
    summary (dram__bytes_read.sum + dram__bytes_write.sum), if present."""
    try:
        for ln in open(PROFILE_TRAFFIC[workload]):
            if ln.startswith("dram_bytes_per_launch:"):
                return float(ln.split(":")[1])
    except (OSError, KeyError):
        pass
    return None


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


def _gen_device():
    try:
        import torch
        return "cuda" if torch.cuda.is_available() else None
    except ImportError:
        return None


class nvtx_range:
    """An NVTX range around a timed region (for ncu --nvtx-include);
    nothing when NVTX is unavailable."""

    def __init__(self, name):
        self.name = name

    def __enter__(self):
        try:
            import torch
            torch.cuda.nvtx.range_push(self.name)
            self.on = True
        except Exception:
            self.on = False
        return self

    def __exit__(self, *a):
        if self.on:
            import torch
            torch.cuda.nvtx.range_pop()


class InFlight:
    """Frames in flight: frame k renders with view k % S on stream k % S, so
    that frame k+1's tiles fill the SMs that frame k's tail leaves idle.  Each
    view and stream has its own RGBA8 frame in device memory and one in
    page-locked host memory (which its launches store into directly)."""

    def __init__(self, ctx, S, stream, h, w):
        import torch
        self.S = max(1, S)
        self.views = [ctx.view() for _ in range(self.S)]
        self.streams = [stream] + [torch.cuda.Stream() for _ in range(self.S - 1)]
        self.dev = [torch.empty((h, w, 4), dtype=torch.uint8, device="cuda") for _ in range(self.S)]
        self.host = [torch.empty((h, w, 4), dtype=torch.uint8).pin_memory() for _ in range(self.S)]

    def render(self, k, vol, state, params, tf, host=False):
        q = k % self.S
        self.views[q].set(vol, state, params)
        self.views[q].render(tf, None, (self.host if host else self.dev)[q].data_ptr(), self.streams[q].cuda_stream)

    def timed(self, ks, run, ev=None):
        """run(k) for k in ks between events on the first stream, which the
        other streams wait on and join: device milliseconds."""
        import torch
        first = self.streams[0]
        start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        start.record(first)
        for q in self.streams[1:]:
            q.wait_event(start)
        t0 = time.perf_counter()
        for n, k in enumerate(ks):
            q = self.streams[k % self.S]
            if ev:
                ev[n][0].record(q)
            run(k)
            if ev:
                ev[n][1].record(q)
        self.host_s = time.perf_counter() - t0  # the host's time to submit the frames
        for q in self.streams[1:]:
            e = torch.cuda.Event()
            e.record(q)
            first.wait_event(e)
        stop.record(first)
        torch.cuda.synchronize()
        return start.elapsed_time(stop)

    def wall(self, ks, run):
        """run(k) for k in ks, host seconds until every stream is done."""
        import torch
        t0 = time.perf_counter()
        for k in ks:
            run(k)
        torch.cuda.synchronize()
        return time.perf_counter() - t0

    def judge_stats(self):
        tot = {}
        for vw in self.views:
            for key, val in vw.judge_stats().items():
                tot[key] = max(tot.get(key, 0), val) if key == "worst" else tot.get(key, 0) + val
        return tot

    def free(self):
        for vw in self.views:
            vw.free()


def band_parity(got32, got8, ref32, ref8, rows):
    """Largest differences of one band of a GPU frame against the oracle's."""
    r0, r1 = rows
    g32, e32 = got32[r0:r1], ref32[r0:r1]
    d8 = int(np.abs(got8[r0:r1].astype(np.int32) - ref8[r0:r1].astype(np.int32)).max())
    rel = float((np.abs(g32 - e32) / np.maximum(np.abs(e32), 1e-6)).max())
    same = bool(np.array_equal(np.ascontiguousarray(g32).view(np.uint32), np.ascontiguousarray(e32).view(np.uint32)))
    return d8, rel, same


def oracle_bands(vol, prep, frames, bricks, step, term, scale, threads, budget_s, min_bands, gpu_frame=None,
                 max_bands=None):
    """The oracle (CONFIG preset, no skipping) on bands of 1/16 of the image
    rows, rotating through the frames [(state, lut)]: frames/s, the bands'
    count and time, and -- with gpu_frame(i) giving the GPU's (rgba32,
    rgba8) of frame i -- each band's largest difference against it."""
    from oracle import oracle
    h = frames[0][0].winheight
    band = h // 16
    t_cpu, nb, rows = 0.0, 0, 0
    par = {"bands": 0, "max_abs_diff_8bit": 0, "max_rel_fp32": 0.0, "bitwise_equal_bands": 0}
    while True:
        fi = (nb // 16) % len(frames)
        b = nb % 16
        st, lut = frames[fi]
        r = (b * band, (b + 1) * band)
        t0 = time.perf_counter()
        ref = oracle.render(vol, st, lut, 0, 6, preset=1, procdims=bricks, step=step, term_alpha=term,
                            lut_scale=scale, rows=r, threads=threads, prepared=prep)
        t_cpu += time.perf_counter() - t0
        rows += band
        nb += 1
        if gpu_frame is not None:
            g32, g8 = gpu_frame(fi)
            d8, rel, same = band_parity(g32, g8, ref["rgba32"], ref["rgba8"], r)
            par["bands"] += 1
            par["max_abs_diff_8bit"] = max(par["max_abs_diff_8bit"], d8)
            par["max_rel_fp32"] = max(par["max_rel_fp32"], rel)
            par["bitwise_equal_bands"] += int(same)
        if max_bands is not None and nb >= max_bands:
            break
        if nb >= min_bands and t_cpu > budget_s:
            break
    return {"fps": (rows / h) / t_cpu, "bands": nb, "band_rows": band, "seconds": t_cpu,
            "parity": par if gpu_frame is not None else None}


# --------------------------------------------------------------------------
# learned_1024: the headline
# --------------------------------------------------------------------------

def tile_order(args):
    """The api tile order of --tiles (resolved per workload in main)."""
    from ivr_gb300 import api
    return api.TILES_RASTER if getattr(args, "tiles", "cost") == "raster" else api.TILES_COST


def learned_config(args, L):
    w, h = L["image"]
    name = [k for k, c in LEARNED_CASES.items() if c is L][0]
    return {"workload": name,
            "volume": "x".join(map(str, L["shape"])) + f" u16, one brick, {L['n_blobs']} blobs, "
                      f"{int(L['zero_fraction'] * 100)}% zero 16^3 macrocells",
            "image": f"{w}x{h}", "tfs": f"{L['tfs']} random 16-knot piecewise-linear TFs, 60% zero opacity knots",
            "lut": "256-entry RGBA FP32, index (int)(v*256/65536)",
            "step_voxels": L["step"], "early_termination_alpha": L["term"],
            "macrocell_voxels": getattr(args, "cell", 16),
            "skip": {"learned": f"learned grid (26-64-64-1 BF16 MLP, trained on "
                                f"{getattr(args, 'train_tfs', 0) or L['train_tfs']} TFs), judged 1 "
                                f"tile in {L['judge_stride']} at 1/255 with exact-grid fallback",
                     "grid": "exact macrocell grid",
                     "none": "none (every lattice point)"}[getattr(args, "skip", "learned")],
            "step": "one frame: a new view under the next TF",
            "tile_order": "costliest first (estimated)" if getattr(args, "tiles", "raster") == "cost" else "row order",
            "frames_in_flight": getattr(args, "inflight", 4),
            "l2": "inputs larger than L2 (2 GiB volume resident)", "parallelism": f"replicas x{args.gpus}"}


def _learned_setup(ctx, L, vol, args):
    """Ingestion through the streamed file load, the TFs, and the predictor
    trained on the device: (volume, tf handles, luts, training summary)."""
    from ivr_gb300 import api
    if int(os.environ.get("RANK", "0")) != 0:  # replicas: one temporary volume file per job is enough
        return _learned_train(ctx, L, ctx.load_volume(vol), args, {"source": "host memory (ivr_volume_load)"})
    ingest = {"bytes": int(vol.nbytes), "source": "raw little-endian file in the page cache"}
    v = None
    try:
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
    return _learned_train(ctx, L, v, args, ingest)


def _learned_train(ctx, L, v, args, ingest):
    """The TFs and the predictor trained on the device for volume v."""
    from ivr_gb300 import api
    if args.linear or args.cell != 16:  # the layout and cells the predictor is trained on
        v.quads(not args.linear).macrocell(args.cell)
    luts = workloads.learned_tfs(L)
    scale = workloads.lut_scale(L["dtype"])
    tfs = [ctx.transfer_function().set_lut(t, 0, scale, api.TF_F2B) for t in luts]
    mlp = ctx.mlp(L["seed"])
    t0 = time.perf_counter()
    n = 0
    for tf in tfs[:args.train_tfs or L["train_tfs"]]:
        n = mlp.add_samples(v, tf)
    t_feat = time.perf_counter() - t0
    t0 = time.perf_counter()
    losses = mlp.train(L["epochs"], batch_rows=L["batch_rows"], lr=L["lr"], wneg=L["wneg"])
    t_train = time.perf_counter() - t0
    margin, recall = mlp.calibrate(L["slack"])
    v.set_mlp(mlp, margin, certify=not args.no_certify)
    training = {"samples": n, "epochs": L["epochs"], "batch_rows": L["batch_rows"],
                "loss_first": float(losses[0]), "loss_last": float(losses[-1]), "features_s": t_feat,
                "train_s": t_train, "margin": margin, "recall_of_transparent_cells": recall}
    return v, tfs, luts, mlp, training, ingest, margin


def _uncertified(ctx, v, mlp, margin, tfs, states, L, args, stream):
    """The same predictor and margin without the cell-by-cell certification
    (the per-frame judge alone guarding the frames), every TF once with the
    same views: frames/s, the judge's verdicts and the cells the network
    called transparent that the exact test calls opaque.  The certified
    grids are restored afterwards."""
    import torch
    from ivr_gb300 import api
    w, h = L["image"]
    sp = stream.cuda_stream
    v.set_mlp(mlp, margin, certify=False)
    view = ctx.view()
    out = torch.empty((h, w, 4), dtype=torch.uint8, device="cuda")
    p = api.config_params(step=L["step"], term_alpha=L["term"], skip=api.SKIP_LEARNED,
                          judge_stride=args.judge_stride or L["judge_stride"], tiles=tile_order(args))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ms = 0.0
    for t in range(len(tfs)):
        view.set(v, states[t], p)
        view.render(tfs[t], None, out.data_ptr(), sp)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(L["frames"]):
            view.render(tfs[t], None, out.data_ptr(), sp)
        e1.record(stream)
        torch.cuda.synchronize()
        ms += e0.elapsed_time(e1) / L["frames"]
    judge = view.judge_stats()
    ls = v.learned_stats()
    view.free()
    v.set_mlp(mlp, margin, certify=True)
    return {"fps": len(tfs) / (ms / 1000.0), "judge": judge, "false_skips": ls["false_skips"],
            "learned_transparent": ls["learned_transparent"],
            "note": "fallbacks = frames whose judged tiles (1 in judge_stride) differed by more than 1/255 from the "
                    "exact grid's (worst = the largest 8-bit difference seen); such a frame is re-rendered with the "
                    "exact grid and its TF's learned grid is not used again; frames whose judged tiles pass are "
                    "not re-rendered"}


def _methods(ctx, v, tfs, states, L, args, stream, device=0):
    """The plain march, the exact grid and the learned grid over every TF:
    the first frame after the TF is set (its grid built inside) and steady
    frames; frames/s, samples and the learned frames' largest difference
    from the plain frames."""
    import torch
    from ivr_gb300 import api
    w, h = L["image"]
    sp = stream.cuda_stream
    methods = {"plain": api.SKIP_NONE, "grid": api.SKIP_GRID, "learned": api.SKIP_LEARNED}
    vw = {m: ctx.view() for m in methods}
    outs = {m: torch.empty((h, w, 4), dtype=torch.uint8, device="cuda") for m in methods}
    ms = {m: [] for m in methods}
    first_ms = {m: [] for m in methods}
    lattice, executed = 0, {m: 0 for m in methods}
    worst = 0
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ntf = len(tfs)
    with ClockSampler(device) as clk:
        for t in range(ntf):
            tf, st = tfs[t], states[t]
            for m, skip in methods.items():
                p = api.config_params(step=L["step"], term_alpha=L["term"], skip=skip,
                                      judge_stride=args.judge_stride or L["judge_stride"], tiles=tile_order(args))
                view = vw[m].set(v, st, p)
                torch.cuda.synchronize()
                with nvtx_range(f"tf_edit_{m}"):  # the TF's grid build and first frame
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
            worst = max(worst, (outs["learned"].int() - outs["plain"].int()).abs().max().item())
            if t < 10:
                for m in methods:
                    c = vw[m].census(tf, sp)
                    executed[m] += c["executed"]
                lattice += c["lattice"]
    judge = vw["learned"].judge_stats()
    for m in methods:
        vw[m].free()
    tot = {m: sum(ms[m]) for m in methods}
    fps = {m: ntf / (tot[m] / 1000.0) for m in methods}
    held = slice(L["train_tfs"], None)
    fps_held = {m: len(ms[m][held]) / (sum(ms[m][held]) / 1000.0) for m in methods}
    ncensus = min(10, ntf)
    ls = v.learned_stats()
    return {
        "fps": fps, "fps_held_out_tfs": fps_held,
        "speedup": {"learned_vs_plain": fps["learned"] / fps["plain"], "learned_vs_grid": fps["learned"] / fps["grid"],
                    "grid_vs_plain": fps["grid"] / fps["plain"]},
        "gsamples_per_s": {m: lattice / ncensus * fps[m] / 1e9 for m in methods},
        "executed_per_frame": {m: executed[m] / ncensus for m in methods}, "lattice_per_frame": lattice / ncensus,
        "max_abs_diff_8bit_vs_plain": worst,
        "first_frame_ms_median": {m: float(np.median(first_ms[m])) for m in methods},
        "frame_ms_median": {m: float(np.median(ms[m])) for m in methods},
        "judge": judge,
        "learned_grid": dict(ls, recall_of_exact=(ls["learned_transparent"] - ls["false_skips"]) /
                             max(ls["exact_transparent"], 1),
                             note="cells over the learned grids; false skips kept opaque by certification"),
        "note": f"every TF once with its own view: first frame after the TF is set (grid built inside), then "
                f"{L['frames']} steady frames; census over the first {ncensus} TFs",
        "clocks": clk.summary(),
    }


def run_learned(args, quiet=False):
    """The headline: learned-skip frames/s at 1024^3 u16 and 1920x1080."""
    import torch
    import torch.distributed as dist
    from ivr_gb300 import api
    L = LEARNED_CASES[args.workload]
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1 and not dist.is_initialized():
        dist.init_process_group("nccl")
    vol = workloads.learned_volume(L, device=f"cuda:{local}")
    torch.cuda.empty_cache()
    ctx = api.Context(local)
    v, tfs, luts, mlp, training, ingest, margin = _learned_setup(ctx, L, vol, args)
    w, h = L["image"]
    ntf = len(tfs)
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream
    # the method comparison renders every TF once with each method (so each
    # TF's grids are resident before the timed region) on views of its own
    states = workloads.learned_views(L, n=max(ntf, args.steps + args.warmup), seed_offset=77 + 7919 * rank)
    methods = None
    if not args.no_methods:
        # the uncertified grids first: re-attaching the predictor drops a
        # volume's learned grids, which the comparison then builds again
        unc = None if args.no_certify else _uncertified(ctx, v, mlp, margin, tfs, states, L, args, stream)
        methods = _methods(ctx, v, tfs, states, L, args, stream, local)
        if unc is not None:
            methods["uncertified"] = unc

    skip = {"learned": api.SKIP_LEARNED, "grid": api.SKIP_GRID, "none": api.SKIP_NONE}[args.skip]
    params = api.config_params(step=L["step"], term_alpha=L["term"], skip=skip,
                               judge_stride=args.judge_stride or L["judge_stride"],
                               tiles=tile_order(args))
    fl = InFlight(ctx, args.inflight, stream, h, w)
    S = fl.S
    view = fl.views[0]
    nsteps = args.steps + args.warmup
    frames = [(states[k], k % ntf) for k in range(nsteps)]

    def frame(k, host=False):
        st, t = frames[k]
        fl.render(k, v, st, params, tfs[t], host)

    timed_ks = range(args.warmup, nsteps)
    with torch.cuda.stream(stream):
        # every TF's grids built before the timed region (the comparison has
        # built them already when it ran)
        for t in sorted({t for _, t in frames}):
            view.set(v, frames[0][0], params)
            view.render(tfs[t], None, fl.dev[0].data_ptr(), sp)
        for k in range(args.warmup):
            frame(k)
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()
        with ClockSampler(local) as clk, nvtx_range("timed"):
            t_ms = fl.timed(timed_ks, frame, ev)
        if world > 1:
            dist.barrier()
        frame_ms = [a.elapsed_time(b) for a, b in ev]
        judge_timed = fl.judge_stats()

        # end to end: the same frames with the STATE from host memory and the
        # RGBA8 frames stored into page-locked host memory by the launches
        # themselves, S in flight, timed until the last frame is in host memory
        for k in range(args.warmup):
            frame(k, True)
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
        e2e_s = fl.wall(timed_ks, lambda k: frame(k, True))
        # and one frame at a time through ivr_render_host (waits for each)
        host8 = fl.host[0].numpy()
        e2e_view = ctx.view()
        for k in range(args.warmup):
            st, t = frames[k]
            e2e_view.render_host(v, tfs[t], st, params, host8, sp)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for k in timed_ks:
            st, t = frames[k]
            e2e_view.render_host(v, tfs[t], st, params, host8, sp)
        sync_s = time.perf_counter() - t0
        e2e_view.free()

    t_ms, e2e_ms, sync_ms = max_over_ranks([t_ms, e2e_s * 1000.0, sync_s * 1000.0], "cuda")
    fps = whole_job_rate(args.steps, world, t_ms)
    e2e_fps = whole_job_rate(args.steps, world, e2e_ms)
    line = None
    if rank == 0:
        # work census of the timed frames (diagnostic launches, outside timing)
        lattice = executed = touched = 0
        for k in range(args.warmup, nsteps):
            st, t = frames[k]
            view.set(v, st, params)
            c = view.census(tfs[t], sp)
            lattice += c["lattice"]
            executed += c["executed"]
            touched += c["touched_bytes"]
        kavg = t_ms / args.steps  # device time per frame, frames overlapping
        peak, how = peaks()
        sample_peak = ctx.sample_peak(api.U16, sp)
        alg_bytes = touched / args.steps + w * h * 4
        achieved = alg_bytes / (kavg / 1000.0) / 1e9
        ex_rate = executed / args.steps / (kavg / 1000.0) / 1e9
        line = {
            "metric": METRIC, "value": fps, "unit": "frames/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u16",
            "data": "synthetic (seeded blobs, 70% zero macrocells, random 16-knot TFs; the reference's datasets "
                    "are not available)",
            "config": learned_config(args, L),
            "gsamples_per_s": lattice / args.steps * fps / 1e9,
            "samples": {"lattice_per_frame": lattice / args.steps, "executed_per_frame": executed / args.steps,
                        "note": "lattice = plain method without skipping or termination"},
            "frame_ms": {"per_frame": kavg, "span_p50": statistics.median(frame_ms), "span_max": max(frame_ms),
                         "host_submit": 1000.0 * fl.host_s / args.steps,
                         "note": f"per_frame = timed region / frames with {S} frames in flight; span = one "
                                 f"frame's own start-to-end on its stream"},
            "e2e": {"value": e2e_fps, "unit": "frames/s", "h2d_bytes_per_step": 184,
                    "d2h_bytes_per_step": w * h * 4,
                    "path": f"ivr_set_view + ivr_render: host STATE in, each RGBA8 frame stored by its launch into "
                            f"page-locked host memory, {S} frames in flight, timed until the last is in host memory",
                    "one_at_a_time": {"value": whole_job_rate(args.steps, world, sync_ms), "unit": "frames/s",
                                      "path": "ivr_render_host, which waits for each frame"}},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": profiled_traffic(args.workload), "peak_source": how,
                         "algorithmic_bytes_per_launch": alg_bytes,
                         "note": "per frame: macrocells an executed sample read + RGBA8 output, over the frame's "
                                 "CUDA-event time (the judged march and its compare and gated launches)"},
            "sample_roofline": {"bound": "sampler", "achieved": ex_rate, "peak": sample_peak, "unit": "Gsamples/s",
                                "frac": ex_rate / sample_peak,
                                "note": "executed samples/s of the frame against ivr_sample_peak (u16): the same "
                                        "sampler, LUT fetch and blend alone on a cache-resident brick"},
            "judge_timed_frames": judge_timed,
            "methods": methods,
            "training": training, "ingest": ingest,
            "gpu_launches": args.steps * ((LAUNCHES_LEARNED if skip == api.SKIP_LEARNED else
                                           LAUNCHES_GRID if skip == api.SKIP_GRID else 1)
                                          - (2 if args.tiles == "raster" and skip != api.SKIP_NONE else 0)),
            "clocks": clk.summary(),
        }
        if not args.no_cpu_baseline and world == 1:
            line["cpu_baseline"] = _learned_cpu_baseline(ctx, v, vol, tfs, luts, frames[args.warmup:], L, params,
                                                         stream, args.cpu_budget)
    fl.free()
    v.set_mlp(None)
    mlp.free()
    for tf in tfs:
        tf.free()
    v.free()
    ctx.close()
    del vol
    torch.cuda.empty_cache()
    if line is not None and not quiet:
        print(json.dumps(line), flush=True)
    return line


def _learned_cpu_baseline(ctx, v, vol, tfs, luts, frames, L, params, stream, budget_s):
    """The oracle on bands of the timed frames (all host threads, then one
    thread), each band compared with the same rows of the GPU's frame."""
    import torch
    from oracle import oracle
    w, h = L["image"]
    scale = workloads.lut_scale(L["dtype"])
    prep = oracle.Prepared(vol, L["bricks"])
    view = ctx.view()
    cache = {}

    def gpu_frame(i):
        if i not in cache:
            cache.clear()
            st, t = frames[i]
            o32 = torch.empty((h, w, 4), dtype=torch.float32, device="cuda")
            o8 = torch.empty((h, w, 4), dtype=torch.uint8, device="cuda")
            view.set(v, st, params)
            view.render(tfs[t], o32.data_ptr(), o8.data_ptr(), stream.cuda_stream)
            torch.cuda.synchronize()
            cache[i] = (o32.cpu().numpy(), o8.cpu().numpy())
        return cache[i]

    cf = [(st, luts[t]) for st, t in frames]
    cores = os.cpu_count() or 1
    allc = oracle_bands(vol, prep, cf, L["bricks"], L["step"], L["term"], scale, cores, budget_s * 0.6, 16,
                        gpu_frame=gpu_frame)
    one = oracle_bands(vol, prep, cf, L["bricks"], L["step"], L["term"], scale, 1, budget_s * 0.2, 2)
    view.free()
    return {"value": allc["fps"], "unit": "frames/s", "cores": cores, "kind": "port",
            "sample": f"{allc['bands']} bands of {allc['band_rows']} of {h} rows of the timed frames (oracle, "
                      f"CONFIG preset, no skipping), {allc['seconds']:.1f} s",
            "one_thread": {"value": one["fps"], "unit": "frames/s", "cores": 1,
                           "sample": f"{one['bands']} bands, {one['seconds']:.1f} s"},
            "parity": dict(allc["parity"], tolerance="max |d| <= 1 on RGBA8 (1/255), <= 1e-4 relative on RGBA32",
                           note="each oracle band against the same rows of the GPU frame (learned skipping, "
                                "judged) of the same view and TF")}


def run_reference_learned(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import oracle
    L = LEARNED_CASES[args.workload]
    vol = workloads.learned_volume(L, device=_gen_device())
    luts = workloads.learned_tfs(L)
    nsteps = args.steps + args.warmup
    states = workloads.learned_views(L, n=max(len(luts), nsteps))
    frames = [(states[k], luts[k % len(luts)]) for k in range(nsteps)]
    w, h = L["image"]
    band = h // 16
    cores = os.cpu_count() or 1
    scale = workloads.lut_scale(L["dtype"])
    prep = oracle.Prepared(vol, L["bricks"])  # volume load: outside the timing, as for the GPU

    def step(k):
        st, lut = frames[k]
        b = k % 16
        oracle.render(vol, st, lut, 0, 6, preset=1, procdims=L["bricks"], step=L["step"], term_alpha=L["term"],
                      lut_scale=scale, rows=(b * band, (b + 1) * band), threads=cores, prepared=prep)

    for k in range(args.warmup):
        step(k)
    t0 = time.perf_counter()
    for k in range(args.steps):
        step(args.warmup + k)
    el = time.perf_counter() - t0
    fps = (args.steps / 16.0) / el
    line = {"impl": "reference", "metric": METRIC, "value": fps, "unit": "frames/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * el / max(args.steps, 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u16",
            "data": "synthetic (seeded blobs, 70% zero macrocells, random 16-knot TFs; the reference's datasets "
                    "are not available)",
            "config": learned_config(args, L),
            "cpu_baseline": {"value": fps, "unit": "frames/s", "cores": cores, "kind": "port",
                             "sample": f"each step renders 1/16 of the rows ({band} of {h}) of the step's frame "
                                       f"(oracle, CONFIG preset, no skipping: the reference samples every lattice "
                                       f"point); value = steps/16 frames over the time"},
            "e2e": {"value": fps, "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------------------
# sorted_brick_512
# --------------------------------------------------------------------------

def sorted_config(args, wl, name):
    w, h = wl["image"]
    return {"workload": name, "volume": "x".join(map(str, wl["shape"][::-1])) + " " + wl["dtype"],
            "bricks": "x".join(map(str, wl["bricks"])) + " + 1-voxel halo", "image": f"{w}x{h}",
            "step_voxels": wl["step"], "early_termination_alpha": wl["term"],
            "skip": f"macrocell grid of {args.cell}^3-voxel cells",
            "tile_order": "costliest first (estimated)" if args.tiles == "cost" else "row order",
            "frames_in_flight": getattr(args, "inflight", 4),
            "tf": "256-entry RGBA FP32 ramp", "l2": "inputs larger than L2 (volume resident, > 129 MB)",
            "parallelism": f"replicas x{args.gpus}"}


def measure_cells(v, fl, view, tf, params, states, args, ref8, cell):
    """frames/s and executed samples of the timed views with the volume's
    macrocell edge switched to `cell` (outside the headline's timed region,
    the same frames in flight), and whether the last frame is the headline's
    frame bit for bit."""
    import torch
    v.macrocell(cell)
    with torch.cuda.stream(fl.streams[0]):
        for k in range(args.warmup):
            fl.render(k, v, states[k], params, tf)
        torch.cuda.synchronize()
        last = args.warmup + args.steps - 1
        ms = fl.timed(range(args.warmup, last + 1), lambda k: fl.render(k, v, states[k], params, tf))
    same = bool(torch.equal(fl.dev[last % fl.S], ref8))
    executed = 0
    for st in states[args.warmup:]:
        view.set(v, st, params)
        executed += view.census(tf, fl.streams[0].cuda_stream)["executed"]
    return {"fps": args.steps / (ms / 1000.0), "executed_per_frame": executed / args.steps,
            "last_frame_equal": same}


def run_sorted(args, quiet=False, name="sorted_brick_512"):
    """The 512^3 f32 sorted-brick workload (or prof_384 / plain_128)."""
    import torch
    import torch.distributed as dist
    from ivr_gb300 import api, synth
    wl = RENDER[name]
    world = int(os.environ.get("WORLD_SIZE", "1")) if not quiet else 1
    rank = int(os.environ.get("RANK", "0")) if not quiet else 0
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1 and not dist.is_initialized():
        dist.init_process_group("nccl")

    vol = workloads.render_volume(wl, f"cuda:{local}")
    torch.cuda.empty_cache()
    w, h = wl["image"]
    nviews = args.steps + args.warmup
    states = workloads.render_views(wl, nviews, seed_offset=100 + 7919 * rank)
    lut = synth.ramp_tf(256)

    ctx = api.Context(local)
    v = ctx.load_volume(vol).bricks(*wl["bricks"], overlap=1).quads(not args.linear).macrocell(args.cell)
    tf = ctx.transfer_function().set_lut(lut, 0, workloads.lut_scale(wl["dtype"]), api.TF_F2B)
    tiles = tile_order(args)
    params = api.config_params(step=wl["step"], term_alpha=wl["term"], skip=True, tiles=tiles)
    view = ctx.view()
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream
    o8 = torch.empty((h, w, 4), dtype=torch.uint8, device="cuda")

    # the plain march (no skipping) on the first views: its executed
    # samples/s against the sample-rate roofline (outside the timed region)
    plain_view = ctx.view()
    plain_params = api.config_params(step=wl["step"], term_alpha=wl["term"], skip=False)
    p_exec, p_touched, p_ms = 0, 0, 0.0
    for st in states[args.warmup:args.warmup + 3]:
        plain_view.set(v, st, plain_params)
        c = plain_view.census(tf, sp)
        p_exec += c["executed"]
        p_touched += c["touched_bytes"]
        plain_view.render(tf, None, o8.data_ptr(), sp)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        plain_view.render(tf, None, o8.data_ptr(), sp)
        e1.record(stream)
        torch.cuda.synchronize()
        p_ms += e0.elapsed_time(e1)
    plain_view.free()
    # the same three views with frames in flight (as the timed frames run):
    # frame k renders view k mod 3 on view and stream k mod S
    pf = InFlight(ctx, args.inflight, stream, h, w)
    preps = 3

    def plain_frame(k):
        pf.render(k, v, states[args.warmup + k % 3], plain_params, tf)

    with torch.cuda.stream(stream):
        for k in range(3):
            plain_frame(k)
        torch.cuda.synchronize()
        pin_ms = pf.timed(range(3 * preps), plain_frame)
    pf.free()

    lattice = executed = touched = 0
    for st in states[args.warmup:]:
        view.set(v, st, params)
        c = view.census(tf, sp)
        lattice += c["lattice"]
        executed += c["executed"]
        touched += c["touched_bytes"]
    torch.cuda.synchronize()

    fl = InFlight(ctx, args.inflight, stream, h, w)
    S = fl.S

    def frame(k, host=False):
        fl.render(k, v, states[k], params, tf, host)

    timed_ks = range(args.warmup, args.warmup + args.steps)
    with torch.cuda.stream(stream):
        for k in range(args.warmup):
            frame(k)
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()
        with ClockSampler(local) as clk, nvtx_range("timed"):
            t_ms = fl.timed(timed_ks, frame, ev)
        if world > 1:
            dist.barrier()
        kern_ms = [a.elapsed_time(b) for a, b in ev]

        for k in range(args.warmup):
            frame(k, True)
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
        e2e_s = fl.wall(timed_ks, lambda k: frame(k, True))
        host8 = fl.host[0].numpy()
        t0 = time.perf_counter()
        for k in timed_ks:
            view.render_host(v, tf, states[k], params, host8, sp)
        sync_s = time.perf_counter() - t0
        o8.copy_(fl.dev[(args.warmup + args.steps - 1) % S])  # the last timed frame (other edges compare with it)

    t_ms, e2e_ms, sync_ms = max_over_ranks([t_ms, e2e_s * 1000.0, sync_s * 1000.0], "cuda")
    fps = whole_job_rate(args.steps, world, t_ms)
    e2e_fps = whole_job_rate(args.steps, world, e2e_ms)
    gsps = lattice * world / (t_ms / 1000.0) / 1e9

    line = None
    if rank == 0:
        kavg = t_ms / args.steps  # device time per frame, frames overlapping
        peak, how = peaks()
        sample_peak = ctx.sample_peak(v.dtype, sp)
        layouts = {}
        for lname, code in (("corner_packed", api.SAMPLER_QUADS), ("bricks", api.SAMPLER_BRICKS),
                            ("texture_point_x8", api.SAMPLER_TEX_POINT),
                            ("texture_filtered", api.SAMPLER_TEX_LINEAR)):
            g, err = ctx.sample_peak_layout(v.dtype, code, sp)
            layouts[lname] = {"gsamples_per_s": g, "max_abs_sample_err": err}
        other_cells = {}
        if world == 1 and not args.no_extras:
            for cell in ((8,) if args.cell != 8 else (16,)):
                other_cells[f"{cell}^3"] = measure_cells(v, fl, view, tf, params, states, args, o8, cell)
            v.macrocell(args.cell)
        alg_bytes = touched / args.steps + w * h * 4
        achieved = alg_bytes / (kavg / 1000.0) / 1e9
        plain_rate = p_exec / (p_ms / 1000.0) / 1e9
        plain_rate_if = p_exec * preps / (pin_ms / 1000.0) / 1e9
        tex_peak = layouts["texture_filtered"]["gsamples_per_s"]
        line = {
            "metric": METRIC, "value": fps, "unit": "frames/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": wl["dtype"],
            "data": "synthetic (seeded blobs + value noise; the reference's datasets are not available)",
            "config": sorted_config(args, wl, name),
            "gsamples_per_s": gsps,
            "samples": {"lattice_per_frame": lattice / args.steps, "executed_per_frame": executed / args.steps,
                        "note": "lattice = plain method without skipping or termination"},
            "frame_ms": {"per_frame": kavg, "span_p50": statistics.median(kern_ms), "span_max": max(kern_ms),
                         "host_submit": 1000.0 * fl.host_s / args.steps,
                         "note": f"per_frame = timed region / frames with {S} frames in flight; span = one "
                                 f"frame's own start-to-end on its stream"},
            "e2e": {"value": e2e_fps, "unit": "frames/s", "h2d_bytes_per_step": 184,
                    "d2h_bytes_per_step": w * h * 4,
                    "path": f"ivr_set_view + ivr_render: host STATE in, each RGBA8 frame stored by its launch into "
                            f"page-locked host memory, {S} frames in flight, timed until the last is in host memory",
                    "one_at_a_time": {"value": whole_job_rate(args.steps, world, sync_ms), "unit": "frames/s",
                                      "path": "ivr_render_host, which waits for each frame"}},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": profiled_traffic(name), "peak_source": how,
                         "algorithmic_bytes_per_launch": alg_bytes,
                         "note": "algorithmic bytes = macrocells an executed sample read + RGBA8 output"},
            "sample_roofline": {"bound": "sampler", "achieved": executed / args.steps / (kavg / 1000.0) / 1e9,
                                "peak": sample_peak, "unit": "Gsamples/s",
                                "frac": executed / args.steps / (kavg / 1000.0) / 1e9 / sample_peak,
                                "note": "executed samples/s of the render launch against ivr_sample_peak"},
            "sampler_layouts": dict(layouts, note="the sampler roofline through each layout of a cache-resident "
                                    "64^3 brick: the march reads corner_packed; bricks (8 gathers) and 8 point "
                                    "texture fetches give the same samples; one filtered texture fetch has "
                                    "fixed-point weights (errors in volume units; values span 0-255)"),
            "plain_kernel": {"executed_gsamples_per_s": plain_rate,
                             "frac_of_sample_roofline": plain_rate / sample_peak,
                             "frac_of_filtered_texture_peak": plain_rate / tex_peak,
                             "hbm_gb_per_s": (p_touched + 3 * w * h * 4) / (p_ms / 1000.0) / 1e9,
                             "frac_of_hbm": (p_touched + 3 * w * h * 4) / (p_ms / 1000.0) / 1e9 / peak,
                             "ms_per_frame": p_ms / 3,
                             "in_flight": {"executed_gsamples_per_s": plain_rate_if,
                                           "frac_of_sample_roofline": plain_rate_if / sample_peak,
                                           "frac_of_filtered_texture_peak": plain_rate_if / tex_peak,
                                           "ms_per_frame": pin_ms / (3 * preps),
                                           "note": f"the same 3 views rendered {preps} times each with "
                                                   f"{pf.S} frames in flight, as the timed frames run"},
                             "note": "the march without skipping (the plain method) on 3 of the views, one "
                                     "frame at a time; "
                                     "filtered-texture peak = one hardware-filtered 3D-texture fetch per sample "
                                     "(the hardware trilinear ceiling); hbm = compulsory bytes (the macrocells an "
                                     "executed sample read + RGBA8 out) over the frame time"},
            "gpu_launches": args.steps * (LAUNCHES_GRID if args.tiles == "cost" else 1),
            "clocks": clk.summary(),
        }
        if other_cells:
            line["other_macrocell_edges"] = dict(other_cells, note=(
                "the same views with the skipping grid's cells of another edge (ivr_volume_set_macrocell); "
                "the line uses the configuration's 16^3-voxel cells; the images are the same"))
        if not args.no_cpu_baseline and world == 1:
            from oracle import oracle
            prep = oracle.Prepared(vol, wl["bricks"])
            cache = {}

            def gpu_frame(i):
                if i not in cache:
                    cache.clear()
                    o32 = torch.empty((h, w, 4), dtype=torch.float32, device="cuda")
                    o8b = torch.empty((h, w, 4), dtype=torch.uint8, device="cuda")
                    view.set(v, states[args.warmup + i], params)
                    view.render(tf, o32.data_ptr(), o8b.data_ptr(), sp)
                    torch.cuda.synchronize()
                    cache[i] = (o32.cpu().numpy(), o8b.cpu().numpy())
                return cache[i]

            cf = [(st, lut) for st in states[args.warmup:]]
            cores = os.cpu_count() or 1
            allc = oracle_bands(vol, prep, cf, wl["bricks"], wl["step"], wl["term"], 1.0, cores,
                                args.cpu_budget * 0.4, 16, gpu_frame=gpu_frame)
            one = oracle_bands(vol, prep, cf, wl["bricks"], wl["step"], wl["term"], 1.0, 1, args.cpu_budget * 0.1, 1)
            line["cpu_baseline"] = {
                "value": allc["fps"], "unit": "frames/s", "cores": cores, "kind": "port",
                "sample": f"{allc['bands']} bands of {allc['band_rows']} of {h} rows of the timed frames (oracle, "
                          f"CONFIG preset, no skipping), {allc['seconds']:.1f} s",
                "one_thread": {"value": one["fps"], "unit": "frames/s", "cores": 1,
                               "sample": f"{one['bands']} bands, {one['seconds']:.1f} s"},
                "parity": dict(allc["parity"], tolerance="max |d| <= 1 on RGBA8 (1/255), <= 1e-4 relative on RGBA32",
                               note="each oracle band against the same rows of the GPU frame of the same view")}
    fl.free()
    view.free()
    tf.free()
    v.free()
    ctx.close()
    del vol
    torch.cuda.empty_cache()
    if line is not None and not quiet:
        print(json.dumps(line), flush=True)
    return line


def run_reference_sorted(args, name):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import oracle
    from ivr_gb300 import synth
    wl = RENDER[name]
    vol = workloads.render_volume(wl, None if wl["shape"][0] <= 160 else _gen_device())
    w, h = wl["image"]
    states = workloads.render_views(wl, max(args.steps + args.warmup, 1))
    lut = synth.ramp_tf(256)
    band = h // 16
    cores = os.cpu_count() or 1
    prep = oracle.Prepared(vol, wl["bricks"])

    def step(k):
        b = k % 16
        oracle.render(vol, states[k % len(states)], lut, 0, 6, preset=1, procdims=wl["bricks"], step=wl["step"],
                      term_alpha=wl["term"], lut_scale=workloads.lut_scale(wl["dtype"]),
                      rows=(b * band, (b + 1) * band), threads=cores, prepared=prep)

    for k in range(args.warmup):
        step(k)
    t0 = time.perf_counter()
    for k in range(args.steps):
        step(args.warmup + k)
    el = time.perf_counter() - t0
    fps = (args.steps / 16.0) / el
    line = {"impl": "reference", "metric": METRIC, "value": fps, "unit": "frames/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * el / max(args.steps, 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": wl["dtype"],
            "data": "synthetic (seeded blobs; the reference's datasets are not available)",
            "config": sorted_config(args, wl, name),
            "cpu_baseline": {"value": fps, "unit": "frames/s", "cores": cores, "kind": "port",
                             "sample": f"each step renders 1/16 of the rows ({band} of {h}); value = steps/16 "
                                       f"frames over the time"},
            "e2e": {"value": fps, "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------------------
# batch_64x4, serve_32, REF preset
# --------------------------------------------------------------------------

def run_batch(args, quiet=False):
    """The batched workload: one batch of 64 views x 4 TFs per step."""
    import torch
    from ivr_gb300 import api, synth
    from ivr_gb300.state import orbit_state
    wl = RENDER[BATCH["base"]]
    torch.cuda.set_device(0)
    vol = workloads.render_volume(wl, "cuda:0")
    torch.cuda.empty_cache()
    ctx = api.Context(0)
    v = ctx.load_volume(vol).bricks(*wl["bricks"], overlap=1)
    del vol
    tfs = [ctx.transfer_function().set_lut(synth.knot_tf(BATCH["seed"] + t)[0], 0, 1.0, api.TF_F2B)
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
    warm = max(args.warmup, 3)
    steps = max(args.steps // 4, 3) if quiet else args.steps
    for _ in range(warm):
        b.render(use_graph=True, stream=sp)
    torch.cuda.synchronize()
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(0) as clk:
        start.record(stream)
        for _ in range(steps):
            b.render(use_graph=True, stream=sp)
        stop.record(stream)
        torch.cuda.synchronize()
    t_ms = start.elapsed_time(stop)
    gsps = lattice * steps / (t_ms / 1000.0) / 1e9
    line = {
        "metric": METRIC, "value": gsps, "unit": "Gsamples/s", "n_gpus": 1, "steps": steps,
        "warmup": warm, "ms_per_step": t_ms / steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded blobs + value noise, random 16-knot TFs)",
        "config": {"workload": "batch_64x4", "volume": "512x512x512 f32, 2x2x2 bricks + halo",
                   "frames_per_step": n, "sizes": "uniform from 256^2, 512^2, 1024^2, 1920x1080",
                   "step_voxels": "uniform 0.25-1.0", "launch": "one persistent launch per step, CUDA-graph replay",
                   "l2": "inputs larger than L2"},
        "frames_per_s": n * steps / (t_ms / 1000.0), "megapixels_per_step": pixels / 1e6,
        "lattice_per_step": lattice, "autotune": {"chosen": api.Batch.VARIANTS[variant],
                                                 "ms": dict(zip(api.Batch.VARIANTS, tune_ms))},
        "graph_replay": True,
        "gpu_launches": steps, "clocks": clk.summary(),
    }
    for view, *_ in frames:
        view.free()
    b.free()
    v.free()
    ctx.close()
    if not quiet:
        print(json.dumps(line), flush=True)
    return line


def run_serve(args, quiet=False, sweep=None):
    """The serving workload: the steering server under Poisson load; with
    `sweep` (rate multipliers) the same server is offered each multiple of
    the per-client rates in turn (the p99 curve)."""
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
        scales.append(workloads.lut_scale(dt))
        names.append("x".join(map(str, shape)) + " " + dt)
    resident = ctx.mem_used
    slots = args.serve_slots or SERVE["slots"]
    batch = args.serve_batch or SERVE["batch"]
    srv = api.Server(ctx, slots=slots, max_batch_frames=batch, arena_mib=SERVE["arena_mib"])
    ids = [srv.add_volume(v) for v in vols]
    rate = tuple(float(x) for x in args.serve_rate.split(",")) if args.serve_rate else SERVE["rate"]
    serve.run(srv, ids, scales, duration=SERVE["warm"], clients=SERVE["clients"], rate=rate, seed=1)

    def one(mult, seed, duration):
        r = (rate[0] * mult, rate[1] * mult)
        with ClockSampler(0) as clk:
            res, wall = serve.run(srv, ids, scales, duration=duration, clients=SERVE["clients"], rate=r, seed=seed)
        ok = [x for x in res if x["status"] == 0]
        lat = np.array([x["latency"] for x in ok]) * 1000.0 if ok else np.zeros(1)
        return res, ok, lat, wall, r, clk

    res, ok, lat, wall, r, clk = one(1.0, 2, SERVE["duration"])
    stats = srv.stats()
    px = sum(x["vw"] * x["vh"] for x in ok)
    curve = []
    for mult in (sweep or []):
        rs, oks, lt, wl_, rr, ck = one(mult, 10 + int(mult * 10), SERVE["duration"] / 2)
        curve.append({"rate_multiplier": mult, "offered_per_s": len(rs) / (SERVE["duration"] / 2),
                      "served_per_s": len(oks) / wl_, "p50_ms": float(np.percentile(lt, 50)),
                      "p99_ms": float(np.percentile(lt, 99)), "rejected": len(rs) - len(oks)})
    srv.close()
    line = {
        "metric": METRIC, "value": len(ok) / wall, "unit": "frames/s", "n_gpus": 1,
        "steps": len(res), "warmup": 0, "ms_per_step": 1000.0 * wall / max(len(res), 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8/u16/f32",
        "data": "synthetic (seeded blobs; Poisson arrivals)",
        "config": {"workload": "serve_32", "volumes": names, "clients": SERVE["clients"],
                   "rate_per_client": list(r), "duration_s": SERVE["duration"],
                   "sizes": "uniform from 256^2, 512^2, 1024^2, 1280x720, 1920x1080",
                   "tf_edit": "every 5th request per client", "slots": slots,
                   "max_batch_frames": batch, "arena_mib": SERVE["arena_mib"],
                   "hbm_budget_gib": SERVE["budget_gib"], "resident_volume_bytes": resident},
        "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                       "max": float(lat.max()), "from": "scheduled arrival to RGBA8 frame in host memory"},
        "latency_parts_ms": {
            k: {"p50": float(np.percentile(a, 50)), "p99": float(np.percentile(a, 99))}
            for k, a in (("generator_late", np.array([x["late"] for x in ok]) * 1000.0),
                         ("queued", np.array([x["t_queue"] for x in ok]) * 1000.0),
                         ("batch_to_host", np.array([x["t_total"] - x["t_queue"] for x in ok]) * 1000.0))},
        "requests": len(res), "rejected": len(res) - len(ok),
        "rejected_status": sorted({x["status"] for x in res if x["status"] != 0}),
        "megapixels_per_s": px / wall / 1e6, "batches": stats["batches"],
        "server_seconds": {k: stats[k] for k in ("gpu_s", "dispatch_s", "finish_s")}, "wall_s": wall,
        "clocks": clk.summary(),
    }
    if curve:
        line["saturation"] = {"points": curve, "note": "the same server offered each multiple of the per-client "
                                                       "rates for half the duration"}
    for v in vols:
        v.free()
    ctx.close()
    if not quiet:
        print(json.dumps(line), flush=True)
    return line


def run_ref_preset(args, quiet=True):
    """The drop-in path with the reference's own semantics (REF preset:
    ray-parameter step 0.001, 256-sample cap, getlinearsample weights, the
    SEISMIC2 transfer function over the seismic colormap) on the
    CPU-runnable workload (plain_128: 128^3 u8, one brick, 512x512): GPU
    frames/s, the CPU restatement on the same frames, and a bitwise check
    of one frame against it."""
    import torch
    from oracle import oracle
    from ivr_gb300 import api
    wl = RENDER["plain_128"]
    vol = workloads.render_volume(wl, None)
    w, h = wl["image"]
    states = workloads.render_views(wl, 8, seed_offset=300)
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


def _extra(fn, args, keys, **kw):
    """A workload's line reduced to `keys`, or the error it raised."""
    import torch
    try:
        full = fn(args, quiet=True, **kw)
        return {k: full[k] for k in keys if k in full}
    except Exception as e:  # reported in the line, not hidden
        return {"error": f"{type(e).__name__}: {e}"}
    finally:
        torch.cuda.empty_cache()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="learned_1024",
                    choices=sorted(LEARNED_CASES) + ["batch_64x4", "serve_32"] + sorted(RENDER))
    ap.add_argument("--skip", default="learned", choices=["learned", "grid", "none"],
                    help="learned workloads: the skipping of the timed frames (learned grid by default)")
    ap.add_argument("--train-tfs", type=int, default=0,
                    help="learned workloads: TFs whose cells train the predictor (0: the workload's 8)")
    ap.add_argument("--inflight", type=int, default=4,
                    help="frames in flight: consecutive frames alternate over this many views and streams "
                         "(measured: 4 renders learned_1024 2-3%% faster than 3, 5 no faster)")
    ap.add_argument("--no-certify", action="store_true",
                    help="learned workloads: learned grids without the cell-by-cell check against the exact test "
                         "(the per-frame judge alone guards the frames)")
    ap.add_argument("--no-methods", action="store_true",
                    help="learned workloads: leave out the comparison of the three methods over every TF")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-budget", type=float, default=20.0)
    ap.add_argument("--serve-slots", type=int, default=0)
    ap.add_argument("--serve-batch", type=int, default=0)
    ap.add_argument("--serve-rate", default="", help="per-client request rate range lo,hi (req/s)")
    ap.add_argument("--judge-stride", type=int, default=0, help="learned skipping: judge 1 in this many tiles")
    ap.add_argument("--tiles", default=None, choices=["cost", "raster"],
                    help="tile order of the skipping launches: costliest first, or row order (default: row "
                         "order for the learned workloads, costliest first for the others; measured)")
    ap.add_argument("--cell", type=int, default=16,
                    help="macrocell edge of the skipping grid in voxels (a power of two, 4-32)")
    ap.add_argument("--linear", action="store_true",
                    help="render from the bricks themselves, without the corner-packed copies")
    ap.add_argument("--no-extras", action="store_true",
                    help="the workload's own line only: no nested summaries of the other workloads")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    args.tiles_given = args.tiles
    if args.tiles is None:
        # measured with three frames in flight: row order is 4-6% faster on
        # learned_1024 (and one frame at a time too); the costliest-first
        # order ties on sorted_brick_512 in flight and wins one at a time
        args.tiles = "raster" if args.workload in LEARNED_CASES else "cost"
    if args.workload == "batch_64x4":
        return run_batch(args)
    if args.workload == "serve_32":
        return run_serve(args, sweep=[] if args.no_extras else [2.0, 3.0])
    learned = args.workload in LEARNED_CASES
    if args.impl == "reference":
        return run_reference_learned(args) if learned else run_reference_sorted(args, args.workload)
    if not learned:
        return run_sorted(args, name=args.workload)

    line = run_learned(args, quiet=True)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if line is not None and world == 1 and args.workload == "learned_1024" and not args.no_extras:
        sargs = argparse.Namespace(**vars(args))
        sargs.tiles = args.tiles_given or "cost"  # the sorted workload's own default
        line["sorted_brick_512"] = _extra(run_sorted, sargs, [
            "value", "unit", "gsamples_per_s", "frame_ms", "e2e", "roofline", "sample_roofline", "plain_kernel",
            "sampler_layouts", "samples", "other_macrocell_edges", "cpu_baseline", "config", "clocks"])
        line["batch_64x4"] = _extra(run_batch, args, ["value", "unit", "frames_per_s", "ms_per_step",
                                                      "megapixels_per_step", "autotune", "graph_replay", "config",
                                                      "clocks"])
        line["serving"] = _extra(run_serve, args, ["value", "unit", "latency_ms", "latency_parts_ms", "requests",
                                                   "rejected", "megapixels_per_s", "saturation", "config", "clocks"],
                                 sweep=[2.0, 3.0])
        line["ref_preset"] = _extra(run_ref_preset, args, ["workload", "fps", "cpu_fps", "cpu_cores", "cpu",
                                                           "bitwise_equal_to_cpu"])
    if line is not None:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        if dist.is_initialized():
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
