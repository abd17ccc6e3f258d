"""Load generator for the steering server (the serving workload).

Simulated clients send requests with Poisson arrivals: each of the
``clients`` draws a rate uniform in ``rate`` (requests/s) and exponential
inter-arrival times.  Each request picks one of the resident volumes, a
random view and an image size from ``sizes``; every 5th request of a client
edits that client's transfer function (a new 16-knot TF).  The generator
submits at the scheduled times and reports latency from the scheduled
arrival to the frame in host memory, so generator lateness counts against
the server.
"""
from __future__ import annotations

import time

import numpy as np

from . import synth
from .state import orbit_state

SIZES = [(256, 256), (512, 512), (1024, 1024), (1280, 720), (1920, 1080)]


def schedule(clients=32, rate=(10.0, 60.0), duration=5.0, seed=0):
    """[(t, client)] sorted by arrival time."""
    rng = np.random.default_rng(seed)
    ev = []
    for c in range(clients):
        lam = rng.uniform(*rate)
        t = rng.exponential(1.0 / lam)
        while t < duration:
            ev.append((t, c))
            t += rng.exponential(1.0 / lam)
    ev.sort()
    return ev


def run(server, volumes, scales, duration=5.0, clients=32, rate=(10.0, 60.0), sizes=SIZES, seed=0,
        tf_every=5, keep_frames=False):
    """Drives `server` (ivr_gb300.api.Server) for `duration` seconds.
    volumes: server volume ids; scales: LUT scale per volume.  Frames land in
    a pool of page-locked buffers that is reused as requests complete (as a
    client reuses its frame buffer).  Returns the completions and the wall
    time."""
    rng = np.random.default_rng(seed + 1)
    events = schedule(clients, rate, duration, seed)
    client_tf = {}
    sent = {}
    # (vh, vw) -> free page-locked frames, kept on the server so that runs
    # after a warm-up one find their buffers allocated
    pool = server.__dict__.setdefault("_frame_pool", {})

    def frame_for(w, h):
        free = pool.setdefault((h, w), [])
        return free.pop() if free else server.ctx.host_frame(h, w)

    def collect(got):
        for r in got:
            f = r.get("frame")
            if f is not None:
                if keep_frames:
                    r["frame"] = f.copy()
                pool.setdefault(f.shape[:2], []).append(f)
            done.append(r)
    for c in range(clients):  # every client starts with its own TF per volume scale
        client_tf[c] = {s: server.add_tf(synth.knot_tf(seed * 1000 + c)[0], 0, s) for s in set(scales)}
    count = {c: 0 for c in range(clients)}
    done = []
    t0 = time.perf_counter()
    for tag, (t_arr, c) in enumerate(events):
        count[c] += 1
        if count[c] % tf_every == 0:
            client_tf[c] = {s: server.add_tf(synth.knot_tf(seed * 1000 + c + 7919 * count[c])[0], 0, s)
                            for s in set(scales)}
        vi = int(rng.integers(len(volumes)))
        w, h = sizes[int(rng.integers(len(sizes)))]
        st = orbit_state(float(rng.uniform(0, 360)), float(rng.uniform(-60, 60)), w, h, fovy=30.0, alpha=1.0)
        now = time.perf_counter() - t0
        if now < t_arr:
            time.sleep(t_arr - now)
        late = max(0.0, time.perf_counter() - t0 - t_arr)
        server.submit(volumes[vi], client_tf[c][scales[vi]], st, tag, out=frame_for(w, h))
        sent[tag] = (late, vi, (w, h), st, client_tf[c][scales[vi]])
        collect(server.poll(wait_ms=0))
    while len(done) < len(events):
        got = server.poll(wait_ms=50)
        if not got and time.perf_counter() - t0 > duration + 60:
            break
        collect(got)
    wall = time.perf_counter() - t0
    out = []
    for r in done:
        late, vi, size, st, tf = sent[r["tag"]]
        r = dict(r)
        r["latency"] = r["t_total"] + late
        r["late"] = late
        r["volume"], r["size"], r["state"], r["tf"] = vi, size, st, tf
        if not keep_frames:
            r.pop("frame", None)
        out.append(r)
    return out, wall
