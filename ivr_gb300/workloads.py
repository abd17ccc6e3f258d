"""The benchmark workloads: volumes, views and transfer functions, seeded.

The reference's datasets are not available, so every workload is a seeded
synthetic input with the shape, size and value distribution it names.  The
benchmark (bench.py) and the workload-scale parity tests build their inputs
from here, so the frames the tests check are the frames the benchmark times.

* ``plain_128``: 128^3 u8, 8 blobs + uniform noise +-0.05, one brick,
  512x512, the 256-entry ramp TF, step 0.5 voxel, termination at 0.99.
* ``sorted_brick_512``: 512^3 f32, 64 blobs + 3-octave value noise (0.1),
  2x2x2 bricks with a one-voxel halo, 1024x1024, 16^3 macrocells.
* ``learned_1024``: 1024^3 u16 (2 GiB), 256 blobs, 70% of the 16^3
  macrocells exactly zero, 1920x1080, 50 random 16-knot TFs (60% of the
  opacity knots zero, the lowest fifteenth of the range transparent).
* ``batch_64x4``: 64 views x 4 TFs on the sorted_brick_512 volume, sizes
  from {256^2, 512^2, 1024^2, 1920x1080}, steps 0.25-1.0 voxel.
* ``serve_32``: 32 Poisson clients at 10-60 requests/s over 4 resident
  volumes (256^3 u8, 512^3 u16, 512^3 f32, 1024^3 u16).
"""
from __future__ import annotations

import numpy as np

from . import synth
from .state import orbit_state

RENDER = {
    "sorted_brick_512": dict(shape=(512, 512, 512), dtype="f32", n_blobs=64, noise=0.0, value_noise=0.1,
                             bricks=(2, 2, 2), image=(1024, 1024), step=0.5, term=0.99, fovy=30.0, seed=2),
    # the same kernel and data type, smaller: the case ncu captures in full
    "prof_384": dict(shape=(384, 384, 384), dtype="f32", n_blobs=64, noise=0.0, value_noise=0.1,
                     bricks=(2, 2, 2), image=(1024, 1024), step=0.5, term=0.99, fovy=30.0, seed=2),
    "plain_128": dict(shape=(128, 128, 128), dtype="u8", n_blobs=8, noise=0.05, value_noise=0.0,
                      bricks=(1, 1, 1), image=(512, 512), step=0.5, term=0.99, fovy=30.0, seed=1),
}

# learned empty-space skipping: 1024^3 u16 of 256 blobs (sigmas scaled by
# (8/256)^(1/3) so they do not sum to saturation) with 70% of the
# macrocells exactly zero, 1920x1080, 50 random 16-knot TFs; the predictor
# is trained on the exact bounds of 8 of them (64^3 cells x 8 = 2.1M samples),
# an opaque cell's under-prediction weighted 16x (measured on GB300 over the
# 42 other TFs: fewer samples than at 4x or 32x, and no TF whose learned grid
# came out nearly all opaque)
LEARNED = dict(shape=(1024, 1024, 1024), dtype="u16", n_blobs=256, sigma_scale=(8 / 256) ** (1 / 3),
               zero_fraction=0.7, image=(1920, 1080), bricks=(1, 1, 1),
               step=0.5, term=0.99, fovy=30.0, seed=3, tfs=50, train_tfs=8, epochs=30, batch_rows=8192, lr=2e-3,
               wneg=16.0, slack=0.02, judge_stride=16, frames=3)
# the same at 256^3 and 1280x720 with 10 TFs: a small case for quick runs
LEARNED_SMALL = dict(LEARNED, shape=(256, 256, 256), n_blobs=32, sigma_scale=(8 / 32) ** (1 / 3), image=(1280, 720),
                     tfs=10, train_tfs=4, epochs=5)
# the learned_1024 volume at half the resolution (the same blobs, 32^3
# macrocells, 256 MiB + 1 GiB of corner-packed copy), the same image and
# TFs: the case ncu captures in full
LEARNED_HALF = dict(LEARNED, shape=(512, 512, 512))
LEARNED_CASES = {"learned_1024": LEARNED, "learned_256": LEARNED_SMALL, "learned_512": LEARNED_HALF}

BATCH = dict(base="sorted_brick_512", views=64, tfs=4, sizes=[(256, 256), (512, 512), (1024, 1024), (1920, 1080)],
             steps=(0.25, 1.0), seed=40)

SERVE = dict(volumes=[((256, 256, 256), "u8", 8, 0.05, 0.0, 0.0), ((512, 512, 512), "u16", 64, 0.0, 0.0, 0.0),
                      ((512, 512, 512), "f32", 64, 0.0, 0.1, 0.0), ((1024, 1024, 1024), "u16", 256, 0.0, 0.0, 0.7)],
             clients=32, rate=(10.0, 60.0), duration=10.0, warm=2.0, slots=4, batch=16, arena_mib=160,
             budget_gib=32)


def lut_scale(dtype: str) -> float:
    """LUT index = (int)(value * scale): 256 entries over the u16 range."""
    return 256.0 / 65536.0 if dtype == "u16" else 1.0


def render_volume(wl: dict, device=None) -> np.ndarray:
    """The volume of a RENDER workload, (d, h, w) in its dtype."""
    return synth.blob_volume(wl["shape"], n_blobs=wl["n_blobs"], seed=wl["seed"], dtype=wl["dtype"],
                             noise=wl["noise"], value_noise=wl["value_noise"], device=device)


def render_views(wl: dict, n: int, seed_offset: int = 100) -> list:
    """n seeded views of a RENDER workload: the camera at distance 5 in a
    seeded azimuth/elevation direction, the workload's field of view."""
    w, h = wl["image"]
    rng = np.random.default_rng(wl["seed"] + seed_offset)
    out = []
    for _ in range(n):
        az, el = float(rng.uniform(0, 360)), float(rng.uniform(-60, 60))
        out.append(orbit_state(az, el, w, h, fovy=wl["fovy"], alpha=1.0))
    return out


def learned_volume(L: dict = LEARNED, device=None) -> np.ndarray:
    return synth.blob_volume(L["shape"], n_blobs=L["n_blobs"], seed=L["seed"], dtype=L["dtype"], noise=0.0,
                             zero_fraction=L["zero_fraction"], device=device, sigma_scale=L["sigma_scale"])


def learned_tfs(L: dict = LEARNED) -> list:
    """The workload's random 16-knot TFs (256-entry RGBA FP32 LUTs)."""
    return [synth.knot_tf(1000 + t, zero_first=True)[0] for t in range(L["tfs"])]


def learned_views(L: dict = LEARNED, n: int = 0, seed_offset: int = 77) -> list:
    """One seeded view per TF (or n views)."""
    w, h = L["image"]
    rng = np.random.default_rng(L["seed"] + seed_offset)
    return [orbit_state(float(rng.uniform(0, 360)), float(rng.uniform(-60, 60)), w, h, fovy=L["fovy"])
            for _ in range(n or L["tfs"])]
