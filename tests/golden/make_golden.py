"""Generates the golden fixtures under tests/golden/ by running the
reference's own C code (O1: oracle/_ref/libivr_ref.so, built from the
reference sources by oracle/Makefile).

Each fixture is one steered frame: the inputs (volume, STATE, colormap or
injected LUT, transfer function id, brick grid, tile size) and the
reference's outputs (composited RGBA32 frame, per-brick sub-images, window
rectangles, LUT).  The reference has no tests or golden data of its own;
these frames are what it computes for seeded synthetic volumes.

Run from the repository root, where the reference checkout is available:
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from ivr_gb300 import synth  # noqa: E402
from ivr_gb300.state import NO_CLIP, orbit_state  # noqa: E402
from oracle import oracle  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))

# name: volume spec, view, colormap, xfer, procdims, tile, extras
CASES = {
    "chem_jet_1brick": dict(shape=(20, 24, 28), seed=3, view=(30, 20), win=(64, 48), cm=4, xfer=3),
    "seismic2_jet_8bricks": dict(shape=(20, 24, 28), seed=3, view=(30, 20), win=(64, 48), cm=4, xfer=2,
                                 procdims=(2, 2, 2)),
    "seismic_base": dict(shape=(22, 18, 26), seed=5, view=(-40, 10), win=(56, 40), cm=0, xfer=0),
    "med_medical": dict(shape=(22, 18, 26), seed=5, view=(120, -15), win=(56, 40), cm=2, xfer=1),
    "blend_jet": dict(shape=(24, 24, 24), seed=7, view=(200, 35), win=(48, 48), cm=4, xfer=4),
    "rgb_seismic": dict(shape=(18, 20, 16), seed=9, view=(75, -30), win=(40, 40), cm=3, xfer=5),
    "chem_clip": dict(shape=(24, 24, 24), seed=11, view=(20, 25), win=(48, 48), cm=4, xfer=3,
                      clip=(0.6, 0.25, 0.9, 0.5, NO_CLIP, 0.7)),
    "chem_f32_values": dict(shape=(20, 22, 18), seed=13, view=(300, 40), win=(48, 40), cm=4, xfer=3,
                            dtype="f32", value_noise=0.1),
    "chem_bigendian": dict(shape=(16, 20, 24), seed=15, view=(45, 0), win=(40, 32), cm=4, xfer=3,
                           big_endian=True),
    "seismic2_injected_lut": dict(shape=(24, 20, 22), seed=17, view=(160, 10), win=(48, 40), cm=-1, xfer=2,
                                  inject="ramp"),
    "chem_bricks_2x3x1_remainder": dict(shape=(19, 25, 29), seed=19, view=(-70, -20), win=(56, 48), cm=4, xfer=3,
                                        procdims=(2, 3, 1), tile=(8, 8)),
    "seismic2_axis_view_ties": dict(shape=(24, 24, 24), seed=21, view=(0, 0), win=(48, 48), cm=4, xfer=2,
                                    procdims=(2, 2, 2)),
    "seismic2_lutoffset_range": dict(shape=(20, 20, 24), seed=23, view=(100, 30), win=(48, 40), cm=4, xfer=2,
                                     value_range=(40, 200), procdims=(1, 2, 1)),
    "chem_lutoffset_medical": dict(shape=(20, 20, 24), seed=25, view=(250, -25), win=(48, 40), cm=2, xfer=3,
                                   value_range=(17, 240)),
}


def make(name, c):
    dtype = c.get("dtype", "u8")
    vol = synth.blob_volume(c["shape"], n_blobs=8, seed=c["seed"], dtype=dtype,
                            value_noise=c.get("value_noise", 0.0))
    if "value_range" in c:  # shift the data so the LUT offset is not zero
        lo, hi = c["value_range"]
        vol = np.rint(lo + vol.astype(np.float64) * (hi - lo) / 255.0).astype(vol.dtype)
    volf = vol.astype(np.float32)
    az, el = c["view"]
    w, h = c["win"]
    st = orbit_state(az, el, w, h, fovy=43.6028, alpha=c.get("alpha", 0.08), clip=c.get("clip"))
    procdims = c.get("procdims", (1, 1, 1))
    tile = c.get("tile", (1, 1))
    inj = None
    if c.get("inject") == "ramp":
        inj = synth.ramp_tf(256)
    r = oracle.ref_render(volf, st, c["cm"], c["xfer"], procdims=procdims, tile=tile, inj_lut=inj,
                          big_endian_file=c.get("big_endian", False), threads=1)
    vw, vh = oracle.viewport(st, tile)
    # createlocalimage writes past the right edge when a brick's rectangle
    # reaches it (main.c:959-962); fixtures keep every rectangle inside
    for k, inf in enumerate(r["info"]):
        x, wdt = inf[0], inf[3]
        assert x + wdt < vw, f"{name}: brick {k} reaches the right edge"
    np.savez_compressed(
        os.path.join(OUT, name + ".npz"),
        volume=vol, state=np.frombuffer(st.to_bytes(), np.uint8), colormap=c["cm"], xfer=c["xfer"],
        procdims=np.array(procdims, np.int32), tile=np.array(tile, np.int32),
        big_endian=bool(c.get("big_endian", False)),
        lut=r["lut"], lutoffset=r["lutoffset"], rgba32=r["rgba32"], bricks=r["bricks"], info=r["info"])
    return r


def main():
    oracle.build(ref=True)
    for name, c in CASES.items():
        r = make(name, c)
        a = r["rgba32"]
        print(f"{name:32s} lut={len(r['lut']):4d} off={r['lutoffset']:3d} mean={a.mean():.4f} "
              f"covered={(a[..., 3] > 0).mean():.2f}")


if __name__ == "__main__":
    main()
