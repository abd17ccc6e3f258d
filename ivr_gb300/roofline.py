"""Sample-rate roofline of the CONFIG sampler on this GPU, per layout.

    python -m ivr_gb300.roofline [--dtype u8|u16|f32|all]

Prints one JSON object: for each dtype and sampler layout
(ivr_sample_peak_layout) the samples/s of the sampler alone on a
cache-resident 64^3 brick and the largest sample error against the exact
trilinear sample.
"""
from __future__ import annotations

import argparse
import json

from . import api

LAYOUTS = {"corner_packed": api.SAMPLER_QUADS, "bricks": api.SAMPLER_BRICKS,
           "texture_point_x8": api.SAMPLER_TEX_POINT, "texture_filtered": api.SAMPLER_TEX_LINEAR}
DTYPES = {"u8": api.U8, "u16": api.U16, "f32": api.F32}


def measure(ctx: api.Context, dtypes) -> dict:
    out = {}
    for dn in dtypes:
        out[dn] = {}
        for ln, code in LAYOUTS.items():
            g, err = ctx.sample_peak_layout(DTYPES[dn], code)
            out[dn][ln] = {"gsamples_per_s": round(g, 1), "max_abs_sample_err": err}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--dtype", default="all", choices=["all", *DTYPES])
    ap.add_argument("--device", type=int, default=0)
    a = ap.parse_args()
    ctx = api.Context(a.device)
    print(json.dumps(measure(ctx, list(DTYPES) if a.dtype == "all" else [a.dtype])))


if __name__ == "__main__":
    main()
