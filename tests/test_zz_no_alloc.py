"""GPU: ivr_volume_histogram_noalloc, the entry point that allocates no
device memory, against the oracle's histogram and ivr_volume_histogram.

It serves callers that cannot call cudaMalloc/cudaFree where they build a
LUT -- a steering server whose HBM budget belongs to resident volumes, a
frame loop that cannot take cudaFree's device-wide wait while other streams
render -- from a fixed static scratch array.  This file is collected last so
that a run stopping at its first failure has already run every other test;
it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

from ivr_gb300 import synth
from ivr_gb300._lib import IvrError

pytestmark = pytest.mark.gpu

MAX_BINS = 65536


def noalloc(ctx, vol, hsize, stream=None):
    hist = np.full(hsize, -1, np.int32)
    mn, mx = ctypes.c_float(), ctypes.c_float()
    rc = ctx.lib.ivr_volume_histogram_noalloc(vol.h, hist.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), hsize,
                                              ctypes.byref(mn), ctypes.byref(mx), stream)
    ctx.check(rc)
    return hist, mn.value, mx.value


def volumes():
    """u8, u16 and f32 blob volumes, and an f32 volume whose minimum is not
    an integer (its bins start at the fractional minimum, mathutil.c:461)."""
    out = {d: synth.blob_volume((40, 36, 44), n_blobs=6, seed=4, dtype=d) for d in ("u8", "u16", "f32")}
    out["f32_frac_min"] = (synth.blob_volume((33, 29, 31), n_blobs=5, seed=6, dtype="f32") * np.float32(0.73)
                           + np.float32(12.37)).astype(np.float32)
    return out


@pytest.mark.parametrize("name", ["u8", "u16", "f32", "f32_frac_min"])
def test_noalloc_histogram_matches_oracle_and_allocating_entry_point(ctx, oracle_mod, name):
    vol = volumes()[name]
    omn, omx, ohist = oracle_mod.minmax_histogram(vol)
    v = ctx.load_volume(vol)
    try:
        mn, mx = v.minmax()
        assert (mn, mx) == (omn, omx)
        hsize = int((mx - mn) + 1)
        assert hsize == len(ohist) <= MAX_BINS
        ref = v.histogram(hsize)
        assert np.array_equal(ref, ohist)
        for _ in range(2):  # two calls in a row share (and reuse) the scratch array
            hist, a, b = noalloc(ctx, v, hsize)
            assert (a, b) == (omn, omx)
            assert np.array_equal(hist, ohist)
    finally:
        v.free()


def test_noalloc_histogram_on_a_stream_of_its_own(ctx, oracle_mod):
    """The work queued on a caller's non-default stream, with other work
    queued on that stream before it; the caller's current device is the
    same afterwards."""
    import torch
    vol = volumes()["u16"]
    omn, omx, ohist = oracle_mod.minmax_histogram(vol)
    v = ctx.load_volume(vol)
    try:
        s = torch.cuda.Stream()
        junk = torch.empty(1 << 22, dtype=torch.float32, device="cuda")
        dev = torch.cuda.current_device()
        for _ in range(2):
            with torch.cuda.stream(s):
                junk.uniform_()  # earlier work on the same stream
            hist, a, b = noalloc(ctx, v, len(ohist), stream=s.cuda_stream)
            assert (a, b) == (omn, omx)
            assert np.array_equal(hist, ohist)
        assert torch.cuda.current_device() == dev
    finally:
        v.free()


def test_noalloc_histogram_smaller_then_larger_bins(ctx):
    # a call with fewer bins leaves stale counts above them; the next call
    # must still start from zero
    vol = synth.blob_volume((30, 30, 30), n_blobs=5, seed=8, dtype="u16")
    v = ctx.load_volume(vol)
    try:
        mn, mx = v.minmax()
        hsize = int((mx - mn) + 1)
        small, _, _ = noalloc(ctx, v, max(1, hsize // 3))
        assert np.array_equal(small, v.histogram(max(1, hsize // 3)))
        full, _, _ = noalloc(ctx, v, hsize)
        assert np.array_equal(full, v.histogram(hsize))
    finally:
        v.free()


def test_noalloc_takes_no_device_memory(ctx):
    import torch
    vol = synth.blob_volume((48, 48, 48), n_blobs=6, seed=9, dtype="u8")
    v = ctx.load_volume(vol)
    try:
        noalloc(ctx, v, 256)  # first call on the device: symbol lookup
        torch.cuda.synchronize()
        used_lib = ctx.mem_used
        free0 = torch.cuda.mem_get_info()[0]
        for _ in range(3):
            noalloc(ctx, v, 256)
        assert torch.cuda.mem_get_info()[0] == free0
        assert ctx.mem_used == used_lib
    finally:
        v.free()


def test_noalloc_rejects_more_bins_than_its_scratch(ctx):
    v = ctx.load_volume(np.zeros((8, 8, 8), np.uint8))
    try:
        with pytest.raises(IvrError) as e:
            noalloc(ctx, v, MAX_BINS + 1)
        assert e.value.code == -1 and "65536" in str(e.value)
    finally:
        v.free()
