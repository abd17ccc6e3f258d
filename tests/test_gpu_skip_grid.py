"""GPU: the skipping grids themselves (ivr_volume_skip_grid).

The exact grid of a TF must be, cell for cell, the capped Chebyshev
distance (in macrocells) from each transparent cell to the nearest opaque
one, where a cell is transparent when every LUT entry its value range can
index has zero opacity (the range of the cell's voxels and of the next voxel
on each high side, widened by one index each way).  The expected grid is
computed here from the oracle's macrocell min/max and a brute-force
distance over all pairs of cells.

A learned grid (certified) must call transparent only cells the exact test
calls transparent, must be the distance transform of its own transparent
set, and must equal the grid built from the same steps run one by one
(ivr_mlp_features, ivr_mlp_forward, the margin and the exact test).
"""
import ctypes

import numpy as np
import pytest

from ivr_gb300 import api, synth, workloads

pytestmark = pytest.mark.gpu

CAP = 8


def chebyshev_capped(transparent):
    """min(CAP, max-norm distance to the nearest opaque cell), 0 on opaque
    cells; cells outside the grid are not opaque."""
    t = np.asarray(transparent, bool)
    idx = np.argwhere(np.ones_like(t))
    opq = np.argwhere(~t)
    out = np.zeros(t.shape, np.int64)
    if len(opq) == 0:
        out[t] = CAP
        return out.astype(np.uint8)
    d = np.empty(len(idx), np.int64)
    for a in range(0, len(idx), 512):  # all pairs, in chunks of cells
        d[a:a + 512] = np.abs(idx[a:a + 512, None, :] - opq[None, :, :]).max(axis=2).min(axis=1)
    out = np.where(t, np.minimum(d.reshape(t.shape), CAP), 0)
    return out.astype(np.uint8)


def exact_transparent(oracle_mod, vol, cell, lut, scale):
    mn, mx = oracle_mod.macrocells(vol, cell)
    n = len(lut)
    a = np.clip(np.trunc(mn.astype(np.float32) * np.float32(scale)).astype(np.int64) - 1, 0, n - 1)
    b = np.clip(np.trunc(mx.astype(np.float32) * np.float32(scale)).astype(np.int64) + 1, 0, n - 1)
    nz = np.concatenate([[0], np.cumsum(lut[:, 3] != 0)])
    return (nz[b + 1] - nz[a]) == 0


CASES = [
    # dtype, shape (d, h, w), macrocell edge, TF seed
    ("u16", (64, 56, 72), 8, 3),
    ("u8", (40, 48, 36), 8, 5),
    ("f32", (36, 44, 40), 4, 7),
    ("u8", (8, 64, 60), 16, 11),   # one cell along z
    ("u8", (8, 8, 6000), 4, 17),   # 1500 cells along x: fewer lines per block of the transform
]


@pytest.mark.parametrize("dtype,shape,cell,seed", CASES, ids=["u16-8", "u8-8", "f32-4", "u8-16-flat", "u8-4-long"])
def test_exact_grid_is_the_capped_distance_transform(ctx, oracle_mod, dtype, shape, cell, seed):
    vol = synth.blob_volume(shape, n_blobs=6, seed=seed, dtype=dtype, zero_fraction=0.4, cell=cell,
                            sigma_scale=0.7)
    lut, _ = synth.knot_tf(seed, zero_first=True)
    scale = workloads.lut_scale(dtype)
    v = ctx.load_volume(vol).macrocell(cell)
    tf = ctx.transfer_function().set_lut(lut, 0, scale, api.TF_F2B)
    try:
        got = v.skip_grid(tf, api.SKIP_GRID)
        t = exact_transparent(oracle_mod, vol, cell, lut, scale)
        assert got.shape == t.shape
        assert 0 < t.sum() < t.size, "the case must mix transparent and opaque cells"
        want = chebyshev_capped(t)
        assert np.array_equal(got, want), f"{np.sum(got != want)} cells differ"
    finally:
        tf.free()
        v.free()


def test_grid_of_bricks_is_its_own_distance_transform(ctx):
    """Bricks with a halo: each brick's grid is the transform of its own
    transparent cells (the brick's voxels decide which those are)."""
    vol = synth.blob_volume((36, 44, 40), n_blobs=8, seed=13, dtype="f32", zero_fraction=0.3, cell=8)
    lut, _ = synth.knot_tf(13, zero_first=True)
    v = ctx.load_volume(vol).bricks(2, 2, 2, overlap=1).macrocell(8)
    tf = ctx.transfer_function().set_lut(lut, 0, 1.0, api.TF_F2B)
    try:
        for k in range(8):
            g = v.skip_grid(tf, api.SKIP_GRID, brick=k)
            assert np.array_equal(g, chebyshev_capped(g > 0)), f"brick {k}"
    finally:
        tf.free()
        v.free()


def _forward_of_cells(mlp, v, tf, ncell):
    """The network's output and the exact bound per cell of a one-brick
    volume, through the separate feature and inference entry points."""
    import torch
    x = torch.zeros((ncell, api.MLP_IN), dtype=torch.int16, device="cuda")
    bound = torch.zeros(ncell, dtype=torch.float32, device="cuda")
    y = torch.zeros(ncell, dtype=torch.float32, device="cuda")
    n = mlp.features(v, tf, x.data_ptr(), bound.data_ptr(), ncell)
    assert n == ncell
    mlp.forward(x.data_ptr(), n, y.data_ptr())
    torch.cuda.synchronize()
    return y.cpu().numpy(), bound.cpu().numpy()


def test_learned_grid_is_certified_and_its_own_distance_transform(ctx, oracle_mod):
    dtype, shape, cell = "u16", (64, 64, 64), 8
    vol = synth.blob_volume(shape, n_blobs=12, seed=21, dtype=dtype, zero_fraction=0.5, cell=cell,
                            sigma_scale=0.7)
    scale = workloads.lut_scale(dtype)
    luts = [synth.knot_tf(30 + s, zero_first=True)[0] for s in range(4)]
    v = ctx.load_volume(vol).macrocell(cell)
    tfs = [ctx.transfer_function().set_lut(t, 0, scale, api.TF_F2B) for t in luts]
    mlp = ctx.mlp(4)
    try:
        for tf in tfs[:3]:
            mlp.add_samples(v, tf)
        mlp.train(40, batch_rows=256, lr=3e-3, wneg=4.0)
        margin, _ = mlp.calibrate(0.05)
        v.set_mlp(mlp, margin, certify=True)
        learned_cells = 0
        for lut, tf in zip(luts, tfs):
            g = v.skip_grid(tf, api.SKIP_LEARNED)
            t = exact_transparent(oracle_mod, vol, cell, lut, scale)
            assert not np.any((g > 0) & ~t), "a learned-transparent cell the exact test calls opaque"
            assert np.array_equal(g, chebyshev_capped(g > 0))
            # the grid's one launch (features, network, flags) against the
            # same steps run one by one: ivr_mlp_features, ivr_mlp_forward
            y, bound = _forward_of_cells(mlp, v, tf, g.size)
            flags = ((y + np.float32(margin)) <= 0) & (bound == 0)
            assert np.array_equal(g, chebyshev_capped(flags.reshape(g.shape)))
            learned_cells += int((g > 0).sum())
        assert learned_cells > 0, "the predictor skipped nothing"
        st = v.learned_stats()
        assert st["learned_transparent"] - st["false_skips"] == learned_cells
    finally:
        v.set_mlp(None)
        mlp.free()
        for tf in tfs:
            tf.free()
        v.free()


def test_skip_grid_arguments(ctx):
    """Wrong arguments are errors with a message, not faults: a skip mode
    without a grid, a brick out of range, an output too small; a learned
    grid needs a predictor."""
    vol = synth.blob_volume((32, 32, 32), n_blobs=4, seed=2, dtype="u8")
    v = ctx.load_volume(vol).macrocell(8)
    tf = ctx.transfer_function().set_lut(synth.ramp_tf(), 0, 1.0, api.TF_F2B)
    lib = ctx.lib
    try:
        dims = (ctypes.c_int * 3)()
        for skip, brick, n, why in ((api.SKIP_NONE, 0, 64, "skip"), (api.SKIP_GRID, 1, 64, "brick"),
                                    (api.SKIP_GRID, -1, 64, "brick"), (api.SKIP_GRID, 0, 63, "bytes")):
            buf = np.zeros(max(n, 1), np.uint8)
            rc = lib.ivr_volume_skip_grid(v.h, tf.h, skip, brick, buf.ctypes.data, n, dims)
            assert rc != 0, why
            assert lib.ivr_last_error(ctx.h).decode(), why
        assert lib.ivr_volume_skip_grid(v.h, tf.h, api.SKIP_GRID, 0, None, 0, dims) == 0
        assert tuple(dims) == (4, 4, 4)
        with pytest.raises(api.IvrError):
            v.skip_grid(tf, api.SKIP_LEARNED)  # no predictor attached
        g = v.skip_grid(tf, api.SKIP_GRID)  # the context still works
        assert g.shape == (4, 4, 4)
    finally:
        tf.free()
        v.free()
