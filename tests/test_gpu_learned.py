"""GPU: learned empty-space skipping.

- features and exact bounds bitwise against the CPU oracle;
- the tensor-core forward pass and training gradient against the float64
  oracle with the kernels' BF16 rounding points (and against plain float64);
- training on the device lowers the loss;
- learned-skip frames stay within 1/255 of the exact grid's frames, a
  predictor that is wrong everywhere is caught by the judge and its frames
  are re-rendered exactly;
- the trained predictor against rendering without skipping and against the
  exact macrocell grid.
"""
import os
import tempfile

import numpy as np
import pytest

from ivr_gb300 import api, synth
from ivr_gb300.state import orbit_state
from oracle import mlp_ref as M

pytestmark = pytest.mark.gpu

RGBA8_TOL = 1


def _torch():
    import torch
    return torch


def _sync_cpu(t):
    torch = _torch()
    torch.cuda.synchronize()
    return t.cpu().numpy()


@pytest.fixture(scope="module")
def scene(ctx):
    """A 64^3 u8 volume (one brick) with most cells zero, and TFs whose low
    values are transparent."""
    vol_np = synth.blob_volume((64, 64, 64), n_blobs=12, seed=5, dtype="u8", zero_fraction=0.6)
    vol = ctx.load_volume(vol_np)
    tfs, luts = [], []
    for s in range(6):
        lut, _ = synth.knot_tf(100 + s, zero_first=True)
        luts.append(lut)
        tfs.append(ctx.transfer_function().set_lut(lut, 0, 1.0, api.TF_F2B))
    yield vol_np, vol, tfs, luts
    for t in tfs:
        t.free()
    vol.free()


def _features(ctx, mlp, vol, tf, cap=4096):
    torch = _torch()
    X = torch.zeros((cap, M.IN), dtype=torch.int16, device="cuda")
    T = torch.zeros(cap, dtype=torch.float32, device="cuda")
    n = mlp.features(vol, tf, X.data_ptr(), T.data_ptr(), cap)
    return X[:n], T[:n], n


def test_features_and_bounds_match_oracle(ctx, scene):
    vol_np, vol, tfs, luts = scene
    mlp = ctx.mlp(1)
    try:
        for tf, lut in zip(tfs[:3], luts[:3]):
            X, T, n = _features(ctx, mlp, vol, tf)
            Xo, To = M.features(vol_np, lut, 0, 1.0)
            assert n == len(To)
            got = _sync_cpu(X).view(np.uint16).astype(np.uint32)
            np.testing.assert_array_equal(got, M.bf16_bits(Xo))
            np.testing.assert_array_equal(_sync_cpu(T), To.astype(np.float32))
    finally:
        mlp.free()


def _random_params(seed):
    rng = np.random.default_rng(seed)
    p = np.zeros(M.NPARAMS, np.float32)
    p[M.OFF_W1:M.OFF_B1] = rng.normal(0, np.sqrt(2 / 26), M.IN * M.HID)
    p[M.OFF_B1:M.OFF_W2] = rng.normal(0, 0.1, M.HID)
    p[M.OFF_W2:M.OFF_B2] = rng.normal(0, np.sqrt(2 / 64), M.HID * M.HID)
    p[M.OFF_B2:M.OFF_W3] = rng.normal(0, 0.1, M.HID)
    p[M.OFF_W3:M.OFF_B3] = rng.normal(0, np.sqrt(1 / 64), M.HID)
    p[M.OFF_B3] = 0.05
    return p


def _random_rows(seed, n):
    rng = np.random.default_rng(seed)
    X = np.zeros((n, M.IN), np.float32)
    X[:, :M.FEAT] = rng.uniform(0, 1, (n, M.FEAT))
    Xb = M.bf16(X)
    T = np.where(rng.uniform(size=n) < 0.5, 0.0, rng.uniform(0.05, 1.0, n)).astype(np.float32)
    return Xb, T


def _dev_rows(Xb, T):
    torch = _torch()
    bits = (Xb.view(np.uint32) >> 16).astype(np.uint16).view(np.int16)
    return torch.from_numpy(bits.copy()).cuda(), torch.from_numpy(T).cuda()


def _near_bf16_tie(p, x):
    """Whether one of the row's first-layer values (before its rounding to
    BF16) lies within FP32 accumulation error of a BF16 rounding tie, so
    that a different FP32 summation order may round it the other way."""
    W1, b1 = M.unpack(p)[:2]
    xe, W1e = M.bf16(x).astype(np.float64), M.bf16(W1).astype(np.float64)
    v = xe @ W1e + b1
    mag = np.abs(xe) @ np.abs(W1e) + np.abs(b1)  # bounds every partial sum
    for j in np.nonzero(v > 0)[0]:
        ulp = 2.0 ** (np.floor(np.log2(v[j])) - 7)  # one BF16 step at v
        frac = v[j] / ulp - np.floor(v[j] / ulp)
        if abs(frac - 0.5) * ulp <= 32 * 2.0 ** -24 * mag[j]:
            return True
    return False


@pytest.mark.parametrize("n", [1, 300, 1000, 50001])
def test_forward_matches_oracle(ctx, n):
    """Inference (the tcgen05 tensor-core kernel: 128-row tiles, a block
    taking several tiles when there are more than two per SM) against the
    float64 oracle with the BF16 rounding points."""
    torch = _torch()
    mlp = ctx.mlp(2)
    try:
        p = _random_params(n)
        mlp.set_params(p)
        p_back = mlp.params()
        p_ref = p.copy()
        p_ref[M.OFF_W1 + M.FEAT * M.HID:M.OFF_B1] = 0.0  # padding rows are cleared
        np.testing.assert_array_equal(p_back, p_ref)
        Xb, T = _random_rows(n + 1, n)
        Xd, _ = _dev_rows(Xb, T)
        y = torch.zeros(n, dtype=torch.float32, device="cuda")
        mlp.forward(Xd.data_ptr(), n, y.data_ptr())
        yo, _ = M.forward(p_ref, Xb, emulate=True)
        got = _sync_cpu(y)
        # FP32 accumulation order is the only difference left.  On a rare
        # row it moves a hidden value across a BF16 rounding tie; every row
        # outside the tight bound must have such a hidden value
        err = np.abs(got - yo)
        tol = 1e-4 * (1 + np.max(np.abs(yo)))
        off = np.nonzero(err > tol)[0]
        assert len(off) <= max(1, n // 1000), (len(off), err.max())
        for r in off:
            assert _near_bf16_tie(p_ref, Xb[r]), (r, err[r])
    finally:
        mlp.free()


@pytest.mark.parametrize("n", [77, 1000])
def test_gradient_matches_oracle(ctx, n):
    torch = _torch()
    mlp = ctx.mlp(3)
    try:
        p = _random_params(10 + n)
        p[M.OFF_W1 + M.FEAT * M.HID:M.OFF_B1] = 0.0
        mlp.set_params(p)
        Xb, T = _random_rows(20 + n, n)
        Xd, Td = _dev_rows(Xb, T)
        grad = torch.zeros(M.NPARAMS, dtype=torch.float32, device="cuda")
        loss = torch.zeros(1, dtype=torch.float32, device="cuda")
        mlp.gradient(Xd.data_ptr(), Td.data_ptr(), n, 4.0, grad.data_ptr(), loss.data_ptr())
        g = _sync_cpu(grad).astype(np.float64)
        lo, go = M.loss_grad(p, Xb, T, 4.0, emulate=True)
        assert float(_sync_cpu(loss)[0]) == pytest.approx(lo, rel=1e-4)
        # same rounding points: agreement to FP32 accumulation error, per layer
        for a, b in [(M.OFF_W1, M.OFF_B1), (M.OFF_B1, M.OFF_W2), (M.OFF_W2, M.OFF_B2), (M.OFF_B2, M.OFF_W3),
                     (M.OFF_W3, M.OFF_B3), (M.OFF_B3, M.NPARAMS)]:
            scale = np.max(np.abs(go[a:b])) + 1e-12
            assert np.max(np.abs(g[a:b] - go[a:b])) <= 2e-3 * scale, (a, b)
        # and against plain float64: the same direction
        _, g64 = M.loss_grad(p, Xb, T, 4.0, emulate=False)
        assert g @ g64 / np.linalg.norm(g) / np.linalg.norm(g64) > 0.995
    finally:
        mlp.free()


def test_save_load_round_trip(ctx):
    a, b = ctx.mlp(4), ctx.mlp(5)
    try:
        with tempfile.TemporaryDirectory() as d:
            path = os.path.join(d, "w.bin")
            a.save(path)
            b.load(path)
            np.testing.assert_array_equal(a.params(), b.params())
            with open(path, "r+b") as f:
                f.write(b"XXXX")
            with pytest.raises(api.IvrError):
                b.load(path)
    finally:
        a.free()
        b.free()


@pytest.fixture(scope="module")
def trained(ctx, scene):
    """A predictor trained on TFs 0-3 of the scene, calibrated."""
    vol_np, vol, tfs, luts = scene
    mlp = ctx.mlp(7)
    for tf in tfs[:4]:
        mlp.add_samples(vol, tf)
    losses = mlp.train(400, batch_rows=64, lr=3e-3, wneg=4.0)
    margin, recall = mlp.calibrate(0.02)
    yield mlp, losses, margin, recall
    vol.set_mlp(None)
    mlp.free()


def test_training_lowers_the_loss(trained):
    mlp, losses, margin, recall = trained
    assert np.all(np.isfinite(losses))
    assert losses[-1] < 0.25 * losses[0], losses
    assert 0.0 <= margin < 1.0
    assert recall > 0.3, recall


def _frame(ctx, view, tf, vh, vw):
    torch = _torch()
    o8 = torch.zeros((vh, vw, 4), dtype=torch.uint8, device="cuda")
    view.render(tf, None, o8.data_ptr())
    return _sync_cpu(o8)


@pytest.mark.parametrize("certify", [True, False])
def test_learned_frames_match_the_exact_grid(ctx, scene, trained, certify):
    vol_np, vol, tfs, luts = scene
    mlp, _, margin, _ = trained
    vol.set_mlp(mlp, margin, certify)
    exact = ctx.view()
    learned = ctx.view()
    try:
        for i, tf in enumerate(tfs):  # 0-3 seen in training, 4-5 not
            st = orbit_state(25 + 40 * i, 15 - 7 * i, 160, 128)
            exact.set(vol, st, api.config_params(skip=api.SKIP_GRID))
            learned.set(vol, st, api.config_params(skip=api.SKIP_LEARNED, judge_stride=1))
            a = _frame(ctx, exact, tf, 128, 160).astype(int)
            b = _frame(ctx, learned, tf, 128, 160).astype(int)
            assert np.abs(a - b).max() <= RGBA8_TOL, i
        st = learned.judge_stats()
        # every learned frame is judged, or rendered with the exact grid
        # once its learned grid is known to be wrong
        assert st["frames"] + st["exact_frames"] >= 1
        assert st["pixels"] == st["frames"] * 160 * 128
        if certify:
            assert st["fallbacks"] == 0 and st["worst"] == 0
    finally:
        exact.free()
        learned.free()


def test_a_wrong_predictor_never_reaches_the_image(ctx, scene):
    """A predictor that calls every cell transparent.  Certified: every false
    skip is kept opaque as the grid is built, so the frame is the exact
    grid's.  Uncertified: the image judge sees the difference, the frame is
    re-rendered with the exact grid and the TF's learned grid is not used
    again."""
    vol_np, vol, tfs, luts = scene
    bad = ctx.mlp(9)
    p = np.zeros(M.NPARAMS, np.float32)
    p[M.OFF_B3] = -10.0
    bad.set_params(p)
    exact, learned = ctx.view(), ctx.view()
    try:
        st = orbit_state(40, 20, 128, 96)
        exact.set(vol, st, api.config_params(skip=api.SKIP_GRID))
        refs = [_frame(ctx, exact, tf, 96, 128) for tf in tfs[:3]]
        assert all(r[..., 3].max() > 0 for r in refs)

        vol.set_mlp(bad, 0.0, certify=True)
        learned.set(vol, st, api.config_params(skip=api.SKIP_LEARNED, judge_stride=1))
        before = learned.judge_stats()
        np.testing.assert_array_equal(_frame(ctx, learned, tfs[0], 96, 128), refs[0])
        after = learned.judge_stats()
        assert after["frames"] == before["frames"] + 1
        assert after["fallbacks"] == before["fallbacks"] and after["worst"] == 0
        ls = vol.learned_stats()
        # every cell called transparent; the opaque ones kept opaque
        assert ls["learned_transparent"] == ls["cells"] > 0
        assert ls["false_skips"] == ls["cells"] - ls["exact_transparent"] > 0

        vol.set_mlp(bad, 0.0, certify=False)
        for k, stride in ((1, 1), (2, 4)):
            learned.set(vol, st, api.config_params(skip=api.SKIP_LEARNED, judge_stride=stride))
            before = learned.judge_stats()
            np.testing.assert_array_equal(_frame(ctx, learned, tfs[k], 96, 128), refs[k])
            after = learned.judge_stats()
            assert after["frames"] == before["frames"] + 1
            assert after["fallbacks"] == before["fallbacks"] + 1
            assert after["worst"] > RGBA8_TOL
        # the rejected grid is replaced by the exact one without judging
        before = learned.judge_stats()
        np.testing.assert_array_equal(_frame(ctx, learned, tfs[2], 96, 128), refs[2])
        assert learned.judge_stats()["frames"] == before["frames"]
    finally:
        vol.set_mlp(None)
        bad.free()
        exact.free()
        learned.free()


def test_learned_skipping_on_8_voxel_cells(ctx):
    """The predictor on 8^3-voxel macrocells (ivr_volume_set_macrocell):
    features and exact bounds bitwise against the oracle on those cells, and
    certified learned frames equal to the exact grid's, bit for bit."""
    vol_np = synth.blob_volume((64, 64, 64), n_blobs=12, seed=6, dtype="u8", zero_fraction=0.6)
    vol = ctx.load_volume(vol_np).macrocell(8)
    assert vol.macrocell_edge() == 8
    tfs, luts = [], []
    for s in range(3):
        lut, _ = synth.knot_tf(200 + s, zero_first=True)
        luts.append(lut)
        tfs.append(ctx.transfer_function().set_lut(lut, 0, 1.0, api.TF_F2B))
    mlp = ctx.mlp(21)
    views = []
    try:
        for tf, lut in zip(tfs, luts):
            X, T, n = _features(ctx, mlp, vol, tf)
            Xo, To = M.features(vol_np, lut, 0, 1.0, cell=8)
            assert n == len(To) == 8 ** 3
            np.testing.assert_array_equal(_sync_cpu(X).view(np.uint16).astype(np.uint32), M.bf16_bits(Xo))
            np.testing.assert_array_equal(_sync_cpu(T), To.astype(np.float32))
            mlp.add_samples(vol, tf)
        mlp.train(300, batch_rows=64, lr=3e-3, wneg=4.0)
        margin, _ = mlp.calibrate(0.02)
        vol.set_mlp(mlp, margin, certify=True)
        exact, learned = ctx.view(), ctx.view()
        views = [exact, learned]
        for i, tf in enumerate(tfs):
            st = orbit_state(30 + 50 * i, 10 + 5 * i, 160, 128)
            exact.set(vol, st, api.config_params(skip=api.SKIP_GRID))
            learned.set(vol, st, api.config_params(skip=api.SKIP_LEARNED, judge_stride=1))
            np.testing.assert_array_equal(_frame(ctx, exact, tf, 128, 160), _frame(ctx, learned, tf, 128, 160))
        ls = vol.learned_stats()
        assert ls["cells"] > 0 and ls["learned_transparent"] > 0
    finally:
        for v in views:
            v.free()
        vol.set_mlp(None)
        mlp.free()
        for t in tfs:
            t.free()
        vol.free()


def test_learned_skip_against_the_plain_grid_and_no_skipping(ctx):
    """The trained predictor against the methods without it.

    Against no skipping (the reference's own method, every lattice point):
    the same frames from far fewer executed samples and less time.  Against
    the plain macrocell grid: certified learned grids skip only cells the
    grid's exact test also skips, so their frames are the grid's bit for bit
    and take at least the grid's samples; the test records how close they
    come (the share of the grid's skipped samples they skip, and the time
    ratio), and requires that they keep most of the grid's gain.  A learned
    grid cannot be faster than the exact grid here: the exact test is one
    prefix-count lookup per cell, as cheap as the network's inference, and
    it is tight -- the trilinear reconstruction inside a cell takes every
    value between the cell's minimum and maximum, so no cell it calls opaque
    is transparent for every ray."""
    torch = _torch()
    vol_np = synth.blob_volume((256, 256, 256), n_blobs=32, seed=11, dtype="u16", zero_fraction=0.7,
                               sigma_scale=(8 / 32) ** (1 / 3))
    vol = ctx.load_volume(vol_np)
    scale = 255.0 / 65535.0
    tfs = [ctx.transfer_function().set_lut(synth.knot_tf(300 + s, zero_first=True)[0], 0, scale, api.TF_F2B)
           for s in range(5)]
    mlp = ctx.mlp(13)
    views = []
    try:
        for tf in tfs[:3]:
            mlp.add_samples(vol, tf)
        mlp.train(200, batch_rows=256, lr=3e-3, wneg=4.0)
        margin, _ = mlp.calibrate(0.02)
        vol.set_mlp(mlp, margin)
        W, H = 1024, 1024
        st = orbit_state(30, 20, W, H)
        plain = ctx.view().set(vol, st, api.config_params(skip=api.SKIP_NONE))
        grid = ctx.view().set(vol, st, api.config_params(skip=api.SKIP_GRID))
        learned = ctx.view().set(vol, st, api.config_params(skip=api.SKIP_LEARNED))
        judged = ctx.view().set(vol, st, api.config_params(skip=api.SKIP_LEARNED, judge_stride=1))
        views = [plain, grid, learned, judged]
        # a TF not seen in training, every pixel judged
        a = _frame(ctx, plain, tfs[4], H, W).astype(int)
        b = _frame(ctx, judged, tfs[4], H, W).astype(int)
        assert np.abs(a - b).max() <= RGBA8_TOL
        tf = tfs[4]
        f_grid = _frame(ctx, grid, tf, H, W)
        np.testing.assert_array_equal(_frame(ctx, plain, tf, H, W), f_grid)
        np.testing.assert_array_equal(_frame(ctx, learned, tf, H, W), f_grid)
        cp, cg, cl = plain.census(tf), grid.census(tf), learned.census(tf)
        assert cp["lattice"] == cl["lattice"] == cg["lattice"]
        assert cl["executed"] < 0.6 * cp["executed"], (cl, cp)
        assert cl["executed"] >= cg["executed"], (cl, cg)
        kept = (cp["executed"] - cl["executed"]) / (cp["executed"] - cg["executed"])
        assert kept > 0.8, kept  # of the samples the exact grid skips, the learned grid skips this share
        o8 = torch.zeros((H, W, 4), dtype=torch.uint8, device="cuda")

        def ms(view, reps=10):
            for _ in range(3):
                view.render(tf, None, o8.data_ptr())
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record()
            for _ in range(reps):
                view.render(tf, None, o8.data_ptr())
            e1.record()
            torch.cuda.synchronize()
            return e0.elapsed_time(e1) / reps

        t_plain, t_grid, t_learned = ms(plain), ms(grid), ms(learned)
        print(f"ms per frame: no skipping {t_plain:.3f}, exact grid {t_grid:.3f}, learned {t_learned:.3f}; "
              f"learned skips {kept:.3f} of the grid's skipped samples")
        assert t_learned < t_plain / 1.3, (t_plain, t_learned)
        assert t_learned < 2.0 * t_grid, (t_grid, t_learned)
    finally:
        for v in views:
            v.free()
        vol.set_mlp(None)
        mlp.free()
        for t in tfs:
            t.free()
        vol.free()
