"""The learned-skip predictor's CPU oracle: BF16 rounding, the exact bound
rule, and the analytic gradient against central finite differences."""
import numpy as np
import pytest

from oracle import mlp_ref as M


def _params(seed):
    rng = np.random.default_rng(seed)
    p = np.zeros(M.NPARAMS)
    p[M.OFF_W1:M.OFF_B1] = rng.normal(0, np.sqrt(2 / 26), M.IN * M.HID)
    p[M.OFF_W1 + M.FEAT * M.HID:M.OFF_B1] = 0.0
    p[M.OFF_B1:M.OFF_W2] = rng.normal(0, 0.1, M.HID)
    p[M.OFF_W2:M.OFF_B2] = rng.normal(0, np.sqrt(2 / 64), M.HID * M.HID)
    p[M.OFF_B2:M.OFF_W3] = rng.normal(0, 0.1, M.HID)
    p[M.OFF_W3:M.OFF_B3] = rng.normal(0, np.sqrt(1 / 64), M.HID)
    p[M.OFF_B3] = 0.05
    return p


def _rows(seed, n):
    rng = np.random.default_rng(seed)
    X = np.zeros((n, M.IN))
    X[:, :M.FEAT] = rng.uniform(0, 1, (n, M.FEAT))
    T = np.where(rng.uniform(size=n) < 0.5, 0.0, rng.uniform(0.05, 1.0, n))
    return X, T


def test_bf16_rounding():
    x = np.array([1.0, 1 + 2 ** -8, 1 + 3 * 2 ** -8, -2.5, 0.0, 1e-30], np.float32)
    r = M.bf16(x)
    assert r[0] == 1.0
    assert r[1] == 1.0                   # tie -> even
    assert r[2] == np.float32(1 + 2 ** -6)  # tie -> even (up)
    assert r[3] == -2.5
    assert r[4] == 0.0
    assert (M.bf16(r) == r).all()        # idempotent


def test_bound_rule_matches_index_range():
    lut = np.zeros((256, 4), np.float32)
    lut[100, 3] = 0.7
    # values 98.x .. 99.x index 97 .. 100 -> sees entry 100
    assert M.bound(98.5, 99.2, lut, 0, 1.0) == pytest.approx(0.7)
    # values 102 .. 110 index 101 .. 111 -> misses it
    assert M.bound(102.0, 110.0, lut, 0, 1.0) == 0.0
    # offset shifts the index
    assert M.bound(110.0, 110.0, lut, 10, 1.0) == pytest.approx(0.7)


@pytest.mark.parametrize("seed", [0, 1])
def test_gradient_matches_finite_differences(seed):
    p = _params(seed)
    X, T = _rows(seed + 10, 48)
    wneg = 4.0
    _, g = M.loss_grad(p, X, T, wneg, emulate=False)
    rng = np.random.default_rng(seed + 20)
    live = np.r_[np.arange(M.OFF_W1, M.OFF_W1 + M.FEAT * M.HID), np.arange(M.OFF_B1, M.NPARAMS)]
    idx = np.r_[rng.choice(live, 300, replace=False), M.OFF_B3]
    eps = 1e-6
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += eps
        pm[i] -= eps
        fd = (M.loss_grad(pp, X, T, wneg, emulate=False)[0] - M.loss_grad(pm, X, T, wneg, emulate=False)[0]) / (2 * eps)
        assert abs(fd - g[i]) <= 1e-6 + 1e-5 * abs(g[i]), (i, fd, g[i])
    # the padding rows of W1 get no gradient (their inputs are zero)
    assert not g[M.OFF_W1 + M.FEAT * M.HID:M.OFF_B1].any()


def test_transparent_rows_are_one_sided():
    p = _params(3)
    X, _ = _rows(4, 32)
    y, _ = M.forward(p, X, emulate=False)
    # bound 0: only y above -gamma costs
    T = np.zeros(32)
    loss, _ = M.loss_grad(p, X, T, 4.0, emulate=False)
    assert loss == pytest.approx(np.mean(np.maximum(y + M.GAMMA, 0) ** 2))
    # bound > 0: under-prediction weighted by wneg
    T = np.full(32, 0.5)
    loss, _ = M.loss_grad(p, X, T, 4.0, emulate=False)
    r = y - 0.5
    assert loss == pytest.approx(np.mean(np.where(r < 0, 4.0, 1.0) * r * r))


def test_emulated_gradient_close_to_exact():
    """BF16 rounding at the tensor-core operands changes the gradient by a
    few parts in a thousand, not its direction."""
    p = _params(5)
    X, T = _rows(6, 256)
    _, g64 = M.loss_grad(p, X, T, 4.0, emulate=False)
    _, gbf = M.loss_grad(p, X, T, 4.0, emulate=True)
    cos = g64 @ gbf / np.linalg.norm(g64) / np.linalg.norm(gbf)
    assert cos > 0.999


def test_features_of_a_tiny_volume():
    rng = np.random.default_rng(7)
    vol = np.zeros((34, 40, 33), np.uint8)
    vol[20:, 20:, 18:] = rng.integers(50, 255, (14, 20, 15))
    lut = np.zeros((256, 4), np.float32)
    lut[60:, 3] = 0.5
    X, T = M.features(vol, lut, 0, 1.0)
    mcx, mcy, mcz = M.cell_grid(33, 40, 34)
    assert X.shape == (mcx * mcy * mcz, M.IN)
    assert (X[:, M.FEAT:] == 0).all()
    # the all-zero cell (0,0,0) is transparent, the full corner is not
    assert T[0] == 0.0 and X[0, 0] == 0.0 and X[0, 1] == 0.0
    assert T[-1] == pytest.approx(0.5)
    # histogram rows are fractions
    np.testing.assert_allclose(X[:, 2:10].sum(axis=1), 1.0, atol=0.03)


@pytest.mark.parametrize("seed", [1000, 1017, 1035])
def test_knot_encoding_reads_a_16_knot_tf(seed):
    """On a piecewise-linear TF of 16 knots (entry 17 k of 256 is knot k),
    feature k < 15 is the larger of knots k and k + 1, and feature 15 the
    LUT's largest opacity; every other LUT size keeps intervals that cover
    the LUT and overlap only at their shared knot."""
    from ivr_gb300 import synth
    lut, ka = synth.knot_tf(seed, zero_first=True)
    kn = M.knots(lut)
    np.testing.assert_allclose(kn[:15], np.maximum(ka[:-1], ka[1:]), rtol=0, atol=1e-6)
    assert kn[15] == lut[:, 3].max()
    for n in (1, 2, 15, 16, 17, 100, 256, 4096):
        last = M.KNOTS - 1
        spans = [(k * (n - 1) // last, ((k + 1) * (n - 1) + last - 1) // last) for k in range(last)]
        assert spans[0][0] == 0 and spans[-1][1] == n - 1
        assert all(a <= b <= n - 1 for a, b in spans)
        assert all(spans[k + 1][0] <= spans[k][1] for k in range(last - 1))
