"""CPU: the O2 restatement against the reference's golden frames (bitwise)
and against the reference itself (O1) where it can be built."""
import numpy as np
import pytest

from conftest import GOLDEN, load_case
from ivr_gb300 import synth
from ivr_gb300.state import orbit_state


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def o2_case(oracle, c, **kw):
    vol = c["volume"]
    if c["colormap"] == -1:
        lut, off = c["lut"], c["lutoffset"]
    else:
        lut, off = oracle.lut_for(vol, c["colormap"])
    return oracle.render(vol, c["state_obj"], lut, off, c["xfer"], procdims=c["procdims"], tile=c["tile"],
                         bricks=True, **kw), lut, off


@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: p.split("/")[-1][:-4])
def test_o2_matches_reference_golden(oracle_mod, path):
    c = load_case(path)
    r, lut, off = o2_case(oracle_mod, c)
    assert off == c["lutoffset"]
    assert np.array_equal(bits(lut), bits(c["lut"])), "LUT differs from the reference's"
    assert np.array_equal(bits(r["rgba32"]), bits(c["rgba32"])), "composited frame differs"
    assert np.array_equal(bits(r["bricks"]), bits(c["bricks"])), "brick sub-images differ"
    K = len(c["procdims"]) and int(np.prod(c["procdims"]))
    for k in range(K):
        assert np.allclose(r["stats"]["wincoord"][k], c["info"][k][:6], rtol=0, atol=0)
    # the reference's composite order (sortboxlist) is recorded per rank
    order = [int(k) for k in np.argsort(c["info"][:K, 6], kind="stable")]
    assert r["stats"]["order"] == order


@pytest.mark.parametrize("path", GOLDEN[:4], ids=lambda p: p.split("/")[-1][:-4])
def test_o2_threads_deterministic(oracle_mod, path):
    c = load_case(path)
    r1, _, _ = o2_case(oracle_mod, c, threads=1)
    r4, _, _ = o2_case(oracle_mod, c, threads=4)
    assert np.array_equal(bits(r1["rgba32"]), bits(r4["rgba32"]))


def test_golden_cover_every_tf_mode():
    modes = {load_case(p)["xfer"] for p in GOLDEN}
    assert modes == {0, 1, 2, 3, 4, 5}
    assert any(load_case(p)["lutoffset"] > 0 for p in GOLDEN)
    assert any(np.prod(load_case(p)["procdims"]) > 1 for p in GOLDEN)


@pytest.mark.parametrize("cm", [0, 1, 2, 3, 4])
@pytest.mark.parametrize("hsize,hmin,hmax", [(256, 0.0, 255.0), (161, 40.0, 200.0), (4096, 3.0, 4098.0)])
def test_colormaps_match_reference(oracle_mod, cm, hsize, hmin, hmax):
    if not oracle_mod.o1_available():
        pytest.skip("reference sources not compiled here")
    import ctypes
    ref = np.zeros((hsize, 4), np.float32)
    oracle_mod.o1().ref_colormap(cm, ref.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), hsize, hmin, hmax)
    ours = oracle_mod.colormap(cm, hsize, hmin, hmax)
    assert np.array_equal(bits(ours), bits(ref))


RANDOM_CASES = [
    # shape, seed, az, el, win, cm, xfer, procdims, alpha
    ((17, 21, 19), 101, 10, 5, (40, 36), 4, 3, (1, 1, 1), 0.1),
    ((26, 16, 20), 102, 210, -35, (44, 40), 4, 2, (2, 2, 2), 0.05),
    ((20, 20, 20), 103, 95, 60, (40, 40), 0, 0, (1, 2, 2), 0.2),
    ((18, 24, 22), 104, 330, -5, (48, 36), 2, 1, (2, 1, 1), 0.3),
    ((22, 22, 18), 105, 140, 15, (40, 40), 3, 5, (1, 1, 2), 0.15),
    ((21, 19, 23), 106, 45, 45, (36, 44), 4, 4, (1, 1, 1), 0.5),
]


@pytest.mark.parametrize("case", RANDOM_CASES, ids=[str(i) for i in range(len(RANDOM_CASES))])
def test_o2_matches_reference_live(oracle_mod, case):
    if not oracle_mod.o1_available():
        pytest.skip("reference sources not compiled here")
    shape, seed, az, el, win, cm, xfer, procdims, alpha = case
    vol = synth.blob_volume(shape, n_blobs=6, seed=seed, dtype="u8")
    st = orbit_state(az, el, win[0], win[1], fovy=43.6028, alpha=alpha)
    ref = oracle_mod.ref_render(vol.astype(np.float32), st, cm, xfer, procdims=procdims, threads=1)
    vw = win[0]
    if any(i[0] + i[3] >= vw for i in ref["info"]):
        pytest.skip("brick rectangle reaches the right edge (reference writes out of bounds there)")
    lut, off = oracle_mod.lut_for(vol, cm)
    ours = oracle_mod.render(vol, st, lut, off, xfer, procdims=procdims, bricks=True)
    assert np.array_equal(bits(ours["rgba32"]), bits(ref["rgba32"]))
    assert np.array_equal(bits(ours["bricks"]), bits(ref["bricks"]))


def test_quantize_rule(oracle_mod):
    rng = np.random.default_rng(0)
    x = np.concatenate([rng.uniform(0, 1, 100000).astype(np.float32),
                        ((np.arange(1, 256) - 0.5) / 255).astype(np.float32),
                        np.array([0.0, 1.0, -0.0, 1e-30, 0.5 / 255], np.float32)])
    # nudge around every rounding boundary
    b = ((np.arange(1, 256) - 0.5) / 255).astype(np.float32)
    x = np.concatenate([x, np.nextafter(b, 0), np.nextafter(b, 1)]).astype(np.float32)
    expect = np.floor(x.astype(np.float64) * 255.0 + 0.5).astype(np.uint8)
    assert np.array_equal(oracle_mod.quantize(x), expect)
    assert oracle_mod.quantize(np.array([1.5, -2.0, np.nan], np.float32)).tolist() == [255, 0, 0]


def test_composite_matches_fused_ref(oracle_mod):
    c = load_case([p for p in GOLDEN if "8bricks" in p][0])
    r, _, _ = o2_case(oracle_mod, c)
    out = oracle_mod.composite(r["bricks"], r["stats"]["order"])
    assert np.array_equal(bits(out), bits(r["rgba32"]))


def test_config_bricked_close_to_single(oracle_mod):
    vol = synth.blob_volume((32, 32, 32), n_blobs=8, seed=5, dtype="u8")
    st = orbit_state(35, 25, 48, 48, fovy=30.0, alpha=1.0)
    lut = synth.ramp_tf(256)
    one = oracle_mod.render(vol, st, lut, 0, 6, preset=1)
    eight = oracle_mod.render(vol, st, lut, 0, 6, preset=1, procdims=(2, 2, 2))
    assert one["stats"]["samples_alg"] > 0
    # same lattice; only the brick-local index mapping and boundary
    # membership differ
    assert np.abs(one["rgba8"].astype(int) - eight["rgba8"].astype(int)).max() <= 2
    # with termination off, compositing per-brick images equals the fused
    # front-to-back march up to rounding
    fused = oracle_mod.render(vol, st, lut, 0, 6, preset=1, procdims=(2, 2, 2), term_alpha=2.0, bricks=True)
    comp = oracle_mod.composite(fused["bricks"], fused["stats"]["order"])
    assert np.allclose(comp, fused["rgba32"], rtol=1e-4, atol=1e-5)


def test_config_early_termination_bound(oracle_mod):
    vol = synth.blob_volume((32, 32, 32), n_blobs=8, seed=6, dtype="u8")
    st = orbit_state(-20, 10, 40, 40, fovy=30.0, alpha=1.0)
    lut = synth.ramp_tf(256)
    a = oracle_mod.render(vol, st, lut, 0, 6, preset=1, term_alpha=0.99)
    b = oracle_mod.render(vol, st, lut, 0, 6, preset=1, term_alpha=2.0)
    assert a["stats"]["samples_exec"] <= b["stats"]["samples_exec"]
    assert np.abs(a["rgba32"] - b["rgba32"]).max() <= 0.0101


@pytest.mark.parametrize("procdims", [(1, 1, 1), (2, 2, 2), (1, 3, 2)])
def test_config_skip_lossless_in_oracle(oracle_mod, procdims):
    vol = synth.blob_volume((48, 48, 48), n_blobs=8, seed=1, dtype="u8", zero_fraction=0.5, cell=8)
    st = orbit_state(35, 20, 64, 64, fovy=30.0, alpha=1.0)
    lut = synth.ramp_tf(256)
    a = oracle_mod.render(vol, st, lut, 0, 6, preset=1, procdims=procdims)
    b = oracle_mod.render(vol, st, lut, 0, 6, preset=1, procdims=procdims, skip=True)
    assert np.array_equal(bits(a["rgba32"]), bits(b["rgba32"]))
    assert b["stats"]["samples_exec"] < a["stats"]["samples_exec"]


def test_gradient_rule(oracle_mod):
    """gradient3d as intended: per axis a halved central difference inside
    and a halved one-sided difference on the faces, on every voxel, edges
    and corners included; w = |g| summed in x, y, z order."""
    rng = np.random.default_rng(3)
    v = rng.random((6, 5, 7)).astype(np.float32) * 100
    g = oracle_mod.gradient(v)

    def axis(a, ax):
        a = np.moveaxis(a, ax, -1)
        out = np.empty_like(a)
        out[..., 1:-1] = (a[..., 2:] - a[..., :-2]) / np.float32(2)
        out[..., 0] = (a[..., 1] - a[..., 0]) / np.float32(2)
        out[..., -1] = (a[..., -1] - a[..., -2]) / np.float32(2)
        return np.moveaxis(out, -1, ax)

    gx, gy, gz = axis(v, 2), axis(v, 1), axis(v, 0)
    assert np.array_equal(g[..., 0], gx) and np.array_equal(g[..., 1], gy) and np.array_equal(g[..., 2], gz)
    mag = np.sqrt((gx * gx + gy * gy) + gz * gz).astype(np.float32)
    assert np.array_equal(g[..., 3], mag)
