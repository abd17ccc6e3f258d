"""GPU: batched rendering (many views, TFs, image sizes and steps in one
persistent launch, optionally a CUDA-graph replay) gives every frame bitwise
the frame rendered alone; the autotuner's choice does not change output."""
import numpy as np
import pytest

from ivr_gb300 import api, synth
from ivr_gb300.state import orbit_state

pytestmark = pytest.mark.gpu

SIZES = [(64, 64), (96, 80), (48, 48), (128, 72)]
STEPS = [0.25, 0.5, 0.75, 1.0]


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


@pytest.fixture(scope="module")
def scene(ctx):
    import torch
    vol = synth.blob_volume((48, 40, 44), n_blobs=8, seed=12, dtype="f32", value_noise=0.1)
    v = ctx.load_volume(vol).bricks(2, 2, 2)
    tfs = [ctx.transfer_function().set_lut(synth.knot_tf(s)[0], 0, 1.0, api.TF_F2B) for s in range(4)]
    rng = np.random.default_rng(3)
    frames = []
    for k in range(12):
        w, h = SIZES[k % 4]
        st = orbit_state(float(rng.uniform(0, 360)), float(rng.uniform(-50, 50)), w, h, fovy=30.0, alpha=1.0)
        view = ctx.view().set(v, st, api.config_params(step=STEPS[(k // 4) % 4]))
        tf = tfs[k % 4]
        o32 = torch.zeros((h, w, 4), dtype=torch.float32, device="cuda")
        o8 = torch.zeros((h, w, 4), dtype=torch.uint8, device="cuda")
        view.render(tf, o32.data_ptr(), o8.data_ptr())
        torch.cuda.synchronize()
        frames.append((view, tf, o32.cpu().numpy(), o8.cpu().numpy(), (w, h)))
    yield v, frames
    v.free()


def run_batch(ctx, frames, variant=None, graph=False, repeat=1):
    import torch
    b = ctx.batch(len(frames))
    outs = []
    for view, tf, _, _, (w, h) in frames:
        o32 = torch.full((h, w, 4), -1.0, dtype=torch.float32, device="cuda")
        o8 = torch.full((h, w, 4), 3, dtype=torch.uint8, device="cuda")
        b.add(view, tf, o32.data_ptr(), o8.data_ptr())
        outs.append((o32, o8))
    if variant is not None:
        b.set_variant(variant)
    for _ in range(repeat):
        b.render(use_graph=graph)
    torch.cuda.synchronize()
    res = [(a.cpu().numpy(), c.cpu().numpy()) for a, c in outs]
    b.free()
    return res


@pytest.mark.parametrize("variant", range(6))
def test_batch_equals_alone(ctx, scene, variant):
    _, frames = scene
    res = run_batch(ctx, frames, variant=variant)
    for (view, tf, a32, a8, _), (b32, b8) in zip(frames, res):
        assert np.array_equal(bits(a32), bits(b32))
        assert np.array_equal(a8, b8)


def test_batch_graph_replay(ctx, scene):
    _, frames = scene
    res = run_batch(ctx, frames, graph=True, repeat=3)
    for (_, _, a32, a8, _), (b32, b8) in zip(frames, res):
        assert np.array_equal(bits(a32), bits(b32))
        assert np.array_equal(a8, b8)


def test_batch_refill_and_autotune(ctx, scene):
    import torch
    _, frames = scene
    b = ctx.batch(8)
    outs = []
    for view, tf, _, _, (w, h) in frames[:8]:
        o8 = torch.zeros((h, w, 4), dtype=torch.uint8, device="cuda")
        b.add(view, tf, None, o8.data_ptr())
        outs.append(o8)
    best, ms = b.autotune()
    assert 0 <= best < 6 and all(m > 0 for m in ms)
    b.render(use_graph=True)
    b.clear()  # waits for the render above, then the staging is refilled
    outs2 = []
    for view, tf, _, _, (w, h) in frames[4:12]:
        o8 = torch.zeros((h, w, 4), dtype=torch.uint8, device="cuda")
        b.add(view, tf, None, o8.data_ptr())
        outs2.append(o8)
    b.render(use_graph=True)
    torch.cuda.synchronize()
    for o, f in zip(outs, frames[:8]):
        assert np.array_equal(o.cpu().numpy(), f[3])
    for o, f in zip(outs2, frames[4:12]):
        assert np.array_equal(o.cpu().numpy(), f[3])
    b.free()


def test_batch_rejects(ctx, scene):
    from ivr_gb300._lib import IvrError
    v, frames = scene
    b = ctx.batch(1)
    b.add(frames[0][0], frames[0][1])
    with pytest.raises(IvrError):
        b.add(frames[1][0], frames[1][1])  # full
    ref_view = ctx.view().set(v, orbit_state(0, 0, 32, 32), api.ref_params())
    b.clear()
    with pytest.raises(IvrError):
        b.add(ref_view, frames[0][1])  # REF preset
    b.free()
