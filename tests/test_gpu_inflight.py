"""GPU: frames in flight.  Consecutive frames rendered by several views on
several streams at once -- so that the next frame's tiles start on the SMs
the last one's tail leaves idle -- are bitwise the frames each view renders
alone, for the exact grid, the learned grid (judged) and no skipping, with
device outputs and with page-locked host outputs written by the launches."""
import numpy as np
import pytest

from ivr_gb300 import api, synth
from ivr_gb300.state import orbit_state

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("skip", [api.SKIP_GRID, api.SKIP_LEARNED, api.SKIP_NONE], ids=["grid", "learned", "none"])
@pytest.mark.parametrize("host_out", [False, True], ids=["device", "pinned"])
def test_frames_in_flight_equal_frames_alone(ctx, skip, host_out):
    import torch
    vol = synth.blob_volume((80, 72, 88), n_blobs=12, seed=31, dtype="u16", zero_fraction=0.6, cell=16)
    v = ctx.load_volume(vol)
    scale = 256.0 / 65536.0
    luts = [synth.knot_tf(700 + t, zero_first=True)[0] for t in range(4)]
    tfs = [ctx.transfer_function().set_lut(lut, 0, scale, api.TF_F2B) for lut in luts]
    mlp = None
    if skip == api.SKIP_LEARNED:
        mlp = ctx.mlp(3)
        for tf in tfs[:2]:
            mlp.add_samples(v, tf)
        mlp.train(4, batch_rows=512)
        margin, _ = mlp.calibrate(0.02)
        v.set_mlp(mlp, margin, certify=True)
    p = api.config_params(skip=skip)
    rng = np.random.default_rng(5)
    frames = [(orbit_state(float(rng.uniform(0, 360)), float(rng.uniform(-60, 60)), 120, 96), k % 4)
              for k in range(9)]
    S = 3
    views = [ctx.view() for _ in range(S)]
    streams = [torch.cuda.Stream() for _ in range(S)]
    outs = []
    for k, (st, t) in enumerate(frames):
        if host_out:
            o = torch.full((96, 120, 4), 7, dtype=torch.uint8).pin_memory()
        else:
            o = torch.full((96, 120, 4), 7, dtype=torch.uint8, device="cuda")
        views[k % S].set(v, st, p)
        views[k % S].render(tfs[t], None, o.data_ptr(), streams[k % S].cuda_stream)
        outs.append(o)
    torch.cuda.synchronize()
    alone = ctx.view()
    for k, (st, t) in enumerate(frames):
        ref = torch.full((96, 120, 4), 9, dtype=torch.uint8, device="cuda")
        alone.set(v, st, p)
        alone.render(tfs[t], None, ref.data_ptr())
        torch.cuda.synchronize()
        assert torch.equal(outs[k].cpu(), ref.cpu()), k
    if skip == api.SKIP_LEARNED:
        assert sum(vw.judge_stats()["frames"] for vw in views) == len(frames)
    for vw in views + [alone]:
        vw.free()
    if mlp is not None:
        v.set_mlp(None)
        mlp.free()
    for tf in tfs:
        tf.free()
    v.free()
