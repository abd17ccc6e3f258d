"""GPU: the steering server.  Each frame served in a mix of concurrent
requests (different volumes, dtypes, sizes, TFs) equals the frame rendered
alone; a frame larger than one slot's share of the output pool waits for
memory and is served, one larger than the pool is rejected without
stopping the server; the TCP
front end speaks the reference's STATE/RGBA8 protocol and survives clients
that disconnect mid-message."""
import socket
import struct

import numpy as np
import pytest

from ivr_gb300 import api, serve, synth
from ivr_gb300.state import orbit_state

pytestmark = pytest.mark.gpu


def render_alone(ctx, vol, lut, scale, st):
    import torch
    tf = ctx.transfer_function().set_lut(lut, 0, scale, api.TF_F2B)
    view = ctx.view().set(vol, st, api.config_params())
    out = torch.zeros((st.winheight, st.winwidth, 4), dtype=torch.uint8, device="cuda")
    view.render(tf, None, out.data_ptr())
    torch.cuda.synchronize()
    view.free()
    tf.free()
    return out.cpu().numpy()


@pytest.fixture(scope="module")
def vols(gpu_lib):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    ctx = api.Context(0)
    a = ctx.load_volume(synth.blob_volume((40, 40, 40), n_blobs=8, seed=31, dtype="u8"))
    b = ctx.load_volume(synth.blob_volume((36, 44, 40), n_blobs=8, seed=32, dtype="f32")).bricks(2, 2, 2)
    c = ctx.load_volume(synth.blob_volume((32, 32, 48), n_blobs=8, seed=33, dtype="u16"))
    yield ctx, [(a, 1.0), (b, 1.0), (c, 256.0 / 65536.0)]
    ctx.close()


@pytest.mark.parametrize("pinned", [False, True], ids=["staged", "page-locked"])
def test_served_frames_equal_frames_rendered_alone(vols, pinned):
    """Pageable output buffers go through the server's staging copy;
    page-locked ones (ivr_host_alloc) receive the frame directly."""
    ctx, vs = vols
    srv = api.Server(ctx, slots=3, max_batch_frames=8, arena_mib=8)
    ids = [srv.add_volume(v) for v, _ in vs]
    luts = [synth.knot_tf(s)[0] for s in range(3)]
    tf_ids = {(t, k): srv.add_tf(luts[t], 0, vs[k][1]) for t in range(3) for k in range(3)}
    rng = np.random.default_rng(5)
    reqs = {}
    for tag in range(60):
        k, t = int(rng.integers(3)), int(rng.integers(3))
        w, h = [(48, 48), (64, 40), (80, 80), (32, 56)][tag % 4]
        st = orbit_state(float(rng.uniform(0, 360)), float(rng.uniform(-50, 50)), w, h, fovy=30.0, alpha=1.0)
        out = ctx.host_frame(h, w) if pinned else None
        srv.submit(ids[k], tf_ids[(t, k)], st, tag, out=out)
        reqs[tag] = (k, t, st)
    done = []
    while len(done) < len(reqs):
        got = srv.poll(wait_ms=200)
        assert got or len(done) < len(reqs)
        done.extend(got)
    stats = srv.stats()
    srv.close()
    assert stats["completed"] == 60 and stats["rejected"] == 0
    assert stats["batches"] >= 60 // 8
    for r in done:
        assert r["status"] == 0
        k, t, st = reqs[r["tag"]]
        alone = render_alone(ctx, vs[k][0], luts[t], vs[k][1], st)
        assert np.array_equal(r["frame"], alone), f"request {r['tag']}"


def test_oversized_request_is_rejected(vols):
    ctx, vs = vols
    srv = api.Server(ctx, slots=1, max_batch_frames=4, arena_mib=1)
    vid = srv.add_volume(vs[0][0])
    tf = srv.add_tf(synth.ramp_tf(), 0, 1.0)
    srv.submit(vid, tf, orbit_state(10, 10, 1024, 1024), 1)  # 4 MiB > 1 MiB arena
    srv.submit(vid, tf, orbit_state(10, 10, 64, 64), 2)
    got = []
    while len(got) < 2:
        got.extend(srv.poll(wait_ms=200))
    srv.close()
    st = {r["tag"]: r["status"] for r in got}
    assert st[1] == -3 and st[2] == 0


def test_pool_admits_a_frame_larger_than_one_arena(vols):
    """The output pool is slots x arena_bytes, shared: a frame larger than
    one slot's share waits for pool memory and is served; only a frame
    larger than the whole pool is refused.  Requests of the three volume
    dtypes share batches."""
    ctx, vs = vols
    srv = api.Server(ctx, slots=4, max_batch_frames=8, arena_mib=1)  # a 4 MiB pool
    ids = [srv.add_volume(v) for v, _ in vs]
    luts = [synth.knot_tf(40 + k)[0] for k in range(3)]
    tfs = [srv.add_tf(luts[k], 0, vs[k][1]) for k in range(3)]
    sizes = [(64, 48), (1024, 768), (80, 80), (1100, 1000), (48, 64), (512, 512)]  # 3 MiB; 4.4 MB > pool
    reqs = {}
    for tag, (w, h) in enumerate(sizes * 2):
        k = tag % 3
        st = orbit_state(20.0 + 37 * tag, 10.0, w, h, fovy=30.0, alpha=1.0)
        srv.submit(ids[k], tfs[k], st, tag)
        reqs[tag] = (k, st, w * h * 4)
    done = []
    while len(done) < len(reqs):
        done.extend(srv.poll(wait_ms=200))
    stats = srv.stats()
    srv.close()
    for r in done:
        k, st, nbytes = reqs[r["tag"]]
        if nbytes > 4 << 20:
            assert r["status"] == -3, r
            continue
        assert r["status"] == 0, r
        assert np.array_equal(r["frame"], render_alone(ctx, vs[k][0], luts[k], vs[k][1], st)), r["tag"]
    assert stats["rejected"] == 2 and stats["completed"] == len(reqs) - 2


def state_bytes(st):
    b = bytearray(st.to_bytes())
    b[0:12] = struct.pack("!iii", st.finish, st.winwidth, st.winheight)  # htonl, connection.c:167-177
    return bytes(b)


def recv_all(sock, n):
    buf = bytearray()
    while len(buf) < n:
        chunk = sock.recv(n - len(buf))
        if not chunk:
            break
        buf.extend(chunk)
    return bytes(buf)


def test_tcp_front_end(vols):
    ctx, vs = vols
    srv = api.Server(ctx, slots=2, max_batch_frames=4, arena_mib=4)
    vid = srv.add_volume(vs[1][0])
    lut = synth.ramp_tf()
    tf = srv.add_tf(lut, 0, 1.0)
    port = srv.listen(vid, tf)
    # a client that disconnects in the middle of a STATE
    bad = socket.create_connection(("127.0.0.1", port))
    bad.sendall(state_bytes(orbit_state(0, 0, 32, 32))[:100])
    bad.close()
    frames = []
    with socket.create_connection(("127.0.0.1", port)) as s:
        for az in (15.0, 75.0):
            st = orbit_state(az, 20, 64, 48, fovy=30.0, alpha=1.0)
            s.sendall(state_bytes(st))
            frames.append((st, recv_all(s, 64 * 48 * 4)))
        fin = orbit_state(0, 0, 8, 8)
        fin.finish = 1
        s.sendall(state_bytes(fin))
    # a client that stays connected without sending: closing the server
    # shuts its connection down instead of waiting for it
    idle = socket.create_connection(("127.0.0.1", port))
    idle.settimeout(30)
    srv.close()
    try:
        assert idle.recv(1) == b""
    except ConnectionResetError:
        pass
    idle.close()
    for st, data in frames:
        assert len(data) == 64 * 48 * 4
        img = np.frombuffer(data, np.uint8).reshape(48, 64, 4)
        assert np.array_equal(img, render_alone(ctx, vs[1][0], lut, 1.0, st))


def test_poisson_load_short(vols):
    ctx, vs = vols
    srv = api.Server(ctx, slots=4, max_batch_frames=32, arena_mib=16)
    ids = [srv.add_volume(v) for v, _ in vs]
    res, wall = serve.run(srv, ids, [s for _, s in vs], duration=1.0, clients=8, rate=(10, 30),
                          sizes=[(64, 64), (128, 96), (192, 192)], seed=3)
    srv.close()
    assert res and all(r["status"] == 0 for r in res)
    lat = np.array([r["latency"] for r in res])
    assert np.percentile(lat, 99) < 1.0
