"""Python handles over the C ABI of libivr_gpu.so.

Device buffers are passed as integer device addresses (for example a torch
tensor's ``data_ptr()``), streams as integer ``cudaStream_t`` handles (for
example ``torch.cuda.current_stream().cuda_stream``); ``None`` means null.
Every call raises ``IvrError`` with the library's message on failure.
"""
from __future__ import annotations

import ctypes
from typing import Optional

import numpy as np

from . import _lib
from ._lib import FrameInfo, IvrError, RenderParams
from .state import IvrState

U8, U16, F32 = 0, 1, 2
DTYPES = {np.dtype(np.uint8): U8, np.dtype(np.uint16): U16, np.dtype(np.float32): F32}
TF_SEISMIC, TF_MED, TF_SEISMIC2, TF_CHEM, TF_BLEND, TF_RGBBLEND, TF_F2B = range(7)
CM_BASE, CM_RAINBOW, CM_MEDICAL, CM_SEISMIC, CM_JET, CM_NOMAP = 0, 1, 2, 3, 4, -1
PRESET_REF, PRESET_CONFIG = 0, 1
ORDER_CENTER, ORDER_AXIS = 0, 1
SKIP_NONE, SKIP_GRID, SKIP_LEARNED = 0, 1, 2
# ivr_tile_order: the order a CONFIG launch hands out its 8x4 tiles
TILES_RASTER, TILES_COST = 0, 1
# ivr_sampler_layout (sample-rate roofline comparisons)
SAMPLER_QUADS, SAMPLER_BRICKS, SAMPLER_TEX_POINT, SAMPLER_TEX_LINEAR = 0, 1, 2, 3
MLP_PARAMS, MLP_IN, MLP_TRANSPARENT = _lib.MLP_PARAMS, _lib.MLP_IN, _lib.MLP_TRANSPARENT


def _vp(x) -> Optional[int]:
    return None if x is None else int(x)


def ref_params(tile=(1, 1)) -> RenderParams:
    """The reference's sampling (ray.c): step 0.001, 256-sample cap."""
    p = RenderParams()
    _lib.load().ivr_params_ref(ctypes.byref(p))
    p.tilew, p.tileh = tile
    return p


def config_params(step=0.5, term_alpha=0.99, skip=True, tile=(1, 1), judge_stride=16,
                  judge_tol=1, tiles=TILES_COST) -> RenderParams:
    """Benchmark sampling: true trilinear, ``step`` voxels, early termination.
    ``skip``: True/False for the exact grid or none, or a SKIP_* value
    (SKIP_LEARNED judges 1 in ``judge_stride`` tiles at ``judge_tol``).
    ``tiles``: TILES_COST hands out the costliest tiles first (with a
    skipping grid), TILES_RASTER in row order; the image is the same."""
    p = RenderParams()
    _lib.load().ivr_params_config(ctypes.byref(p))
    p.step = step
    p.term_alpha = term_alpha
    p.skip = (SKIP_GRID if skip else SKIP_NONE) if isinstance(skip, bool) else int(skip)
    p.tilew, p.tileh = tile
    p.judge_stride, p.judge_tol = judge_stride, judge_tol
    p.tile_order = int(tiles)
    return p


class Context:
    """ivr_create / ivr_destroy: one GPU, an optional HBM budget in bytes."""

    def __init__(self, device: int = 0, hbm_budget: int = 0):
        self.lib = _lib.load()
        h = ctypes.c_void_p()
        rc = self.lib.ivr_create(device, hbm_budget, ctypes.byref(h))
        if rc != 0:
            raise IvrError(rc, f"ivr_create(device={device}) failed")
        self.h = h

    def check(self, rc: int):
        if rc != 0:
            raise IvrError(rc, self.lib.ivr_last_error(self.h).decode())

    def close(self):
        if self.h:
            self.lib.ivr_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def mem_used(self) -> int:
        v = ctypes.c_size_t()
        self.check(self.lib.ivr_mem_used(self.h, ctypes.byref(v)))
        return v.value

    def host_frame(self, vh: int, vw: int) -> np.ndarray:
        """A (vh, vw, 4) uint8 frame in page-locked host memory (ivr_host_alloc),
        freed when the array is collected."""
        p = ctypes.c_void_p()
        n = vh * vw * 4
        self.check(self.lib.ivr_host_alloc(self.h, n, ctypes.byref(p)))
        buf = (ctypes.c_uint8 * n).from_address(p.value)
        arr = np.frombuffer(buf, dtype=np.uint8).reshape(vh, vw, 4)
        import weakref
        weakref.finalize(buf, self.lib.ivr_host_free, None, p.value)
        return arr

    def load_volume(self, vol: np.ndarray, byteswap: bool = False) -> "Volume":
        """readvoldata: a (d, h, w) uint8/uint16/float32 array to the device."""
        vol = np.ascontiguousarray(vol)
        if vol.ndim != 3 or vol.dtype not in DTYPES:
            raise ValueError("volume must be a 3-D uint8, uint16 or float32 array (d, h, w)")
        d, h, w = vol.shape
        out = ctypes.c_void_p()
        self.check(self.lib.ivr_volume_load(self.h, vol.ctypes.data, w, h, d, DTYPES[vol.dtype], int(byteswap),
                                            ctypes.byref(out)))
        return Volume(self, out, (d, h, w), DTYPES[vol.dtype])

    def load_volume_file(self, path: str, w: int, h: int, d: int, dtype: int,
                         file_little_endian: bool = True) -> "Volume":
        out = ctypes.c_void_p()
        self.check(self.lib.ivr_volume_load_file(self.h, path.encode(), w, h, d, dtype, int(file_little_endian),
                                                 ctypes.byref(out)))
        return Volume(self, out, (d, h, w), dtype)

    def transfer_function(self) -> "TransferFunction":
        out = ctypes.c_void_p()
        self.check(self.lib.ivr_tf_create(self.h, ctypes.byref(out)))
        return TransferFunction(self, out)

    def view(self) -> "View":
        out = ctypes.c_void_p()
        self.check(self.lib.ivr_view_create(self.h, ctypes.byref(out)))
        return View(self, out)

    def mlp(self, seed: int = 0) -> "Mlp":
        """A learned empty-space predictor (He-initialised)."""
        h = ctypes.c_void_p()
        self.check(self.lib.ivr_mlp_create(self.h, seed, ctypes.byref(h)))
        return Mlp(self, h)

    def batch(self, max_frames: int) -> "Batch":
        out = ctypes.c_void_p()
        self.check(self.lib.ivr_batch_create(self.h, max_frames, ctypes.byref(out)))
        return Batch(self, out)

    def composite(self, tilebuf, rcolorbuf, num: int, w: int, h: int, stream=None):
        """compositetiles: num w*h RGBA sub-images (near -> far) over tilebuf."""
        self.check(self.lib.ivr_composite(self.h, _vp(tilebuf), _vp(rcolorbuf), num, w, h, _vp(stream)))

    def sample_peak(self, dtype: int, stream=None) -> float:
        """Sample-rate roofline of the march's sampler (Gsamples/s)."""
        g = ctypes.c_double()
        self.check(self.lib.ivr_sample_peak(self.h, dtype, ctypes.byref(g), _vp(stream)))
        return g.value

    def sample_peak_layout(self, dtype: int, layout: int, stream=None) -> tuple:
        """(Gsamples/s, largest |sample - exact trilinear|) of the sampler
        roofline through a SAMPLER_* layout."""
        g, err = ctypes.c_double(), ctypes.c_double()
        self.check(self.lib.ivr_sample_peak_layout(self.h, dtype, layout, ctypes.byref(g), ctypes.byref(err),
                                                   _vp(stream)))
        return g.value, err.value

    def quantize(self, src, dst, n: int, stream=None):
        self.check(self.lib.ivr_quantize(self.h, _vp(src), _vp(dst), n, _vp(stream)))


class Volume:
    def __init__(self, ctx: Context, h, shape, dtype):
        self.ctx, self.h, self.shape, self.dtype = ctx, h, shape, dtype

    def bricks(self, py: int, px: int, pz: int, overlap: int = 1) -> "Volume":
        """initvolbbox/getlocalbrick: py rows x px columns x pz slabs."""
        self.ctx.check(self.ctx.lib.ivr_bricks_setup(self.h, py, px, pz, overlap))
        return self

    def gradient(self, out_dev, stream=None):
        """Per-voxel (gx, gy, gz, |g|) into out_dev: float32 [d][h][w][4]."""
        self.ctx.check(self.ctx.lib.ivr_volume_gradient(self.h, _vp(out_dev), _vp(stream)))

    def quads(self, on: bool) -> "Volume":
        """Corner-packed brick copies on/off (on by default)."""
        self.ctx.check(self.ctx.lib.ivr_volume_set_quads(self.h, int(on)))
        return self

    def macrocell(self, cell: int) -> "Volume":
        """Macrocell edge of the skipping grids in voxels (a power of two in
        [4, 32]; 16 by default).  The images do not depend on it."""
        self.ctx.check(self.ctx.lib.ivr_volume_set_macrocell(self.h, int(cell)))
        return self

    def macrocell_edge(self) -> int:
        c = ctypes.c_int()
        self.ctx.check(self.ctx.lib.ivr_volume_macrocell(self.h, ctypes.byref(c)))
        return c.value

    def quad_bytes(self) -> int:
        n = ctypes.c_size_t()
        self.ctx.check(self.ctx.lib.ivr_volume_quad_bytes(self.h, ctypes.byref(n)))
        return n.value

    def minmax(self):
        mn, mx = ctypes.c_float(), ctypes.c_float()
        self.ctx.check(self.ctx.lib.ivr_volume_minmax(self.h, ctypes.byref(mn), ctypes.byref(mx)))
        return mn.value, mx.value

    def histogram(self, hsize: int) -> np.ndarray:
        hist = np.zeros(hsize, dtype=np.int32)
        self.ctx.check(self.ctx.lib.ivr_volume_histogram(
            self.h, hist.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), hsize))
        return hist

    def set_mlp(self, mlp: Optional["Mlp"], margin: float = 0.0, certify: bool = True) -> "Volume":
        """Attaches the predictor used by SKIP_LEARNED views (None detaches);
        ``certify`` checks each learned grid against the exact test as it is
        built and keeps false skips opaque."""
        self.ctx.check(self.ctx.lib.ivr_volume_set_mlp(self.h, mlp.h if mlp else None, margin, int(certify)))
        return self

    def learned_stats(self) -> dict:
        """Cell counts over the learned grids built since set_mlp."""
        st = (ctypes.c_ulonglong * 4)()
        self.ctx.check(self.ctx.lib.ivr_volume_learned_stats(self.h, st))
        return {"cells": st[0], "exact_transparent": st[1], "learned_transparent": st[2], "false_skips": st[3]}

    def skip_grid(self, tf, skip=None, brick=0):
        """The skipping grid frames of `skip` (SKIP_GRID or SKIP_LEARNED) use
        for tf, one brick's macrocells as uint8 [z][y][x]: 0 where a sample
        can be opaque, r >= 1 where every cell within r - 1 is transparent."""
        skip = SKIP_GRID if skip is None else skip
        dims = (ctypes.c_int * 3)()
        lib = self.ctx.lib
        self.ctx.check(lib.ivr_volume_skip_grid(self.h, tf.h, skip, brick, None, 0, dims))
        out = np.zeros((dims[2], dims[1], dims[0]), np.uint8)
        self.ctx.check(lib.ivr_volume_skip_grid(self.h, tf.h, skip, brick, out.ctypes.data, out.size, dims))
        return out

    def free(self):
        if self.h:
            self.ctx.lib.ivr_volume_free(self.h)
            self.h = None


class TransferFunction:
    def __init__(self, ctx: Context, h):
        self.ctx, self.h = ctx, h

    def set_lut(self, rgba: np.ndarray, offset: int = 0, scale: float = 1.0, mode: int = TF_F2B):
        lut = np.ascontiguousarray(rgba, dtype=np.float32).reshape(-1, 4)
        self.ctx.check(self.ctx.lib.ivr_tf_set_lut(self.h, lut.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                                   len(lut), offset, scale, mode))
        return self

    def set_colormap(self, vol: Volume, colormap: int, mode: int):
        """initcolormap + initvolluts + inittransferfunc."""
        self.ctx.check(self.ctx.lib.ivr_tf_set_colormap(self.h, vol.h, colormap, mode))
        return self

    def get_lut(self):
        n, off = ctypes.c_int(), ctypes.c_int()
        self.ctx.check(self.ctx.lib.ivr_tf_get_lut(self.h, None, 0, ctypes.byref(n), ctypes.byref(off)))
        out = np.zeros((n.value, 4), dtype=np.float32)
        self.ctx.check(self.ctx.lib.ivr_tf_get_lut(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                                   n.value, None, None))
        return out, off.value

    def free(self):
        if self.h:
            self.ctx.lib.ivr_tf_free(self.h)
            self.h = None


class View:
    def __init__(self, ctx: Context, h):
        self.ctx, self.h = ctx, h

    def set(self, vol: Volume, state: IvrState, params: RenderParams) -> "View":
        """setviewport/setplaneconst/setmvm/setpm/setfrustum/updatevolbbox."""
        self.ctx.check(self.ctx.lib.ivr_set_view(self.h, vol.h, ctypes.byref(state), ctypes.byref(params)))
        return self

    def info(self) -> dict:
        fi = FrameInfo()
        self.ctx.check(self.ctx.lib.ivr_view_info(self.h, ctypes.byref(fi)))
        n = fi.nbricks
        return {"vw": fi.vw, "vh": fi.vh, "nbricks": n, "order": list(fi.order[:n]),
                "wincoord": [list(fi.wincoord[k]) for k in range(n)], "rect": [list(fi.rect[k]) for k in range(n)]}

    def render(self, tf: TransferFunction, rgba32=None, rgba8=None, stream=None):
        self.ctx.check(self.ctx.lib.ivr_render(self.h, tf.h, _vp(rgba32), _vp(rgba8), _vp(stream)))

    def render_tile(self, tf: TransferFunction, x, y, w, h, rgba32=None, rgba8=None, stream=None):
        self.ctx.check(self.ctx.lib.ivr_render_tile(self.h, tf.h, x, y, w, h, _vp(rgba32), _vp(rgba8), _vp(stream)))

    def render_brick(self, tf: TransferFunction, brick: int, rgba32, stream=None):
        """createlocalimage(rank): one brick's sub-image over the viewport."""
        self.ctx.check(self.ctx.lib.ivr_render_brick(self.h, tf.h, brick, _vp(rgba32), _vp(stream)))

    def census(self, tf: TransferFunction, stream=None) -> dict:
        """Plain-method lattice points, executed samples and touched volume
        bytes of this CONFIG frame (diagnostic launch)."""
        a, e, t = ctypes.c_ulonglong(), ctypes.c_ulonglong(), ctypes.c_ulonglong()
        self.ctx.check(self.ctx.lib.ivr_census(self.h, tf.h, ctypes.byref(a), ctypes.byref(e), ctypes.byref(t),
                                               _vp(stream)))
        return {"lattice": a.value, "executed": e.value, "touched_bytes": t.value}

    def judge_stats(self) -> dict:
        """Totals of the learned-skip judge over this view's frames."""
        st = _lib.JudgeStats()
        self.ctx.check(self.ctx.lib.ivr_view_judge_stats(self.h, ctypes.byref(st)))
        return {"frames": st.frames, "fallbacks": st.fallbacks, "pixels": st.pixels, "worst": st.worst,
                "exact_frames": st.exact_frames}

    def render_host(self, vol: Volume, tf: TransferFunction, state: IvrState, params: RenderParams,
                    out: np.ndarray, stream=None):
        """End to end: STATE in, RGBA8 frame to host memory (out: uint8 [vh, vw, 4])."""
        if out.dtype != np.uint8 or not out.flags.c_contiguous:
            raise ValueError("out must be a C-contiguous uint8 array")
        self.ctx.check(self.ctx.lib.ivr_render_host(self.h, vol.h, tf.h, ctypes.byref(state), ctypes.byref(params),
                                                    out.ctypes.data, _vp(stream)))
        return out

    def free(self):
        if self.h:
            self.ctx.lib.ivr_view_free(self.h)
            self.h = None


class Mlp:
    """The learned empty-space predictor (ivr_mlp_*).  Device arrays are
    integer addresses: features bf16 [n][MLP_IN] (uint16 storage), bounds
    and predictions float32 [n]."""

    def __init__(self, ctx: Context, h):
        self.ctx, self.h = ctx, h

    def _fp(self, a: np.ndarray):
        return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))

    def params(self) -> np.ndarray:
        p = np.zeros(MLP_PARAMS, dtype=np.float32)
        self.ctx.check(self.ctx.lib.ivr_mlp_get_params(self.h, self._fp(p)))
        return p

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, dtype=np.float32)
        if p.size != MLP_PARAMS:
            raise ValueError(f"{MLP_PARAMS} parameters expected")
        self.ctx.check(self.ctx.lib.ivr_mlp_set_params(self.h, self._fp(p)))

    def save(self, path: str):
        self.ctx.check(self.ctx.lib.ivr_mlp_save(self.h, path.encode()))

    def load(self, path: str):
        self.ctx.check(self.ctx.lib.ivr_mlp_load(self.h, path.encode()))

    def features(self, vol: Volume, tf: TransferFunction, x_dev, bound_dev, cap: int, stream=None) -> int:
        n = ctypes.c_longlong()
        self.ctx.check(self.ctx.lib.ivr_mlp_features(self.h, vol.h, tf.h, _vp(x_dev), _vp(bound_dev), cap,
                                                     ctypes.byref(n), _vp(stream)))
        return n.value

    def forward(self, x_dev, n: int, y_dev, stream=None):
        self.ctx.check(self.ctx.lib.ivr_mlp_forward(self.h, _vp(x_dev), n, _vp(y_dev), _vp(stream)))

    def gradient(self, x_dev, bound_dev, n: int, wneg: float, grad_dev, loss_dev, stream=None):
        self.ctx.check(self.ctx.lib.ivr_mlp_gradient(self.h, _vp(x_dev), _vp(bound_dev), n, wneg, _vp(grad_dev),
                                                     _vp(loss_dev), _vp(stream)))

    def add_samples(self, vol: Volume, tf: TransferFunction) -> int:
        n = ctypes.c_longlong()
        self.ctx.check(self.ctx.lib.ivr_mlp_add_samples(self.h, vol.h, tf.h, ctypes.byref(n)))
        return n.value

    def clear_samples(self):
        self.ctx.check(self.ctx.lib.ivr_mlp_clear_samples(self.h))

    def train(self, epochs: int, batch_rows: int = 8192, lr: float = 2e-3, wneg: float = 4.0) -> np.ndarray:
        losses = np.zeros(epochs, dtype=np.float32)
        self.ctx.check(self.ctx.lib.ivr_mlp_train(self.h, epochs, batch_rows, lr, wneg, self._fp(losses)))
        return losses

    def calibrate(self, slack: float = 0.02):
        """(margin, recall): the margin that keeps every training cell with a
        bound above 0 opaque, and the share of transparent cells it keeps."""
        m, r = ctypes.c_float(), ctypes.c_float()
        self.ctx.check(self.ctx.lib.ivr_mlp_calibrate(self.h, slack, ctypes.byref(m), ctypes.byref(r)))
        return m.value, r.value

    def free(self):
        if self.h:
            self.ctx.lib.ivr_mlp_free(self.h)
            self.h = None


class Batch:
    """Many CONFIG frames in one persistent launch (ivr_batch_*)."""

    VARIANTS = ["8x4 pair", "8x4", "4x8 pair", "4x8", "16x2 pair", "16x2"]

    def __init__(self, ctx: Context, h):
        self.ctx, self.h = ctx, h

    def clear(self):
        self.ctx.check(self.ctx.lib.ivr_batch_clear(self.h))

    def add(self, view: View, tf: TransferFunction, rgba32=None, rgba8=None):
        self.ctx.check(self.ctx.lib.ivr_batch_add(self.h, view.h, tf.h, _vp(rgba32), _vp(rgba8)))

    def render(self, use_graph: bool = False, stream=None):
        self.ctx.check(self.ctx.lib.ivr_batch_render(self.h, int(use_graph), _vp(stream)))

    def autotune(self, stream=None):
        v = ctypes.c_int()
        ms = (ctypes.c_float * 6)()
        self.ctx.check(self.ctx.lib.ivr_batch_autotune(self.h, _vp(stream), ctypes.byref(v), ms))
        return v.value, list(ms)

    def set_variant(self, v: int):
        self.ctx.check(self.ctx.lib.ivr_batch_set_variant(self.h, v))

    def free(self):
        if self.h:
            self.ctx.lib.ivr_batch_free(self.h)
            self.h = None


class Server:
    """The steering server (ivr_server_*): continuous batching over resident
    volumes.  While it runs, its context belongs to the server's threads."""

    def __init__(self, ctx: Context, slots=4, max_batch_frames=64, arena_mib=96, step=0.5, term_alpha=0.99,
                 poll_us=100):
        self.ctx = ctx
        self.lib = ctx.lib
        cfg = _lib.ServerConfig()
        self.lib.ivr_server_config_default(ctypes.byref(cfg))
        cfg.slots, cfg.max_batch_frames = slots, max_batch_frames
        cfg.arena_bytes = int(arena_mib) << 20
        cfg.step, cfg.term_alpha, cfg.poll_us = step, term_alpha, poll_us
        self.cfg = cfg
        h = ctypes.c_void_p()
        ctx.check(self.lib.ivr_server_create(ctx.h, ctypes.byref(cfg), ctypes.byref(h)))
        self.h = h
        self.keep = {}  # tag -> host buffer, alive until completion

    def add_volume(self, vol: Volume) -> int:
        i = ctypes.c_int()
        self.ctx.check(self.lib.ivr_server_add_volume(self.h, vol.h, vol.dtype, ctypes.byref(i)))
        return i.value

    def add_tf(self, rgba: np.ndarray, offset: int = 0, scale: float = 1.0) -> int:
        lut = np.ascontiguousarray(rgba, dtype=np.float32).reshape(-1, 4)
        i = ctypes.c_int()
        self.ctx.check(self.lib.ivr_server_add_tf(self.h, lut.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                                  len(lut), offset, scale, ctypes.byref(i)))
        return i.value

    def submit(self, volume: int, tf: int, state: IvrState, tag: int, out: np.ndarray = None) -> np.ndarray:
        vw = (state.winwidth // self.cfg.tilew) * self.cfg.tilew
        vh = (state.winheight // self.cfg.tileh) * self.cfg.tileh
        if out is None:
            out = np.empty((vh, vw, 4), np.uint8)
        r = _lib.Request()
        r.volume, r.tf, r.state, r.tag = volume, tf, state, tag
        r.rgba8_host = out.ctypes.data
        self.keep[tag] = out
        self.ctx.check(self.lib.ivr_server_submit(self.h, ctypes.byref(r)))
        return out

    def poll(self, max_n: int = 256, wait_ms: int = 10):
        buf = (_lib.Completion * max_n)()
        n = ctypes.c_int()
        self.ctx.check(self.lib.ivr_server_poll(self.h, buf, max_n, ctypes.byref(n), wait_ms))
        res = []
        for k in range(n.value):
            c = buf[k]
            out = self.keep.pop(c.tag, None)
            res.append({"tag": c.tag, "status": c.status, "vw": c.vw, "vh": c.vh, "t_queue": c.t_queue,
                        "t_total": c.t_total, "frame": out})
        return res

    def stats(self) -> dict:
        c, r, b = ctypes.c_longlong(), ctypes.c_longlong(), ctypes.c_longlong()
        q = ctypes.c_int()
        self.ctx.check(self.lib.ivr_server_stats(self.h, ctypes.byref(c), ctypes.byref(r), ctypes.byref(b),
                                                 ctypes.byref(q)))
        g, d, f = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        self.ctx.check(self.lib.ivr_server_times(self.h, ctypes.byref(g), ctypes.byref(d), ctypes.byref(f)))
        return {"completed": c.value, "rejected": r.value, "batches": b.value, "queued": q.value,
                "gpu_s": g.value, "dispatch_s": d.value, "finish_s": f.value}

    def listen(self, volume: int, tf: int, port: int = 0) -> int:
        p = ctypes.c_int()
        self.ctx.check(self.lib.ivr_server_listen(self.h, port, volume, tf, ctypes.byref(p)))
        return p.value

    def close(self):
        if self.h:
            self.lib.ivr_server_destroy(self.h)
            self.h = None
