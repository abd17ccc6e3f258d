"""ctypes bindings of the CPU oracles.  TEST INFRASTRUCTURE ONLY.

O2 (liboracle.so, ivr_oracle.c) is this project's CPU restatement of the
hot path; O1 (_ref/libivr_ref.so) is the reference's own C code driven by
ref_driver.c, present only where the reference sources could be compiled.
Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline use these.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import tempfile

import numpy as np

from ivr_gb300.state import IvrState

HERE = os.path.dirname(os.path.abspath(__file__))
O2_PATH = os.path.join(HERE, "liboracle.so")
O1_PATH = os.path.join(HERE, "_ref", "libivr_ref.so")
# where the reference checkout lies: IVR_REFERENCE_SRC, else the checkout this
# build was set up with
REF_SRC = os.environ.get("IVR_REFERENCE_SRC") or "/root/reference"

U8, U16, F32 = 0, 1, 2
PRESET_REF, PRESET_CONFIG = 0, 1
ORDER_CENTER, ORDER_AXIS = 0, 1
DT_CODE = {np.dtype(np.uint8): U8, np.dtype(np.uint16): U16, np.dtype(np.float32): F32}


class OrcScene(ctypes.Structure):
    _fields_ = [("data", ctypes.c_void_p), ("dtype", ctypes.c_int), ("gw", ctypes.c_int), ("gh", ctypes.c_int),
                ("gd", ctypes.c_int), ("procdims", ctypes.c_int * 3), ("overlap", ctypes.c_int),
                ("state", IvrState), ("tilew", ctypes.c_int), ("tileh", ctypes.c_int),
                ("lut", ctypes.POINTER(ctypes.c_float)), ("lut_n", ctypes.c_int), ("lut_offset", ctypes.c_int),
                ("lut_scale", ctypes.c_float), ("tf_mode", ctypes.c_int), ("preset", ctypes.c_int),
                ("step", ctypes.c_float), ("max_samples", ctypes.c_int), ("term_alpha", ctypes.c_float),
                ("order", ctypes.c_int), ("row0", ctypes.c_int), ("row1", ctypes.c_int), ("skip", ctypes.c_int)]


class OrcStats(ctypes.Structure):
    _fields_ = [("samples_alg", ctypes.c_longlong), ("samples_exec", ctypes.c_longlong), ("vw", ctypes.c_int),
                ("vh", ctypes.c_int), ("nbricks", ctypes.c_int), ("wincoord", (ctypes.c_float * 6) * 64),
                ("order", ctypes.c_int * 64), ("rect", (ctypes.c_int * 4) * 64)]


class RefFrame(ctypes.Structure):
    _fields_ = [("width", ctypes.c_int), ("height", ctypes.c_int), ("depth", ctypes.c_int),
                ("dataendian", ctypes.c_int), ("colormap", ctypes.c_int), ("xfer", ctypes.c_int),
                ("procdims", ctypes.c_int * 3), ("tilew", ctypes.c_int), ("tileh", ctypes.c_int),
                ("winwidth", ctypes.c_int), ("winheight", ctypes.c_int), ("alpha", ctypes.c_float),
                ("newconst", ctypes.c_float * 6), ("vv", ctypes.c_float * 4), ("mvm", ctypes.c_float * 16),
                ("pm", ctypes.c_float * 16), ("inj_lut", ctypes.POINTER(ctypes.c_float)), ("inj_n", ctypes.c_int),
                ("inj_offset", ctypes.c_int)]


_FP = ctypes.POINTER(ctypes.c_float)


def _fp(a):
    return None if a is None else a.ctypes.data_as(_FP)


def build(ref: bool | None = None) -> None:
    """make the oracles: O2 always, O1 when the reference sources exist."""
    subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True)
    if ref is None:
        ref = os.path.isdir(REF_SRC)
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={REF_SRC}"], check=True)


_o2 = None
_o1 = None


def o2():
    global _o2
    if _o2 is None:
        if not os.path.exists(O2_PATH):
            build(ref=False)
        lib = ctypes.CDLL(O2_PATH)
        lib.orc_render.restype = ctypes.c_int
        lib.orc_render.argtypes = [ctypes.POINTER(OrcScene), ctypes.c_int, _FP, ctypes.c_void_p, _FP,
                                   ctypes.POINTER(OrcStats)]
        lib.orc_prepare.restype = ctypes.c_void_p
        lib.orc_prepare.argtypes = [ctypes.POINTER(OrcScene)]
        lib.orc_prepared_free.argtypes = [ctypes.c_void_p]
        lib.orc_render_prepared.restype = ctypes.c_int
        lib.orc_render_prepared.argtypes = [ctypes.POINTER(OrcScene), ctypes.c_void_p, ctypes.c_int, _FP,
                                            ctypes.c_void_p, _FP, ctypes.POINTER(OrcStats)]
        lib.orc_composite.argtypes = [_FP, _FP, ctypes.POINTER(ctypes.c_int), ctypes.c_int, ctypes.c_int]
        lib.orc_quantize.argtypes = [_FP, ctypes.c_void_p, ctypes.c_longlong]
        lib.orc_colormap.argtypes = [ctypes.c_int, _FP, ctypes.c_int, ctypes.c_float, ctypes.c_float]
        lib.orc_minmax.restype = ctypes.c_int
        lib.orc_minmax.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_longlong, _FP, _FP]
        lib.orc_histogram.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_longlong, ctypes.c_float,
                                      ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
        lib.orc_macrocells.argtypes = [_FP, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, _FP, _FP]
        lib.orc_gradient.argtypes = [_FP, ctypes.c_int, ctypes.c_int, ctypes.c_int, _FP]
        _o2 = lib
    return _o2


def o1_available() -> bool:
    return os.path.exists(O1_PATH)


def o1():
    global _o1
    if _o1 is None:
        lib = ctypes.CDLL(O1_PATH)
        lib.ref_render.restype = ctypes.c_int
        lib.ref_render.argtypes = [ctypes.c_char_p, ctypes.POINTER(RefFrame), ctypes.c_int, _FP, _FP, _FP, _FP,
                                   ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
        lib.ref_colormap.argtypes = [ctypes.c_int, _FP, ctypes.c_int, ctypes.c_float, ctypes.c_float]
        lib.ref_quantize.argtypes = [_FP, ctypes.c_void_p, ctypes.c_longlong]
        _o1 = lib
    return _o1


def viewport(state: IvrState, tile) -> tuple:
    return (state.winwidth // tile[0]) * tile[0], (state.winheight // tile[1]) * tile[1]


class Prepared:
    """Brick arrays of one volume and brick grid, extracted once."""

    def __init__(self, vol: np.ndarray, procdims=(1, 1, 1)):
        self.vol = np.ascontiguousarray(vol)
        self.procdims = tuple(procdims)
        sc = _scene(self.vol, None, None, 0, 0, procdims, (1, 1))
        self.h = o2().orc_prepare(ctypes.byref(sc))
        if not self.h:
            raise RuntimeError("orc_prepare failed")

    def __del__(self):
        if getattr(self, "h", None):
            o2().orc_prepared_free(self.h)
            self.h = None


def _scene(vol, state, lut_arr, lut_offset, tf_mode, procdims, tile):
    d, h, w = vol.shape
    sc = OrcScene()
    sc.data = vol.ctypes.data
    sc.dtype = DT_CODE[vol.dtype]
    sc.gw, sc.gh, sc.gd = w, h, d
    for i in range(3):
        sc.procdims[i] = procdims[i]
    sc.overlap = 1
    if state is not None:
        sc.state = state
    else:
        sc.state.winwidth = sc.state.winheight = 1
    sc.tilew, sc.tileh = tile
    if lut_arr is not None:
        sc.lut = lut_arr.ctypes.data_as(_FP)
        sc.lut_n = len(lut_arr)
    sc.lut_offset = lut_offset
    sc.tf_mode = tf_mode
    return sc


def render(vol: np.ndarray, state: IvrState, lut: np.ndarray, lut_offset: int, tf_mode: int, *,
           procdims=(1, 1, 1), tile=(1, 1), preset=PRESET_REF, step=None, max_samples=None, term_alpha=None,
           order=None, lut_scale=1.0, rows=None, threads=0, bricks=False, prepared: "Prepared" = None,
           skip=False):
    """O2 frame.  Returns dict(rgba32, rgba8, bricks, stats)."""
    if prepared is not None:
        vol = prepared.vol
        assert tuple(procdims) == prepared.procdims
    vol = np.ascontiguousarray(vol)
    d, h, w = vol.shape
    sc = OrcScene()
    sc.data = vol.ctypes.data
    sc.dtype = DT_CODE[vol.dtype]
    sc.gw, sc.gh, sc.gd = w, h, d
    for i in range(3):
        sc.procdims[i] = procdims[i]
    sc.overlap = 1
    sc.state = state
    sc.tilew, sc.tileh = tile
    lut_arr = np.ascontiguousarray(lut if lut is not None else np.zeros((1, 4)), dtype=np.float32)
    sc.lut = lut_arr.ctypes.data_as(_FP)
    sc.lut_n = len(lut_arr)
    sc.lut_offset = lut_offset
    sc.lut_scale = lut_scale
    sc.tf_mode = tf_mode
    sc.preset = preset
    ref = preset == PRESET_REF
    sc.step = step if step is not None else (0.001 if ref else 0.5)
    sc.max_samples = max_samples if max_samples is not None else (256 if ref else 0)
    sc.term_alpha = term_alpha if term_alpha is not None else (2.0 if ref else 0.99)
    sc.order = order if order is not None else (ORDER_CENTER if ref else ORDER_AXIS)
    sc.row0, sc.row1 = rows if rows is not None else (0, 0)
    sc.skip = int(skip)
    vw, vh = viewport(state, tile)
    K = procdims[0] * procdims[1] * procdims[2]
    rgba32 = np.zeros((vh, vw, 4), np.float32)
    rgba8 = np.zeros((vh, vw, 4), np.uint8)
    bimg = np.zeros((K, vh, vw, 4), np.float32) if bricks else None
    st = OrcStats()
    rc = o2().orc_render_prepared(ctypes.byref(sc), prepared.h if prepared is not None else None, threads,
                                  _fp(rgba32), rgba8.ctypes.data, _fp(bimg), ctypes.byref(st))
    if rc != K:
        raise RuntimeError(f"orc_render failed: {rc}")
    stats = {"samples_alg": st.samples_alg, "samples_exec": st.samples_exec, "order": list(st.order[:K]),
             "wincoord": [list(st.wincoord[k]) for k in range(K)], "rect": [list(st.rect[k]) for k in range(K)]}
    return {"rgba32": rgba32, "rgba8": rgba8, "bricks": bimg, "stats": stats}


def colormap(cm: int, hsize: int, hmin: float, hmax: float) -> np.ndarray:
    out = np.zeros((hsize, 4), np.float32)
    o2().orc_colormap(cm, _fp(out), hsize, hmin, hmax)
    return out


def lut_for(vol: np.ndarray, cm: int):
    """initvolluts over the whole volume: (lut, lutoffset)."""
    v = np.ascontiguousarray(vol)
    mn, mx = ctypes.c_float(), ctypes.c_float()
    hsize = o2().orc_minmax(v.ctypes.data, DT_CODE[v.dtype], v.size, ctypes.byref(mn), ctypes.byref(mx))
    lut = colormap(cm, hsize, mn.value, mx.value)
    return lut, int(mn.value + 0.5)


def minmax_histogram(vol: np.ndarray, hsize: int = 0):
    """initvolluts' min, max and histogram (mathutil.c:444-470) over the
    whole volume: (mn, mx, hist) with hsize bins (0: (int)(max-min+1))."""
    v = np.ascontiguousarray(vol)
    mn, mx = ctypes.c_float(), ctypes.c_float()
    full = o2().orc_minmax(v.ctypes.data, DT_CODE[v.dtype], v.size, ctypes.byref(mn), ctypes.byref(mx))
    n = hsize or full
    hist = np.zeros(n, np.int32)
    o2().orc_histogram(v.ctypes.data, DT_CODE[v.dtype], v.size, mn.value, n,
                       hist.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
    return mn.value, mx.value, hist


def quantize(x: np.ndarray) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float32)
    out = np.zeros(x.shape, np.uint8)
    o2().orc_quantize(_fp(x), out.ctypes.data, x.size)
    return out


def composite(sub: np.ndarray, order, base=None) -> np.ndarray:
    """compositetiles over whole frames: sub [K, h, w, 4], order near -> far."""
    K = sub.shape[0]
    npix = sub.shape[1] * sub.shape[2]
    dst = np.zeros(sub.shape[1:], np.float32) if base is None else np.array(base, np.float32)
    s = np.ascontiguousarray(sub, np.float32)
    o = np.array(order, np.int32)
    o2().orc_composite(_fp(dst), _fp(s), o.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), K, npix)
    return dst


def macrocells(vol: np.ndarray, cell=16):
    v = np.ascontiguousarray(vol, np.float32)
    d, h, w = v.shape
    shp = ((d + cell - 1) // cell, (h + cell - 1) // cell, (w + cell - 1) // cell)
    mn = np.zeros(shp, np.float32)
    mx = np.zeros(shp, np.float32)
    o2().orc_macrocells(_fp(v), w, h, d, cell, _fp(mn), _fp(mx))
    return mn, mx


def gradient(vol: np.ndarray) -> np.ndarray:
    """Per-voxel (gx, gy, gz, |g|) of the volume as float32 [d][h][w][4]."""
    v = np.ascontiguousarray(vol, np.float32)
    d, h, w = v.shape
    out = np.zeros((d, h, w, 4), np.float32)
    o2().orc_gradient(_fp(v), w, h, d, _fp(out))
    return out


def ref_render(vol: np.ndarray, state: IvrState, colormap_id: int, xfer: int, procdims=(1, 1, 1), tile=(1, 1),
               inj_lut=None, inj_offset=0, big_endian_file=False, threads=1):
    """O1: the reference's own code for one frame (vol written as float32)."""
    d, h, w = vol.shape
    fd, path = tempfile.mkstemp(suffix=".raw")
    os.close(fd)
    try:
        np.ascontiguousarray(vol, dtype=">f4" if big_endian_file else "<f4").tofile(path)
        f = RefFrame()
        f.width, f.height, f.depth = w, h, d
        f.dataendian = 0 if big_endian_file else 1  # endianness(): 1 = little
        f.colormap = colormap_id
        f.xfer = xfer
        for i in range(3):
            f.procdims[i] = procdims[i]
        f.tilew, f.tileh = tile
        f.winwidth, f.winheight, f.alpha = state.winwidth, state.winheight, state.alpha
        for i in range(6):
            f.newconst[i] = state.newconst[i]
        for i in range(4):
            f.vv[i] = state.vv[i]
        for i in range(16):
            f.mvm[i] = state.mvm[i]
            f.pm[i] = state.pm[i]
        lut_keep = None
        if inj_lut is not None:
            lut_keep = np.ascontiguousarray(inj_lut, np.float32)
            f.inj_lut = lut_keep.ctypes.data_as(_FP)
            f.inj_n = len(lut_keep)
            f.inj_offset = inj_offset
        vw, vh = viewport(state, tile)
        K = procdims[0] * procdims[1] * procdims[2]
        out = np.zeros((vh, vw, 4), np.float32)
        bimg = np.zeros((K, vh, vw, 4), np.float32)
        info = np.zeros((K, 8), np.float32)
        lut = np.zeros((1 << 17, 4), np.float32)
        lutinfo = np.zeros(2, np.int32)
        vp = np.zeros(2, np.int32)
        rc = o1().ref_render(path.encode(), ctypes.byref(f), threads, _fp(out), _fp(bimg), _fp(info), _fp(lut),
                             lutinfo.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                             vp.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
        if rc != K:
            raise RuntimeError(f"ref_render failed: {rc}")
        return {"rgba32": out, "bricks": bimg, "info": info, "lut": lut[:lutinfo[0]].copy(),
                "lutoffset": int(lutinfo[1])}
    finally:
        os.unlink(path)
