"""ctypes binding of libivr_gpu.so (include/ivr_gpu.h).

The library is built in-tree by ``ivr_gb300.build``.  Loading fails loudly
when it is missing: there is no CPU path behind this package.
"""
from __future__ import annotations

import ctypes
import os

from .state import IvrState

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libivr_gpu.so")

IVR_OK = 0
ERRORS = {-1: "IVR_ERR_INVALID", -2: "IVR_ERR_CUDA", -3: "IVR_ERR_NOMEM", -4: "IVR_ERR_IO",
          -5: "IVR_ERR_UNSUPPORTED", -6: "IVR_ERR_TIMEOUT"}
MAX_BRICKS = 64


class RenderParams(ctypes.Structure):
    _fields_ = [
        ("preset", ctypes.c_int),
        ("step", ctypes.c_float),
        ("max_samples", ctypes.c_int),
        ("term_alpha", ctypes.c_float),
        ("order", ctypes.c_int),
        ("skip", ctypes.c_int),
        ("tilew", ctypes.c_int),
        ("tileh", ctypes.c_int),
        ("judge_stride", ctypes.c_int),
        ("judge_tol", ctypes.c_int),
        ("tile_order", ctypes.c_int),
    ]


class JudgeStats(ctypes.Structure):
    _fields_ = [
        ("frames", ctypes.c_ulonglong),
        ("fallbacks", ctypes.c_ulonglong),
        ("pixels", ctypes.c_ulonglong),
        ("worst", ctypes.c_int),
        ("pad", ctypes.c_int),
        ("exact_frames", ctypes.c_ulonglong),
    ]


MLP_PARAMS = 6337
MLP_IN = 32
MLP_TRANSPARENT = 0.5


class ServerConfig(ctypes.Structure):
    _fields_ = [
        ("slots", ctypes.c_int),
        ("max_batch_frames", ctypes.c_int),
        ("arena_bytes", ctypes.c_size_t),
        ("poll_us", ctypes.c_int),
        ("step", ctypes.c_float),
        ("term_alpha", ctypes.c_float),
        ("tilew", ctypes.c_int),
        ("tileh", ctypes.c_int),
        ("variant", ctypes.c_int),
    ]


class Request(ctypes.Structure):
    _fields_ = [
        ("volume", ctypes.c_int),
        ("tf", ctypes.c_int),
        ("state", IvrState),
        ("rgba8_host", ctypes.c_void_p),
        ("tag", ctypes.c_ulonglong),
    ]


class Completion(ctypes.Structure):
    _fields_ = [
        ("tag", ctypes.c_ulonglong),
        ("status", ctypes.c_int),
        ("vw", ctypes.c_int),
        ("vh", ctypes.c_int),
        ("t_queue", ctypes.c_double),
        ("t_total", ctypes.c_double),
    ]


class FrameInfo(ctypes.Structure):
    _fields_ = [
        ("vw", ctypes.c_int),
        ("vh", ctypes.c_int),
        ("nbricks", ctypes.c_int),
        ("order", ctypes.c_int * MAX_BRICKS),
        ("wincoord", (ctypes.c_float * 6) * MAX_BRICKS),
        ("rect", (ctypes.c_int * 4) * MAX_BRICKS),
    ]


# name -> (restype, argtypes); every function the header declares
_P = ctypes.c_void_p
_I = ctypes.c_int
_F = ctypes.c_float
_PF = ctypes.POINTER(ctypes.c_float)
_PI = ctypes.POINTER(ctypes.c_int)
SIGNATURES = {
    "ivr_params_ref": (None, [ctypes.POINTER(RenderParams)]),
    "ivr_params_config": (None, [ctypes.POINTER(RenderParams)]),
    "ivr_create": (_I, [_I, ctypes.c_size_t, ctypes.POINTER(_P)]),
    "ivr_destroy": (_I, [_P]),
    "ivr_last_error": (ctypes.c_char_p, [_P]),
    "ivr_mem_used": (_I, [_P, ctypes.POINTER(ctypes.c_size_t)]),
    "ivr_volume_load": (_I, [_P, _P, _I, _I, _I, _I, _I, ctypes.POINTER(_P)]),
    "ivr_volume_load_file": (_I, [_P, ctypes.c_char_p, _I, _I, _I, _I, _I, ctypes.POINTER(_P)]),
    "ivr_volume_free": (_I, [_P]),
    "ivr_bricks_setup": (_I, [_P, _I, _I, _I, _I]),
    "ivr_volume_set_quads": (_I, [_P, _I]),
    "ivr_volume_set_macrocell": (_I, [_P, _I]),
    "ivr_volume_macrocell": (_I, [_P, ctypes.POINTER(ctypes.c_int)]),
    "ivr_volume_gradient": (_I, [_P, _P, _P]),
    "ivr_volume_quad_bytes": (_I, [_P, ctypes.POINTER(ctypes.c_size_t)]),
    "ivr_volume_minmax": (_I, [_P, _PF, _PF]),
    "ivr_volume_histogram": (_I, [_P, _PI, _I]),
    "ivr_volume_histogram_noalloc": (_I, [_P, _PI, _I, _PF, _PF, _P]),
    "ivr_tf_create": (_I, [_P, ctypes.POINTER(_P)]),
    "ivr_tf_free": (_I, [_P]),
    "ivr_tf_set_lut": (_I, [_P, _PF, _I, _I, _F, _I]),
    "ivr_tf_set_colormap": (_I, [_P, _P, _I, _I]),
    "ivr_tf_get_lut": (_I, [_P, _PF, _I, _PI, _PI]),
    "ivr_view_create": (_I, [_P, ctypes.POINTER(_P)]),
    "ivr_view_free": (_I, [_P]),
    "ivr_set_view": (_I, [_P, _P, ctypes.POINTER(IvrState), ctypes.POINTER(RenderParams)]),
    "ivr_view_info": (_I, [_P, ctypes.POINTER(FrameInfo)]),
    "ivr_render": (_I, [_P, _P, _P, _P, _P]),
    "ivr_render_tile": (_I, [_P, _P, _I, _I, _I, _I, _P, _P, _P]),
    "ivr_render_brick": (_I, [_P, _P, _I, _P, _P]),
    "ivr_render_host": (_I, [_P, _P, _P, ctypes.POINTER(IvrState), ctypes.POINTER(RenderParams), _P, _P]),
    "ivr_census": (_I, [_P, _P, ctypes.POINTER(ctypes.c_ulonglong), ctypes.POINTER(ctypes.c_ulonglong),
                        ctypes.POINTER(ctypes.c_ulonglong), _P]),
    "ivr_batch_create": (_I, [_P, _I, ctypes.POINTER(_P)]),
    "ivr_batch_free": (_I, [_P]),
    "ivr_batch_clear": (_I, [_P]),
    "ivr_batch_add": (_I, [_P, _P, _P, _P, _P]),
    "ivr_batch_render": (_I, [_P, _I, _P]),
    "ivr_batch_autotune": (_I, [_P, _P, ctypes.POINTER(_I), _PF]),
    "ivr_batch_set_variant": (_I, [_P, _I]),
    "ivr_device_alloc": (_I, [_P, ctypes.c_size_t, ctypes.POINTER(_P)]),
    "ivr_device_free": (_I, [_P, _P, ctypes.c_size_t]),
    "ivr_host_alloc": (_I, [_P, ctypes.c_size_t, ctypes.POINTER(_P)]),
    "ivr_host_free": (_I, [_P, _P]),
    "ivr_server_config_default": (None, [ctypes.POINTER(ServerConfig)]),
    "ivr_server_create": (_I, [_P, ctypes.POINTER(ServerConfig), ctypes.POINTER(_P)]),
    "ivr_server_destroy": (_I, [_P]),
    "ivr_server_add_volume": (_I, [_P, _P, _I, ctypes.POINTER(_I)]),
    "ivr_server_add_tf": (_I, [_P, _PF, _I, _I, _F, ctypes.POINTER(_I)]),
    "ivr_server_submit": (_I, [_P, ctypes.POINTER(Request)]),
    "ivr_server_poll": (_I, [_P, ctypes.POINTER(Completion), _I, ctypes.POINTER(_I), _I]),
    "ivr_server_stats": (_I, [_P, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong),
                              ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(_I)]),
    "ivr_server_listen": (_I, [_P, _I, _I, _I, ctypes.POINTER(_I)]),
    "ivr_server_times": (_I, [_P, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                              ctypes.POINTER(ctypes.c_double)]),
    "ivr_mlp_create": (_I, [_P, ctypes.c_ulonglong, ctypes.POINTER(_P)]),
    "ivr_mlp_free": (_I, [_P]),
    "ivr_mlp_get_params": (_I, [_P, _PF]),
    "ivr_mlp_set_params": (_I, [_P, _PF]),
    "ivr_mlp_save": (_I, [_P, ctypes.c_char_p]),
    "ivr_mlp_load": (_I, [_P, ctypes.c_char_p]),
    "ivr_mlp_features": (_I, [_P, _P, _P, _P, _P, ctypes.c_longlong, ctypes.POINTER(ctypes.c_longlong), _P]),
    "ivr_mlp_forward": (_I, [_P, _P, ctypes.c_longlong, _P, _P]),
    "ivr_mlp_gradient": (_I, [_P, _P, _P, ctypes.c_longlong, _F, _P, _P, _P]),
    "ivr_mlp_add_samples": (_I, [_P, _P, _P, ctypes.POINTER(ctypes.c_longlong)]),
    "ivr_mlp_clear_samples": (_I, [_P]),
    "ivr_mlp_train": (_I, [_P, _I, _I, _F, _F, _PF]),
    "ivr_mlp_calibrate": (_I, [_P, _F, _PF, _PF]),
    "ivr_volume_set_mlp": (_I, [_P, _P, _F, _I]),
    "ivr_view_judge_stats": (_I, [_P, ctypes.POINTER(JudgeStats)]),
    "ivr_volume_learned_stats": (_I, [_P, ctypes.POINTER(ctypes.c_ulonglong)]),
    "ivr_volume_skip_grid": (_I, [_P, _P, _I, _I, _P, ctypes.c_longlong, _PI]),
    "ivr_sample_peak": (_I, [_P, _I, ctypes.POINTER(ctypes.c_double), _P]),
    "ivr_sample_peak_layout": (_I, [_P, _I, _I, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double), _P]),
    "ivr_composite": (_I, [_P, _P, _P, _I, _I, _I, _P]),
    "ivr_quantize": (_I, [_P, _P, _P, ctypes.c_longlong, _P]),
    "ivr_copy": (_I, [_P, _P, _P, ctypes.c_size_t, _P]),
    "ivr_stream_wait": (_I, [_P, _P]),
}

_lib = None


def load(path: str = LIB_PATH) -> ctypes.CDLL:
    """Loads the library (once) and declares every signature."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with `python -m ivr_gb300.build` "
                           "(or __graft_entry__.build()); there is no CPU fallback")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class IvrError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code
