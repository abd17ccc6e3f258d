"""CPU: the C-ABI library loads and exports every function include/ivr_gpu.h
declares, with the declared record sizes (no device calls)."""
import ctypes
import os
import re

import pytest

from conftest import ROOT


def declared_functions():
    src = open(os.path.join(ROOT, "include", "ivr_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_ \*]*?\b(ivr_[a-z0-9_]+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ["ivr_create", "ivr_volume_load", "ivr_bricks_setup", "ivr_set_view", "ivr_tf_set_colormap",
                 "ivr_render", "ivr_render_tile", "ivr_render_brick", "ivr_composite", "ivr_quantize"]:
        assert must in names


def test_library_exports_every_declared_symbol(gpu_lib):
    missing = [n for n in declared_functions() if not hasattr(gpu_lib, n)]
    assert not missing, missing


def test_python_binding_covers_header(gpu_lib):
    from ivr_gb300 import _lib
    assert set(declared_functions()) <= set(_lib.SIGNATURES)


def test_record_sizes():
    from ivr_gb300._lib import FrameInfo, RenderParams
    from ivr_gb300.state import IvrState
    assert ctypes.sizeof(IvrState) == 184
    assert ctypes.sizeof(RenderParams) == 44
    assert ctypes.sizeof(FrameInfo) == 12 + 64 * 4 + 64 * 24 + 64 * 16
    from ivr_gb300._lib import Completion, Request, ServerConfig
    assert ctypes.sizeof(Request) == 4 + 4 + 184 + 8 + 8
    assert ctypes.sizeof(Completion) == 8 + 4 * 3 + 4 + 16
    assert ctypes.sizeof(ServerConfig) == 40
    from ivr_gb300._lib import JudgeStats
    assert ctypes.sizeof(JudgeStats) == 40


def test_record_layout_matches_the_c_compiler(tmp_path):
    """sizeof of every record as gcc lays it out from the header, against
    the ctypes mirrors."""
    import shutil
    import subprocess
    if shutil.which("gcc") is None:
        pytest.skip("no C compiler")
    from ivr_gb300 import _lib
    from ivr_gb300.state import IvrState
    recs = {"ivr_state": IvrState, "ivr_render_params": _lib.RenderParams, "ivr_frame_info": _lib.FrameInfo,
            "ivr_server_config": _lib.ServerConfig, "ivr_request": _lib.Request, "ivr_completion": _lib.Completion,
            "ivr_judge_stats": _lib.JudgeStats}
    src = tmp_path / "sizes.c"
    src.write_text('#include <stdio.h>\n#include "ivr_gpu.h"\nint main(void){\n' +
                   "".join(f'printf("{k} %zu\\n", sizeof({k}));\n' for k in recs) + "return 0;}\n")
    exe = tmp_path / "sizes"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    got = dict(zip(out[0::2], (int(x) for x in out[1::2])))
    for k, rec in recs.items():
        assert got[k] == ctypes.sizeof(rec), k


def test_errors_without_device(gpu_lib):
    # argument checks that return before any CUDA call
    assert gpu_lib.ivr_destroy(None) == -1
    assert gpu_lib.ivr_create(0, 0, None) == -1
    assert gpu_lib.ivr_last_error(None) == b"null context"
    assert gpu_lib.ivr_volume_set_macrocell(None, 8) == -1
    assert gpu_lib.ivr_volume_macrocell(None, None) == -1
    assert gpu_lib.ivr_volume_set_quads(None, 1) == -1
