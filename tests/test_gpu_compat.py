"""GPU: the reference's steered frame through its own function names.

A C program (tests/compat/compat_driver.c) calls init, then the frame
sequence of main.c:226-248 -- setviewport, setplaneconst, setmvm, setpm,
setfrustum, updatevolbbox, initcolbufs, createlocalimage for every rank,
compositelocalimage -- and writetomemory, all from include/ivr_compat.h over
libivr_compat.so.  Every brick's sub-image, the composited frame and its
RGBA8 must equal the reference's golden output bit for bit.
"""
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT, load_case

pytestmark = pytest.mark.gpu

INC = os.path.join(ROOT, "include")
LIBDIR = os.path.join(ROOT, "ivr_gb300")


@pytest.fixture(scope="module")
def driver(tmp_path_factory, gpu_lib):
    from ivr_gb300 import build
    if not os.path.exists(build.COMPAT_LIB):
        build.build()
    exe = tmp_path_factory.mktemp("compat") / "compat_driver"
    subprocess.run(["gcc", "-std=gnu99", "-O2", "-I", INC, os.path.join(ROOT, "tests", "compat", "compat_driver.c"),
                    "-o", str(exe), "-L", LIBDIR, "-l:libivr_compat.so", "-l:libivr_gpu.so",
                    "-Wl,-rpath," + LIBDIR], check=True)
    return str(exe)


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: p.split("/")[-1][:-4])
def test_reference_names_render_the_golden_frame(driver, oracle_mod, tmp_path, path):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    c = load_case(path)
    d, h, w = c["volume"].shape
    big = bool(c["big_endian"])
    vol = tmp_path / "vol.raw"
    np.ascontiguousarray(c["volume"], dtype=">f4" if big else "<f4").tofile(vol)
    st = tmp_path / "state.bin"
    st.write_bytes(c["state"].tobytes())
    lut = tmp_path / "lut.bin"
    if c["colormap"] == -1:
        np.ascontiguousarray(c["lut"], np.float32).tofile(lut)
    prefix = str(tmp_path / "out")
    p = c["procdims"]
    args = [driver, str(vol), w, h, d, 0 if big else 1, c["colormap"], c["xfer"], p[0], p[1], p[2], c["tile"][0],
            c["tile"][1], str(st), str(lut) if c["colormap"] == -1 else "-", c["lutoffset"], prefix]
    r = subprocess.run([str(a) for a in args], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    vw, vh, K = (int(x) for x in open(prefix + ".info").read().split())
    assert (vh, vw) == c["rgba32"].shape[:2] and K == int(np.prod(p))
    frame = np.fromfile(prefix + ".frame", np.float32).reshape(vh, vw, 4)
    assert np.array_equal(bits(frame), bits(c["rgba32"])), f"max |d| {np.abs(frame - c['rgba32']).max()}"
    bricks = np.fromfile(prefix + ".bricks", np.float32).reshape(K, vh, vw, 4)
    for k in range(K):
        assert np.array_equal(bits(bricks[k]), bits(c["bricks"][k])), f"brick {k}"
    rgba8 = np.fromfile(prefix + ".rgba8", np.uint8).reshape(vh, vw, 4)
    assert np.array_equal(rgba8, oracle_mod.quantize(c["rgba32"]))
