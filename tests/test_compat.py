"""CPU: the reference-name layer (include/ivr_compat.h, libivr_compat.so)
exports every function and global its header declares; a C program in the
reference's steered-frame order compiles and links against it; and the C
snippets of INTEGRATION.md compile against the headers (no device calls)."""
import os
import re
import shutil
import subprocess

import pytest

from conftest import ROOT

INC = os.path.join(ROOT, "include")
LIBDIR = os.path.join(ROOT, "ivr_gb300")
DRIVER = os.path.join(ROOT, "tests", "compat", "compat_driver.c")


def compat_lib():
    path = os.path.join(LIBDIR, "libivr_compat.so")
    if not os.path.exists(path):
        from ivr_gb300 import build
        build.build()
    return path


def declared():
    src = open(os.path.join(INC, "ivr_compat.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    src = re.sub(r"#ifndef IBM_Ray_Caster_mathutil_h.*?#endif", "", src, flags=re.S)  # static inlines
    funcs = set(re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_ \*]*?\b([a-z_][a-z0-9_]*)\s*\(", src, flags=re.M))
    globs = set()
    for line in re.findall(r"^extern\s+(.*?);", src, flags=re.M):
        for name in line.split(","):
            m = re.search(r"\**\s*([A-Za-z_][A-Za-z0-9_]*)\s*(\[[^\]]*\])?\s*$", name.strip())
            if m:
                globs.add(m.group(1))
    return funcs - {"if", "for", "return"}, globs


def exported(path):
    out = subprocess.run(["nm", "-D", "--defined-only", path], check=True, capture_output=True, text=True).stdout
    return {ln.split()[-1] for ln in out.splitlines() if ln.strip()}


def test_compat_exports_the_reference_names():
    if shutil.which("nm") is None:
        pytest.skip("no nm")
    funcs, globs = declared()
    for must in ["createlocalimage", "compositetiles", "readvoldata", "initvolluts", "inittransferfunc",
                 "initcolormap", "setplaneconst", "updatevolbbox", "compositelocalimage", "initvolattrs",
                 "initvolbbox", "initcolbufs", "writetomemory", "init", "freeall"]:
        assert must in funcs, must
    for must in ["mystate", "viewport", "mvm", "pm", "viewvolume", "pzero", "lut", "lutoffset", "maxlutindx",
                 "colorbuf", "tiffimage", "winwidth", "winheight"]:
        assert must in globs, must
    names = exported(compat_lib())
    assert not (funcs - names), sorted(funcs - names)
    assert not (globs - names), sorted(globs - names)


def test_compat_driver_links(tmp_path):
    if shutil.which("gcc") is None:
        pytest.skip("no C compiler")
    compat_lib()
    exe = tmp_path / "compat_driver"
    subprocess.run(["gcc", "-std=gnu99", "-O2", "-Wall", "-Wextra", "-Werror", "-I", INC, DRIVER, "-o", str(exe),
                    "-L", LIBDIR, "-l:libivr_compat.so", "-l:libivr_gpu.so", "-Wl,-rpath," + LIBDIR],
                   check=True)
    assert exe.exists()


def test_compat_record_layouts(tmp_path):
    """The reference's records, as the compat header lays them out: CMDARGS
    (types.h:128-141) 80 + 6*4 + 3*4 + 2*4 + 4 + 12 bytes, WINDOW 32, FRUSTUM 24,
    color4f 16, STATE 184."""
    if shutil.which("gcc") is None:
        pytest.skip("no C compiler")
    src = tmp_path / "sizes.c"
    src.write_text('#include <stdio.h>\n#include "ivr_compat.h"\nint main(void){printf("%zu %zu %zu %zu %zu\\n",'
                   'sizeof(ivr_cmdargs), sizeof(ivr_window), sizeof(ivr_frustum), sizeof(ivr_color4f),'
                   'sizeof(ivr_state));return 0;}\n')
    exe = tmp_path / "sizes"
    subprocess.run(["gcc", "-I", INC, str(src), "-o", str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()]
    assert got == [140, 32, 24, 16, 184]


def integration_snippets():
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    return re.findall(r"```c\n(.*?)```", text, flags=re.S)


# What a snippet finds around it in the reference's main.c: its records
# (types.h, connection.h) and the handles a previous snippet declared.
PRELUDE = """#include <stdio.h>
#include <stdint.h>
#include <stdlib.h>
#include "ivr_compat.h"
typedef ivr_cmdargs CMDARGS;
typedef ivr_state STATE;
static ivr_ctx *ctx; static ivr_volume *vol; static ivr_view *view; static ivr_tf *tf;
static ivr_view *views[4]; static ivr_tf *tfs[4]; static ivr_tf *train_tfs[4];
static uint8_t *rgba8_dev[4]; static ivr_state state; static ivr_render_params params;
static void *stream; static int nframes, ntrain, w, h;
static ivr_state states[8];
static const float *rgba;
"""


@pytest.mark.parametrize("k", range(len(integration_snippets())))
def test_integration_snippet_compiles(tmp_path, k):
    if shutil.which("gcc") is None:
        pytest.skip("no C compiler")
    body = integration_snippets()[k]
    src = tmp_path / f"snippet{k}.c"
    if re.search(r"^\s*(static\s+)?[A-Za-z_][\w \*]*\([^;]*\)\s*(/\*.*\*/)?\s*$\s*\{", body, flags=re.M) or \
            body.lstrip().startswith("#include"):
        src.write_text(PRELUDE + body)  # top-level definitions
    else:
        src.write_text(PRELUDE + "void snippet(void) {\n" + body + "\n}\n")  # statements
    subprocess.run(["gcc", "-std=gnu99", "-fsyntax-only", "-Wall", "-Wno-unused-variable",
                    "-Wno-unused-function", "-Wno-unused-but-set-variable", "-I", INC, str(src)], check=True)
