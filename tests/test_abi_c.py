"""The boundary is a C ABI: include/gs_abi.h and include/gs_setup.h compile as C99, and a C
program links against libgsolver_gb300.so and calls it (the calls here need no GPU)."""
import os
import shutil
import subprocess
import tempfile

import pytest

import gsolver_gb300 as gs

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = os.path.join(ROOT, "include")

PROG = r"""
#include <stdio.h>
#include <string.h>
#include "gs_abi.h"
#include "gs_setup.h"

int main(void) {
    printf("%d\n", GS_ABI_VERSION);
    printf("%s\n", gs_status_string(GS_ERR_COLLAPSE));
    printf("%d\n", gs_check_build());
    printf("%zu\n", gs_noalloc_max_samples());
    gs_handle* h = 0;
    printf("%d\n", gs_create(0, &h));   /* a null parameter block is refused before any GPU work */
    return 0;
}
"""


@pytest.mark.skipif(shutil.which("gcc") is None, reason="gcc not found")
def test_headers_are_c99_and_a_c_program_links():
    for h in ("gs_abi.h", "gs_setup.h"):
        r = subprocess.run(["gcc", "-x", "c", "-std=c99", "-Wall", "-Werror", "-fsyntax-only", os.path.join(INC, h)],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
    lib = gs.LIB_PATH
    assert os.path.exists(lib)
    d = tempfile.mkdtemp(prefix="gs_cabi_")
    src, exe = os.path.join(d, "main.c"), os.path.join(d, "main")
    with open(src, "w") as f:
        f.write(PROG)
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", INC, src, "-o", exe, lib,
                        "-Wl,-rpath," + os.path.dirname(lib)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    out = r.stdout.splitlines()
    assert int(out[0]) >= 2
    assert out[1] == "Minimum Z step size reached, collapse is possible!"
    assert out[2] == "0"
    assert int(out[3]) == 524280
    assert int(out[4]) == gs.GS_ERR_ARG
