"""The C ABI from C: include/gpumatfun.h compiles as C99, a C program links
against the library and gets the documented status codes from the argument
checks that run before any device call, and the struct layout seen by C
matches the ctypes mirror (no GPU needed)."""
import ctypes as ct
import os
import shutil
import subprocess

import pytest

from gpumatfun_gb300 import engine as E

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r"""
#include <stddef.h>
#include <stdio.h>
#include <string.h>
#include "gpumatfun.h"

int main(void) {
  gm_create_args a;
  gm_handle h = 0;
  gm_default_args(&a);
  printf("sizeof %zu\n", sizeof(gm_create_args));
  printf("off_precision %zu\n", offsetof(gm_create_args, precision));
  printf("off_row_weight %zu\n", offsetof(gm_create_args, row_weight));
  printf("off_reorth %zu\n", offsetof(gm_create_args, reorth));
  printf("off_val_prefetch %zu\n", offsetof(gm_create_args, val_prefetch));
  printf("version_ok %d\n", strstr(gm_version(), "sm_103a") != NULL);
  printf("null_args %d\n", gm_lanczos_create(NULL, &h));
  a.n = 0;
  printf("bad_n %d\n", gm_lanczos_create(&a, &h));
  printf("handle_null %d\n", h == 0);
  printf("null_handle_calls %d %d %d\n", gm_build_subspace(NULL), gm_get_U(NULL, NULL), gm_set_state(NULL, NULL, NULL));
  return 0;
}
"""


@pytest.fixture(scope="module")
def c_output(tmp_path_factory, engine_lib):
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    d = tmp_path_factory.mktemp("cabi")
    src = d / "t.c"
    src.write_text(PROGRAM)
    lib = os.path.dirname(engine_lib._name)
    exe = d / "t"
    subprocess.run([cc, "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), str(src),
                    "-L", lib, "-lgpumatfun", f"-Wl,-rpath,{lib}", "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    return dict(line.split(" ", 1) for line in out.strip().splitlines())


def test_struct_layout_c_vs_ctypes(c_output):
    assert int(c_output["sizeof"]) == ct.sizeof(E.CreateArgs)
    for field in ("precision", "row_weight", "reorth", "val_prefetch"):
        assert int(c_output[f"off_{field}"]) == getattr(E.CreateArgs, field).offset, field


def test_status_codes_from_c(c_output):
    assert c_output["version_ok"] == "1"
    assert c_output["null_args"] == "1"          # GM_ERR_ARG
    assert c_output["bad_n"] == "1"
    assert c_output["handle_null"] == "1"
    assert c_output["null_handle_calls"].split() == ["1", "1", "1"]
