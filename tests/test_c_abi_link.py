"""The C ABI is consumable from plain C: a C99 program includes include/hora_gb300.h, links
libhora_gb300.so and gets integer statuses back (no device is needed for these calls)."""
import os
import shutil
import subprocess

import pytest

from ptctcl_gb300 import build as libbuild

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r"""
#include <stdio.h>
#include "hora_gb300.h"
int main(void) {
  hora_handle h = 0;
  int32_t n = -1, r = 0;
  printf("abi %d\n", (int)hora_gb_abi_version());
  const int32_t rc = hora_gb_device_count(&n);
  printf("count %d %d\n", (int)rc, n >= 0);
  const int32_t ro = hora_gb_open(NULL, NULL, &h);
  printf("open %d %d\n", (int)ro, h == 0);
  printf("run %d\n", (int)hora_gb_run(NULL, &r, NULL));
  printf("close %d\n", (int)hora_gb_close(NULL));
  printf("batch %d\n", (int)hora_gb_batch_run(-1, NULL, NULL, NULL, NULL, NULL));
  printf("error %s\n", hora_gb_last_error());
  return 0;
}
"""


@pytest.mark.skipif(shutil.which("gcc") is None, reason="needs gcc")
def test_c_program_links_and_calls_the_library(tmp_path):
    lib = libbuild.build()
    src = tmp_path / "abi.c"
    src.write_text(PROGRAM)
    exe = tmp_path / "abi"
    libdir = os.path.dirname(lib)
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), str(src), "-o",
                    str(exe), "-L", libdir, "-lhora_gb300", f"-Wl,-rpath,{libdir}"], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines()
    got = dict(line.split(" ", 1) for line in out)
    assert got["abi"] == "2"
    assert got["count"] == "0 1"
    assert got["open"] == "1 1"       # HORA_E_INVALID, handle left null
    assert got["run"] == "1" and got["close"] == "1" and got["batch"] == "1"
    assert got["error"].strip()
