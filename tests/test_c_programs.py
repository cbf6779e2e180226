"""C and C++ callers of the boundary, built the way a maintainer would build
them (no GPU work: argument checks only).

  * a plain C program that includes include/spacelab_gpu.h and links
    libspacelab_gb300.so;
  * the reference's translation unit after the two-line edit that switches
    its sim_looper to the GPU (include/spacelab_sim_one_step_gpu.hpp),
    compiled from the reference's sources and linked with the library.
    Running it is tests/test_gpu_dropin.py."""
import subprocess
from pathlib import Path

import pytest

from spacelab_gb300 import _lib

ROOT = Path(__file__).resolve().parents[1]
ORACLE = ROOT / "oracle"

C_PROGRAM = r"""
#include <stdio.h>
#include "spacelab_gpu.h"
#include "spacelab_host.h"

int main(void)
{
    sl_material mat = {6.674e-8, 4e-13, 0.3, 1e-5, 1e-5};
    sl_handle* h = NULL;
    if (sl_version() != SL_API_VERSION) return 10;
    if (sl_create(0, &mat, SL_MODE_EXACT, &h) != SL_ERR_ARG || h != NULL) return 11;
    printf("%s\n", sl_last_error());
    if (sl_destroy(NULL) != SL_OK) return 12;
    if (sl_step(NULL, 1, 0, NULL) != SL_ERR_ARG) return 13;
    if (sl_step_host(NULL, NULL, NULL, NULL, NULL, NULL, 0, NULL) != SL_ERR_ARG) return 16;
    double kin = 0, kout = 0, dt = 0;
    if (slh_spring_and_dt(1e-4, 7e-12, 10.0, 1.7, 0.4096, 50.0, &kin, &kout, &dt) != 0) return 14;
    if (!(kin > 0 && kout > 0 && dt > 0)) return 15;
    printf("ok %.17g %.17g %.17g\n", kin, kout, dt);
    return 0;
}
"""


def test_c_program_includes_header_and_links_library(tmp_path):
    src = tmp_path / "caller.c"
    src.write_text(C_PROGRAM)
    exe = tmp_path / "caller"
    libdir = _lib.LIB_PATH.parent
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", str(ROOT / "include"), str(src), "-o", str(exe),
                    "-L", str(libdir), "-lspacelab_gb300", f"-Wl,-rpath,{libdir}"], check=True)
    out = subprocess.run([str(exe)], stdout=subprocess.PIPE, text=True, timeout=60)
    assert out.returncode == 0, out.stdout
    assert out.stdout.splitlines()[-1].startswith("ok ")


def test_reference_tu_with_gpu_adapter_compiles():
    if not (ORACLE / "_ref" / "src" / "ColliderSingleCore" / "ColliderSingleCore.cpp").exists():
        pytest.skip("the reference's sources are not at hand (oracle/_ref/src)")
    proc = subprocess.run(["make", "-s", "-C", str(ORACLE), "adapter"], stdout=subprocess.PIPE,
                          stderr=subprocess.STDOUT, text=True)
    assert proc.returncode == 0, proc.stdout
    adapted = (ORACLE / "_ref" / "adapted" / "ColliderSingleCore" / "ColliderSingleCore.cpp").read_text()
    assert adapted.count("sim_one_step_gpu(writeStep);") == 1
    assert adapted.count('#include "spacelab_sim_one_step_gpu.hpp"') == 1
