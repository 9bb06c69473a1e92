"""The public header is plain C: a C99 program compiles against it, links the
library and calls it without a GPU (version query and host-side argument
validation of a host-pointer and a device-pointer entry)."""
import os
import shutil
import subprocess

import pytest

from tests.conftest import ROOT

C_PROGRAM = r"""
#include <stdio.h>
#include <string.h>
#include "phinfortran_gb300.h"

int main(void) {
  if (pf_version() != PF_ABI_VERSION) return 10;
  /* n = 0 is refused on the host before any device work */
  int rc = pf_transport_tdb(0, 1, 1, 1, 1, NULL, NULL, NULL, NULL, NULL, NULL, NULL, NULL,
                            0, NULL, NULL, NULL, 0.0, 0.0, 1.0, 1e-14, 10, 0,
                            NULL, NULL, NULL, NULL);
  if (rc != PF_ERR_ARG) return 11;
  if (strstr(pf_last_error(), "positive") == NULL) return 12;
  /* a device-pointer entry with a void* stream: also refused on the host */
  rc = pf_transport_tdb_tiled_dev(0, 1, 1, 1, 1, NULL, NULL, NULL, NULL, NULL, NULL, NULL, NULL,
                                  0, NULL, NULL, NULL, 0.0, 0.0, 1.0, 1e-14, 10, PF_ARITH_FP64,
                                  NULL, NULL, NULL, NULL, 0, (void*)0);
  if (rc != PF_ERR_ARG) return 13;
  if (pf_transport_tdb_tiled_workspace_size(0, 1, 1, 1, 1, 1, PF_ARITH_FP64) != 0) return 14;
  rc = pf_dense_to_tdb_dev(0, 1, NULL, 1, 1, 0, 0, 1, NULL, 1, NULL, NULL, NULL, NULL, NULL, NULL,
                           NULL, NULL, NULL, (void*)0);
  if (rc != PF_ERR_ARG) return 15;
  printf("ok %d\n", pf_version());
  return 0;
}
"""


@pytest.mark.skipif(shutil.which("gcc") is None, reason="no C compiler")
def test_header_compiles_as_c99_and_links(built_lib, tmp_path):
    src = tmp_path / "abi_check.c"
    src.write_text(C_PROGRAM)
    exe = tmp_path / "abi_check"
    libdir = os.path.dirname(built_lib)
    cmd = ["gcc", "-std=c99", "-Wall", "-Werror", "-pedantic", "-I", os.path.join(ROOT, "include"), str(src),
           "-o", str(exe), "-L", libdir, "-lphinfortran_gb300", f"-Wl,-rpath,{libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)
    assert r.stdout.strip() == "ok 1"


@pytest.mark.skipif(shutil.which("gcc") is None, reason="no C compiler")
def test_header_has_no_cuda_types():
    """Every stream parameter is a void* (a cudaStream_t handle), so the
    header needs no CUDA include."""
    src = open(os.path.join(ROOT, "include", "phinfortran_gb300.h")).read()
    code = "\n".join(ln for ln in src.splitlines() if not ln.lstrip().startswith("*"))
    assert "cudaStream_t" not in code
    r = subprocess.run(["gcc", "-std=c99", "-fsyntax-only", "-x", "c", "-I", os.path.join(ROOT, "include"), "-"],
                       input='#include "phinfortran_gb300.h"\n', capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
