"""Build the in-tree C-ABI shared library ``libphinfortran_gb300.so``.

One nvcc invocation per translation unit, compiled in parallel, for sm_103a
only.  The library has no torch dependency: it is the same object a Fortran
driver links against.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT_DIR, "libphinfortran_gb300.so")

SOURCES = ["negf_abi.cu", "negf_mixed.cu", "negf_fused.cu", "dyn_abi.cu", "cond_abi.cu", "grad_abi.cu", "grad_fp64.cu", "grad_df64.cu", "modes_abi.cu", "tiled_abi.cu", "tb_abi.cu", "fullh_abi.cu", "probe_abi.cu", "tc_abi.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-I", os.path.join(ROOT, "include")]


def nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _compile(src, extra):
    obj = os.path.join(OUT_DIR, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def build(verbose=False, ptxas_info=False):
    """Compile every .cu under csrc/ and link the shared library."""
    os.makedirs(OUT_DIR, exist_ok=True)
    extra = ["-Xptxas", "-v"] if ptxas_info else []
    with ThreadPoolExecutor(max_workers=max(1, min(len(SOURCES), os.cpu_count() or 1))) as ex:
        results = list(ex.map(lambda s: _compile(s, extra), SOURCES))
    objs = [o for o, _ in results]
    if verbose or ptxas_info:
        for _, err in results:
            if err:
                sys.stderr.write(err)
    tmp = LIB + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, ptxas_info="-v" in sys.argv))
