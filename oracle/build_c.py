"""Compile the C restatement of the transmission oracle (oracle/negf_c.c)
into oracle/_lib/liboracle_negf.so: test infrastructure and the CPU
baseline of bench.py, never part of the product."""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_lib", "liboracle_negf.so")


def build(quiet=True):
    src = os.path.join(HERE, "negf_c.c")
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(src):
        return LIB
    cmd = ["gcc", "-O3", "-std=c11", "-fopenmp", "-fcx-limited-range", "-fPIC", "-shared", src, "-o", LIB, "-lm"]
    subprocess.run(cmd, check=True, capture_output=quiet)
    return LIB


if __name__ == "__main__":
    print(build(quiet=False))
