"""Compile tests/native/host_pair.cu into a host shared library (test-only)."""

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build", "libhost_pair.so")


def build():
    src = os.path.join(HERE, "host_pair.cu")
    csrc = os.path.join(os.path.dirname(os.path.dirname(HERE)), "harmonica_gb300", "csrc")
    deps = [src] + [os.path.join(csrc, f) for f in os.listdir(csrc)
                    if f.endswith((".cuh", ".inc"))]
    if os.path.exists(OUT) and os.path.getmtime(OUT) > max(os.path.getmtime(d) for d in deps):
        return OUT
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    subprocess.run(
        ["nvcc", "-O2", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off", "-shared",
         "-gencode", "arch=compute_103a,code=sm_103a", "-o", OUT, src],
        check=True,
    )
    return OUT
