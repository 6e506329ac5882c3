"""Builds the test-only native library (TEST INFRASTRUCTURE, never shipped):

  tests/native/build/libopencal_probes.so  the engine probe rules of
                                           tests/native/probes.cu, linked
                                           against opencal_gb300's C-ABI library

Same compiler flags as the model library (sm_103a, no FP contraction), so
that the probes restate the oracle's arithmetic operation by operation.
"""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "build")
PROBES_LIB = os.path.join(OUT_DIR, "libopencal_probes.so")


def build(force: bool = False) -> str:
    from opencal_gb300 import nvbuild
    src = os.path.join(HERE, "probes.cu")
    core = os.path.join(nvbuild.LIB, "libopencal_gb300.so")
    deps = [src, core] + nvbuild._headers()
    if (not force and os.path.exists(PROBES_LIB) and
            all(os.path.getmtime(d) <= os.path.getmtime(PROBES_LIB) for d in deps)):
        return PROBES_LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    cmd = ([nvbuild.nvcc()] + nvbuild.COMMON + nvbuild.MODEL_FLAGS +
           ["-I" + os.path.join(nvbuild.CSRC, "models"), "-shared", "-o", PROBES_LIB, src,
            "-L" + nvbuild.LIB, "-lopencal_gb300", "-Xlinker", "-rpath," + nvbuild.LIB])
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr}")
    return PROBES_LIB


if __name__ == "__main__":
    print(build(force=True))
