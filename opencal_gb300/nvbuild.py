"""Build the opencal-gb300 shared libraries in-tree (nvcc, sm_103a only).

  opencal_gb300/lib/libopencal_gb300.so  the C-ABI library (include/opencal/*.h)
  opencal_gb300/lib/libopencal_models.so the models shipped with it (SCIDDICA-T,
                                         SCIARA-fv2, mbusu, Life 2D/3D) and their
                                         driver entry points, linked against the
                                         former

Compiles translation units in parallel and skips those whose object is newer
than the source and every header.  No cmake.

    python -m opencal_gb300.nvbuild [--force] [--verbose]
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OBJ = os.path.join(PKG, "lib", "obj")
LIB = os.path.join(PKG, "lib")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-cudart", "shared",
                 "-I" + INCLUDE, "-I" + CSRC, "-diag-suppress", "550,177"]
# model kernels restate reference arithmetic operation by operation: no FMA contraction
MODEL_FLAGS = ["--fmad=false", "-Xcompiler=-ffp-contract=off"]  # no contraction on the device or host side

CORE_SOURCES = ["cal_core.cu", "cal2D.cu", "cal3D.cu", "cal2DRun.cu", "cal3DRun.cu", "calIO.cu", "calReduction.cu", "cal_noalloc.cu"]
MODEL_SOURCES = ["models/sciddicaT.cu", "models/sciddicaT_adjoint.cu", "models/sciddicaT_batch.cu",
                 "models/sciddicaT_unsafe.cu", "models/sciara.cu", "models/sciara_batch.cu", "models/sciara_io.cu", "models/mbusu.cu",
                 "models/life.cu", "models/life3d.cu", "models/fp64_peak.cu"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _headers() -> list[str]:
    return (glob.glob(os.path.join(INCLUDE, "opencal", "*")) + glob.glob(os.path.join(CSRC, "*.cuh")) +
            glob.glob(os.path.join(CSRC, "models", "*.cuh")))


def _stale(src: str, obj: str, deps: list[str]) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in [src] + deps)


def _compile(src: str, obj: str, extra: list[str], verbose: bool) -> str:
    cmd = [nvcc()] + COMMON + extra + ["-c", src, "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr}")
    return r.stderr


def build(force: bool = False, verbose: bool = False) -> dict[str, str]:
    os.makedirs(OBJ, exist_ok=True)
    deps = _headers()
    jobs = []
    for rel in CORE_SOURCES:
        src = os.path.join(CSRC, rel)
        jobs.append((src, os.path.join(OBJ, rel.replace("/", "_").replace(".cu", ".o")), []))
    for rel in MODEL_SOURCES:
        src = os.path.join(CSRC, rel)
        jobs.append((src, os.path.join(OBJ, rel.replace("/", "_").replace(".cu", ".o")), MODEL_FLAGS))
    todo = [j for j in jobs if force or _stale(j[0], j[1], deps)]
    logs = {}
    if todo:
        with cf.ThreadPoolExecutor(max_workers=min(8, len(todo))) as ex:
            futs = {ex.submit(_compile, s, o, e, verbose): s for s, o, e in todo}
            for f in cf.as_completed(futs):
                logs[futs[f]] = f.result()
    core = os.path.join(LIB, "libopencal_gb300.so")
    models = os.path.join(LIB, "libopencal_models.so")
    core_objs = [j[1] for j in jobs[: len(CORE_SOURCES)]]
    model_objs = [j[1] for j in jobs[len(CORE_SOURCES):]]
    if todo or not os.path.exists(core) or not os.path.exists(models):
        subprocess.run([nvcc()] + ARCH + ["-shared", "-cudart", "shared", "-o", core] + core_objs, check=True)
        subprocess.run([nvcc()] + ARCH + ["-shared", "-cudart", "shared", "-o", models] + model_objs +
                       ["-L" + LIB, "-lopencal_gb300", "-Xlinker", "-rpath,$ORIGIN"], check=True)
    return logs


if __name__ == "__main__":
    out = build(force="--force" in sys.argv, verbose="--verbose" in sys.argv)
    for src, log in sorted(out.items()):
        if log.strip():
            print(f"== {os.path.relpath(src, ROOT)}\n{log}")
    print("built", os.path.join(LIB, "libopencal_gb300.so"), os.path.join(LIB, "libopencal_models.so"))
