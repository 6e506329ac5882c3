"""Regenerate the committed golden fixtures from the REFERENCE itself.

Needs the reference source tree, named by the OPENCAL_REFERENCE environment
variable; nothing that runs on the GPU machine calls this script.

1. Compiles the reference library and its two SCIDDICA-T examples from their
   own sources (oracle/ref/Makefile), runs them on the examples' shipped
   610x496 DEM/source, and checks that they reproduce the shipped goldens:
     OpenCAL-OMP/examples/calomp_sciddicaT/data/width_final.txt   (%.9f, plain)
     OpenCAL/examples/cal_sciddicaT-activecells-glut/data/width_final.txt (%f, AC)
   Writes sciddicaT_610x496.npz (inputs + both goldens, parsed) and records
   the sha256 of the plain golden text in manifest.json.
2. Runs the reference library (oracle/_ref/libref.so) on small seeded
   synthetic cases -- every neighbourhood, both boundaries, active cells on
   and off, 2D and 3D -- and writes their outputs to synthetic_cases.npz.
   FLAT cases are chosen so that no state reaches the outer band of the grid,
   where the reference reads outside its buffers.

Run:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import json
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from opencal_gb300 import workloads as W  # noqa: E402

REF = os.environ.get("OPENCAL_REFERENCE") or ""  # required when run as a script (checked in main)
PLAIN_DATA = os.path.join(REF, "OpenCAL-OMP/examples/calomp_sciddicaT/data")
AC_DATA = os.path.join(REF, "OpenCAL/examples/cal_sciddicaT-activecells-glut/data")


def sha256_file(path: str) -> str:
    h = hashlib.sha256()
    with open(path, "rb") as f:
        h.update(f.read())
    return h.hexdigest()


def run_example(binary: str, data_dir: str) -> str:
    """Run a reference example in a scratch copy of its data dir; return the output path."""
    work = tempfile.mkdtemp(prefix="opencal_golden_")
    shutil.copytree(data_dir, os.path.join(work, "data"))
    os.remove(os.path.join(work, "data", "width_final.txt"))
    subprocess.run([binary], cwd=work, check=True, stdout=subprocess.DEVNULL)
    return os.path.join(work, "data", "width_final.txt")


def shipped_goldens(manifest: dict) -> None:
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle", "ref"), f"REF={REF}", "all", "examples"],
                   check=True)
    refdir = os.path.join(ROOT, "oracle", "_ref")

    out_plain = run_example(os.path.join(refdir, "sciddicaT_plain"), PLAIN_DATA)
    golden_plain = os.path.join(PLAIN_DATA, "width_final.txt")
    assert sha256_file(out_plain) == sha256_file(golden_plain), "reference build does not reproduce its golden"

    out_ac = run_example(os.path.join(refdir, "sciddicaT_ac"), AC_DATA)
    ac_ref = np.loadtxt(out_ac)
    ac_golden = np.loadtxt(os.path.join(AC_DATA, "width_final.txt"))
    ac_err = float(np.abs(ac_ref - ac_golden).max())
    assert ac_err <= 1e-6, ac_err

    z = np.loadtxt(os.path.join(PLAIN_DATA, "dem.txt"))
    h = np.loadtxt(os.path.join(PLAIN_DATA, "source.txt"))
    assert np.array_equal(z, np.loadtxt(os.path.join(AC_DATA, "dem.txt")))
    assert np.array_equal(h, np.loadtxt(os.path.join(AC_DATA, "source.txt")))
    np.savez_compressed(os.path.join(HERE, "sciddicaT_610x496.npz"), z=z, h0=h,
                        h_plain=np.loadtxt(golden_plain), h_ac=ac_golden, h_ac_ref_run=ac_ref)
    manifest["sciddicaT_610x496"] = {
        "rows": 610, "cols": 496, "steps": 4000, "p_r": 0.5, "p_eps": 0.001, "toroidal": True,
        "plain_text_sha256": sha256_file(golden_plain),
        "plain_format": "%.9f followed by two spaces per value, newline per row",
        "ac_max_abs_err_ref_vs_shipped": ac_err,
        "source": "reference examples' shipped data and goldens; reference examples rerun here",
    }


def synthetic_cases():
    """(name, kwargs) for each fixture; kept small so the oracle checks them in seconds."""
    cases = []
    for tor in (0, 1):
        for ac in (0, 1):
            cases.append(("sdt", dict(rows=160, cols=144, seed=11, steps=30, toroidal=tor, ac=ac)))
    for tor in (1,):
        for as_int in (0, 1):
            cases.append(("life", dict(rows=96, cols=80, seed=1, steps=60, toroidal=tor, as_int=as_int)))
    for nb in (oracle.NB_VN, oracle.NB_MOORE, oracle.NB_HEX, oracle.NB_HEX_ALT):
        cases.append(("nb", dict(rows=40, cols=36, seed=3, steps=5, nbhd=nb, toroidal=1)))
    for nb in (oracle.NB_VN, oracle.NB_MOORE, oracle.NB_HEX, oracle.NB_HEX_ALT):
        for tor in (0, 1):
            cases.append(("acp2", dict(rows=48, cols=40, seed=4, steps=6 if not tor else 20, nbhd=nb,
                                       toroidal=tor)))
    for nb in (1, 2):
        for tor in (0, 1):
            cases.append(("acp3", dict(rows=18, cols=20, slices=16, seed=6, steps=2 if not tor else 10,
                                       nbhd=nb, toroidal=tor)))
    cases.append(("life3d", dict(rows=12, cols=10, slices=8, seed=7, steps=10, toroidal=1)))
    return cases


def case_inputs(kind: str, kw: dict):
    if kind == "sdt":
        return W.sciddicaT_inputs(kw["rows"], kw["cols"], seed=kw["seed"])
    if kind == "life":
        return W.life_state(kw["rows"], kw["cols"], seed=kw["seed"])
    if kind == "nb":
        return W.random_field((kw["rows"], kw["cols"]), seed=kw["seed"])
    if kind == "acp2":
        return W.sparse_blobs((kw["rows"], kw["cols"]), seed=kw["seed"], margin=10)
    if kind == "acp3":
        return W.sparse_blobs((kw["slices"], kw["rows"], kw["cols"]), seed=kw["seed"], radius=2.5, margin=6)
    if kind == "life3d":
        return W.life3d_state(kw["rows"], kw["cols"], kw["slices"], p=0.2, seed=kw["seed"])
    raise ValueError(kind)


def run_case(kind: str, kw: dict, impl: str):
    """Outputs of one case on the oracle ('serial'/'omp') or the reference ('ref')."""
    x = case_inputs(kind, kw)
    if kind == "sdt":
        z, h, cells = oracle.sciddicaT(x[0], x[1], kw["steps"], toroidal=kw["toroidal"], ac=kw["ac"], kind=impl)
        return {"z": z, "h": h, "cells": cells}
    if kind == "life":
        return {"s": oracle.life2d(x, kw["steps"], toroidal=kw["toroidal"], as_int=kw["as_int"], kind=impl)}
    if kind == "nb":
        return {"v": oracle.nbprobe2d(x, kw["steps"], nbhd=kw["nbhd"], toroidal=kw["toroidal"], kind=impl)}
    if kind in ("acp2", "acp3"):
        v, cells = oracle.acprobe(x, kw["steps"], nbhd=kw["nbhd"], toroidal=kw["toroidal"], kind=impl)
        return {"v": v, "cells": cells}
    if kind == "life3d":
        return {"s": oracle.life3d(x, kw["steps"], toroidal=kw["toroidal"], kind=impl)}
    raise ValueError(kind)


def edge_band_clear(kind: str, out: dict, band: int = 2) -> bool:
    """True when nothing non-zero reaches the outer `band` cells (2D) / faces (3D)."""
    key = "h" if kind == "sdt" else ("v" if "v" in out else "s")
    a = np.array(out[key], dtype=np.float64)
    inner = np.zeros_like(a, dtype=bool)
    sl = tuple(slice(band, -band) for _ in a.shape)
    inner[sl] = True
    return not np.any(a[~inner] != 0)


def synthetic_goldens(manifest: dict) -> None:
    arrays = {}
    meta = []
    for idx, (kind, kw) in enumerate(synthetic_cases()):
        out = run_case(kind, kw, "ref")
        if not kw.get("toroidal", 1):
            assert edge_band_clear(kind, out), f"flat case {kind} {kw} reaches the edge band"
        for k, v in out.items():
            arrays[f"c{idx}_{k}"] = v
        meta.append({"kind": kind, "kw": kw, "keys": sorted(out)})
    np.savez_compressed(os.path.join(HERE, "synthetic_cases.npz"), **arrays)
    manifest["synthetic_cases"] = meta


def main() -> None:
    if not os.path.isdir(os.path.join(REF, "OpenCAL-OMP")):
        sys.exit(f"reference tree not found at {REF}")
    oracle.build(ref=True)
    path = os.path.join(HERE, "manifest.json")
    manifest = json.load(open(path)) if os.path.exists(path) else {}
    if "--synthetic-only" not in sys.argv:
        shipped_goldens(manifest)
    synthetic_goldens(manifest)
    manifest["generator"] = "tests/golden/make_golden.py (reference compiled by oracle/ref/Makefile)"
    with open(path, "w") as f:
        json.dump(manifest, f, indent=1, sort_keys=True)
    print("wrote", path)


if __name__ == "__main__":
    main()
