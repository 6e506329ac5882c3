"""Regenerate the unsafe-operation fixtures from the REFERENCE itself.

Runs the reference library (OpenCAL-OMP sources including cal2DUnsafe.c,
compiled serially into oracle/_ref/libref.so by oracle/ref/Makefile) on the
unsafe-operation probe (every neighbourhood, toroidal) and on SCIDDICA-T in
the unsafe form of OpenCAL/examples/cal_sciddicaT-unsafe, checks that the
oracle restatement reproduces them bit for bit, and writes unsafe_cases.npz.
Needs the reference source tree, named by the OPENCAL_REFERENCE environment
variable.

Run:  python tests/golden/make_unsafe_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from opencal_gb300 import workloads as W  # noqa: E402


def probe_inputs(rows, cols, seed):
    g = W.SplitMix64(seed)
    u = W.uniform_array(seed, (rows, cols))
    v0 = np.where(u < 0.3, 1 + (W.uniform_array(seed + 1, (rows, cols)) * 19).astype(np.int32), 0).astype(np.int32)
    b0 = (W.uniform_array(seed + 2, (rows, cols)) < 0.2).astype(np.int8)
    w0 = W.quantise(W.uniform_array(seed + 3, (rows, cols)))
    del g
    return v0, b0, w0


def main():
    if not REF or not os.path.isdir(os.path.join(REF, "OpenCAL-OMP")):
        sys.exit("set OPENCAL_REFERENCE to the OpenCAL source tree")
    oracle.build(ref=True)
    out = {}
    for nb in (1, 2, 3, 4):
        v0, b0, w0 = probe_inputs(40, 52, 60 + nb)
        ref = oracle.unsafe2d(v0, b0, w0, 12, nbhd=nb, toroidal=True, kind="ref")
        orc = oracle.unsafe2d(v0, b0, w0, 12, nbhd=nb, toroidal=True)
        assert all(a.tobytes() == b.tobytes() for a, b in zip(ref, orc)), nb
        for name, a in zip(("v0", "b0", "w0"), (v0, b0, w0)):
            out[f"probe{nb}_{name}"] = a
        for name, a in zip(("v", "b", "w", "u", "x"), ref):
            out[f"probe{nb}_{name}"] = a
    z, h = W.sciddicaT_inputs(64, 80, seed=3)
    ref = oracle.sciddicaT_unsafe(z, h, 50, toroidal=True, kind="ref")
    orc = oracle.sciddicaT_unsafe(z, h, 50, toroidal=True)
    assert all(a.tobytes() == b.tobytes() for a, b in zip(ref, orc))
    out["sdtu_z0"], out["sdtu_h0"], out["sdtu_z"], out["sdtu_h"] = z, h, ref[0], ref[1]
    np.savez_compressed(os.path.join(HERE, "unsafe_cases.npz"), **out)
    print("unsafe fixtures written; oracle == reference bit for bit")


if __name__ == "__main__":
    main()
