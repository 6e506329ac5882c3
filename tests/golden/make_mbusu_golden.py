"""Regenerate the mbusu golden fixtures from the REFERENCE itself.

Needs the reference source tree, named by the OPENCAL_REFERENCE environment
variable; nothing that runs on the GPU machine calls this script.

Compiles the reference's mbusu example (OpenCAL/examples/cal_mbusu-glut/
source/mbusu.c, unmodified) against the serially built reference library
with a headless driver (oracle/ref/Makefile, target `mbusu`) and runs it:

* for 0 (the initial state) and 40 steps: records the SHA-256 of each of the
  eight substates and checks that the oracle restatement
  (oracle/oracle_mbusu.c) reproduces them bit for bit;
* until its stop condition (10 days of simulated time, about 35 minutes on
  one core): records the step reached, delta_t and the accumulated time,
  the SHA-256 of each substate, and the y = 14 slice (the one the program
  prints to ris10g.txt) of moist_cont and h at full precision; the printed
  ris10g.txt of this run is compared with the two OpenCAL outputs shipped
  in the reference (ris10g-orig-opencal.txt, ris10g-orig-opencal-omp.txt),
  and the largest differences are recorded.

Run:  python tests/golden/make_mbusu_golden.py [--reuse <full-run state file>]
"""
from __future__ import annotations

import argparse
import hashlib
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402

REF = os.environ.get("OPENCAL_REFERENCE") or ""  # required when run as a script (checked in main)
SHIPPED = os.path.join(REF, "OpenCAL", "examples", "cal_mbusu-glut")
N = 130 * 160 * 30


def run_ref(steps: int, workdir: str) -> np.ndarray:
    exe = os.path.join(ROOT, "oracle", "_ref", "mbusu_ref")
    out = os.path.join(workdir, "state.bin")
    subprocess.run([exe, str(steps), out], cwd=workdir, check=True)
    return np.fromfile(out)


def hashes(raw: np.ndarray) -> np.ndarray:
    return np.array([hashlib.sha256(raw[q * N:(q + 1) * N].tobytes()).hexdigest() for q in range(8)])


def main() -> None:
    if not REF or not os.path.isdir(os.path.join(REF, "OpenCAL-OMP")):
        sys.exit("set OPENCAL_REFERENCE to the OpenCAL source tree")
    ap = argparse.ArgumentParser()
    ap.add_argument("--reuse", help="state file of a finished full reference run (skips the 35-minute run)")
    ap.add_argument("--reuse-ris", help="ris10g.txt written by that run")
    args = ap.parse_args()
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle", "ref"), f"REF={REF}", "mbusu"], check=True)
    oracle.build()
    fx = {}
    with tempfile.TemporaryDirectory() as tmp:
        for steps, key in ((-1, "init"), (40, "s40")):
            raw = run_ref(steps, tmp)
            fx[f"{key}_sha256"] = hashes(raw)
            fx[f"{key}_tail"] = raw[8 * N:]
            o = oracle.mbusu(steps)
            mine = np.concatenate([o[f].ravel() for f in oracle.MBUSU_FIELDS])
            assert hashes(mine).tolist() == fx[f"{key}_sha256"].tolist(), f"oracle differs from the reference ({key})"
            print(f"{key}: oracle == reference bit for bit")
        if args.reuse:
            raw = np.fromfile(args.reuse)
            ris = args.reuse_ris
        else:
            raw = run_ref(0, tmp)
            ris = os.path.join(tmp, "ris10g.txt")
        fx["full_sha256"] = hashes(raw)
        fx["full_tail"] = raw[8 * N:]
        state = raw[:8 * N].reshape(8, 130, 160, 30)
        fx["full_moist_cont_y14"] = state[oracle.MBUSU_FIELDS.index("moist_cont"), :, :, 14].copy()
        fx["full_h_y14"] = state[oracle.MBUSU_FIELDS.index("h"), :, :, 14].copy()
        printed = np.loadtxt(ris)
        assert np.abs(printed - fx["full_moist_cont_y14"]).max() <= 5e-7, "ris10g.txt is not the y = 14 slice"
        for name in ("ris10g-orig-opencal.txt", "ris10g-orig-opencal-omp.txt"):
            shipped = np.loadtxt(os.path.join(SHIPPED, name))
            d = float(np.abs(shipped - printed).max())
            fx["shipped_maxdiff_" + name.split("-")[-1].replace(".txt", "").replace("opencal", "serial")] = d
            print(f"{name}: max |this run - shipped| = {d:.3e}")
    np.savez_compressed(os.path.join(HERE, "mbusu_cases.npz"), **fx)
    print("wrote", os.path.join(HERE, "mbusu_cases.npz"), "steps", fx["full_tail"])


if __name__ == "__main__":
    main()
