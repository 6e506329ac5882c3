"""Golden fixture of the benchmarked SCIDDICA-T run: 2048 x 2048 FP64, von
Neumann, flat, p_r = 0.5, p_epsilon = 0.001, the seeded inputs of
opencal_gb300.workloads.sciddicaT_inputs(2048, 2048, seed=2), 4000 steps,
with active cells off and on.

The oracle (the OpenMP build of oracle/, which gives the serial build's bits:
tests/test_oracle_pins.py::test_oracle_serial_equals_openmp) runs both
forms; the script records SHA-256 digests of the final h (and of the active
list), the input digests, the first step after which the two-cell edge band
holds h != 0, and the mass leaving the grid in every step (the outflows of
border cells towards absent neighbours).  The GPU test
(tests/test_sciddicaT_2048.py) compares the benchmarked kernels with these.

With OPENCAL_REFERENCE set it also runs the reference library itself
(OpenCAL-OMP, compiled serially by oracle/ref/Makefile with the guard-row
allocator) on the same inputs: up to the edge step it must give the oracle's
bits; past it the reference's unchecked flat reads (row -1 and row `rows`
outside the buffer, columns -1 and `columns` wrapping into the adjacent row,
OpenCAL-OMP/source/cal2D.c:866-867) make the two differ, and the script
records by how much.

Run (about 30 minutes on 8 cores):
    OPENCAL_REFERENCE=<OpenCAL tree> python tests/golden/make_sciddicaT_2048_golden.py
"""
from __future__ import annotations

import hashlib
import json
import math
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

ROWS = COLS = 2048
SEED = 2
STEPS = 4000
P_R, P_EPS = 0.5, 0.001
PAST_EDGE = 200  # steps past the edge step compared against the reference
REF = os.environ.get("OPENCAL_REFERENCE") or ""


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def write(out: dict) -> None:
    with open(os.path.join(HERE, "sciddicaT_2048.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
        f.write("\n")


def main() -> None:
    import oracle
    from opencal_gb300 import workloads as W

    oracle.build(ref=bool(REF), ref_tree=REF or None)
    z, h = W.sciddicaT_inputs(ROWS, COLS, seed=SEED)
    out = {"rows": ROWS, "cols": COLS, "seed": SEED, "steps": STEPS, "p_r": P_R, "p_eps": P_EPS,
           "z0_sha256": sha(z), "h0_sha256": sha(h), "mass0": math.fsum(h.ravel())}
    t = time.time()
    zt, ht, outflux, edge = oracle.sciddicaT_trace(z, h, STEPS, p_r=P_R, p_eps=P_EPS, kind="omp")
    out["plain"] = {"h_sha256": sha(ht), "z_sha256": sha(zt), "edge_step": edge, "mass": math.fsum(ht.ravel()),
                    "outflux_total": math.fsum(outflux), "seconds": time.time() - t}
    m0, mt, of = out["mass0"], out["plain"]["mass"], out["plain"]["outflux_total"]
    out["plain"]["mass_balance_rel"] = (m0 - of - mt) / m0
    np.save(os.path.join(HERE, "sciddicaT_2048_outflux.npy"), outflux)
    print("plain", out["plain"], flush=True)

    t = time.time()
    za, ha, cells = oracle.sciddicaT(z, h, STEPS, toroidal=False, ac=True, p_r=P_R, p_eps=P_EPS, kind="omp")
    out["active_cells"] = {"h_sha256": sha(ha), "z_sha256": sha(za), "cells_sha256": sha(cells.astype(np.int32)),
                           "n_active": int(len(cells)), "seconds": time.time() - t,
                           "h_equals_plain": bool(ha.tobytes() == ht.tobytes())}
    print("active cells", out["active_cells"], flush=True)
    write(out)  # the GPU test needs only this much; the reference comparison follows

    if REF and edge > 0:
        # the reference itself up to the edge step, and past it
        t = time.time()
        _, ho, _ = oracle.sciddicaT(z, h, edge, toroidal=False, p_r=P_R, p_eps=P_EPS, kind="omp")
        _, hr, _ = oracle.sciddicaT(z, h, edge, toroidal=False, p_r=P_R, p_eps=P_EPS, kind="ref")
        cmp = {"steps": edge, "bit_identical": bool(ho.tobytes() == hr.tobytes())}
        later = min(edge + PAST_EDGE, STEPS)
        _, ho2, _ = oracle.sciddicaT(z, h, later, toroidal=False, p_r=P_R, p_eps=P_EPS, kind="omp")
        _, hr2, _ = oracle.sciddicaT(z, h, later, toroidal=False, p_r=P_R, p_eps=P_EPS, kind="ref")
        diff = ho2 != hr2
        cmp["past_edge"] = {"steps": later, "cells_differing": int(np.count_nonzero(diff)),
                            "max_abs_diff": float(np.max(np.abs(ho2 - hr2))) if diff.any() else 0.0,
                            "mass_oracle": math.fsum(ho2.ravel()), "mass_reference": math.fsum(hr2.ravel())}
        cmp["seconds"] = time.time() - t
        out["reference"] = cmp
        print("reference", cmp, flush=True)
        write(out)


if __name__ == "__main__":
    main()
