"""Regenerate the SCIARA-fv2 golden fixtures from the REFERENCE itself.

Needs the reference source tree, named by the OPENCAL_REFERENCE environment
variable; nothing that runs on the GPU machine calls this script.

Compiles the reference's SCIARA-fv2 example (OpenCAL-OMP/examples/
calomp_sciara-fv2, its own sources, unmodified) against the serially built
reference library with a headless driver (oracle/ref/Makefile, target
`sciara`), writes each seeded synthetic case in the example's own input
formats (parameter file, GIS morphology and vent grids, emission-rate
file), runs the reference program on it, checks that the oracle restatement
(oracle/oracle_sciara.c) reproduces the reference's final Sz, Slt, St and
Msl bit for bit, and writes the reference outputs to sciara_cases.npz.

The parameters are those of the example's 2006 configuration file; the
morphology is a synthetic cone with fractal noise (opencal_gb300.workloads.
sciara_inputs); there is no SCIARA output golden in the reference.

Run:  python tests/golden/make_sciara_golden.py
"""
from __future__ import annotations

import os
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
CFG_KEYS = ["Pclock", "PTsol", "PTvent", "Pr(Tsol)", "Pr(Tvent)", "Phc(Tsol)", "Phc(Tvent)", "Pcool", "Prho",
            "Pepsilon", "Psigma", "Pcv"]

# (rows, cols, seed, emission_time [s], max steps (0: until the emission ends), active cells)
CASES = [
    (64, 80, 5, 600, 0, 0),
    (64, 80, 5, 600, 0, 1),
    (96, 128, 6, 900, 0, 0),
    (96, 128, 6, 900, 0, 1),
    (77, 101, 7, 1200, 70, 1),
    (120, 90, 8, 300, 0, 0),
]


def write_case(prefix: str, z, vents, rates, emission_time, params):
    rows, cols = z.shape
    with open(prefix + "_000000000000.cfg", "w") as f:
        f.write("maximum_steps_(0_for_loop) 0\nstopping_threshold_(height) 0.00\nrefreshing_step 0\n"
                "thickness_visual_threshold 0.00\n")
        for k, v in zip(CFG_KEYS, params[:12]):
            f.write(f"{k} {v!r}\n")
        f.write("algorithm MIN\n")
    header = (f"ncols {cols}\nnrows {rows}\nxllcorner 0.0\nyllcorner 0.0\ncellsize {params[12]!r}\n"
              f"NODATA_value -9999.0\n")
    with open(prefix + "_000000000000_Morphology.stt", "w") as f:
        f.write(header)
        for row in z:
            f.write(" ".join(repr(float(x)) for x in row) + "\n")
    mv = np.zeros((rows, cols), dtype=np.int64)
    for vid, (x, y) in enumerate(vents, start=1):
        mv[y, x] = vid
    with open(prefix + "_000000000000_Vents.stt", "w") as f:
        f.write(header)
        for row in mv:
            f.write(" ".join(str(int(x)) for x in row) + "\n")
    # vents are numbered in the row-major order the reference scans the grid
    order = sorted(range(len(vents)), key=lambda k: (vents[k][1], vents[k][0]))
    with open(prefix + "_000000000000_EmissionRate.txt", "w") as f:
        f.write(f"[TIME]\n{int(emission_time)}\n\n")
        for vid in range(1, len(vents) + 1):
            f.write(f"[VENT_ID]\n{vid}\n\n[EMISSION_RATE]\n")
            for r in rates[vid - 1]:
                f.write(f"{r!r}\n")
            f.write("\n")
        f.write("[END]\n")
    return [vents[k] for k in order], [rates[k] for k in order]


def main():
    if not REF or not os.path.isdir(os.path.join(REF, "OpenCAL-OMP")):
        sys.exit("set OPENCAL_REFERENCE to the OpenCAL source tree")
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle", "ref"), f"REF={REF}", "all", "sciara"],
                   check=True)
    oracle.build()
    binary = os.path.join(ROOT, "oracle", "_ref", "sciara_ref")
    params = W.SCIARA_PARAMS
    out = {}
    work = tempfile.mkdtemp(prefix="opencal_sciara_")
    for idx, (rows, cols, seed, et, steps, ac) in enumerate(CASES):
        z, vents, rates = W.sciara_inputs(rows, cols, seed=seed)
        prefix = os.path.join(work, f"case{idx}")
        vents_ord, rates_ord = write_case(prefix, z, vents, rates, et, params)
        res = os.path.join(work, f"case{idx}.bin")
        subprocess.run([binary, prefix, str(steps if steps else 1000000), str(ac), res], check=True,
                       stdout=subprocess.DEVNULL)
        raw = np.fromfile(res, dtype=np.float64)
        n = rows * cols
        ref = {k: raw[q * n:(q + 1) * n].reshape(rows, cols) for q, k in enumerate(("z", "slt", "st", "msl"))}
        ref_steps, ref_active = int(raw[4 * n]), int(raw[4 * n + 1])
        orc = oracle.sciara(z, vents_ord, rates_ord, et, steps, ac=bool(ac))
        for k in ("z", "slt", "st", "msl"):
            assert orc[k].tobytes() == ref[k].tobytes(), (idx, k, np.abs(orc[k] - ref[k]).max())
        # the reference's step counter ends one past the last step run when the stop condition fires
        assert orc["steps"] in (ref_steps, ref_steps - 1), (idx, orc["steps"], ref_steps)
        if ac:
            assert len(orc["cells"]) == ref_active, (idx, len(orc["cells"]), ref_active)
        pfx = f"c{idx}_"
        out[pfx + "dims"] = np.array([rows, cols, seed, et, steps, ac], dtype=np.int64)
        out[pfx + "z0"] = z
        out[pfx + "vents"] = np.asarray(vents_ord, dtype=np.int32)
        out[pfx + "rates"] = np.asarray(rates_ord, dtype=np.float64)
        for k in ("z", "slt", "st", "msl"):
            out[pfx + k] = ref[k]
        out[pfx + "steps"] = np.array([orc["steps"]], dtype=np.int64)
        out[pfx + "active"] = np.array([ref_active if ac else 0], dtype=np.int64)
        print(f"case {idx}: {rows}x{cols} ac={ac} steps={orc['steps']} lava cells={(ref['slt'] > 0).sum()} "
              f"solid={ref['msl'].sum():.3f} -- oracle == reference bit for bit")
    out["params"] = np.asarray(params, dtype=np.float64)
    np.savez_compressed(os.path.join(HERE, "sciara_cases.npz"), **out)


if __name__ == "__main__":
    main()
