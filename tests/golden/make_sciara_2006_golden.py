"""Golden fixture of SCIARA-fv2 on the reference's own input files: the
2006 configuration the reference ships (OpenCAL/examples/cal_sciara-fv2/
data/2006: parameter file, GIS morphology and vent grids, emission rates).

Stores the four input files byte for byte (compressed), and the final Sz,
Slt, St and Msl of the reference's SCIARA-fv2 program (compiled unmodified
from its sources by oracle/ref/Makefile, target `sciara`) run on them for
STEPS steps with active cells off and on; checks that the oracle
restatement, fed by the library's reader (cal_sciara_read), gives the
reference's bits.  Needs the reference source tree, named by the
OPENCAL_REFERENCE environment variable.

Run:  OPENCAL_REFERENCE=<OpenCAL tree> python tests/golden/make_sciara_2006_golden.py
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

REF = os.environ.get("OPENCAL_REFERENCE") or ""  # required when run as a script (checked in main)
DATA = "OpenCAL/examples/cal_sciara-fv2/data/2006"
FILES = ["2006_000000000000.cfg", "2006_000000000000_Morphology.stt", "2006_000000000000_Vents.stt",
         "2006_000000000000_EmissionRate.txt"]
STEPS = 1000


def main():
    if not REF or not os.path.isdir(os.path.join(REF, "OpenCAL-OMP")):
        sys.exit("set OPENCAL_REFERENCE to the OpenCAL source tree")
    import oracle
    import opencal_gb300 as cal
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle", "ref"), f"REF={REF}", "all", "sciara"],
                   check=True)
    oracle.build()
    cal.build()
    work = tempfile.mkdtemp(prefix="opencal_sciara2006_")
    out = {}
    for name in FILES:
        shutil.copy(os.path.join(REF, DATA, name), os.path.join(work, name))
        out["file_" + name.split("_")[-1].replace(".", "_")] = np.frombuffer(
            open(os.path.join(REF, DATA, name), "rb").read(), dtype=np.uint8)
    prefix = os.path.join(work, "2006")
    cfg = cal.sciara_read(prefix)
    z0 = cfg["z"]
    for ac in (0, 1):
        res = os.path.join(work, f"out{ac}.bin")
        subprocess.run([os.path.join(ROOT, "oracle", "_ref", "sciara_ref"), prefix, str(STEPS), str(ac), res],
                       check=True, stdout=subprocess.DEVNULL)
        raw = np.fromfile(res, dtype=np.float64)
        n = z0.size
        ref = {k: raw[q * n:(q + 1) * n].reshape(z0.shape) for q, k in enumerate(("z", "slt", "st", "msl"))}
        orc = oracle.sciara(z0, cfg["vents"], cfg["rates"], cfg["emission_time"], STEPS, ac=bool(ac),
                            params=cfg["params"])
        for k in ("z", "slt", "st", "msl"):
            assert orc[k].tobytes() == ref[k].tobytes(), (ac, k, float(np.abs(orc[k] - ref[k]).max()))
        p = f"ac{ac}_"
        out[p + "dz"] = ref["z"] - z0  # zero except where lava solidified
        for k in ("slt", "st", "msl"):
            out[p + k] = ref[k]
        out[p + "steps"] = np.array([orc["steps"], int(raw[4 * n])], dtype=np.int64)
        print(f"active cells {ac}: {STEPS} steps, lava cells {(ref['slt'] > 0).sum()}, "
              f"oracle == reference bit for bit")
    out["steps"] = np.array([STEPS], dtype=np.int64)
    np.savez_compressed(os.path.join(HERE, "sciara_2006.npz"), **out)
    print("wrote", os.path.join(HERE, "sciara_2006.npz"), os.path.getsize(os.path.join(HERE, "sciara_2006.npz")))


if __name__ == "__main__":
    main()
