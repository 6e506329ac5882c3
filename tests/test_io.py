"""Substate text files on the GPU path (cal2DIO.h / cal3DIO.h) against the
oracle's restatement of the reference's format (oracle/cal_oracle.c,
orc_save_text / orc_load_text, pinned to the reference's own
calSaveSubstate / calLoadSubstate in tests/test_oracle_pins.py):

* calLoadSubstate* -> a device update -> calSaveSubstate*, byte, int and
  real substates, 2D and 3D: the file written is byte for byte the oracle's
  file of the same values, and the values loaded are the oracle's;
* the reference SCIDDICA-T example's main() as written (z and h from text
  files, calRun2D, h saved with calSaveSubstate2Dr) on its shipped 610 x 496
  data, 4000 steps: the file it writes is the reference's shipped golden
  width_final.txt byte for byte (its SHA-256 is in tests/golden/manifest.json).
"""
import ctypes as C
import hashlib
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")


def _arrays():
    from opencal_gb300 import workloads as W
    u2, u3 = W.uniform_array(61, (37, 29)), W.uniform_array(62, (6, 13, 17))
    return [
        (u2 * 120 - 60).astype(np.int8), (u2 * 2e6 - 1e6).astype(np.int32), (u2 - 0.5) * 3e3,
        (u3 * 120 - 60).astype(np.int8), (u3 * 2e6 - 1e6).astype(np.int32), (u3 - 0.5) * 3e3,
    ]


@pytest.fixture(scope="module")
def libs():
    import oracle
    import opencal_gb300 as cal
    import probes
    cal.build()
    oracle.build()
    probes.lib()
    return probes, oracle


@pytest.mark.parametrize("idx", range(6))
def test_load_save_roundtrip_matches_oracle(libs, tmp_path, idx):
    probes, oracle = libs
    a = _arrays()[idx]
    oracle.save_text(a, tmp_path / "in.txt")
    want = oracle.load_text(a.shape, a.dtype, tmp_path / "in.txt")
    got = probes.io_roundtrip(a, tmp_path / "in.txt", tmp_path / "out.txt")
    assert got.tobytes() == want.tobytes()
    oracle.save_text(want, tmp_path / "want.txt")
    assert (tmp_path / "out.txt").read_bytes() == (tmp_path / "want.txt").read_bytes()


def test_reference_example_main_writes_the_shipped_golden(libs, tmp_path):
    import opencal_gb300 as cal
    probes, oracle = libs
    with open(os.path.join(GOLDEN, "manifest.json")) as f:
        meta = json.load(f)["sciddicaT_610x496"]
    g = np.load(os.path.join(GOLDEN, "sciddicaT_610x496.npz"))
    # the shipped DEM and source, written back in the reference's text format
    # (their values round-trip through "%.9f": checked)
    for name, key in (("dem.txt", "z"), ("source.txt", "h0")):
        oracle.save_text(g[key], tmp_path / name)
        assert oracle.load_text(g[key].shape, np.float64, tmp_path / name).tobytes() == g[key].tobytes()
    m = cal.models()
    f = m.cal_sciddicaT_run_files
    f.restype = C.c_int
    f.argtypes = [C.c_int] * 4 + [C.c_double] * 2 + [C.c_char_p] * 3 + [C.c_int]
    for graph in (0, 1):
        out = tmp_path / f"width_final_{graph}.txt"
        rc = f(meta["rows"], meta["cols"], int(meta["toroidal"]), meta["steps"], meta["p_r"], meta["p_eps"],
               str(tmp_path / "dem.txt").encode(), str(tmp_path / "source.txt").encode(), str(out).encode(), graph)
        assert rc == 0
        assert hashlib.sha256(out.read_bytes()).hexdigest() == meta["plain_text_sha256"]
