"""The benchmarked configuration against the oracle, at its full size:
SCIDDICA-T 2048 x 2048 FP64, von Neumann, flat, p_r = 0.5, p_epsilon = 0.001,
the bench's seeded inputs (workloads.sciddicaT_inputs(2048, 2048, seed=2)),
4000 steps.

tests/golden/sciddicaT_2048.json holds SHA-256 digests of the oracle's final
h (and active list) for this run, and sciddicaT_2048_outflux.npy the mass
that left the grid in each step; both are made on the CPU by
tests/golden/make_sciddicaT_2048_golden.py (the oracle is built with
-ffp-contract=off and the inputs are quantised to 2^-10, so every machine
computes the same bits).  Checked here:

* the persistent split step (the bench's timed form, every step in one
  cooperative launch) and the persistent active-cells split step give the
  oracle's final h bit for bit, and the active list;
* the traced run (split step one launch pair at a time, with the boundary
  trace): the same final bits, the oracle's first step at which the two-cell
  edge band gets wet, the mass leaving the grid per step within 1e-12
  relative of the oracle's (the sums run in another order), and the mass
  balance M0 - outflux - M_T within 1e-12 of M0.
"""
import ctypes as C
import hashlib
import json
import math
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
RTOL = 1e-12  # mass terms: per-step outflux and the balance, relative


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.fixture(scope="module")
def setup():
    import opencal_gb300 as cal
    from opencal_gb300 import workloads as W
    cal.build()
    with open(os.path.join(GOLDEN, "sciddicaT_2048.json")) as f:
        g = json.load(f)
    z, h = W.sciddicaT_inputs(g["rows"], g["cols"], seed=g["seed"])
    assert sha(z) == g["z0_sha256"] and sha(h) == g["h0_sha256"], "input generator drifted"
    return cal, g, z, h


def test_persistent_split_step_matches_oracle(setup):
    cal, g, z, h = setup
    zt, ht, _ = cal.sciddicaT(z, h, g["steps"], toroidal=False, ac=False, p_r=g["p_r"], p_eps=g["p_eps"],
                              mode=cal.MODE_FUSED, graph=4)
    assert sha(ht) == g["plain"]["h_sha256"], "final h differs from the oracle's"
    assert sha(zt) == g["plain"]["z_sha256"]


def test_persistent_active_cells_split_step_matches_oracle(setup):
    cal, g, z, h = setup
    za, ha, cells = cal.sciddicaT(z, h, g["steps"], toroidal=False, ac=True, p_r=g["p_r"], p_eps=g["p_eps"],
                                  mode=cal.MODE_FUSED, graph=4)
    ac = g["active_cells"]
    assert len(cells) == ac["n_active"]
    assert sha(cells.astype(np.int32)) == ac["cells_sha256"], "active list differs from the oracle's"
    assert sha(ha) == ac["h_sha256"], "final h differs from the oracle's"


def test_traced_run_edge_step_and_mass_balance(setup):
    cal, g, z, h = setup
    m = cal.models()
    m.cal_sciddicaT_open.restype = C.c_void_p
    m.cal_sciddicaT_open.argtypes = [C.c_int] * 4 + [C.c_double] * 2 + [C.c_void_p] * 2 + [C.c_int]
    m.cal_sciddicaT_trace.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    m.cal_sciddicaT_read.argtypes = [C.c_void_p, C.c_void_p]
    m.cal_sciddicaT_close.argtypes = [C.c_void_p]
    steps = g["steps"]
    sess = m.cal_sciddicaT_open(g["rows"], g["cols"], 0, 0, g["p_r"], g["p_eps"], z.ctypes.data, h.ctypes.data,
                                cal.MODE_FUSED)
    assert sess, "cal_sciddicaT_open failed"
    outflux = np.zeros(steps)
    wet = np.zeros(steps, np.int32)
    edge = C.c_int(-1)
    ht = np.empty_like(h)
    try:
        assert m.cal_sciddicaT_trace(sess, steps, outflux.ctypes.data, wet.ctypes.data, C.byref(edge)) == 0
        assert m.cal_sciddicaT_read(sess, ht.ctypes.data) == 0
    finally:
        m.cal_sciddicaT_close(sess)
    plain = g["plain"]
    assert sha(ht) == plain["h_sha256"], "traced run: final h differs from the oracle's"
    assert edge.value == plain["edge_step"], "first step with a wet edge band differs from the oracle's"
    ref_out = np.load(os.path.join(GOLDEN, "sciddicaT_2048_outflux.npy"))
    assert ref_out.shape == outflux.shape
    # per step: the same border outflows summed in another order
    scale = max(float(np.abs(ref_out).max()), 1e-300)
    assert np.all(np.abs(outflux - ref_out) <= RTOL * scale), "per-step outflux differs from the oracle's"
    assert (outflux[: plain["edge_step"] - 1] == 0.0).all() or plain["edge_step"] < 0
    m0 = math.fsum(h.ravel())
    mt = math.fsum(ht.ravel())
    of = math.fsum(outflux)
    assert abs(m0 - of - mt) <= RTOL * m0, "mass balance M0 - outflux - M_T"
    assert abs(of - plain["outflux_total"]) <= RTOL * m0
    assert (wet > 0).all(), "every step of the run has wet cells"
