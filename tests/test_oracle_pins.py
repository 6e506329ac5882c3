"""The oracle (CPU restatement, oracle/) pinned against the reference.

* the reference's shipped SCIDDICA-T golden (610x496, toroidal, 4000 steps):
  the oracle's %.9f text must hash to the golden file's sha256, byte for byte;
* the shipped active-cells golden (printed with %f) and the reference's own
  rerun of that example (tests/golden/make_golden.py);
* fixtures generated by running the reference library itself on seeded
  synthetic cases: every neighbourhood, both boundaries, active cells on and
  off, 2D and 3D -- bit-exact, active lists included;
* when the reference tree is present (not on the GPU machine), extra seeds are
  checked against the live reference build.
"""
import hashlib
import io
import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")


def _manifest():
    with open(os.path.join(GOLDEN, "manifest.json")) as f:
        return json.load(f)


def format_pct9(h):
    """calSaveSubstate2Dr's text format (OpenCAL-OMP/source/cal2DBufferIO.c:142)."""
    out = io.StringIO()
    for row in h:
        out.write("".join("%.9f  " % v for v in row))
        out.write("\n")
    return out.getvalue().encode()


def bits_equal(a, b):
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(b)
    return a.shape == b.shape and a.dtype == b.dtype and a.tobytes() == b.tobytes()


@pytest.mark.slow
def test_oracle_reproduces_shipped_plain_golden(oracle_lib):
    g = np.load(os.path.join(GOLDEN, "sciddicaT_610x496.npz"))
    meta = _manifest()["sciddicaT_610x496"]
    _, h, _ = oracle_lib.sciddicaT(g["z"], g["h0"], meta["steps"], toroidal=True, ac=False,
                                   p_r=meta["p_r"], p_eps=meta["p_eps"], kind="omp")
    assert hashlib.sha256(format_pct9(h)).hexdigest() == meta["plain_text_sha256"]


@pytest.mark.slow
def test_oracle_reproduces_shipped_ac_golden(oracle_lib):
    g = np.load(os.path.join(GOLDEN, "sciddicaT_610x496.npz"))
    meta = _manifest()["sciddicaT_610x496"]
    _, h, cells = oracle_lib.sciddicaT(g["z"], g["h0"], meta["steps"], toroidal=True, ac=True,
                                       p_r=meta["p_r"], p_eps=meta["p_eps"])
    printed = np.array([[float("%.9f" % v) for v in row] for row in h])
    assert np.array_equal(printed, g["h_ac_ref_run"])   # the reference rerun here, %.9f
    assert np.abs(h - g["h_ac"]).max() <= 5e-7            # the shipped %f golden
    assert len(cells) > 0 and np.all(h[cells[:, 0], cells[:, 1]] > meta["p_eps"])


def _cases():
    import sys
    sys.path.insert(0, GOLDEN)
    import make_golden  # noqa: E402  (the generator defines the case list and inputs)
    return make_golden


@pytest.mark.parametrize("idx", range(len(_manifest()["synthetic_cases"])))
def test_oracle_matches_reference_fixtures(oracle_lib, idx):
    mg = _cases()
    meta = _manifest()["synthetic_cases"][idx]
    fx = np.load(os.path.join(GOLDEN, "synthetic_cases.npz"))
    out = mg.run_case(meta["kind"], meta["kw"], "serial")
    for key in meta["keys"]:
        assert bits_equal(out[key], fx[f"c{idx}_{key}"]), (meta, key)


def test_oracle_serial_equals_openmp(oracle_lib):
    from opencal_gb300 import workloads as W
    z, h = W.sciddicaT_inputs(192, 160, seed=21)
    for ac in (0, 1):
        a = oracle_lib.sciddicaT(z, h, 40, toroidal=False, ac=ac, kind="serial")
        b = oracle_lib.sciddicaT(z, h, 40, toroidal=False, ac=ac, kind="omp")
        assert bits_equal(a[1], b[1]) and np.array_equal(a[2], b[2])


@pytest.mark.parametrize("seed", [31, 32])
def test_oracle_vs_live_reference(reference_oracle, seed):
    oracle = reference_oracle
    from opencal_gb300 import workloads as W
    z, h = W.sciddicaT_inputs(200, 176, seed=seed)
    for tor in (0, 1):
        for ac in (0, 1):
            a = oracle.sciddicaT(z, h, 35, toroidal=tor, ac=ac)
            b = oracle.sciddicaT(z, h, 35, toroidal=tor, ac=ac, kind="ref")
            inner = a[1].copy()
            inner[2:-2, 2:-2] = 0
            if not tor:
                assert not inner.any(), "flat case reached the edge band"
            assert bits_equal(a[1], b[1]) and bits_equal(a[0], b[0]) and np.array_equal(a[2], b[2])
    v = W.random_field((30, 26), seed=seed)
    for nb in (1, 2, 3, 4):
        assert bits_equal(oracle.nbprobe2d(v, 4, nbhd=nb), oracle.nbprobe2d(v, 4, nbhd=nb, kind="ref"))


CUSTOM_NEIGHBOURHOODS = [
    [(0, 0), (-1, 0), (0, 2), (2, -1), (1, 1)],
    [(0, 0), (-2, -2), (-2, 2), (2, -2), (2, 2), (0, -3), (3, 0)],
    [(1, 0), (0, 0), (0, -1)],  # the cell itself need not come first
]


@pytest.mark.parametrize("idx", range(len(CUSTOM_NEIGHBOURHOODS)))
def test_oracle_custom_neighbourhood_vs_live_reference(reference_oracle, idx):
    """calAddNeighbor2D on a CAL_CUSTOM_NEIGHBORHOOD_2D model (OpenCAL-OMP/
    source/cal2D.c:444-466), toroidal (the reference's flat reads outside the
    grid are unchecked)."""
    oracle = reference_oracle
    from opencal_gb300 import workloads as W
    v = W.random_field((23, 29), seed=40 + idx)
    offs = CUSTOM_NEIGHBOURHOODS[idx]
    a = oracle.nbprobe2d_custom(v, 5, offs, toroidal=True)
    b = oracle.nbprobe2d_custom(v, 5, offs, toroidal=True, kind="ref")
    assert bits_equal(a, b)


def _reduction_data(kind, op, rows, cols, seed):
    from opencal_gb300.workloads import uniform_array
    u = uniform_array(seed, (rows, cols))
    if kind == 0:
        d = (u * 7).astype(np.int8) + 1
        if op == 4:
            d = np.where(u < 0.5, 1, 3).astype(np.int8)
    elif kind == 1:
        d = (u * 1000 - 300).astype(np.int32)
        if op == 4:
            d = np.where(u < 0.5, 1, 3).astype(np.int32)
    else:
        d = u * 10.0 - 2.0
        if op == 4:
            d = 1.0 + (u - 0.5) * 1e-3
    return np.ascontiguousarray(d)


@pytest.mark.parametrize("op", range(1, 11))
@pytest.mark.parametrize("kind", [0, 1, 2])
def test_oracle_reduction_vs_live_reference(reference_oracle, kind, op):
    """The reference's serial calReductionOperation2D* folds elements
    0 .. rows-1 (cal2DReduction.c:45-47); on a one-column grid that is every
    cell, and the oracle (which folds every cell) must give its bits."""
    oracle = reference_oracle
    d = _reduction_data(kind, op, 173, 1, 300 + op + 10 * kind)
    a = oracle.reduce2d(kind, d, op)
    b = oracle.reduce2d(kind, d, op, kind="ref")
    assert bits_equal(np.float64(a), np.float64(b)), (a, b)


def _sciara_cases():
    fx = np.load(os.path.join(GOLDEN, "sciara_cases.npz"))
    n = len([k for k in fx.files if k.endswith("_dims")])
    return fx, n


@pytest.mark.parametrize("idx", range(6))
def test_oracle_sciara_matches_reference_fixtures(oracle_lib, idx):
    """oracle_sciara.c against the reference's own SCIARA-fv2 program
    (compiled from its sources, run on the same synthetic inputs): Sz, Slt,
    St and Msl bit for bit.  The transcendental functions are the C
    library's on both sides (same machine class as the fixtures: x86-64
    glibc)."""
    fx, n = _sciara_cases()
    assert idx < n
    p = f"c{idx}_"
    rows, cols, seed, et, steps, ac = (int(v) for v in fx[p + "dims"])
    vents = [tuple(v) for v in fx[p + "vents"]]
    rates = fx[p + "rates"].tolist()
    out = oracle_lib.sciara(fx[p + "z0"], vents, rates, et, steps, ac=bool(ac))
    for k in ("z", "slt", "st", "msl"):
        assert out[k].tobytes() == fx[p + k].tobytes(), k
    assert out["steps"] == int(fx[p + "steps"][0])
    if ac:
        assert len(out["cells"]) == int(fx[p + "active"][0])


@pytest.mark.parametrize("nb", [1, 2, 3, 4])
def test_oracle_unsafe_probe_matches_reference_fixtures(oracle_lib, nb):
    """the unsafe-operation probe (calAddNext*, calSetX*, calGetNextX*,
    calSetCurrentX*, calInitX*) against the reference library's run"""
    fx = np.load(os.path.join(GOLDEN, "unsafe_cases.npz"))
    p = f"probe{nb}_"
    got = oracle_lib.unsafe2d(fx[p + "v0"], fx[p + "b0"], fx[p + "w0"], 12, nbhd=nb, toroidal=True)
    for name, a in zip(("v", "b", "w", "u", "x"), got):
        assert a.tobytes() == fx[p + name].tobytes(), name


def test_oracle_sciddicaT_unsafe_matches_reference_fixture(oracle_lib):
    fx = np.load(os.path.join(GOLDEN, "unsafe_cases.npz"))
    z, h = oracle_lib.sciddicaT_unsafe(fx["sdtu_z0"], fx["sdtu_h0"], 50, toroidal=True)
    assert z.tobytes() == fx["sdtu_z"].tobytes() and h.tobytes() == fx["sdtu_h"].tobytes()


def _io_arrays():
    from opencal_gb300 import workloads as W
    u2, u3 = W.uniform_array(61, (17, 23)), W.uniform_array(62, (5, 9, 11))
    return [
        (u2 * 120 - 60).astype(np.int8), (u2 * 2e6 - 1e6).astype(np.int32), (u2 - 0.5) * 3e3,
        (u3 * 120 - 60).astype(np.int8), (u3 * 2e6 - 1e6).astype(np.int32), (u3 - 0.5) * 3e3,
    ]


@pytest.mark.parametrize("idx", range(6))
def test_oracle_text_files_vs_live_reference(reference_oracle, tmp_path, idx):
    """Substate text files: the oracle's writer gives the reference's bytes
    (calSaveSubstate2D* "%.9f " / 3D "%f " / "%d " plus a space, newline per
    row, empty line per slice), and both readers give the same values."""
    oracle = reference_oracle
    a = _io_arrays()[idx]
    oracle.save_text(a, tmp_path / "o.txt")
    oracle.save_text(a, tmp_path / "r.txt", kind="ref")
    assert (tmp_path / "o.txt").read_bytes() == (tmp_path / "r.txt").read_bytes()
    x = oracle.load_text(a.shape, a.dtype, tmp_path / "r.txt")
    y = oracle.load_text(a.shape, a.dtype, tmp_path / "r.txt", kind="ref")
    assert x.tobytes() == y.tobytes()
