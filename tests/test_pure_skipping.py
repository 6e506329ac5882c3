"""Performance declarations of elementary processes, which must not change
any result.

Tile skipping of processes declared pure (calSetElementaryProcessPure2D):
the process kernel skips the 32 x 8 tiles where the process changed nothing
the last time and whose 3 x 3 tile neighbourhood has not changed since.  The
results must be the dense run's bits: checked here against the oracle on
SCIDDICA-T (the reference program with both processes declared pure, flat
and toroidal grids, per-step launches, recorded-step replay and the
device-driven loop, including the reference's shipped 610 x 496 golden) and
on Life defined from Python, and for a custom neighbourhood that reaches
further than one tile (skipping refused, still exact).  Also the active-cell
counterpart: the compaction after a process that changed no flag keeps the
list (a session reset that rewrites the flags through their device pointer
must still be seen).

Guards (calSetElementaryProcessGuard2Dr): SCIDDICA-T's flows process with
its early return on dry cells declared, alone and with the other
declarations, against the same oracle runs and the shipped golden; a guard
on a substate of another type is refused.

TMA staging of the substates a process declared it reads
(calSetElementaryProcessReads2D): SCIDDICA-T (doubles, von Neumann, flat and
toroidal: border tiles of toroidal grids read global memory), Life (bytes,
Moore, boxes 64 cells wide), an integer rule on a hexagonal neighbourhood,
each against the oracle or the same program without the declaration; rows
that are not a multiple of 16 bytes keep global reads.
"""
import hashlib
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(params=[(1, 0, 0), (0, 1, 0), (1, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1)],
                ids=["pure", "staged", "pure+staged", "guard", "pure+guard", "pure+staged+guard"])
def pure_sdt(request):
    import opencal_gb300 as cal
    cal.build()
    m = cal.models()
    pure, staged, guard = request.param
    m.cal_sciddicaT_set_pure(pure)
    m.cal_sciddicaT_set_staged(staged)
    m.cal_sciddicaT_set_guard(guard)
    yield cal
    m.cal_sciddicaT_set_pure(0)
    m.cal_sciddicaT_set_staged(0)
    m.cal_sciddicaT_set_guard(0)


@pytest.mark.parametrize("rows,cols,seed,steps,tor", [(160, 144, 11, 60, 0), (203, 177, 13, 90, 1),
                                                      (256, 256, 5, 150, 0)])
@pytest.mark.parametrize("graph", [0, 1, 2])
def test_sciddicaT_pure_processes_bit_exact(pure_sdt, rows, cols, seed, steps, tor, graph):
    import oracle
    from opencal_gb300 import workloads as W
    cal = pure_sdt
    oracle.build()
    z, h = W.sciddicaT_inputs(rows, cols, seed=seed)
    ref = oracle.sciddicaT(z, h, steps, toroidal=bool(tor), ac=False)
    got = cal.sciddicaT(z, h, steps, toroidal=bool(tor), ac=False, mode=cal.MODE_PROCESSES, graph=graph)
    assert got[1].tobytes() == ref[1].tobytes()
    assert got[0].tobytes() == ref[0].tobytes()


def test_sciddicaT_pure_processes_shipped_golden(pure_sdt):
    cal = pure_sdt
    g = np.load(os.path.join(GOLDEN, "sciddicaT_610x496.npz"))
    meta = json.load(open(os.path.join(GOLDEN, "manifest.json")))["sciddicaT_610x496"]
    _, h, _ = cal.sciddicaT(g["z"], g["h0"], 4000, toroidal=True, ac=False, mode=cal.MODE_PROCESSES, graph=1)
    text = "".join("".join("%.9f  " % v for v in row) + "\n" for row in h).encode()
    assert hashlib.sha256(text).hexdigest() == meta["plain_text_sha256"]


LIFE_BODY = """
    int sum = 0;
    for (int n = 1; n < ca->sizeof_X; n++)
        sum += calGetX2Db(ca, Q.alive, i, j, n);
    const CALbyte a = calGet2Db(ca, Q.alive, i, j);
    calSet2Db(ca, Q.alive, i, j, (sum == 3 || (a == 1 && sum == 2)) ? 1 : 0);
"""


@pytest.mark.parametrize("staged", [False, True])
@pytest.mark.parametrize("shape,tor,graph", [((96, 80), True, False), ((130, 70), False, True),
                                            ((72, 256), True, True), ((64, 96), False, False)])
def test_life_pure_from_python(shape, tor, graph, staged):
    """Life on a sparse field (most tiles dead and skipped after their first
    generation) declared pure from Python, with and without its substate
    staged (byte rows of 80, 256, 96 cells are staged, 70 are not)."""
    import oracle
    import opencal_gb300 as cal
    from opencal_gb300 import program as P
    cal.build()
    oracle.build()
    rng = np.random.default_rng(3)
    s0 = np.zeros(shape, np.uint8)
    s0[10:30, 12:40] = rng.random((20, 28)) < 0.35  # one live patch
    lib = P.Program("pylife_pure").substates(alive="b").process("pylife_pure_rule", LIFE_BODY).build()
    model = P.Model2D(shape[0], shape[1], P.CAL_MOORE_NEIGHBORHOOD_2D,
                      P.CAL_SPACE_TOROIDAL if tor else P.CAL_SPACE_FLAT)
    alive = model.add_substate("b")
    lib.bind(alive=alive)
    rule = lib.process("pylife_pure_rule")
    model.add_process(rule)
    model.set_pure(rule)
    if staged:
        model.set_reads(rule, [alive])
    model.load(alive, s0.astype(np.int8))
    run = P.Run2D(model, 1, 60, graph=graph)
    try:
        run.run()
        got = model.read(alive).astype(np.uint8)
    finally:
        run.close()
        model.close()
    assert np.array_equal(got, oracle.life2d(s0, 60, toroidal=tor))


def test_life_pure_grid_too_large_to_deal():
    """6144 x 6400 cells: 200 x 768 tiles (4800 bitmap words, 63 tiles per
    block of the launch) is past what a skipping launch deals over its
    blocks (4096 words), so the blocks walk their own tiles instead; three
    sparse patches, 12 generations, against the oracle."""
    import oracle
    import opencal_gb300 as cal
    from opencal_gb300 import program as P
    cal.build()
    oracle.build()
    rows, cols = 6144, 6400
    rng = np.random.default_rng(7)
    s0 = np.zeros((rows, cols), np.uint8)
    for (i, j) in ((40, 60), (3000, 3100), (6100, 6350)):
        s0[i:i + 30, j:j + 40] = rng.random((30, 40)) < 0.4
    lib = P.Program("pylife_large").substates(alive="b").process("pylife_large_rule", LIFE_BODY).build()
    model = P.Model2D(rows, cols, P.CAL_MOORE_NEIGHBORHOOD_2D, P.CAL_SPACE_TOROIDAL)
    alive = model.add_substate("b")
    lib.bind(alive=alive)
    rule = lib.process("pylife_large_rule")
    model.add_process(rule)
    model.set_pure(rule)
    model.load(alive, s0.astype(np.int8))
    run = P.Run2D(model, 1, 12, graph=False)
    try:
        run.run()
        got = model.read(alive).astype(np.uint8)
    finally:
        run.close()
        model.close()
    assert np.array_equal(got, oracle.life2d(s0, 12, toroidal=True))


def test_far_reaching_custom_neighbourhood_is_not_skipped():
    """A custom neighbourhood 12 rows tall reaches past the adjacent tile:
    the declaration is accepted but tiles are not skipped, and the run
    matches a dense run of the same program."""
    import opencal_gb300 as cal
    from opencal_gb300 import program as P
    cal.build()
    body = """
        CALint s = calGet2Di(ca, Q.v, i, j);
        for (int n = 1; n < ca->sizeof_X; n++) s += calGetX2Di(ca, Q.v, i, j, n);
        calSet2Di(ca, Q.v, i, j, s % 7);
    """
    lib = P.Program("pyfar").substates(v="i").process("pyfar_rule", body).build()
    capi = P.capi()
    import ctypes as C
    capi.calAddNeighbor2D.argtypes = [C.c_void_p, C.c_int, C.c_int]
    capi.calAddNeighbor2D.restype = C.c_void_p
    out = []
    for pure in (False, True):
        model = P.Model2D(64, 96, P.CAL_CUSTOM_NEIGHBORHOOD_2D, P.CAL_SPACE_FLAT)
        for di, dj in ((0, 0), (-12, 0), (12, 0), (0, 1)):
            capi.calAddNeighbor2D(model, di, dj)
        v = model.add_substate("i")
        lib.bind(v=v)
        rule = lib.process("pyfar_rule")
        model.add_process(rule)
        if pure:
            model.set_pure(rule)
        v0 = np.zeros((64, 96), np.int32)
        v0[30:34, 40:44] = 1
        model.load(v, v0)
        run = P.Run2D(model, 1, 15)
        try:
            run.run()
            out.append(model.read(v))
        finally:
            run.close()
            model.close()
    assert out[0].tobytes() == out[1].tobytes()
    assert out[0].any()


def test_active_cells_session_reset_and_rerun():
    """The active-cells program through a session: run, reset (the flags
    restored through their device pointer, then calUpdateActiveCells2D),
    run again.  The compactions after processes that changed no flag keep
    the list; both runs must give the oracle's h and active set."""
    import ctypes as C
    import oracle
    import opencal_gb300 as cal
    from opencal_gb300 import workloads as W
    cal.build()
    oracle.build()
    z, h = W.sciddicaT_inputs(160, 144, seed=11)
    steps = 50
    ref = oracle.sciddicaT(z, h, steps, toroidal=False, ac=True)
    m = cal.models()
    m.cal_sciddicaT_open.restype = C.c_void_p
    m.cal_sciddicaT_open.argtypes = [C.c_int] * 4 + [C.c_double] * 2 + [C.c_void_p] * 2 + [C.c_int]
    for fn in ("cal_sciddicaT_reset", "cal_sciddicaT_close"):
        getattr(m, fn).argtypes = [C.c_void_p]
    m.cal_sciddicaT_steps.argtypes = [C.c_void_p, C.c_int, C.c_int]
    m.cal_sciddicaT_read.argtypes = [C.c_void_p, C.c_void_p]
    sess = m.cal_sciddicaT_open(160, 144, 0, 1, 0.5, 0.001, z.ctypes.data, h.ctypes.data, cal.MODE_PROCESSES)
    assert sess
    try:
        for loop in (0, 1, 2):
            assert m.cal_sciddicaT_reset(sess) == 0
            assert m.cal_sciddicaT_steps(sess, steps, loop) == 0
            out = np.empty_like(h)
            assert m.cal_sciddicaT_read(sess, out.ctypes.data) == 0
            assert out.tobytes() == ref[1].tobytes(), loop
    finally:
        m.cal_sciddicaT_close(sess)


def test_staged_hexagonal_integer_rule_equals_global_reads():
    """An integer rule over the hexagonal neighbourhood (both layouts), with
    and without its substate staged: the same bits, flat and toroidal."""
    from opencal_gb300 import program as P
    import opencal_gb300 as cal
    cal.build()
    body = """
        CALint s = 3 * calGet2Di(ca, Q.v, i, j);
        for (int n = 1; n < ca->sizeof_X; n++) s += n * calGetX2Di(ca, Q.v, i, j, n);
        calSet2Di(ca, Q.v, i, j, s % 1009);
    """
    lib = P.Program("pyhexint").substates(v="i").process("pyhexint_rule", body).build()
    rng = np.random.default_rng(9)
    v0 = rng.integers(0, 1009, size=(72, 96)).astype(np.int32)
    for nb in (P.CAL_HEXAGONAL_NEIGHBORHOOD_2D, P.CAL_HEXAGONAL_NEIGHBORHOOD_ALT_2D):
        for space in (P.CAL_SPACE_FLAT, P.CAL_SPACE_TOROIDAL):
            out = []
            for staged in (False, True):
                model = P.Model2D(72, 96, nb, space)
                v = model.add_substate("i")
                lib.bind(v=v)
                rule = lib.process("pyhexint_rule")
                model.add_process(rule)
                if staged:
                    model.set_reads(rule, [v])
                model.load(v, v0)
                run = P.Run2D(model, 1, 12)
                try:
                    run.run()
                    out.append(model.read(v))
                finally:
                    run.close()
                    model.close()
            assert out[0].tobytes() == out[1].tobytes(), (nb, space)


@pytest.mark.parametrize("flags", [1, 2, 3])
@pytest.mark.parametrize("shape,tor", [((96, 80), True), ((128, 256), False), ((100, 72), True)])
def test_life_program_declarations(flags, shape, tor):
    """The reference Life program (calModels.h) with its process declared
    pure (1), its reads declared (2) or both (3): the oracle's bits."""
    import oracle
    import opencal_gb300 as cal
    from opencal_gb300 import workloads as W
    cal.build()
    oracle.build()
    m = cal.models()
    s0 = W.life_state(shape[0], shape[1], p=0.3, seed=5)
    m.cal_life2d_set_declarations(flags)
    try:
        got = cal.life2d(s0, 40, toroidal=tor, mode=cal.MODE_PROCESSES)
    finally:
        m.cal_life2d_set_declarations(0)
    assert np.array_equal(got, oracle.life2d(s0, 40, toroidal=tor))
