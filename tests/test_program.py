"""Models defined from Python (opencal_gb300.program): elementary-process
bodies as CUDA C strings compiled at run time against the C ABI, the model,
substates and run loop (with Python init / steering / stop callbacks) driven
from Python -- this library's counterpart of the reference's SWIG binding
(OpenCAL/include/opencal.i, ElementaryProcessFunctor2D.i).

CPU: a program compiles for sm_103a and loads (its processes register with
the library) without a GPU; a body that does not compile raises with nvcc's
message; bad names and types are refused.  GPU: Life B3/S23 defined in
Python gives the oracle's bits (recorded-step replay, a Python stop
condition, a device stop condition); SCIDDICA-T defined in Python (the
reference example's processes, init and steering, OpenCAL-OMP/examples/
calomp_sciddicaT/source/sciddicaT.c) reproduces the reference's shipped
610 x 496 golden byte for byte.
"""
import hashlib
import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")

LIFE_BODY = """
    int sum = 0;
    for (int n = 1; n < ca->sizeof_X; n++)
        sum += calGetX2Db(ca, Q.alive, i, j, n);
    const CALbyte a = calGet2Db(ca, Q.alive, i, j);
    calSet2Db(ca, Q.alive, i, j, (sum == 3 || (a == 1 && sum == 2)) ? 1 : 0);
"""

# the reference example's processes (sciddicaT.c:20-101), as bodies
SDT_FLOWS = """
    CALbyte eliminated_cells[5] = {CAL_FALSE, CAL_FALSE, CAL_FALSE, CAL_FALSE, CAL_FALSE};
    CALbyte again;
    CALint cells_count;
    CALreal average, m, u[5], z, h;
    CALint n;
    if (calGet2Dr(ca, Q.h, i, j) <= P.epsilon)
        return;
    m = calGet2Dr(ca, Q.h, i, j) - P.epsilon;
    u[0] = calGet2Dr(ca, Q.z, i, j) + P.epsilon;
    for (n = 1; n < ca->sizeof_X; n++) {
        z = calGetX2Dr(ca, Q.z, i, j, n);
        h = calGetX2Dr(ca, Q.h, i, j, n);
        u[n] = z + h;
    }
    do {
        again = CAL_FALSE;
        average = m;
        cells_count = 0;
        for (n = 0; n < ca->sizeof_X; n++)
            if (!eliminated_cells[n]) {
                average += u[n];
                cells_count++;
            }
        if (cells_count != 0)
            average /= cells_count;
        for (n = 0; n < ca->sizeof_X; n++)
            if ((average <= u[n]) && (!eliminated_cells[n])) {
                eliminated_cells[n] = CAL_TRUE;
                again = CAL_TRUE;
            }
    } while (again);
    for (n = 1; n < ca->sizeof_X; n++)
        calSet2Dr(ca, outflow(n - 1), i, j, eliminated_cells[n] ? 0.0 : (average - u[n]) * P.r);
"""
SDT_WIDTH = """
    CALreal h_next = calGet2Dr(ca, Q.h, i, j);
    for (int n = 1; n < ca->sizeof_X; n++)
        h_next += calGetX2Dr(ca, outflow(4 - n), i, j, n) - calGet2Dr(ca, outflow(n - 1), i, j);
    calSet2Dr(ca, Q.h, i, j, h_next);
"""
SDT_INIT = """
    const CALreal h = calGet2Dr(ca, Q.h, i, j);
    if (h > 0.0)
        calSet2Dr(ca, Q.z, i, j, calGet2Dr(ca, Q.z, i, j) - h);
"""
SDT_HELPERS = """
static __device__ __forceinline__ struct CALSubstate2Dr* outflow(int q)
{
    return q == 0 ? Q.f0 : (q == 1 ? Q.f1 : (q == 2 ? Q.f2 : Q.f3));
}
"""


def life_program(name="pylife"):
    from opencal_gb300.program import Program
    return (Program(name).substates(alive="b").process(f"{name}_rule", LIFE_BODY)
            .stop_condition(f"{name}_stop", "return calRunGetStep2D(ca) >= 17;"))


def sciddicaT_program():
    from opencal_gb300.program import Program
    return (Program("pysdt").substates(z="r", h="r", f0="r", f1="r", f2="r", f3="r")
            .parameters(epsilon="r", r="r").device(SDT_HELPERS)
            .process("pysdt_flows", SDT_FLOWS).process("pysdt_width", SDT_WIDTH)
            .process("pysdt_init_cell", SDT_INIT))


def test_program_builds_and_registers_without_gpu():
    import opencal_gb300 as cal
    cal.build()
    prog = life_program()
    src = prog.source()
    assert "CAL_ELEMENTARY_PROCESS_2D(pylife_rule)" in src
    assert "CAL_DEVICE_STOP_CONDITION_2D(pylife_stop)" in src
    lib = prog.build()
    assert lib.process("pylife_rule")
    assert lib.stop_condition("pylife_stop")
    with pytest.raises(KeyError):
        lib.process("missing")
    # a second build of the same source is the cached library
    assert prog.build().path == lib.path
    sdt = sciddicaT_program().build()
    for p in ("pysdt_flows", "pysdt_width", "pysdt_init_cell"):
        assert sdt.process(p)


def test_program_compile_error_is_reported():
    from opencal_gb300 import CALError
    from opencal_gb300.program import Program
    bad = Program("pybroken").substates(v="r").process("pybroken_rule", "this is not C;")
    with pytest.raises(CALError, match="nvcc failed"):
        bad.build()


def test_program_refuses_bad_names_and_types():
    from opencal_gb300 import CALError
    from opencal_gb300.program import Program
    with pytest.raises(CALError):
        Program("two words")
    with pytest.raises(CALError):
        Program("ok").substates(x="f")
    with pytest.raises(CALError):
        Program("ok").parameters(y="double")
    with pytest.raises(CALError):
        Program("ok").process("1st", "")


@pytest.fixture(scope="module")
def gpu():
    import opencal_gb300 as cal
    import oracle
    cal.build()
    oracle.build()
    return cal, oracle


def _life_model(lib, s0):
    from opencal_gb300 import program as P
    model = P.Model2D(s0.shape[0], s0.shape[1], P.CAL_MOORE_NEIGHBORHOOD_2D, P.CAL_SPACE_TOROIDAL)
    alive = model.add_substate("b")
    lib.bind(alive=alive)
    model.add_process(lib.process("pylife_rule"))
    model.load(alive, s0.astype(np.int8))
    return model, alive


@pytest.mark.gpu
@pytest.mark.parametrize("graph", [False, True])
def test_life_from_python_matches_oracle(gpu, graph):
    from opencal_gb300 import program as P
    from opencal_gb300 import workloads as W
    _, oracle = gpu
    s0 = W.life_state(96, 80, seed=1)
    lib = life_program().build()
    model, alive = _life_model(lib, s0)
    run = P.Run2D(model, 1, 20, graph=graph)
    try:
        run.run()
        got = model.read(alive).astype(np.uint8)
        if graph:
            assert run.graph_replays() > 0
    finally:
        run.close()
        model.close()
    assert np.array_equal(got, oracle.life2d(s0, 20))


@pytest.mark.gpu
def test_life_from_python_stop_conditions(gpu):
    """A Python stop condition (host) and the program's device stop
    condition (one device-driven launch) end the run at the same step."""
    from opencal_gb300 import program as P
    from opencal_gb300 import workloads as W
    _, oracle = gpu
    s0 = W.life_state(64, 64, seed=3)
    lib = life_program().build()
    seen = []

    def steer(model):
        seen.append(1)

    results = []
    for host in (True, False):
        model, alive = _life_model(lib, s0)
        kw = {"stop": (lambda m: len(seen) >= 12)} if host else {"device_stop": lib.stop_condition("pylife_stop")}
        seen.clear()
        run = P.Run2D(model, 1, 100, steering=steer if host else None, **kw)
        try:
            run.run() if host else run.run_device()
            results.append((run.step, model.read(alive).astype(np.uint8)))
        finally:
            run.close()
            model.close()
    (step_h, got_h), (step_d, got_d) = results
    assert np.array_equal(got_h, oracle.life2d(s0, 12))
    assert np.array_equal(got_d, oracle.life2d(s0, step_d))
    assert step_d == 17


@pytest.mark.gpu
@pytest.mark.parametrize("declared", [False, True], ids=["as_written", "pure+guard"])
def test_sciddicaT_from_python_reproduces_shipped_golden(gpu, declared):
    """The reference's SCIDDICA-T example written in Python (processes as
    bodies, init and steering as Python callbacks) on its shipped 610 x 496
    data: 4000 steps, toroidal, the final h printed %.9f is the shipped
    golden byte for byte; also with both processes declared pure and the
    flows process's early return (h <= epsilon) declared as its guard."""
    from opencal_gb300 import program as P
    g = np.load(os.path.join(GOLDEN, "sciddicaT_610x496.npz"))
    meta = json.load(open(os.path.join(GOLDEN, "manifest.json")))["sciddicaT_610x496"]
    lib = sciddicaT_program().build()
    lib.set(epsilon=meta["p_eps"], r=meta["p_r"])
    assert lib.get("epsilon") == meta["p_eps"]
    model = P.Model2D(meta["rows"], meta["cols"], P.CAL_VON_NEUMANN_NEIGHBORHOOD_2D, P.CAL_SPACE_TOROIDAL)
    subs = {n: model.add_substate("r") for n in ("z", "h", "f0", "f1", "f2", "f3")}
    lib.bind(**subs)
    model.add_process(lib.process("pysdt_flows"))
    model.add_process(lib.process("pysdt_width"))
    if declared:
        model.set_pure(lib.process("pysdt_flows"))
        model.set_pure(lib.process("pysdt_width"))
        model.set_guard(lib.process("pysdt_flows"), subs["h"], "<=", meta["p_eps"])
        with pytest.raises(P.CALError):  # not a substate handle of the model
            model.set_guard(lib.process("pysdt_flows"), P.Substate(subs["h"].ptr + 1, "r"), "<=", 0.0)
        P.core().calClearError()
    model.load(subs["z"], g["z"])
    model.load(subs["h"], g["h0"])

    def init(m):  # sciddicaT.c:104-131
        for q in range(4):
            m.init(subs[f"f{q}"], 0.0)
        m.apply(lib.process("pysdt_init_cell"))

    def steering(m):  # sciddicaT.c:133-138
        for q in range(4):
            m.init(subs[f"f{q}"], 0.0)

    run = P.Run2D(model, 1, meta["steps"], init=init, steering=steering, graph=True)
    try:
        run.run()
        h = model.read(subs["h"])
    finally:
        run.close()
        model.close()
    text = "".join("".join("%.9f  " % v for v in row) + "\n" for row in h).encode()
    assert hashlib.sha256(text).hexdigest() == meta["plain_text_sha256"]
