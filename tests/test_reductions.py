"""Device reductions (cal2DReduction.h) against the oracle's fold
(oracle/cal_oracle.c, orc_reduce2d: the serial calReductionOperation2D* of
OpenCAL-OMP/source/cal2DReduction.c over every cell, pinned to the reference
itself on one-column grids in tests/test_oracle_pins.py) and against a
direct fold of the same values: exact for byte/int and for min/max, logical
and binary operations; real sums and products within 1e-12 relative (the
device folds in a fixed tree order, the oracle in index order).

Which semantics: the reference's serial build folds elements 0 .. rows-1
only (the last thread's end index is `rows`, cal2DReduction.c:45-47) and its
OpenMP build drops the last thread's share the same way; this library folds
every cell, as the oracle does."""
import operator
from functools import reduce

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

OPS = {1: "max", 2: "min", 3: "sum", 4: "prod", 5: "land", 6: "band", 7: "lor", 8: "bor", 9: "lxor", 10: "bxor"}


def fold(values, op, kind):
    """The reference's fold (cal2DReduction.c): start from element 0."""
    v = [int(x) if kind != 2 else float(x) for x in values.ravel()]
    name = OPS[op]
    if name == "max":
        return reduce(lambda a, b: b if a < b else a, v)
    if name == "min":
        return reduce(lambda a, b: b if a > b else a, v)
    if name in ("sum", "prod"):
        if kind == 2:
            return float(np.sum(values) if name == "sum" else np.prod(values))
        f = operator.add if name == "sum" else operator.mul
        bits = 8 if kind == 0 else 32
        r = reduce(lambda a, b: f(a, b) % (1 << bits), v)
        return r - (1 << bits) if r >= 1 << (bits - 1) else r
    if name == "land":
        return reduce(lambda a, b: int(bool(a) and bool(b)), v)
    if name == "lor":
        return reduce(lambda a, b: int(bool(a) or bool(b)), v)
    if name == "lxor":
        return reduce(lambda a, b: int(bool(a) != bool(b)), v)
    cast = (lambda x: int(x)) if kind == 2 else (lambda x: x)
    f = {"band": operator.and_, "bor": operator.or_, "bxor": operator.xor}[name]
    return reduce(lambda a, b: f(cast(a), cast(b)), v)


@pytest.fixture(scope="module")
def lib():
    import opencal_gb300 as cal
    import oracle
    import probes
    cal.build()
    oracle.build()
    probes.lib()
    return probes, oracle


@pytest.mark.parametrize("op", list(OPS))
@pytest.mark.parametrize("kind", [0, 1, 2])
def test_reduction(lib, kind, op):
    from opencal_gb300.workloads import uniform_array
    rows, cols = 97, 131
    u = uniform_array(100 + op + 10 * kind, (rows, cols))
    if kind == 0:
        data = np.ascontiguousarray((u * 7).astype(np.int8) + 1)  # 1..7, no zeros for the logical ops
        if op in (4,):
            data[:] = np.where(u < 0.5, 1, 3).astype(np.int8)
    elif kind == 1:
        data = np.ascontiguousarray((u * 1000 - 300).astype(np.int32))
        if op == 4:
            data[:] = np.where(u < 0.5, 1, 3).astype(np.int32)
    else:
        data = np.ascontiguousarray(u * 10.0 - 2.0)
        if op == 4:
            data[:] = 1.0 + (u - 0.5) * 1e-3
    probes, oracle = lib
    got = probes.reduce2d(kind, data, op)
    want = fold(data, op, kind)
    orc = oracle.reduce2d(kind, data, op)
    if kind == 2 and OPS[op] in ("sum", "prod"):
        assert abs(got - want) <= 1e-12 * abs(want)
        assert abs(got - orc) <= 1e-12 * abs(orc)
    elif kind == 0 and OPS[op] in ("sum", "prod"):
        # CALbyte is char: its signedness is the platform's, compare modulo 256
        assert int(got) % 256 == want % 256 == int(orc) % 256
    else:
        assert got == want == orc, (OPS[op], got, want, orc)
