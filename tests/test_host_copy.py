"""calCopySubstateFromHost* / calCopySubstateToHost* (2D and 3D, byte, int,
real): a caller's array becomes both layers of a substate on the device and
comes back bit for bit -- through the direct copy, through the host
accessors (which refresh the mirror from the device), and after an update of
the substate (next -> current, so the next layer holds the array too)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

VN_2D, VN_3D, FLAT, NO_OPT = 1, 1, 0, 0


@pytest.fixture(scope="module")
def lib():
    import opencal_gb300 as cal
    cal.build()
    L = cal.core()
    for name in ("calCADef2D", "calCADef3D", "calAddSubstate2Db", "calAddSubstate2Di", "calAddSubstate2Dr",
                 "calAddSubstate3Db", "calAddSubstate3Di", "calAddSubstate3Dr"):
        getattr(L, name).restype = C.c_void_p
    L.calCADef2D.argtypes = [C.c_int] * 5
    L.calCADef3D.argtypes = [C.c_int] * 6
    for d in ("2D", "3D"):
        for t in "bir":
            getattr(L, f"calAddSubstate{d}{t}").argtypes = [C.c_void_p]
            getattr(L, f"calCopySubstateFromHost{d}{t}").argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
            getattr(L, f"calCopySubstateToHost{d}{t}").argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
            getattr(L, f"calUpdateSubstate{d}{t}").argtypes = [C.c_void_p, C.c_void_p]
        getattr(L, f"calFinalize{d}").argtypes = [C.c_void_p]
    L.calGet2Dr.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int]
    L.calGet2Dr.restype = C.c_double
    L.calGet3Di.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int]
    L.calGet3Di.restype = C.c_int
    return L


TYPES = {"b": np.int8, "i": np.int32, "r": np.float64}


def _data(shape, t, seed):
    rng = np.random.default_rng(seed)
    if t == "r":
        return rng.standard_normal(shape)
    info = np.iinfo(TYPES[t])
    return rng.integers(0, info.max, size=shape, dtype=TYPES[t])


@pytest.mark.parametrize("dim", ["2D", "3D"])
def test_copy_round_trip(lib, dim):
    shape = (45, 37) if dim == "2D" else (11, 23, 17)  # (rows, cols) or (slices, rows, cols)
    if dim == "2D":
        m = lib.calCADef2D(shape[0], shape[1], VN_2D, FLAT, NO_OPT)
    else:
        m = lib.calCADef3D(shape[1], shape[2], shape[0], VN_3D, FLAT, NO_OPT)
    assert m
    try:
        for k, t in enumerate("bir"):
            q = getattr(lib, f"calAddSubstate{dim}{t}")(m)
            x = np.ascontiguousarray(_data(shape, t, 7 + k))
            getattr(lib, f"calCopySubstateFromHost{dim}{t}")(m, q, x.ctypes.data)
            y = np.zeros_like(x)
            getattr(lib, f"calCopySubstateToHost{dim}{t}")(m, q, y.ctypes.data)
            assert x.tobytes() == y.tobytes(), t
            getattr(lib, f"calUpdateSubstate{dim}{t}")(m, q)  # next -> current: next holds x too
            y[...] = 0
            getattr(lib, f"calCopySubstateToHost{dim}{t}")(m, q, y.ctypes.data)
            assert x.tobytes() == y.tobytes(), t
            if dim == "2D" and t == "r":
                assert lib.calGet2Dr(m, q, 13, 29) == x[13, 29]
            if dim == "3D" and t == "i":
                assert lib.calGet3Di(m, q, 5, 11, 9) == x[9, 5, 11]
        assert lib.calGetLastError() == 0
    finally:
        getattr(lib, f"calFinalize{dim}")(m)
