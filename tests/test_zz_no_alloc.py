"""calCompactActiveCellsNoAlloc2D: the active-cell compaction for callers
that cannot allocate device memory (for example a host whose device memory
is all owned by its own allocator, or a loop that must not call
cudaMalloc/cudaFree because they can synchronise the device).  It must give
exactly what calUpdateActiveCells2D gives, on consecutive calls that share
its fixed scratch array.  This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CAL_MOORE, CAL_TOROIDAL, CAL_OPT_ACTIVE_CELLS = 2, 1, 1
CAL_ERROR_LIMIT = 5


class CALActiveCells2D(C.Structure):
    _fields_ = [("flags", C.c_void_p), ("size_next", C.c_void_p), ("cells", C.POINTER(C.c_int)),
                ("size_current", C.c_int), ("num_threads", C.c_int)]


class CALModel2D(C.Structure):
    """Leading fields of struct CALModel2D (include/opencal/cal2D.h)."""
    _fields_ = [("rows", C.c_int), ("columns", C.c_int), ("T", C.c_int), ("is_safe", C.c_int),
                ("OPTIMIZATION", C.c_int), ("A", CALActiveCells2D)]


class _DeviceArray:
    def __init__(self, ptr, shape, typestr):
        self.__cuda_array_interface__ = {"shape": shape, "typestr": typestr, "data": (ptr, False), "version": 2}


@pytest.fixture(scope="module")
def lib():
    import opencal_gb300 as cal
    cal.build()
    L = cal.core()
    L.calCADef2D.restype = C.POINTER(CALModel2D)
    L.calCADef2D.argtypes = [C.c_int] * 5
    for fn in ("calUpdateActiveCells2D", "calSync2D", "calFinalize2D", "calFinish2D"):
        getattr(L, fn).argtypes = [C.POINTER(CALModel2D)]
    L.calAddActiveCell2D.argtypes = [C.POINTER(CALModel2D), C.c_int, C.c_int]
    L.calRemoveActiveCell2D.argtypes = [C.POINTER(CALModel2D), C.c_int, C.c_int]
    L.calGetStream2D.argtypes = [C.POINTER(CALModel2D)]
    L.calGetStream2D.restype = C.c_void_p
    L.calGetDeviceActiveCells2D.argtypes = [C.POINTER(CALModel2D), C.POINTER(C.c_void_p), C.POINTER(C.c_void_p),
                                            C.POINTER(C.c_void_p)]
    L.calCompactActiveCellsNoAlloc2D.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                                 C.c_void_p]
    L.calCompactActiveCellsNoAlloc2D.restype = C.c_int
    return L


def _reference_list(L, ca):
    """The existing entry point: calUpdateActiveCells2D, read back with calSync2D."""
    L.calUpdateActiveCells2D(ca)
    L.calSync2D(ca)
    n = ca.contents.A.size_current
    if n == 0:
        return np.zeros((0, 2), np.int32)
    return np.ctypeslib.as_array(ca.contents.A.cells, shape=(n * 2,)).reshape(n, 2).copy()


def _no_alloc_list(L, ca, rows, cols):
    import torch
    flags = C.c_void_p()
    L.calGetDeviceActiveCells2D(ca, C.byref(flags), None, None)
    cells = torch.full((rows * cols, 2), -1, dtype=torch.int32, device="cuda")
    linear = torch.full((rows * cols,), -1, dtype=torch.int32, device="cuda")
    count = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    rc = L.calCompactActiveCellsNoAlloc2D(flags, rows, cols, cells.data_ptr(), linear.data_ptr(), count.data_ptr(),
                                          L.calGetStream2D(ca))
    assert rc == 0
    L.calFinish2D(ca)
    n = int(count.cpu()[0])
    got = cells[:n].cpu().numpy()
    lin = linear[:n].cpu().numpy()
    assert np.array_equal(lin, got[:, 0] * cols + got[:, 1])
    return got


def _random_cells(rows, cols, frac, seed):
    from opencal_gb300.workloads import uniform_array
    return np.argwhere(uniform_array(seed, (rows, cols)) < frac)


@pytest.mark.parametrize("rows,cols", [(517, 389), (1024, 768)])
def test_no_alloc_matches_update_active_cells_on_consecutive_calls(lib, rows, cols):
    L = lib
    ca = L.calCADef2D(rows, cols, CAL_MOORE, CAL_TOROIDAL, CAL_OPT_ACTIVE_CELLS)
    assert ca
    try:
        for i, j in _random_cells(rows, cols, 0.2, 5):
            L.calAddActiveCell2D(ca, int(i), int(j))
        ref1 = _reference_list(L, ca)
        got1 = _no_alloc_list(L, ca, rows, cols)
        assert len(ref1) > 0 and np.array_equal(got1, ref1)

        # second call in a row, on a different pattern: the scratch array keeps
        # the previous call's contents, which must not leak into the result
        for i, j in _random_cells(rows, cols, 0.5, 6):
            L.calRemoveActiveCell2D(ca, int(i), int(j))
        for i, j in _random_cells(rows, cols, 0.01, 7):
            L.calAddActiveCell2D(ca, int(i), int(j))
        ref2 = _reference_list(L, ca)
        got2 = _no_alloc_list(L, ca, rows, cols)
        assert np.array_equal(got2, ref2) and not np.array_equal(ref1, ref2)
    finally:
        L.calFinalize2D(ca)


def test_no_alloc_rejects_grids_beyond_its_limit(lib):
    L = lib
    ca = L.calCADef2D(64, 64, CAL_MOORE, CAL_TOROIDAL, CAL_OPT_ACTIVE_CELLS)
    try:
        flags = C.c_void_p()
        cells = C.c_void_p()
        count = C.c_void_p()
        L.calGetDeviceActiveCells2D(ca, C.byref(flags), C.byref(cells), C.byref(count))
        rc = L.calCompactActiveCellsNoAlloc2D(flags, 20000, 20000, cells, cells, count, None)
        assert rc == CAL_ERROR_LIMIT
    finally:
        L.calFinalize2D(ca)
