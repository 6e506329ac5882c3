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
CAL_ERROR_INVALID_ARGUMENT, CAL_ERROR_LIMIT = 1, 5


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


def _no_alloc_list(L, ca, rows, cols, stream=None, flag_offset=0):
    """The no-allocation entry point on the model's flags (copied to an
    address `flag_offset` bytes past an allocation when that is non-zero),
    on the model's stream or on a caller's torch stream."""
    import torch
    flags = C.c_void_p()
    L.calGetDeviceActiveCells2D(ca, C.byref(flags), None, None)
    L.calFinish2D(ca)
    flag_ptr = flags.value
    if flag_offset:
        shifted = torch.zeros(rows * cols + flag_offset, dtype=torch.uint8, device="cuda")
        src = torch.as_tensor(_DeviceArray(flags.value, (rows * cols,), "|u1"), device="cuda")
        shifted[flag_offset:].copy_(src)
        flag_ptr = shifted.data_ptr() + flag_offset
    cells = torch.full((rows * cols, 2), -1, dtype=torch.int32, device="cuda")
    linear = torch.full((rows * cols,), -1, dtype=torch.int32, device="cuda")
    count = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    st = stream.cuda_stream if stream is not None else L.calGetStream2D(ca)
    rc = L.calCompactActiveCellsNoAlloc2D(flag_ptr, rows, cols, cells.data_ptr(), linear.data_ptr(),
                                          count.data_ptr(), st)
    assert rc == 0
    if stream is not None:
        stream.synchronize()
    L.calFinish2D(ca)
    n = int(count.cpu()[0])
    got = cells[:n].cpu().numpy()
    lin = linear[:n].cpu().numpy()
    assert np.array_equal(lin, got[:, 0] * cols + got[:, 1])
    if n < rows * cols:
        # nothing written past the list
        assert (cells[n:].cpu().numpy() == -1).all() and (linear[n:].cpu().numpy() == -1).all()
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


def test_no_alloc_empty_set_caller_stream_and_unaligned_flags(lib):
    """An empty flag set gives count 0 and writes nothing; the call runs on a
    stream the caller created; flags at an odd address give the same list."""
    import torch
    L = lib
    rows, cols = 301, 255
    ca = L.calCADef2D(rows, cols, CAL_MOORE, CAL_TOROIDAL, CAL_OPT_ACTIVE_CELLS)
    assert ca
    try:
        assert len(_reference_list(L, ca)) == 0
        assert len(_no_alloc_list(L, ca, rows, cols)) == 0
        for i, j in _random_cells(rows, cols, 0.07, 8):
            L.calAddActiveCell2D(ca, int(i), int(j))
        ref = _reference_list(L, ca)
        assert len(ref) > 0
        stream = torch.cuda.Stream()
        assert np.array_equal(_no_alloc_list(L, ca, rows, cols, stream=stream), ref)
        for off in (1, 3, 8):
            assert np.array_equal(_no_alloc_list(L, ca, rows, cols, flag_offset=off), ref)
    finally:
        L.calFinalize2D(ca)


def test_no_alloc_rejects_misaligned_outputs(lib):
    """cells, linear and count must be 4-byte aligned: an offset pointer is
    refused with CAL_ERROR_INVALID_ARGUMENT before anything is launched."""
    import torch
    L = lib
    rows, cols = 64, 64
    ca = L.calCADef2D(rows, cols, CAL_MOORE, CAL_TOROIDAL, CAL_OPT_ACTIVE_CELLS)
    try:
        flags = C.c_void_p()
        L.calGetDeviceActiveCells2D(ca, C.byref(flags), None, None)
        buf = torch.zeros(4 * rows * cols + 64, dtype=torch.int32, device="cuda")
        base = buf.data_ptr()
        cells, linear, count = base, base + 8 * rows * cols, base + 12 * rows * cols
        for bad in ((cells + 2, linear, count), (cells, linear + 1, count), (cells, linear, count + 3)):
            rc = L.calCompactActiveCellsNoAlloc2D(flags, rows, cols, bad[0], bad[1], bad[2], None)
            assert rc == CAL_ERROR_INVALID_ARGUMENT
        torch.cuda.synchronize()
        assert int(buf.abs().sum().item()) == 0  # nothing was written
    finally:
        L.calFinalize2D(ca)
