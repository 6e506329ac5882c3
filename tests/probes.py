"""ctypes front end of the test-only probe library (tests/native/probes.cu).

TEST INFRASTRUCTURE: the probe rules exercise the engine's semantics through
the public C API; each function has the contract of the oracle's function of
the same name (oracle/__init__.py).
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
if os.path.dirname(HERE) not in sys.path:
    sys.path.insert(0, os.path.dirname(HERE))

NB_CUSTOM, NB_VN, NB_MOORE, NB_HEX, NB_HEX_ALT = 0, 1, 2, 3, 4

_lib = None
_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_pl = C.POINTER(C.c_long)


def lib() -> C.CDLL:
    """Builds (when stale) and loads libopencal_probes.so after the product library."""
    global _lib
    if _lib is None:
        import opencal_gb300 as cal
        sys.path.insert(0, os.path.join(HERE, "native"))
        try:
            import build as native_build
        finally:
            sys.path.pop(0)
        cal.core()
        m = C.CDLL(native_build.build())
        m.cal_nbprobe2d_run.argtypes = [C.c_int] * 5 + [_dp, _dp, C.c_int]
        m.cal_nbprobe2d_custom_run.argtypes = [C.c_int] * 5 + [C.c_void_p, _dp, _dp, C.c_int]
        m.cal_acprobe_run.argtypes = [C.c_int] * 7 + [C.c_double, _dp, _dp, _pl, C.c_void_p, C.c_int]
        for f in ("cal_nbprobe2d_run", "cal_nbprobe2d_custom_run", "cal_acprobe_run"):
            getattr(m, f).restype = C.c_int
        _lib = m
    return _lib


def _check(rc: int, what: str) -> None:
    if rc != 0:
        import opencal_gb300 as cal
        msg = cal.core().calGetErrorString()
        raise cal.CALError(f"{what} failed (CALError {rc}): {msg.decode() if msg else ''}")


def nbprobe2d(v0, steps, *, nbhd=NB_HEX, toroidal=True, graph=False):
    v0 = np.ascontiguousarray(v0, dtype=np.float64)
    rows, cols = v0.shape
    out = np.empty_like(v0)
    _check(lib().cal_nbprobe2d_run(rows, cols, int(nbhd), int(toroidal), int(steps), v0, out, int(graph)),
           "cal_nbprobe2d_run")
    return out


def nbprobe2d_custom(v0, steps, offsets, *, toroidal=True, graph=False):
    """The probe rule on a neighbourhood built with calAddNeighbor2D from
    `offsets`, a sequence of (di, dj) in index order."""
    v0 = np.ascontiguousarray(v0, dtype=np.float64)
    rows, cols = v0.shape
    offs = np.ascontiguousarray(np.asarray(offsets, dtype=np.int32).reshape(-1))
    out = np.empty_like(v0)
    _check(lib().cal_nbprobe2d_custom_run(rows, cols, int(toroidal), int(steps), len(offs) // 2, offs.ctypes.data,
                                          v0, out, int(graph)), "cal_nbprobe2d_custom_run")
    return out


def acprobe(v0, steps, *, nbhd=NB_MOORE, toroidal=True, thr=0.5, graph=False):
    v0 = np.ascontiguousarray(v0, dtype=np.float64)
    dim = v0.ndim
    if dim == 2:
        rows, cols = v0.shape
        slices = 1
    else:
        slices, rows, cols = v0.shape
    out = np.empty_like(v0)
    n = C.c_long(0)
    cells = np.zeros((v0.size, dim), dtype=np.int32)
    _check(lib().cal_acprobe_run(dim, rows, cols, slices, int(nbhd), int(toroidal), int(steps), thr, v0, out,
                                 C.byref(n), cells.ctypes.data, int(graph)), "cal_acprobe_run")
    return out, cells[: n.value].copy()


def unsafe2d(v0, b0, w0, steps, *, nbhd=NB_MOORE, toroidal=True, graph=False):
    """The unsafe-operation probe on the GPU; same contract as oracle.unsafe2d."""
    v0 = np.ascontiguousarray(v0, dtype=np.int32)
    b0 = np.ascontiguousarray(b0, dtype=np.int8)
    w0 = np.ascontiguousarray(w0, dtype=np.float64)
    rows, cols = v0.shape
    v, b, w = np.empty_like(v0), np.empty_like(b0), np.empty_like(w0)
    u, x = np.empty_like(w0), np.empty_like(w0)
    f = lib().cal_unsafe2d_run
    f.restype = C.c_int
    f.argtypes = [C.c_int] * 5 + [C.c_void_p] * 8 + [C.c_int]
    _check(f(rows, cols, int(nbhd), int(toroidal), int(steps), v0.ctypes.data, b0.ctypes.data, w0.ctypes.data,
             v.ctypes.data, b.ctypes.data, w.ctypes.data, u.ctypes.data, x.ctypes.data, int(bool(graph))),
           "cal_unsafe2d_run")
    return v, b, w, u, x


def reduce2d(kind: int, data, op: int) -> float:
    """A device reduction (cal2DReduction.h) of `data` (type by `kind`:
    0 byte, 1 int, 2 real) into a double."""
    f = lib().cal_reduce2d_run
    f.restype = C.c_int
    f.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_int, C.POINTER(C.c_double)]
    rows, cols = data.shape
    out = C.c_double(0.0)
    _check(f(kind, rows, cols, data.ctypes.data, op, C.byref(out)), "cal_reduce2d_run")
    return out.value


def exact_div_mismatches(x, c, y) -> int:
    f = lib().cal_test_exact_div
    f.restype = C.c_long
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_longlong]
    return f(x.ctypes.data, c.ctypes.data, y.ctypes.data, len(x))


def io_roundtrip(data, in_path, out_path):
    """calLoadSubstate* from in_path into a GPU model, an update, then
    calSaveSubstate* to out_path; returns the model's current layer."""
    data = np.ascontiguousarray(data)
    dim = data.ndim
    slices, rows, cols = (1,) + data.shape if dim == 2 else data.shape
    kind = {1: 0, 4: 1, 8: 2}[data.dtype.itemsize]
    out = np.zeros_like(data)
    f = lib().cal_io_roundtrip
    f.restype = C.c_int
    f.argtypes = [C.c_int] * 5 + [C.c_char_p, C.c_char_p, C.c_void_p]
    _check(f(dim, kind, rows, cols, slices, str(in_path).encode(), str(out_path).encode(), out.ctypes.data),
           "cal_io_roundtrip")
    return out
