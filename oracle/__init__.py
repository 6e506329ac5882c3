"""ctypes front end of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import this package: it is the checker, never the thing
measured or shipped.

Three interchangeable back ends expose the same entry points:
  * ``serial``  -- oracle/build/liboracle.so: the C restatement (the checker)
  * ``omp``     -- oracle/build/liboracle_omp.so: the same code with OpenMP
  * ``ref``     -- oracle/_ref/libref.so: the reference library itself,
                   compiled from its own sources by oracle/ref/Makefile; exists
                   only where the reference tree is present
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# the reference source tree, for the reference build that pins the oracle:
# given by the OPENCAL_REFERENCE environment variable (no default)
REF_TREE = os.environ.get("OPENCAL_REFERENCE")

_LIBS: dict[str, C.CDLL] = {}

NB_CUSTOM, NB_VN, NB_MOORE, NB_HEX, NB_HEX_ALT = 0, 1, 2, 3, 4

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_u8 = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")
_i32 = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_pl = C.POINTER(C.c_long)


def build(ref: bool = False, ref_tree: str | None = None) -> None:
    """Compile the oracle and, when asked and the reference tree is given
    (argument or OPENCAL_REFERENCE) and present, the reference build."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    tree = ref_tree or REF_TREE
    if ref and tree and os.path.isdir(os.path.join(tree, "OpenCAL-OMP", "source")):
        subprocess.run(["make", "-s", "-C", os.path.join(HERE, "ref"), f"REF={tree}"], check=True)


def ref_available() -> bool:
    return os.path.exists(os.path.join(HERE, "_ref", "libref.so"))


def _bind(lib: C.CDLL, prefix: str) -> C.CDLL:
    f = getattr(lib, prefix + "sciddicaT")
    f.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                  _dp, _dp, _dp, _dp, _pl, C.c_void_p]
    f.restype = C.c_int
    f = getattr(lib, prefix + "life2d")
    f.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _u8, _u8]
    f.restype = C.c_int
    f = getattr(lib, prefix + "nbprobe2d")
    f.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _dp, _dp]
    f.restype = C.c_int
    f = getattr(lib, prefix + "acprobe")
    f.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double,
                  _dp, _dp, _pl, C.c_void_p]
    f.restype = C.c_int
    f = getattr(lib, prefix + "life3d")
    f.argtypes = [C.c_int] * 10 + [_u8, _u8]
    f.restype = C.c_int
    f = getattr(lib, prefix + "nbprobe2d_custom")
    f.argtypes = [C.c_int] * 5 + [C.c_void_p, _dp, _dp]
    f.restype = C.c_int
    f = getattr(lib, prefix + "reduce2d")
    f.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_int, C.POINTER(C.c_double)]
    f.restype = C.c_int
    return lib


def lib(kind: str = "serial") -> C.CDLL:
    if kind not in _LIBS:
        if kind == "ref":
            path = os.path.join(HERE, "_ref", "libref.so")
        else:
            path = os.path.join(HERE, "build", "liboracle.so" if kind == "serial" else "liboracle_omp.so")
        if not os.path.exists(path):
            build(ref=(kind == "ref"))
        _LIBS[kind] = _bind(C.CDLL(path), "ref_" if kind == "ref" else "orc_")
    return _LIBS[kind]


def _fn(kind: str, name: str):
    return getattr(lib(kind), ("ref_" if kind == "ref" else "orc_") + name)


def sciddicaT(z0, h0, steps, *, toroidal=False, ac=False, p_r=0.5, p_eps=0.001, kind="serial",
              want_cells=True):
    """Run SCIDDICA-T; returns (z, h, cells) with cells an (n, 2) int32 array of (i, j)."""
    z0 = np.ascontiguousarray(z0, dtype=np.float64)
    h0 = np.ascontiguousarray(h0, dtype=np.float64)
    rows, cols = z0.shape
    z = np.empty_like(z0)
    h = np.empty_like(h0)
    n = C.c_long(0)
    cells = np.zeros((rows * cols if (ac and want_cells) else 1, 2), dtype=np.int32)
    rc = _fn(kind, "sciddicaT")(rows, cols, int(toroidal), int(ac), int(steps), p_r, p_eps,
                                z0, h0, z, h, C.byref(n),
                                cells.ctypes.data if (ac and want_cells) else None)
    if rc:
        raise RuntimeError(f"oracle sciddicaT failed ({rc})")
    return z, h, (cells[: n.value].copy() if (ac and want_cells) else np.zeros((0, 2), np.int32))


def sciddicaT_trace(z0, h0, steps, *, p_r=0.5, p_eps=0.001, kind="serial"):
    """Plain SCIDDICA-T on a flat grid with its boundary trace: returns
    (z, h, outflux, edge_step): outflux[s - 1] is the mass that left the grid
    in step s (outflows of border cells towards absent neighbours), edge_step
    the first step after which a cell of the two-cell edge band is wet (-1:
    never).  Serial or OpenMP build only."""
    z0 = np.ascontiguousarray(z0, dtype=np.float64)
    h0 = np.ascontiguousarray(h0, dtype=np.float64)
    rows, cols = z0.shape
    z, h = np.empty_like(z0), np.empty_like(h0)
    out = np.zeros(max(int(steps), 1))
    edge = C.c_int(-1)
    f = _fn(kind, "sciddicaT_trace")
    f.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double] + [C.c_void_p] * 5 + [C.POINTER(C.c_int)]
    f.restype = C.c_int
    if f(rows, cols, int(steps), p_r, p_eps, z0.ctypes.data, h0.ctypes.data, z.ctypes.data, h.ctypes.data,
         out.ctypes.data, C.byref(edge)):
        raise RuntimeError("oracle sciddicaT_trace failed")
    return z, h, out[: int(steps)], edge.value


_KINDS = {np.dtype(np.int8): 0, np.dtype(np.uint8): 0, np.dtype(np.int32): 1, np.dtype(np.float64): 2}


def save_text(data, path, *, kind="serial"):
    """A 2D (rows, cols) or 3D (slices, rows, cols) array of int8/uint8,
    int32 or float64 written in the reference's substate text format."""
    data = np.ascontiguousarray(data)
    dim = data.ndim
    slices, rows, cols = (1,) + data.shape if dim == 2 else data.shape
    f = _fn(kind, "save_text")
    f.argtypes = [C.c_int] * 5 + [C.c_void_p, C.c_char_p]
    if f(dim, _KINDS[data.dtype], rows, cols, slices, data.ctypes.data, str(path).encode()):
        raise RuntimeError("save_text failed")


def load_text(shape, dtype, path, *, kind="serial"):
    """The reference's substate text format read into an array of `shape`
    ((rows, cols) or (slices, rows, cols)) and `dtype`."""
    out = np.zeros(shape, dtype=dtype)
    dim = len(shape)
    slices, rows, cols = (1,) + tuple(shape) if dim == 2 else tuple(shape)
    f = _fn(kind, "load_text")
    f.argtypes = [C.c_int] * 5 + [C.c_void_p, C.c_char_p]
    if f(dim, _KINDS[np.dtype(dtype)], rows, cols, slices, out.ctypes.data, str(path).encode()):
        raise RuntimeError("load_text failed")
    return out


def life2d(s0, steps, *, toroidal=True, as_int=False, kind="serial"):
    s0 = np.ascontiguousarray(s0, dtype=np.uint8)
    out = np.empty_like(s0)
    rows, cols = s0.shape
    if _fn(kind, "life2d")(rows, cols, int(toroidal), int(as_int), int(steps), s0, out):
        raise RuntimeError("oracle life2d failed")
    return out


def nbprobe2d(v0, steps, *, nbhd=NB_HEX, toroidal=True, kind="serial"):
    v0 = np.ascontiguousarray(v0, dtype=np.float64)
    out = np.empty_like(v0)
    rows, cols = v0.shape
    if _fn(kind, "nbprobe2d")(rows, cols, int(nbhd), int(toroidal), int(steps), v0, out):
        raise RuntimeError("oracle nbprobe2d failed")
    return out


def nbprobe2d_custom(v0, steps, offsets, *, toroidal=True, kind="serial"):
    """The probe rule on a custom neighbourhood: `offsets` (di, dj) appended
    in order, as calAddNeighbor2D does."""
    v0 = np.ascontiguousarray(v0, dtype=np.float64)
    offs = np.ascontiguousarray(np.asarray(offsets, dtype=np.int32).reshape(-1))
    out = np.empty_like(v0)
    rows, cols = v0.shape
    if _fn(kind, "nbprobe2d_custom")(rows, cols, int(toroidal), int(steps), len(offs) // 2, offs.ctypes.data, v0,
                                     out):
        raise RuntimeError("oracle nbprobe2d_custom failed")
    return out


def reduce2d(kind_of_data: int, data, op: int, *, kind="serial") -> float:
    """calReductionOperation2D{b,i,r} over `data` (kind_of_data: 0 byte, 1
    int, 2 real; op: the REDUCTION_OPERATION value).  The serial oracle folds
    every cell; the reference build folds elements 0 .. rows-1 only."""
    data = np.ascontiguousarray(data)
    rows, cols = data.shape
    out = C.c_double(0.0)
    if _fn(kind, "reduce2d")(int(kind_of_data), rows, cols, data.ctypes.data, int(op), C.byref(out)):
        raise RuntimeError("oracle reduce2d failed")
    return out.value


def acprobe(v0, steps, *, nbhd=NB_MOORE, toroidal=True, thr=0.5, kind="serial"):
    """2D: v0 shape (rows, cols); 3D: v0 shape (slices, rows, cols).  Returns (v, cells)."""
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
    if _fn(kind, "acprobe")(dim, rows, cols, slices, int(nbhd), int(toroidal), int(steps), thr,
                            v0, out, C.byref(n), cells.ctypes.data):
        raise RuntimeError("oracle acprobe failed (active-cell count mismatch)")
    return out, cells[: n.value].copy()


def life3d(s0, steps, *, nbhd=NB_MOORE - 0, toroidal=True, rule=(5, 7, 6, 6), kind="serial"):
    """s0 shape (slices, rows, cols) uint8 in OpenCAL's slice-major layout."""
    s0 = np.ascontiguousarray(s0, dtype=np.uint8)
    slices, rows, cols = s0.shape
    out = np.empty_like(s0)
    # 3D neighbourhood enum: 1 = von Neumann, 2 = Moore (OpenCAL-OMP/include/cal3D.h)
    if _fn(kind, "life3d")(rows, cols, slices, int(nbhd), int(toroidal), int(steps), *rule, s0, out):
        raise RuntimeError("oracle life3d failed")
    return out


def sciara(z0, vents, rates, emission_time, steps, *, ac=False, params=None, slt0=None, st0=None,
           kind="serial", want_cells=True):
    """Run SCIARA-fv2 (oracle_sciara.c).  vents: [(x, y)], rates: [nvents][nphases]
    m^3/s, emission_time: seconds per phase, steps: maximum steps (0 = until
    the emission ends).  Returns dict(z, slt, st, msl, steps, cells)."""
    from opencal_gb300.workloads import SCIARA_PARAMS
    z0 = np.ascontiguousarray(z0, dtype=np.float64)
    rows, cols = z0.shape
    p = np.ascontiguousarray(params if params is not None else SCIARA_PARAMS, dtype=np.float64)
    v = np.ascontiguousarray(np.asarray(vents, dtype=np.int32).reshape(-1))
    r = np.ascontiguousarray(np.asarray(rates, dtype=np.float64).reshape(-1))
    nphases = len(rates[0]) if len(rates) else 0
    outs = {k: np.empty_like(z0) for k in ("z", "slt", "st", "msl")}
    done = C.c_int(0)
    n = C.c_long(0)
    cells = np.zeros((rows * cols if (ac and want_cells) else 1, 2), dtype=np.int32)
    f = _fn(kind, "sciara")
    f.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_uint, C.c_int, C.c_void_p,
                  C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                  C.POINTER(C.c_int), C.POINTER(C.c_long), C.c_void_p]
    slt0 = None if slt0 is None else np.ascontiguousarray(slt0, dtype=np.float64)
    st0 = None if st0 is None else np.ascontiguousarray(st0, dtype=np.float64)
    rc = f(rows, cols, int(ac), int(steps), p.ctypes.data, len(vents), v.ctypes.data, int(emission_time), nphases,
           r.ctypes.data, z0.ctypes.data, None if slt0 is None else slt0.ctypes.data,
           None if st0 is None else st0.ctypes.data, outs["z"].ctypes.data, outs["slt"].ctypes.data,
           outs["st"].ctypes.data, outs["msl"].ctypes.data, C.byref(done), C.byref(n),
           cells.ctypes.data if (ac and want_cells) else None)
    if rc:
        raise RuntimeError(f"oracle sciara failed ({rc})")
    outs["steps"] = done.value
    outs["cells"] = cells[: n.value].copy() if (ac and want_cells) else np.zeros((0, 2), np.int32)
    return outs


MBUSU_SHAPE = (130, 160, 30)  # slices, rows, cols
MBUSU_FIELDS = ("teta", "moist_cont", "psi", "k", "h", "dqdh", "convergence", "moist_diff")


def mbusu(steps, *, kind="serial"):
    """Run the mbusu subsurface-flow program (oracle_mbusu.c) for `steps`
    steps (0: until its stop condition at 10 days).  Returns a dict of the
    eight substates, each (slices, rows, cols), plus steps, delta_t and
    delta_t_cum."""
    n = MBUSU_SHAPE[0] * MBUSU_SHAPE[1] * MBUSU_SHAPE[2]
    state = np.empty(8 * n)
    tail = np.zeros(3)
    f = _fn(kind, "mbusu")
    f.argtypes = [C.c_int, C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    if f(int(steps), state.ctypes.data, tail.ctypes.data):
        raise RuntimeError("oracle mbusu failed")
    out = {name: state[q * n:(q + 1) * n].reshape(MBUSU_SHAPE).copy() for q, name in enumerate(MBUSU_FIELDS)}
    out["steps"], out["delta_t"], out["delta_t_cum"] = int(tail[0]), float(tail[1]), float(tail[2])
    return out


def unsafe2d(v0, b0, w0, steps, *, nbhd=NB_MOORE, toroidal=True, kind="serial"):
    """The unsafe-operation probe (oracle_models.c): returns v, b, w, u, x."""
    v0 = np.ascontiguousarray(v0, dtype=np.int32)
    b0 = np.ascontiguousarray(b0, dtype=np.int8)
    w0 = np.ascontiguousarray(w0, dtype=np.float64)
    rows, cols = v0.shape
    v, b, w = np.empty_like(v0), np.empty_like(b0), np.empty_like(w0)
    u, x = np.empty_like(w0), np.empty_like(w0)
    f = _fn(kind, "unsafe2d")
    f.argtypes = [C.c_int] * 5 + [C.c_void_p] * 8
    if f(rows, cols, int(nbhd), int(toroidal), int(steps), v0.ctypes.data, b0.ctypes.data, w0.ctypes.data,
         v.ctypes.data, b.ctypes.data, w.ctypes.data, u.ctypes.data, x.ctypes.data):
        raise RuntimeError("oracle unsafe2d failed")
    return v, b, w, u, x


def sciddicaT_unsafe(z0, h0, steps, *, toroidal=True, p_r=0.5, p_eps=0.001, kind="serial"):
    """SCIDDICA-T in the reference's unsafe form; returns (z, h)."""
    z0 = np.ascontiguousarray(z0, dtype=np.float64)
    h0 = np.ascontiguousarray(h0, dtype=np.float64)
    rows, cols = z0.shape
    z, h = np.empty_like(z0), np.empty_like(h0)
    f = _fn(kind, "sciddicaT_unsafe")
    f.argtypes = [C.c_int] * 4 + [C.c_double, C.c_double] + [C.c_void_p] * 4
    if f(rows, cols, int(toroidal), int(steps), p_r, p_eps, z0.ctypes.data, h0.ctypes.data, z.ctypes.data,
         h.ctypes.data):
        raise RuntimeError("oracle sciddicaT_unsafe failed")
    return z, h
