"""opencal-gb300: OpenCAL's cellular-automaton global transition on GB300.

The product is the C-ABI library ``lib/libopencal_gb300.so`` (headers in
``include/opencal``): OpenCAL's C API with the work on the GPU.  This module
is a thin ctypes front end used by the tests and the benchmark; it calls the
model drivers in ``lib/libopencal_models.so``, which are ordinary C-API
programs (device elementary processes registered with
``calAddElementaryProcess2D``, or the fused kernels).

There is no CPU fallback: if the CUDA libraries are missing or no GPU is
present every call raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_DIR = os.path.join(PKG, "lib")
CORE_LIB = os.path.join(LIB_DIR, "libopencal_gb300.so")
MODELS_LIB = os.path.join(LIB_DIR, "libopencal_models.so")

NB_CUSTOM, NB_VN, NB_MOORE, NB_HEX, NB_HEX_ALT = 0, 1, 2, 3, 4
MODE_PROCESSES, MODE_FUSED, MODE_FUSED_BLOCKED = 0, 1, 2
MODE_BITS = 3  # Life only: bit-sliced fused launches (32 cells per word)

_core = None
_models = None

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_u8 = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")
_pl = C.POINTER(C.c_long)
_pd = C.POINTER(C.c_double)


class CALError(RuntimeError):
    pass


def build(force: bool = False) -> None:
    """Compile the CUDA libraries in-tree (opencal_gb300/nvbuild.py)."""
    import importlib
    importlib.import_module(__name__ + ".nvbuild").build(force=force)


def core() -> C.CDLL:
    """The C-ABI library (loaded once, RTLD_GLOBAL so the models resolve to it)."""
    global _core
    if _core is None:
        if not os.path.exists(CORE_LIB):
            raise CALError(f"{CORE_LIB} is missing: build it with `python -m opencal_gb300.nvbuild`")
        _core = C.CDLL(CORE_LIB, mode=C.RTLD_GLOBAL)
        _core.calGetErrorString.restype = C.c_char_p
        _core.calGetLastError.restype = C.c_int
    return _core


def models() -> C.CDLL:
    global _models
    if _models is None:
        core()
        if not os.path.exists(MODELS_LIB):
            raise CALError(f"{MODELS_LIB} is missing: build it with `python -m opencal_gb300.nvbuild`")
        m = C.CDLL(MODELS_LIB)
        m.cal_sciddicaT_run.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                                        _dp, _dp, _dp, _dp, _pl, C.c_void_p, C.c_int, C.c_int, _pd]
        m.cal_life2d_run.argtypes = [C.c_int] * 5 + [_u8, _u8, C.c_int, C.c_int, C.c_int, _pd]
        m.cal_life3d_run.argtypes = [C.c_int] * 10 + [_u8, _u8, C.c_int]
        for f in ("cal_sciddicaT_run", "cal_life2d_run", "cal_life3d_run"):
            getattr(m, f).restype = C.c_int
        _models = m
    return _models


def __getattr__(name):
    # opencal_gb300.adjoint imports torch: load it on first use only
    if name == "adjoint":
        import importlib
        return importlib.import_module(__name__ + ".adjoint")
    raise AttributeError(name)


def _check(rc: int, what: str) -> None:
    if rc != 0:
        msg = core().calGetErrorString()
        raise CALError(f"{what} failed (CALError {rc}): {msg.decode() if msg else ''}")


def sciddicaT(z0, h0, steps, *, toroidal=False, ac=False, p_r=0.5, p_eps=0.001, mode=MODE_FUSED, graph=False,
              timing=False):
    """SCIDDICA-T on the GPU.  Returns (z, h, cells) like oracle.sciddicaT,
    plus the device milliseconds of the step loop when timing=True."""
    z0 = np.ascontiguousarray(z0, dtype=np.float64)
    h0 = np.ascontiguousarray(h0, dtype=np.float64)
    rows, cols = z0.shape
    z = np.empty_like(z0)
    h = np.empty_like(h0)
    n = C.c_long(0)
    ms = C.c_double(0.0)
    cells = np.zeros((rows * cols if ac else 1, 2), dtype=np.int32)
    rc = models().cal_sciddicaT_run(rows, cols, int(toroidal), int(ac), int(steps), p_r, p_eps, z0, h0, z, h,
                                    C.byref(n), cells.ctypes.data if ac else None, int(mode), int(graph),
                                    C.byref(ms))
    _check(rc, "cal_sciddicaT_run")
    out = (z, h, cells[: n.value].copy() if ac else np.zeros((0, 2), np.int32))
    return out + (ms.value,) if timing else out


def life2d(s0, steps, *, toroidal=True, as_int=False, mode=MODE_FUSED_BLOCKED, block=8, graph=False, timing=False):
    s0 = np.ascontiguousarray(s0, dtype=np.uint8)
    rows, cols = s0.shape
    out = np.empty_like(s0)
    ms = C.c_double(0.0)
    rc = models().cal_life2d_run(rows, cols, int(toroidal), int(as_int), int(steps), s0, out, int(mode), int(block),
                                 int(graph), C.byref(ms))
    _check(rc, "cal_life2d_run")
    return (out, ms.value) if timing else out


def life3d(s0, steps, *, nbhd=2, toroidal=True, rule=(5, 7, 6, 6), graph=False):
    s0 = np.ascontiguousarray(s0, dtype=np.uint8)
    slices, rows, cols = s0.shape
    out = np.empty_like(s0)
    _check(models().cal_life3d_run(rows, cols, slices, int(nbhd), int(toroidal), int(steps), *rule, s0, out,
                                   int(graph)), "cal_life3d_run")
    return out


def sciara(z0, vents, rates, emission_time, steps, *, ac=False, params=None, slt0=None, st0=None, graph=False,
           timing=False, libm=False):
    """SCIARA-fv2 on the GPU (csrc/models/sciara.cu): the reference program's
    elementary processes as device processes behind the C API.  Same
    arguments and result as oracle.sciara (dict z, slt, st, msl, steps,
    cells), plus the device milliseconds of the step loop with timing=True.
    libm=True evaluates pow / atan / cos as the reference writes them
    instead of the identity forms."""
    from .workloads import SCIARA_PARAMS
    z0 = np.ascontiguousarray(z0, dtype=np.float64)
    rows, cols = z0.shape
    p = np.ascontiguousarray(params if params is not None else SCIARA_PARAMS, dtype=np.float64)
    v = np.ascontiguousarray(np.asarray(vents, dtype=np.int32).reshape(-1))
    r = np.ascontiguousarray(np.asarray(rates, dtype=np.float64).reshape(-1))
    nphases = len(rates[0]) if len(rates) else 0
    outs = {k: np.empty_like(z0) for k in ("z", "slt", "st", "msl")}
    done = C.c_int(0)
    n = C.c_long(0)
    ms = C.c_double(0.0)
    cells = np.zeros((rows * cols if ac else 1, 2), dtype=np.int32)
    m = models()
    m.cal_sciara_set_math.argtypes = [C.c_int]
    _check(m.cal_sciara_set_math(1 if libm else 0), "cal_sciara_set_math")
    f = m.cal_sciara_run
    f.restype = C.c_int
    f.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_uint, C.c_int, C.c_void_p,
                  C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                  C.POINTER(C.c_int), C.POINTER(C.c_long), C.c_void_p, C.c_int, C.POINTER(C.c_double)]
    slt0 = None if slt0 is None else np.ascontiguousarray(slt0, dtype=np.float64)
    st0 = None if st0 is None else np.ascontiguousarray(st0, dtype=np.float64)
    rc = f(rows, cols, int(ac), int(steps), p.ctypes.data, len(vents), v.ctypes.data, int(emission_time), nphases,
           r.ctypes.data, z0.ctypes.data, None if slt0 is None else slt0.ctypes.data,
           None if st0 is None else st0.ctypes.data, outs["z"].ctypes.data, outs["slt"].ctypes.data,
           outs["st"].ctypes.data, outs["msl"].ctypes.data, C.byref(done), C.byref(n),
           cells.ctypes.data if ac else None, int(bool(graph)), C.byref(ms))
    _check(rc, "cal_sciara_run")
    outs["steps"] = done.value
    outs["cells"] = cells[: n.value].copy() if ac else np.zeros((0, 2), np.int32)
    if timing:
        outs["ms"] = ms.value
    return outs


def sciara_read(path):
    """A SCIARA-fv2 configuration in the reference example's files (.cfg,
    Morphology.stt, Vents.stt, EmissionRate.txt, optional Thickness /
    Temperature / SolidifiedLavaThickness.stt) as
    dict(params, z, vents, rates, emission_time, slt0, st0, msl0), ready for
    ``sciara``."""
    m = models()
    rows, cols, nv, nph = (C.c_int() for _ in range(4))
    f = m.cal_sciara_read_sizes
    f.restype = C.c_int
    f.argtypes = [C.c_char_p] + [C.POINTER(C.c_int)] * 4
    _check(f(str(path).encode(), C.byref(rows), C.byref(cols), C.byref(nv), C.byref(nph)), "cal_sciara_read_sizes")
    params = np.zeros(13)
    z = np.zeros((rows.value, cols.value))
    vent_xy = np.zeros((max(nv.value, 1), 2), dtype=np.int32)
    rates = np.zeros((max(nv.value, 1), max(nph.value, 1)))
    grids = [np.zeros_like(z) for _ in range(3)]
    present = (C.c_int * 3)()
    et = C.c_uint(0)
    g = m.cal_sciara_read
    g.restype = C.c_int
    g.argtypes = [C.c_char_p] + [C.c_void_p] * 4 + [C.POINTER(C.c_uint)] + [C.c_void_p] * 4
    _check(g(str(path).encode(), params.ctypes.data, z.ctypes.data, vent_xy.ctypes.data, rates.ctypes.data,
             C.byref(et), grids[0].ctypes.data, grids[1].ctypes.data, grids[2].ctypes.data, present),
           "cal_sciara_read")
    return {"params": params, "z": z, "vents": [tuple(v) for v in vent_xy[: nv.value]],
            "rates": rates[: nv.value, : nph.value].tolist(), "emission_time": et.value,
            "slt0": grids[0] if present[0] else None, "st0": grids[1] if present[1] else None,
            "msl0": grids[2] if present[2] else None}


def sciddicaT_unsafe(z0, h0, steps, *, toroidal=True, p_r=0.5, p_eps=0.001, graph=False):
    """SCIDDICA-T in the reference's unsafe form on the GPU; returns (z, h)."""
    z0 = np.ascontiguousarray(z0, dtype=np.float64)
    h0 = np.ascontiguousarray(h0, dtype=np.float64)
    rows, cols = z0.shape
    z, h = np.empty_like(z0), np.empty_like(h0)
    f = models().cal_sciddicaT_unsafe_run
    f.restype = C.c_int
    f.argtypes = [C.c_int] * 4 + [C.c_double, C.c_double] + [C.c_void_p] * 4 + [C.c_int]
    _check(f(rows, cols, int(toroidal), int(steps), p_r, p_eps, z0.ctypes.data, h0.ctypes.data, z.ctypes.data,
             h.ctypes.data, int(bool(graph))), "cal_sciddicaT_unsafe_run")
    return z, h


MBUSU_SHAPE = (130, 160, 30)  # slices, rows, cols
MBUSU_FIELDS = ("teta", "moist_cont", "psi", "k", "h", "dqdh", "convergence", "moist_diff")


def mbusu(steps=0, *, mode=2, timing=False):
    """The reference's mbusu subsurface-flow program on the GPU through the
    3D C API (csrc/models/mbusu.cu).  steps: 0 = until its stop condition at
    10 days, > 0 = at most that many, < 0 = none.  mode: 0 = launches per
    step, 1 = recorded step replayed, 2 = one device-driven loop.  Returns a
    dict of the eight substates (slices, rows, cols) plus steps, delta_t,
    delta_t_cum (and ms with timing=True)."""
    n = MBUSU_SHAPE[0] * MBUSU_SHAPE[1] * MBUSU_SHAPE[2]
    state = np.empty(8 * n)
    tail = np.zeros(3)
    ms = C.c_double(0.0)
    m = models()
    m.cal_mbusu_run.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.POINTER(C.c_double)]
    _check(m.cal_mbusu_run(int(steps), int(mode), state.ctypes.data, tail.ctypes.data, C.byref(ms)),
           "cal_mbusu_run")
    out = {name: state[q * n:(q + 1) * n].reshape(MBUSU_SHAPE).copy() for q, name in enumerate(MBUSU_FIELDS)}
    out["steps"], out["delta_t"], out["delta_t_cum"] = int(tail[0]), float(tail[1]), float(tail[2])
    if timing:
        out["ms"] = ms.value
    return out


class SciaraBatch:
    """SCIARA-fv2 scenarios on the device, advanced together by the split step
    (csrc/models/sciara_batch.cu): created once, then run (always from the
    initial state), read back and differentiated as often as wanted.
    scenarios: [(z0, vents [(x, y)], rates [nvents][nphases], emission_time)]
    sharing the emission schedule.  close() (or ``with``) frees the device
    memory."""

    def __init__(self, scenarios, *, params=None, list_fraction=0.0):
        from .workloads import SCIARA_PARAMS
        self.shapes = [tuple(np.shape(s[0])) for s in scenarios]
        self.vents_per = [len(s[1]) for s in scenarios]
        ets = {int(s[3]) for s in scenarios}
        nph = {len(s[2][0]) for s in scenarios}
        if len(ets) != 1 or len(nph) != 1:
            raise ValueError("scenarios must share the emission schedule (emission_time, number of phases)")
        et, self.nphases = ets.pop(), nph.pop()
        self.cells = int(sum(r * c for r, c in self.shapes))
        dims = np.ascontiguousarray(np.array(self.shapes, dtype=np.int32).reshape(-1))
        z = np.empty(self.cells)
        pos = 0
        for s in scenarios:
            n = int(np.size(s[0]))
            z[pos:pos + n] = np.asarray(s[0], np.float64).ravel()
            pos += n
        vinst, vxy, rates = [], [], []
        for b, s in enumerate(scenarios):
            for v, r in zip(s[1], s[2]):
                vinst.append(b)
                vxy.extend(v)
                rates.extend(r)
        self.nvents = len(vinst)
        vinst = np.ascontiguousarray(np.array(vinst, dtype=np.int32))
        vxy = np.ascontiguousarray(np.array(vxy, dtype=np.int32))
        rates = np.ascontiguousarray(np.array(rates, dtype=np.float64))
        p = np.ascontiguousarray(params if params is not None else SCIARA_PARAMS, dtype=np.float64)
        m = models()
        m.cal_sciara_batch_create.restype = C.c_void_p
        m.cal_sciara_batch_create.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                              C.c_int, C.c_void_p, C.c_void_p, C.c_uint, C.c_int, C.c_void_p,
                                              C.c_double]
        m.cal_sciara_batch_run.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_float)]
        m.cal_sciara_batch_read.argtypes = [C.c_void_p] + [C.c_void_p] * 4
        m.cal_sciara_batch_destroy.argtypes = [C.c_void_p]
        m.cal_sciara_batch_lava_cells.argtypes = [C.c_void_p]
        m.cal_sciara_batch_loss_grad.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p,
                                                 C.POINTER(C.c_int), C.c_longlong, C.POINTER(C.c_float)]
        self._m = m
        self._h = m.cal_sciara_batch_create(len(scenarios), dims.ctypes.data, z.ctypes.data, None, None,
                                            p.ctypes.data, self.nvents, vinst.ctypes.data, vxy.ctypes.data, et,
                                            self.nphases, rates.ctypes.data, float(list_fraction))
        if not self._h:
            raise CALError("cal_sciara_batch_create failed (bad argument or out of device memory)")

    def run(self, steps=0):
        """Run every scenario from its initial state (steps 0: until the
        emission ends).  Returns (steps run, device milliseconds)."""
        done, ms = C.c_int(0), C.c_float(0.0)
        _check(self._m.cal_sciara_batch_run(self._h, int(steps), C.byref(done), C.byref(ms)),
               "cal_sciara_batch_run")
        return done.value, ms.value

    def read(self, *names):
        """The final grids named ("z", "slt", "st", "msl"), each a list of
        per-scenario arrays; default all four as a list of dicts."""
        want = names or ("z", "slt", "st", "msl")
        outs = {k: np.empty(self.cells) for k in want}
        ptr = [outs[k].ctypes.data if k in outs else None for k in ("z", "slt", "st", "msl")]
        _check(self._m.cal_sciara_batch_read(self._h, *ptr), "cal_sciara_batch_read")
        per = {k: self._unpack(v) for k, v in outs.items()}
        if names:
            return per[names[0]] if len(names) == 1 else [per[k] for k in names]
        return [{k: per[k][b] for k in per} for b in range(len(self.shapes))]

    def lava_cells(self):
        return int(self._m.cal_sciara_batch_lava_cells(self._h))

    def loss_grad(self, targets, steps=0, *, tape_slots=0):
        """L_b = sum (Slt_T - target_b)^2 and dL/drate of every vent and phase
        (adjoint with the forward's decisions frozen).  targets: per-scenario
        grids or one flat array.  Returns (loss[B], [grad_b (nvents_b x
        nphases)], device milliseconds of forward + adjoint)."""
        if isinstance(targets, np.ndarray) and targets.ndim == 1:
            tgt = np.ascontiguousarray(targets, dtype=np.float64)
        else:
            tgt = np.ascontiguousarray(np.concatenate([np.asarray(t, np.float64).ravel() for t in targets]))
        if tgt.size != self.cells:
            raise ValueError("targets do not match the scenarios' grids")
        loss = np.zeros(len(self.shapes))
        grad = np.zeros(max(1, self.nvents * self.nphases))
        done, ms = C.c_int(0), C.c_float(0.0)
        _check(self._m.cal_sciara_batch_loss_grad(self._h, tgt.ctypes.data, int(steps), loss.ctypes.data,
                                                  grad.ctypes.data, C.byref(done), int(tape_slots), C.byref(ms)),
               "cal_sciara_batch_loss_grad")
        grads, pos = [], 0
        for k in self.vents_per:
            grads.append(grad[pos * self.nphases:(pos + k) * self.nphases].reshape(k, self.nphases).copy())
            pos += k
        return loss, grads, ms.value

    def _unpack(self, flat):
        res, pos = [], 0
        for r, c in self.shapes:
            res.append(flat[pos:pos + r * c].reshape(r, c))
            pos += r * c
        return res

    def close(self):
        if self._h:
            self._m.cal_sciara_batch_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def sciara_batch(scenarios, steps=0, *, params=None, list_fraction=0.0, timing=False):
    """SCIARA-fv2 scenarios advanced together by the split step
    (csrc/models/sciara_batch.cu).  scenarios: [(z0, vents, rates,
    emission_time)], sharing the emission schedule.  Returns a list of dicts
    (z, slt, st, msl) and the steps run (and the device milliseconds with
    timing=True)."""
    with SciaraBatch(scenarios, params=params, list_fraction=list_fraction) as sb:
        done, ms = sb.run(steps)
        res = sb.read()
    return (res, done, ms) if timing else (res, done)


def sciara_loss_grad(scenarios, targets, steps=0, *, params=None, list_fraction=0.0, tape_slots=0, timing=False):
    """L_b = sum (Slt_T - target_b)^2 for every scenario and dL/drate for
    every vent and phase (csrc/models/sciara_batch.cu, adjoint with the
    forward's decisions frozen).  Returns (loss[B], [grad_b (nvents_b x
    nphases)]) (and the device milliseconds with timing=True)."""
    with SciaraBatch(scenarios, params=params, list_fraction=list_fraction) as sb:
        loss, grads, ms = sb.loss_grad(targets, steps, tape_slots=tape_slots)
    return (loss, grads, ms) if timing else (loss, grads)
