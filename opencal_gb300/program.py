"""Models defined from Python: this library's counterpart of the reference's
SWIG binding (OpenCAL/include/opencal.i, ElementaryProcessFunctor2D.i), where
a Python class subclasses the elementary-process functor
(``%feature("director")``) and the C library calls back into Python for
every cell.

A process body cannot run in the Python interpreter on the GPU, so here it
is given as the CUDA C statements of the per-cell function -- what a C
program wraps in ``CAL_ELEMENTARY_PROCESS_2D`` -- and compiled for sm_103a
at run time against the C ABI (``include/opencal``), cached by the hash of
the generated source.  Everything else is Python: the model, its substates,
the process list, host data in and out, and the run loop with its init,
steering and stop-condition callbacks (ctypes function pointers handed to
``calRunAdd*Func2D``, as the SWIG module hands its directors).

    prog = (Program("life").substates(alive="b")
            .process("life_rule", '''
                int sum = 0;
                for (int n = 1; n < ca->sizeof_X; n++) sum += calGetX2Db(ca, Q.alive, i, j, n);
                const CALbyte a = calGet2Db(ca, Q.alive, i, j);
                calSet2Db(ca, Q.alive, i, j, (sum == 3 || (a == 1 && sum == 2)) ? 1 : 0);'''))
    lib = prog.build()
    model = Model2D(1024, 1024, CAL_MOORE_NEIGHBORHOOD_2D, CAL_SPACE_TOROIDAL)
    alive = model.add_substate("b")
    lib.bind(alive=alive)
    model.add_process(lib.process("life_rule"))
    model.load(alive, grid)
    Run2D(model, 1, 1000, graph=True).run()
    grid = model.read(alive)

Inside a body: ``ca`` (the model), ``i``, ``j`` (the cell), ``Q.<substate>``
(the handles bound with ``ProgramLib.bind``) and ``P.<parameter>`` (set with
``ProgramLib.set``), and every accessor of ``cal2D.h``.
"""
from __future__ import annotations

import ctypes as C
import hashlib
import os
import re
import subprocess

import numpy as np

from . import CALError, LIB_DIR, core
from . import nvbuild

# enumerators of include/opencal/cal2D.h and calCommon.h
CAL_CUSTOM_NEIGHBORHOOD_2D, CAL_VON_NEUMANN_NEIGHBORHOOD_2D, CAL_MOORE_NEIGHBORHOOD_2D = 0, 1, 2
CAL_HEXAGONAL_NEIGHBORHOOD_2D, CAL_HEXAGONAL_NEIGHBORHOOD_ALT_2D = 3, 4
CAL_SPACE_FLAT, CAL_SPACE_TOROIDAL = 0, 1
CAL_NO_OPT, CAL_OPT_ACTIVE_CELLS = 0, 1
CAL_UPDATE_EXPLICIT, CAL_UPDATE_IMPLICIT = 0, 1
CAL_RUN_LOOP = -1

PROGRAM_DIR = os.path.join(LIB_DIR, "programs")

_KINDS = {"b": ("CALSubstate2Db", "CALbyte", C.c_byte, np.int8),
          "i": ("CALSubstate2Di", "CALint", C.c_int, np.int32),
          "r": ("CALSubstate2Dr", "CALreal", C.c_double, np.float64)}
_PARAM_TYPES = {"r": ("CALreal", C.c_double), "i": ("CALint", C.c_int), "b": ("CALbyte", C.c_byte)}
_IDENT = re.compile(r"^[A-Za-z_][A-Za-z0-9_]*$")

_CB_MODEL = C.CFUNCTYPE(None, C.c_void_p)
_CB_STOP = C.CFUNCTYPE(C.c_byte, C.c_void_p)


def _ident(name: str, what: str) -> str:
    if not _IDENT.match(name or ""):
        raise CALError(f"{what} {name!r} is not a C identifier")
    return name


_capi = None


def capi() -> C.CDLL:
    """The C API (libopencal_gb300.so) with argument types set for the
    functions this module calls, under the reference's names."""
    global _capi
    if _capi is not None:
        return _capi
    lib = core()
    vp, i, d = C.c_void_p, C.c_int, C.c_double
    sig = {
        "calCADef2D": ([i, i, i, i, i], vp),
        "calFinalize2D": ([vp], None),
        "calAddElementaryProcess2D": ([vp, vp], vp),
        "calSetElementaryProcessPure2D": ([vp, vp, C.c_byte], i),
        "calSetElementaryProcessReads2D": ([vp, vp, vp, i], i),
        "calSetElementaryProcessGuard2Dr": ([vp, vp, vp, i, C.c_double], i),
        "calApplyElementaryProcess2D": ([vp, vp], None),
        "calUpdate2D": ([vp], None),
        "calAddActiveCell2D": ([vp, i, i], None),
        "calUpdateActiveCells2D": ([vp], None),
        "calGetActiveCellCount2D": ([vp], i),
        "calSync2D": ([vp], None),
        "calRunDef2D": ([vp, i, i, i], vp),
        "calRunAddInitFunc2D": ([vp, vp], None),
        "calRunAddGlobalTransitionFunc2D": ([vp, vp], None),
        "calRunAddSteeringFunc2D": ([vp, vp], None),
        "calRunAddStopConditionFunc2D": ([vp, vp], None),
        "calRunAddDeviceStopConditionFunc2D": ([vp, vp], None),
        "calRunAddFinalizeFunc2D": ([vp, vp], None),
        "calRunSetGraph2D": ([vp, C.c_byte], None),
        "calRunGraphReplays2D": ([vp], C.c_long),
        "calRunInitSimulation2D": ([vp], None),
        "calRunCAStep2D": ([vp], C.c_byte),
        "calRun2D": ([vp], None),
        "calRunDevice2D": ([vp], None),
        "calRunFinalize2D": ([vp], None),
        "calGetStream2D": ([vp], vp),
    }
    for s in "bir":
        t = _KINDS[s][2]
        sig[f"calAddSubstate2D{s}"] = ([vp], vp)
        sig[f"calAddSingleLayerSubstate2D{s}"] = ([vp], vp)
        sig[f"calInitSubstate2D{s}"] = ([vp, vp, t], None)
        sig[f"calCopySubstateFromHost2D{s}"] = ([vp, vp, vp], None)
        sig[f"calCopySubstateToHost2D{s}"] = ([vp, vp, vp], None)
    for name, (args, res) in sig.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = res
    _capi = lib
    return lib


def _raise_on_error(what: str) -> None:
    lib = core()
    rc = lib.calGetLastError()
    if rc:
        msg = lib.calGetErrorString()
        raise CALError(f"{what} failed (CALError {rc}): {msg.decode() if msg else ''}")


class Substate:
    """A substate handle (struct CALSubstate2D{b,i,r}*) and its type letter."""

    def __init__(self, ptr: int, kind: str):
        self.ptr = ptr
        self.kind = kind

    @property
    def _as_parameter_(self):  # ctypes passes the handle
        return C.c_void_p(self.ptr)


class Program:
    """Elementary processes, device stop conditions and device helpers given
    as CUDA C source, with the substate handles (Q) and parameters (P) they
    read.  ``build()`` compiles them into a shared library that registers
    its processes with the C API when loaded."""

    def __init__(self, name: str):
        self.name = _ident(name, "program name")
        self._subs: list[tuple[str, str]] = []
        self._params: list[tuple[str, str]] = []
        self._helpers: list[str] = []
        self._procs: list[tuple[str, str]] = []
        self._stops: list[tuple[str, str]] = []

    def substates(self, **kinds: str) -> "Program":
        """Q's fields: name="b" | "i" | "r" (CALbyte, CALint, CALreal)."""
        for n, k in kinds.items():
            if k not in _KINDS:
                raise CALError(f"substate {n}: type {k!r} is not one of b, i, r")
            self._subs.append((_ident(n, "substate"), k))
        return self

    def parameters(self, **types: str) -> "Program":
        """P's fields: name="r" | "i" | "b"."""
        for n, k in types.items():
            if k not in _PARAM_TYPES:
                raise CALError(f"parameter {n}: type {k!r} is not one of r, i, b")
            self._params.append((_ident(n, "parameter"), k))
        return self

    def device(self, code: str) -> "Program":
        """Device helper code (functions, constants) placed before the processes."""
        self._helpers.append(code)
        return self

    def process(self, name: str, body: str) -> "Program":
        """An elementary process: the statements of its per-cell body."""
        self._procs.append((_ident(name, "process"), body))
        return self

    def stop_condition(self, name: str, body: str) -> "Program":
        """A device stop condition (CAL_DEVICE_STOP_CONDITION_2D): statements
        that return a CALbyte, evaluated by one thread after every step of
        Run2D.device()."""
        self._stops.append((_ident(name, "stop condition"), body))
        return self

    def source(self) -> str:
        p = self.name
        out = ["/* generated by opencal_gb300.program */", "#include <opencal/cal2D.h>",
               "#include <opencal/cal2DRun.h>", ""]
        q = "".join(f" struct {_KINDS[k][0]}* {n};" for n, k in self._subs) or " int unused_;"
        out.append(f"__managed__ struct {{{q} }} Q;")
        par = "".join(f" {_PARAM_TYPES[k][0]} {n};" for n, k in self._params) or " int unused_;"
        out.append(f"__managed__ struct {{{par} }} P;")
        out.append("")
        out.append(f'extern "C" int cal_prog_{p}_bind(int k, void* handle)')
        out.append("{\n    cudaDeviceSynchronize(); /* no process reads Q meanwhile */\n    switch (k) {")
        for k, (n, kind) in enumerate(self._subs):
            out.append(f"    case {k}: Q.{n} = (struct {_KINDS[kind][0]}*)handle; return 0;")
        out.append("    }\n    return 1;\n}")
        for n, k in self._params:
            t = _PARAM_TYPES[k][0]
            out.append(f'extern "C" void cal_prog_{p}_set_{n}({t} v)\n{{\n    cudaDeviceSynchronize();\n'
                       f"    P.{n} = v;\n}}")
            out.append(f'extern "C" {t} cal_prog_{p}_get_{n}(void) {{ return P.{n}; }}')
        out.append("")
        out.extend(self._helpers)
        for n, body in self._procs:
            out.append(f"CAL_ELEMENTARY_PROCESS_2D({n})(struct CALModel2D* ca, int i, int j)\n{{\n{body}\n}}")
        for n, body in self._stops:
            out.append(f"CAL_DEVICE_STOP_CONDITION_2D({n})(struct CALModel2D* ca)\n{{\n{body}\n}}")
        return "\n".join(out) + "\n"

    def build(self, *, exact: bool = True, verbose: bool = False, extra_flags=()) -> "ProgramLib":
        """Compile (or reuse the cached build of) the program for sm_103a and
        load it.  exact: no FMA contraction (--fmad=false), so that FP64
        arithmetic follows the source operation by operation, as the
        reference's C compiler evaluates it."""
        src = self.source()
        flags = nvbuild.COMMON + (nvbuild.MODEL_FLAGS if exact else []) + list(extra_flags)
        key = hashlib.sha256((src + "\0" + " ".join(flags)).encode()).hexdigest()[:16]
        os.makedirs(PROGRAM_DIR, exist_ok=True)
        base = os.path.join(PROGRAM_DIR, f"{self.name}_{key}")
        so = base + ".so"
        if not os.path.exists(so):
            with open(base + ".cu", "w") as f:
                f.write(src)
            tmp = f"{base}.{os.getpid()}.so"
            cmd = ([nvbuild.nvcc()] + flags + ["-shared", "-o", tmp, base + ".cu", "-L" + LIB_DIR,
                                                "-lopencal_gb300", "-Xlinker", "-rpath," + LIB_DIR])
            if verbose:
                cmd.insert(1, "-Xptxas=-v")
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise CALError(f"nvcc failed on program {self.name}:\n{r.stderr}")
            os.replace(tmp, so)
        return ProgramLib(self, so)


class ProgramLib:
    """A built program, loaded: its processes are registered with the C API."""

    def __init__(self, prog: Program, path: str):
        capi()  # the C API first (RTLD_GLOBAL), then the program linked to it
        self.path = path
        self.prog = prog
        self.lib = C.CDLL(path)
        self._subs = {n: (k, idx) for idx, (n, k) in enumerate(prog._subs)}
        self._params = dict(prog._params)
        self._procs = {n for n, _ in prog._procs}
        self._stops = {n for n, _ in prog._stops}
        self._bind = getattr(self.lib, f"cal_prog_{prog.name}_bind")
        self._bind.argtypes = [C.c_int, C.c_void_p]
        self._bind.restype = C.c_int

    def _symbol(self, name: str) -> int:
        return C.cast(getattr(self.lib, name), C.c_void_p).value

    def process(self, name: str) -> int:
        """The host name of process `name` (what calAddElementaryProcess2D takes)."""
        if name not in self._procs:
            raise KeyError(name)
        return self._symbol(name)

    def stop_condition(self, name: str) -> int:
        if name not in self._stops:
            raise KeyError(name)
        return self._symbol(name)

    def bind(self, **handles: Substate) -> None:
        """Q.<name> = handle, for the substates the processes read."""
        for n, h in handles.items():
            if n not in self._subs:
                raise KeyError(n)
            kind, idx = self._subs[n]
            if not isinstance(h, Substate) or h.kind != kind:
                raise CALError(f"Q.{n} is a {kind} substate")
            if self._bind(idx, h.ptr):
                raise CALError(f"binding Q.{n} failed")

    def set(self, **values) -> None:
        """P.<name> = value."""
        for n, v in values.items():
            if n not in self._params:
                raise KeyError(n)
            f = getattr(self.lib, f"cal_prog_{self.prog.name}_set_{n}")
            f.argtypes = [_PARAM_TYPES[self._params[n]][1]]
            f.restype = None
            f(v)

    def get(self, name: str):
        f = getattr(self.lib, f"cal_prog_{self.prog.name}_get_{name}")
        f.restype = _PARAM_TYPES[self._params[name]][1]
        f.argtypes = []
        return f()


class Model2D:
    """calCADef2D and the calls on a model, with numpy in and out."""

    def __init__(self, rows: int, cols: int, neighborhood: int = CAL_VON_NEUMANN_NEIGHBORHOOD_2D,
                 space: int = CAL_SPACE_TOROIDAL, optimization: int = CAL_NO_OPT):
        self._c = capi()
        self.rows, self.cols = int(rows), int(cols)
        self.ptr = self._c.calCADef2D(self.rows, self.cols, int(neighborhood), int(space), int(optimization))
        if not self.ptr:
            _raise_on_error("calCADef2D")
            raise CALError("calCADef2D failed")

    @property
    def _as_parameter_(self):
        return C.c_void_p(self.ptr)

    def add_substate(self, kind: str, single_layer: bool = False) -> Substate:
        if kind not in _KINDS:
            raise CALError(f"substate type {kind!r} is not one of b, i, r")
        fn = "calAddSingleLayerSubstate2D" if single_layer else "calAddSubstate2D"
        h = getattr(self._c, fn + kind)(self)
        if not h:
            _raise_on_error(fn + kind)
        return Substate(h, kind)

    def add_process(self, process: int) -> None:
        """calAddElementaryProcess2D with a process of a built program."""
        self._c.calAddElementaryProcess2D(self, process)
        _raise_on_error("calAddElementaryProcess2D")

    def set_pure(self, process: int, pure: bool = True) -> None:
        """calSetElementaryProcessPure2D: the process is a pure function of
        its neighbourhood and of values constant during the run, so the
        engine may skip tiles where it would change nothing."""
        if self._c.calSetElementaryProcessPure2D(self, process, 1 if pure else 0):
            _raise_on_error("calSetElementaryProcessPure2D")

    def set_reads(self, process: int, substates) -> None:
        """calSetElementaryProcessReads2D: the substates the process reads
        (current layer, calGet / calGetX), staged into shared memory by TMA
        tile by tile."""
        subs = list(substates)
        arr = (C.c_void_p * max(len(subs), 1))(*[h.ptr for h in subs])
        if self._c.calSetElementaryProcessReads2D(self, process, arr, len(subs)):
            _raise_on_error("calSetElementaryProcessReads2D")

    GUARD_OPS = {"<=": 1, "<": 2, ">=": 3, ">": 4, "==": 5, "!=": 6}

    def set_guard(self, process: int, sub: Substate, op: str, value: float) -> None:
        """calSetElementaryProcessGuard2Dr: the process returns at once,
        changing nothing, where the real substate's current value v
        satisfies ``v op value`` (op one of <=, <, >=, >, ==, !=; None
        withdraws the declaration); the kernel then runs it on each tile's
        other cells packed into consecutive threads."""
        code = 0 if op is None else self.GUARD_OPS[op]
        if self._c.calSetElementaryProcessGuard2Dr(self, process, sub, code, float(value)):
            _raise_on_error("calSetElementaryProcessGuard2Dr")

    def apply(self, process: int) -> None:
        """calApplyElementaryProcess2D: one process over the grid now (then
        calUpdate2D, as the reference does when it is called from init)."""
        self._c.calApplyElementaryProcess2D(self, process)
        _raise_on_error("calApplyElementaryProcess2D")

    def update(self) -> None:
        self._c.calUpdate2D(self)

    def init(self, sub: Substate, value) -> None:
        """calInitSubstate2D{b,i,r}: both layers = value."""
        getattr(self._c, "calInitSubstate2D" + sub.kind)(self, sub, value)

    def add_active(self, i: int, j: int) -> None:
        self._c.calAddActiveCell2D(self, int(i), int(j))

    def update_active(self) -> None:
        self._c.calUpdateActiveCells2D(self)

    def active_count(self) -> int:
        return int(self._c.calGetActiveCellCount2D(self))

    def load(self, sub: Substate, data) -> None:
        """A (rows, cols) array into both layers of `sub` on the device."""
        a = np.ascontiguousarray(data, dtype=_KINDS[sub.kind][3])
        if a.shape != (self.rows, self.cols):
            raise CALError(f"expected a {self.rows}x{self.cols} array, got {a.shape}")
        getattr(self._c, "calCopySubstateFromHost2D" + sub.kind)(self, sub, a.ctypes.data)
        _raise_on_error("calCopySubstateFromHost2D" + sub.kind)

    def read(self, sub: Substate) -> np.ndarray:
        """The current layer of `sub` as a (rows, cols) array (waits for the
        device work queued so far)."""
        a = np.empty((self.rows, self.cols), dtype=_KINDS[sub.kind][3])
        getattr(self._c, "calCopySubstateToHost2D" + sub.kind)(self, sub, a.ctypes.data)
        _raise_on_error("calCopySubstateToHost2D" + sub.kind)
        return a

    def close(self) -> None:
        if getattr(self, "ptr", None):
            self._c.calFinalize2D(self)
            self.ptr = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class _RunHead(C.Structure):
    """The leading fields of struct CALRun2D (include/opencal/cal2DRun.h)."""
    _fields_ = [("ca2D", C.c_void_p), ("step", C.c_int), ("initial_step", C.c_int), ("final_step", C.c_int)]


class Run2D:
    """calRunDef2D with Python callbacks: init(model), steering(model),
    global_transition(model), finalize(model) and stop(model) -> bool, each
    called by the C run loop through a ctypes function pointer, as the SWIG
    module's directors are.  A callback issues its device work through the
    Model2D methods (which queue it on the model's stream); with graph=True
    the first step is recorded as a CUDA graph and replayed, which requires
    the steering to queue the same work every step.  A device stop condition
    (a process library's stop_condition) makes run_device() one graph launch
    for the whole loop."""

    def __init__(self, model: Model2D, initial_step: int, final_step: int, *, init=None, steering=None,
                 global_transition=None, finalize=None, stop=None, device_stop: int | None = None,
                 graph: bool = False, update: int = CAL_UPDATE_IMPLICIT):
        self._c = capi()
        self.model = model
        self.ptr = self._c.calRunDef2D(model, int(initial_step), int(final_step), int(update))
        if not self.ptr:
            _raise_on_error("calRunDef2D")
        self._keep = []  # the ctypes callbacks must outlive the run

        def wrap(fn):
            def cb(_ca):
                fn(model)
            f = _CB_MODEL(cb)
            self._keep.append(f)
            return C.cast(f, C.c_void_p)

        if init is not None:
            self._c.calRunAddInitFunc2D(self.ptr, wrap(init))
        if global_transition is not None:
            self._c.calRunAddGlobalTransitionFunc2D(self.ptr, wrap(global_transition))
        if steering is not None:
            self._c.calRunAddSteeringFunc2D(self.ptr, wrap(steering))
        if finalize is not None:
            self._c.calRunAddFinalizeFunc2D(self.ptr, wrap(finalize))
        if stop is not None:
            f = _CB_STOP(lambda _ca: 1 if stop(model) else 0)
            self._keep.append(f)
            self._c.calRunAddStopConditionFunc2D(self.ptr, C.cast(f, C.c_void_p))
        if device_stop is not None:
            self._c.calRunAddDeviceStopConditionFunc2D(self.ptr, device_stop)
        self._c.calRunSetGraph2D(self.ptr, 1 if graph else 0)
        _raise_on_error("calRunDef2D")

    @property
    def step(self) -> int:
        """CALRun2D::step (the step the loop is on / ended on)."""
        return C.cast(self.ptr, C.POINTER(_RunHead)).contents.step if self.ptr else 0

    def run(self) -> None:
        """calRun2D: init, steps until the final step or the stop condition, finalize."""
        self._c.calRun2D(self.ptr)
        _raise_on_error("calRun2D")

    def run_device(self) -> None:
        """calRunDevice2D: the step loop as one device-driven graph launch."""
        self._c.calRunDevice2D(self.ptr)
        _raise_on_error("calRunDevice2D")

    def init_simulation(self) -> None:
        self._c.calRunInitSimulation2D(self.ptr)

    def ca_step(self) -> bool:
        """calRunCAStep2D: one step; False once the stop condition holds."""
        return bool(self._c.calRunCAStep2D(self.ptr))

    def graph_replays(self) -> int:
        return int(self._c.calRunGraphReplays2D(self.ptr))

    def close(self) -> None:
        if getattr(self, "ptr", None):
            self._c.calRunFinalize2D(self.ptr)
            self.ptr = None
