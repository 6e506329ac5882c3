"""Batched SCIDDICA-T ensembles and their calibration.

``Ensemble`` wraps the ensemble entry points of ``libopencal_models.so``
(csrc/models/sciddicaT_batch.cu): many independent plain-mode SCIDDICA-T
instances (flat boundary; each with its own grid size, DEM, source, p_r and
p_epsilon) advanced by one launch per step over a packed tile work-list, with
a hand-written adjoint giving every instance's dL/dp_r and dL/dp_eps of
L = sum (h_T - target)^2 in one backward pass.

``calibrate`` fits (p_r, p_eps) of every instance to its target map with a
per-instance quasi-Newton iteration (BFGS on log-parameters with a
backtracking line search); one iteration is one batched loss+gradient call.
``FDSession`` is the comparison: the plain C-API program run per instance,
with central finite-difference gradients (five forward runs per instance
per iteration).

Torch holds device buffers only.  There is no CPU path: every call runs the
CUDA library and raises if it is missing.
"""
from __future__ import annotations

import ctypes as C
import time

import numpy as np
import torch

from . import CALError, models as _models

SHAPES = ("32x16", "64x16", "64x32", "16x8", "32x8")
_bound = False
_pd = C.POINTER(C.c_double)
_pi = C.POINTER(C.c_int)
_pll = C.POINTER(C.c_longlong)


def _lib():
    global _bound
    m = _models()
    if not _bound:
        m.cal_sdt_batch_create.restype = C.c_void_p
        m.cal_sdt_batch_create.argtypes = [C.c_int, _pi, _pd, _pd, _pd, C.c_int]
        m.cal_sdt_batch_destroy.argtypes = [C.c_void_p]
        m.cal_sdt_batch_cells.restype = C.c_longlong
        m.cal_sdt_batch_cells.argtypes = [C.c_void_p, _pll]
        m.cal_sdt_batch_stream.restype = C.c_void_p
        m.cal_sdt_batch_stream.argtypes = [C.c_void_p]
        m.cal_sdt_batch_shape.argtypes = [C.c_void_p]
        m.cal_sdt_batch_set_params.argtypes = [C.c_void_p, _pd]
        m.cal_sdt_batch_forward.argtypes = [C.c_void_p, C.c_void_p]
        m.cal_sdt_batch_active_tiles.argtypes = [C.c_void_p, _pi]
        m.cal_sdt_batch_loss_grad.argtypes = [C.c_void_p, C.c_void_p, _pd, _pd, C.c_void_p]
        m.cal_sdt_batch_set_graph.argtypes = [C.c_void_p, C.c_int]
        m.cal_sdt_batch_graph_stats.argtypes = [C.c_void_p, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]
        m.cal_sdt_batch_set_tape.argtypes = [C.c_void_p, C.c_int]
        m.cal_sdt_batch_tape_info.argtypes = [C.c_void_p, C.POINTER(C.c_longlong)]
        m.cal_sdt_batch_autotune.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_float)]
        m.cal_sdt_batch_set_shape.argtypes = [C.c_void_p, C.c_int]
        m.cal_sciddicaT_open.restype = C.c_void_p
        m.cal_sciddicaT_open.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, _pd, _pd,
                                         C.c_int]
        m.cal_sciddicaT_reset.argtypes = [C.c_void_p]
        m.cal_sciddicaT_steps.argtypes = [C.c_void_p, C.c_int, C.c_int]
        m.cal_sciddicaT_set_params.argtypes = [C.c_void_p, C.c_double, C.c_double]
        m.cal_sciddicaT_read.argtypes = [C.c_void_p, _pd]
        m.cal_sciddicaT_close.argtypes = [C.c_void_p]
        m.cal_sciddicaT_stream.restype = C.c_void_p
        m.cal_sciddicaT_stream.argtypes = [C.c_void_p]
        m.cal_sciddicaT_persist_failed.argtypes = [C.c_void_p]
        m.cal_sciddicaT_host_run.argtypes = [C.c_void_p, _pd, _pd, C.c_int, C.c_int, _pd]
        _bound = True
    return m


def _ptr(a: np.ndarray, ctype):
    return a.ctypes.data_as(C.POINTER(ctype))


class Ensemble:
    """B SCIDDICA-T instances (plain mode, flat boundary) on one GPU.

    dims: [(rows, cols)], params: [(p_r, p_eps)], zs / hs: per-instance DEM
    and initial thickness (float64 arrays of shape (rows, cols)), steps: the
    rollout length.  Device arrays use the padded packed layout: instance b
    occupies [offsets[b], offsets[b] + rows*cols) of ``cells`` values.
    """

    def __init__(self, dims, params, zs, hs, steps: int, device="cuda"):
        self.B = len(dims)
        self.dims = [(int(r), int(c)) for r, c in dims]
        self.steps = int(steps)
        self.device = torch.device(device)
        d = np.ascontiguousarray(np.asarray(self.dims, dtype=np.int32).reshape(-1))
        p = np.ascontiguousarray(np.asarray(params, dtype=np.float64).reshape(-1))
        z = np.ascontiguousarray(np.concatenate([np.asarray(a, np.float64).ravel() for a in zs]))
        h = np.ascontiguousarray(np.concatenate([np.asarray(a, np.float64).ravel() for a in hs]))
        for (r, c), a, b in zip(self.dims, zs, hs):
            if np.shape(a) != (r, c) or np.shape(b) != (r, c):
                raise ValueError("every z and h must have its instance's (rows, cols) shape")
        self._lib = _lib()
        self.handle = self._lib.cal_sdt_batch_create(self.B, _ptr(d, C.c_int), _ptr(p, C.c_double),
                                                     _ptr(z, C.c_double), _ptr(h, C.c_double), self.steps)
        if not self.handle:
            raise CALError("cal_sdt_batch_create failed (bad argument or out of device memory)")
        self.offsets = np.zeros(self.B + 1, dtype=np.int64)
        self.cells = int(self._lib.cal_sdt_batch_cells(self.handle, _ptr(self.offsets, C.c_longlong)))
        self.params = np.asarray(params, dtype=np.float64).reshape(self.B, 2).copy()

    def close(self):
        if getattr(self, "handle", None):
            self._lib.cal_sdt_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        self.close()

    # ---- layout ----------------------------------------------------------
    def pack(self, arrays) -> torch.Tensor:
        """Per-instance arrays -> one padded device tensor."""
        out = np.zeros(self.cells, dtype=np.float64)
        for b, a in enumerate(arrays):
            n = self.dims[b][0] * self.dims[b][1]
            out[self.offsets[b]:self.offsets[b] + n] = np.asarray(a, np.float64).ravel()
        return torch.from_numpy(out).to(self.device)

    def unpack(self, t: torch.Tensor):
        """Padded device tensor -> per-instance host arrays."""
        a = t.detach().cpu().numpy()
        return [a[self.offsets[b]:self.offsets[b] + r * c].reshape(r, c).copy()
                for b, (r, c) in enumerate(self.dims)]

    def _sync_torch(self):
        torch.cuda.current_stream(self.device).synchronize()

    # ---- runs ------------------------------------------------------------
    def set_params(self, params):
        p = np.ascontiguousarray(np.asarray(params, dtype=np.float64).reshape(-1))
        rc = self._lib.cal_sdt_batch_set_params(self.handle, _ptr(p, C.c_double))
        if rc:
            raise CALError(f"cal_sdt_batch_set_params failed ({rc})")
        self.params = p.reshape(self.B, 2).copy()

    def forward(self) -> torch.Tensor:
        """h_T of every instance (padded device tensor)."""
        hT = torch.empty(self.cells, dtype=torch.float64, device=self.device)
        self._sync_torch()
        rc = self._lib.cal_sdt_batch_forward(self.handle, C.c_void_p(hT.data_ptr()))
        torch.cuda.synchronize(self.device)
        if rc:
            raise CALError(f"cal_sdt_batch_forward failed ({rc})")
        return hT

    def loss_grad(self, target: torch.Tensor, want_h0_grad: bool = False):
        """(loss[B], grad[B, 2] = dL/dp_r, dL/dp_eps[, dL/dh0 padded tensor])."""
        assert target.dtype == torch.float64 and target.numel() == self.cells and target.is_cuda
        target = target.contiguous()
        loss = np.zeros(self.B)
        grad = np.zeros(2 * self.B)
        gh0 = torch.empty(self.cells, dtype=torch.float64, device=self.device) if want_h0_grad else None
        self._sync_torch()
        rc = self._lib.cal_sdt_batch_loss_grad(self.handle, C.c_void_p(target.data_ptr()), _ptr(loss, C.c_double),
                                               _ptr(grad, C.c_double),
                                               C.c_void_p(gh0.data_ptr()) if gh0 is not None else None)
        if rc:
            raise CALError(f"cal_sdt_batch_loss_grad failed ({rc})")
        grad = grad.reshape(self.B, 2)
        return (loss, grad, gh0) if want_h0_grad else (loss, grad)

    def set_graph(self, on: bool) -> None:
        """loss_grad as one launch of a recorded graph (default) or launch by launch."""
        self._lib.cal_sdt_batch_set_graph(self.handle, 1 if on else 0)

    def set_tape(self, mode: str) -> None:
        """What the adjoint's tape holds: "auto" (the whole rollout while it fits in
        half of the free device memory, else sqrt(T) segments), "segments", "full"."""
        code = {"auto": -1, "segments": 0, "full": 1}[mode]
        if self._lib.cal_sdt_batch_set_tape(self.handle, code):
            raise CALError(f"bad tape mode {mode}")

    def tape_info(self) -> dict:
        """{"full": the last evaluation taped the whole rollout, "capacity_bytes",
        "need_bytes": tape the last evaluation needed}"""
        info = (C.c_longlong * 3)()
        self._lib.cal_sdt_batch_tape_info(self.handle, info)
        return {"full": bool(info[0]), "capacity_bytes": int(info[1]), "need_bytes": int(info[2])}

    def graph_stats(self) -> tuple[int, int]:
        """(graph launches made by loss_grad so far, nodes of the recorded evaluation)"""
        a, b = C.c_longlong(0), C.c_longlong(0)
        self._lib.cal_sdt_batch_graph_stats(self.handle, C.byref(a), C.byref(b))
        return a.value, b.value

    def active_tiles(self) -> np.ndarray:
        out = np.zeros(self.steps + 1, dtype=np.int32)
        self._lib.cal_sdt_batch_active_tiles(self.handle, _ptr(out, C.c_int))
        return out

    def autotune(self, probe_steps: int = 50):
        """Time each tile shape on a forward probe; keep the fastest.
        Returns (shape name, {shape: ms})."""
        ms = (C.c_float * len(SHAPES))()
        best = self._lib.cal_sdt_batch_autotune(self.handle, int(probe_steps), ms)
        if best < 0:
            raise CALError("cal_sdt_batch_autotune failed")
        return SHAPES[best], {SHAPES[k]: float(ms[k]) for k in range(3)}

    def set_shape(self, name: str):
        if self._lib.cal_sdt_batch_set_shape(self.handle, SHAPES.index(name)):
            raise CALError("cal_sdt_batch_set_shape failed")


# ---- calibration -------------------------------------------------------


class _BFGS:
    """Per-instance BFGS on x = log(p) (two parameters each), vectorised over
    instances, with Armijo backtracking.  ``propose`` returns the points to
    evaluate next; ``accept`` takes their loss and gradient."""

    def __init__(self, x0: np.ndarray, step0: float = 0.05):
        self.x = x0.copy()
        self.B = x0.shape[0]
        self.H = np.repeat(np.eye(2)[None], self.B, axis=0)
        self.f = None
        self.g = None
        self.d = None
        self.alpha = np.ones(self.B)
        self.step0 = step0
        self.trial = x0.copy()
        self.done = np.zeros(self.B, dtype=bool)

    def first(self, f, g):
        self.f, self.g = f.copy(), g.copy()
        gn = np.linalg.norm(g, axis=1) + 1e-300
        # first direction: a step of step0 in log space along -g
        self.H = self.H * (self.step0 / gn)[:, None, None]
        self._new_direction()

    def _new_direction(self):
        self.d = -np.einsum("bij,bj->bi", self.H, self.g)
        self.alpha[:] = 1.0
        self.trial = self.x + self.alpha[:, None] * self.d

    def accept(self, f, g):
        armijo = f <= self.f + 1e-4 * self.alpha * np.einsum("bi,bi->b", self.g, self.d)
        ok = armijo & ~self.done
        if ok.any():
            s = (self.trial - self.x)[ok]
            y = (g - self.g)[ok]
            sy = np.einsum("bi,bi->b", s, y)
            H = self.H[ok]
            good = sy > 1e-300
            rho = np.where(good, 1.0 / np.where(good, sy, 1.0), 0.0)
            I = np.eye(2)[None]
            V = I - rho[:, None, None] * np.einsum("bi,bj->bij", s, y)
            Hn = np.einsum("bij,bjk,blk->bil", V, H, V) + rho[:, None, None] * np.einsum("bi,bj->bij", s, s)
            H = np.where(good[:, None, None], Hn, H)
            self.H[ok] = H
            self.x[ok] = self.trial[ok]
            self.f[ok] = f[ok]
            self.g[ok] = g[ok]
            d = -np.einsum("bij,bj->bi", self.H[ok], self.g[ok])
            self.d[ok] = d
            self.alpha[ok] = 1.0
        bad = ~armijo & ~self.done
        self.alpha[bad] *= 0.5
        self.trial = self.x + self.alpha[:, None] * self.d
        self.trial[self.done] = self.x[self.done]


def identifiable(ens: Ensemble, target: torch.Tensor, p_true, rel: float = 1e-3) -> np.ndarray:
    """(B, 2) booleans: whether h_T tells p_r (column 0) and p_eps (column 1)
    apart at relative resolution `rel` -- i.e. the forward runs at the true
    parameters with that parameter scaled by (1 - rel) and by (1 + rel) both
    give an h_T whose bits differ from the target's.  Where one of them does
    not, the loss is exactly 0 over part of the bracket and no method can
    recover that parameter to `rel` from h_T.  Four batched forwards."""
    p_true = np.asarray(p_true, dtype=np.float64).reshape(ens.B, 2)
    tgt = ens.unpack(target)
    out = np.ones((ens.B, 2), dtype=bool)
    for k in (0, 1):
        for sgn in (-1.0, 1.0):
            p = p_true.copy()
            p[:, k] *= 1.0 + sgn * rel
            ens.set_params(p)
            hT = ens.unpack(ens.forward())
            for b in range(ens.B):
                out[b, k] &= hT[b].tobytes() != tgt[b].tobytes()
    ens.set_params(p_true)
    return out


def recovered_fraction(params, p_true, mask, tol: float = 1e-3) -> float:
    """Fraction of instances whose identifiable parameters (mask) are all
    within `tol` relative of the truth."""
    rel = np.abs(np.asarray(params) - np.asarray(p_true)) / np.abs(np.asarray(p_true))
    return float(np.mean(np.all((rel < tol) | ~mask, axis=1)))


def calibrate(ens: Ensemble, target: torch.Tensor, p0, iters: int, p_true=None, tol: float = 1e-3,
              log=None, mask=None, stop_at: float | None = None):
    """Fit every instance's (p_r, p_eps) to ``target`` (padded h_T maps).
    One iteration = one batched forward + adjoint.  Returns a dict with the
    final parameters, the iterations used and the per-iteration wall time;
    with p_true also the relative errors and, after each iteration, the
    fraction of instances whose parameters -- the identifiable ones when
    `mask` (B x 2, see ``identifiable``) is given -- are all within ``tol``;
    the run stops early once that fraction reaches ``stop_at`` (or 1)."""
    p0 = np.asarray(p0, dtype=np.float64).reshape(ens.B, 2)
    mask = np.ones((ens.B, 2), dtype=bool) if mask is None else np.asarray(mask, dtype=bool)
    opt = _BFGS(np.log(p0))
    times, recovered, each = [], [], []
    converged_at = None
    for it in range(iters):
        p = np.exp(opt.trial if it else opt.x)
        ens.set_params(p)
        t0 = time.perf_counter()
        loss, gp = ens.loss_grad(target)
        times.append(time.perf_counter() - t0)
        gx = gp * p  # d/dlog(p)
        if it == 0:
            opt.first(loss, gx)
        else:
            opt.accept(loss, gx)
        if p_true is not None:
            frac = recovered_fraction(np.exp(opt.x), p_true, mask, tol)
            recovered.append(frac)
            rel = np.abs(np.exp(opt.x) - np.asarray(p_true)) / np.abs(np.asarray(p_true))
            each.append(np.all((rel < tol) | ~mask, axis=1))
            if log:
                log(f"iter {it + 1}: recovered {frac:.3f}, median loss {np.median(opt.f):.3e}")
            if frac >= (1.0 if stop_at is None else stop_at):
                converged_at = it + 1
                break
    out = {"params": np.exp(opt.x), "iterations": len(times), "iter_s": times, "converged_at": converged_at,
           "loss": opt.f.copy()}
    if p_true is not None:
        out["rel_err"] = np.abs(out["params"] - np.asarray(p_true)) / np.abs(np.asarray(p_true))
        out["recovered"] = recovered
        out["recovered_each"] = each  # per iteration: (B,) booleans
    return out


def calibrate_fd(instances, steps: int, iters: int, tol: float = 1e-3, rel_step: float = 1e-6, loop: int = 1):
    """The same optimiser driven by the plain drop-in's central differences
    (``FDSession.fd_grad``: five forward runs per instance and iteration):
    the comparison arm's own trajectory.  `instances`: (z, h, target, p0,
    p_true, mask) per instance; they run one after another (the drop-in
    program keeps its state in globals: one session at a time).  Returns the
    recovered fraction after each iteration and the wall time of each
    iteration summed over the instances."""
    rec = np.zeros((len(instances), iters), dtype=bool)
    times = np.zeros(iters)
    for b, (z, h, target, p0, p_true, mask) in enumerate(instances):
        p0 = np.asarray(p0, dtype=np.float64).reshape(1, 2)
        sess = FDSession(z, h, p0[0, 0], p0[0, 1], steps, target, loop=loop)
        try:
            opt = _BFGS(np.log(p0))
            for it in range(iters):
                p = np.exp(opt.trial if it else opt.x)
                t0 = time.perf_counter()
                f, g = sess.fd_grad(p[0, 0], p[0, 1], rel_step)
                times[it] += time.perf_counter() - t0
                gx = (np.asarray(g) * p[0])[None]
                if it == 0:
                    opt.first(np.array([f]), gx)
                else:
                    opt.accept(np.array([f]), gx)
                rec[b, it] = recovered_fraction(np.exp(opt.x), np.asarray(p_true).reshape(1, 2),
                                                np.asarray(mask).reshape(1, 2), tol) == 1.0
        finally:
            sess.close()
    return {"recovered": rec.mean(axis=0).tolist(), "iter_s": times.tolist()}


class FDSession:
    """The comparison arm: one instance as the plain GPU drop-in (the C-API
    program of the reference's SCIDDICA-T example, split step, recorded step
    replayed), with losses from host-side read-back.  The example program
    keeps its substates in globals, as the reference's does: one session is
    open at a time."""

    def __init__(self, z, h, p_r, p_eps, steps, target: np.ndarray, loop: int = 1):
        """loop: 1 = the recorded step replayed (the drop-in's run loop), 4 =
        every step in one cooperative launch (the fastest single-grid loop)"""
        self._lib = _lib()
        self.loop = int(loop)
        z = np.ascontiguousarray(z, np.float64)
        h = np.ascontiguousarray(h, np.float64)
        self.rows, self.cols = z.shape
        self.steps = int(steps)
        self.target = np.ascontiguousarray(target, np.float64)
        self.out = np.empty_like(self.target)
        self.handle = self._lib.cal_sciddicaT_open(self.rows, self.cols, 0, 0, float(p_r), float(p_eps),
                                                   _ptr(z, C.c_double), _ptr(h, C.c_double), 1)
        if not self.handle:
            raise CALError("cal_sciddicaT_open failed")

    def loss(self, p_r, p_eps) -> float:
        lib = self._lib
        lib.cal_sciddicaT_set_params(self.handle, float(p_r), float(p_eps))
        lib.cal_sciddicaT_reset(self.handle)
        if lib.cal_sciddicaT_steps(self.handle, self.steps, self.loop):
            raise CALError("cal_sciddicaT_steps failed")
        if lib.cal_sciddicaT_read(self.handle, _ptr(self.out, C.c_double)):
            raise CALError("cal_sciddicaT_read failed")
        d = self.out - self.target
        return float(np.dot(d.ravel(), d.ravel()))

    def fd_grad(self, p_r, p_eps, rel_step: float = 1e-6):
        """loss and central-difference gradient: five forward runs"""
        f0 = self.loss(p_r, p_eps)
        hr = rel_step * p_r
        he = rel_step * p_eps
        gr = (self.loss(p_r + hr, p_eps) - self.loss(p_r - hr, p_eps)) / (2 * hr)
        ge = (self.loss(p_r, p_eps + he) - self.loss(p_r, p_eps - he)) / (2 * he)
        return f0, np.array([gr, ge])

    def close(self):
        if getattr(self, "handle", None):
            self._lib.cal_sciddicaT_close(self.handle)
            self.handle = None

    def __del__(self):
        self.close()
