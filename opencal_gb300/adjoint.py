"""SCIDDICA-T rollout as a differentiable torch function (calibration only).

``rollout(z_dem, h0, p_r, p_eps, steps)`` runs ``steps`` plain-mode steps
on the GPU (the bit-exact fused step kernel) and returns h_T; its backward
calls the hand-written adjoint kernels of ``libopencal_models.so``
(csrc/models/sciddicaT_adjoint.cu): elimination sets recomputed from the
forward states and frozen, sqrt(T) checkpointing, gradients with respect to
h0 (including the initialisation's z -= h0), p_r and p_eps.  Torch is used
for device memory and streams only; the library itself stays C.
"""
from __future__ import annotations

import ctypes as C

import torch

from . import models as _models

_bound = False


def _lib():
    global _bound
    m = _models()
    if not _bound:
        m.cal_sdt_adj_create.restype = C.c_void_p
        m.cal_sdt_adj_create.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int]
        m.cal_sdt_adj_destroy.argtypes = [C.c_void_p]
        m.cal_sdt_adj_forward.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_void_p,
                                          C.c_void_p]
        m.cal_sdt_adj_backward.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_double),
                                           C.POINTER(C.c_double), C.c_void_p]
        _bound = True
    return m


class _Workspace:
    def __init__(self, rows, cols, steps, toroidal):
        self.handle = _lib().cal_sdt_adj_create(rows, cols, steps, int(toroidal))
        if not self.handle:
            raise MemoryError("cal_sdt_adj_create failed")

    def __del__(self):
        if getattr(self, "handle", None):
            _lib().cal_sdt_adj_destroy(self.handle)
            self.handle = None


class SciddicaTRollout(torch.autograd.Function):
    @staticmethod
    def forward(ctx, z_dem, h0, p_r, p_eps, steps, toroidal):
        assert z_dem.is_cuda and z_dem.dtype == torch.float64 and h0.shape == z_dem.shape
        z_dem = z_dem.contiguous()
        h0 = h0.contiguous()
        rows, cols = h0.shape
        ws = _Workspace(rows, cols, int(steps), toroidal)
        hT = torch.empty_like(h0)
        stream = torch.cuda.current_stream().cuda_stream
        rc = _lib().cal_sdt_adj_forward(ws.handle, z_dem.data_ptr(), h0.data_ptr(), float(p_r), float(p_eps),
                                        hT.data_ptr(), stream)
        if rc:
            raise RuntimeError(f"cal_sdt_adj_forward failed ({rc})")
        ctx.ws = ws
        ctx.keep = (z_dem, h0)
        ctx.p_dtype = p_r.dtype if torch.is_tensor(p_r) else torch.float64
        return hT

    @staticmethod
    def backward(ctx, grad_hT):
        grad_hT = grad_hT.contiguous()
        g_h0 = torch.empty_like(grad_hT)
        gr = C.c_double(0.0)
        ge = C.c_double(0.0)
        stream = torch.cuda.current_stream().cuda_stream
        rc = _lib().cal_sdt_adj_backward(ctx.ws.handle, grad_hT.data_ptr(), g_h0.data_ptr(), C.byref(gr),
                                         C.byref(ge), stream)
        if rc:
            raise RuntimeError(f"cal_sdt_adj_backward failed ({rc})")
        dev = grad_hT.device
        return (None, g_h0, torch.tensor(gr.value, dtype=torch.float64, device=dev),
                torch.tensor(ge.value, dtype=torch.float64, device=dev), None, None)


def rollout(z_dem, h0, p_r, p_eps, steps, toroidal=False):
    """h_T of a SCIDDICA-T run; differentiable w.r.t. h0, p_r and p_eps."""
    if not torch.is_tensor(p_r):
        p_r = torch.tensor(float(p_r), dtype=torch.float64, device=h0.device)
    if not torch.is_tensor(p_eps):
        p_eps = torch.tensor(float(p_eps), dtype=torch.float64, device=h0.device)
    return SciddicaTRollout.apply(z_dem, h0, p_r, p_eps, steps, toroidal)
