"""Continuous correlator of the fine search: power, gradient, Hessian, Newton refinement and
the adjoint with respect to the samples (C ABI ``acq_corr_*`` in include/acqgb300.h).

The grid search reports code phase and Doppler on the plan's bins and refines them by a
parabola through neighbouring bins (src/acquire.jl:9-13,713-740). This module evaluates the
correlator power P(code phase, Doppler) = |sum_n x[n] c(phi_n) exp(-i theta_n)|^2 at any
continuous point, with its closed-form derivatives, and refines peaks by batched Newton steps.

``CorrelatorPower`` is the ``torch.autograd.Function`` of P: its backward pass calls the
adjoint kernel, which recomputes the code replica instead of storing it, for the cotangent of
the samples, and uses the forward pass's closed-form gradient for code phase and Doppler.

Device memory is torch's; every call runs on torch's current stream of the tensor's device.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib as L
from .api import ArgumentError, GNSSSystem, _check

CELL_DTYPE = np.dtype([("prn", "<i4"), ("reserved", "<i4"), ("code_phase", "<f8"), ("doppler_hz", "<f8")])
RESULT_DTYPE = np.dtype([("power", "<f8"), ("grad", "<f8", (2,)), ("hess", "<f8", (3,)), ("z_re", "<f8"),
                         ("z_im", "<f8"), ("iterations", "<i4"), ("status", "<i4")])
assert CELL_DTYPE.itemsize == C.sizeof(L.CorrCell) and RESULT_DTYPE.itemsize == C.sizeof(L.CorrResult)

_DT = {"complex64": L.ACQ_CF32, "complex128": L.ACQ_CF64}


def _torch():
    import torch
    return torch


def _stream(t) -> int:
    torch = _torch()
    return torch.cuda.current_stream(t.device).cuda_stream


def _samples(x):
    """(device tensor, dtype code, n) for a CUDA tensor: complex64/complex128, or (n, 2) int16 / int8."""
    torch = _torch()
    if not isinstance(x, torch.Tensor) or not x.is_cuda:
        raise ArgumentError("samples must be a CUDA tensor")
    x = x.contiguous()
    if x.dtype == torch.complex64:
        return x, L.ACQ_CF32, x.numel()
    if x.dtype == torch.complex128:
        return x, L.ACQ_CF64, x.numel()
    if x.dim() == 2 and x.shape[1] == 2 and x.dtype in (torch.int16, torch.int8):
        return x, (L.ACQ_CI16 if x.dtype == torch.int16 else L.ACQ_CI8), x.shape[0]
    raise ArgumentError(f"unsupported sample tensor {x.dtype} {tuple(x.shape)}")


def pack_cells(prns, code_phase, doppler) -> np.ndarray:
    prns, code_phase, doppler = np.broadcast_arrays(np.asarray(prns), np.asarray(code_phase, dtype=np.float64),
                                                    np.asarray(doppler, dtype=np.float64))
    c = np.zeros(prns.size, dtype=CELL_DTYPE)
    c["prn"] = prns.reshape(-1)
    c["code_phase"] = code_phase.reshape(-1)
    c["doppler_hz"] = doppler.reshape(-1)
    return c


@dataclass
class CorrEval:
    """Per-cell results (numpy arrays): power, grad (n, 2), hess (n, 3) = (tt, tf, ff), z (complex)."""
    power: np.ndarray
    grad: np.ndarray
    hess: np.ndarray
    z: np.ndarray
    iterations: np.ndarray
    status: np.ndarray
    code_phase: np.ndarray | None = None
    doppler: np.ndarray | None = None


def _unpack(raw: np.ndarray, cells: np.ndarray | None = None) -> CorrEval:
    r = raw.view(RESULT_DTYPE)
    return CorrEval(r["power"].copy(), r["grad"].copy(), r["hess"].copy(), r["z_re"] + 1j * r["z_im"],
                    r["iterations"].copy(), r["status"].copy(),
                    None if cells is None else cells["code_phase"].copy(),
                    None if cells is None else cells["doppler_hz"].copy())


class Correlator:
    """Context for one system and sampling rate over a PRN set (chip tables on the device)."""

    def __init__(self, system: GNSSSystem, sampling_freq: float, prns, *, device: int = 0, codes=None):
        torch = _torch()
        self.system, self.fs, self.prns = system, float(sampling_freq), [int(p) for p in prns]
        self.device = torch.device("cuda", device)
        lib = L.load()
        pa = (C.c_int32 * len(self.prns))(*self.prns)
        cp = None
        if codes is not None:
            self._codes = np.ascontiguousarray(codes, dtype=np.int8)
            cp = self._codes.ctypes.data_as(C.POINTER(C.c_int8))
        h = C.c_void_p()
        with torch.cuda.device(self.device):
            _check(lib.acq_corr_create(system.sid, self.fs, pa, len(self.prns), cp, C.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            L.load().acq_corr_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- device-level calls (tensors in, tensors out) -------------------------------------------
    def _cells_dev(self, cells: np.ndarray):
        torch = _torch()
        return torch.from_numpy(cells.view(np.uint8).copy()).to(self.device)

    def eval_device(self, x, cells_dev, n_cells: int, hessian: bool = False, interm_freq: float = 0.0):
        """Raw results (uint8 tensor of n_cells x 72 bytes) for cells already on the device."""
        torch = _torch()
        xs, dt, n = _samples(x)
        out = torch.empty(n_cells * RESULT_DTYPE.itemsize, dtype=torch.uint8, device=self.device)
        _check(L.load().acq_corr_eval(self._h, C.c_void_p(xs.data_ptr()), dt, int(n), float(interm_freq),
                                      C.c_void_p(cells_dev.data_ptr()), int(n_cells), int(bool(hessian)),
                                      C.c_void_p(out.data_ptr()), C.c_void_p(_stream(xs))))
        return out

    def vjp_device(self, n: int, cells_dev, n_cells: int, zbar, interm_freq: float = 0.0):
        """x_bar (complex64 tensor of n) = sum_c zbar_c conj(dz_c/dx) for device cells and cotangents."""
        torch = _torch()
        zb = torch.view_as_real(zbar.to(torch.complex64).contiguous()).contiguous()
        xbar = torch.empty(int(n), dtype=torch.complex64, device=self.device)
        _check(L.load().acq_corr_vjp_samples(self._h, int(n), float(interm_freq), C.c_void_p(cells_dev.data_ptr()),
                                             C.c_void_p(zb.data_ptr()), int(n_cells), C.c_void_p(xbar.data_ptr()),
                                             C.c_void_p(_stream(xbar))))
        return xbar

    def refine_device(self, x, cells_dev, n_cells: int, *, max_iterations=20, tol_chips=1e-4, tol_hz=1e-3,
                      max_step_chips=0.25, max_step_hz=None, interm_freq=0.0):
        torch = _torch()
        xs, dt, n = _samples(x)
        if max_step_hz is None:
            max_step_hz = 0.25 * self.fs / n     # a quarter of a Doppler bin of the coherent time
        out = torch.empty(n_cells * RESULT_DTYPE.itemsize, dtype=torch.uint8, device=self.device)
        _check(L.load().acq_corr_refine(self._h, C.c_void_p(xs.data_ptr()), dt, int(n), float(interm_freq),
                                        C.c_void_p(cells_dev.data_ptr()), int(n_cells), int(max_iterations),
                                        float(tol_chips), float(tol_hz), float(max_step_chips), float(max_step_hz),
                                        C.c_void_p(out.data_ptr()), C.c_void_p(_stream(xs))))
        return out

    # -- host conveniences --------------------------------------------------------------------
    def eval(self, x, prns, code_phase, doppler, *, hessian=False, interm_freq=0.0) -> CorrEval:
        cells = pack_cells(prns, code_phase, doppler)
        raw = self.eval_device(x, self._cells_dev(cells), cells.size, hessian, interm_freq)
        return _unpack(raw.cpu().numpy())

    def refine(self, x, prns, code_phase, doppler, **kw) -> CorrEval:
        cells = pack_cells(prns, code_phase, doppler)
        cd = self._cells_dev(cells)
        raw = self.refine_device(x, cd, cells.size, **kw)
        out = _unpack(raw.cpu().numpy(), cd.cpu().numpy().view(CELL_DTYPE))
        return out

    def vjp_samples(self, n, prns, code_phase, doppler, zbar, *, interm_freq=0.0):
        torch = _torch()
        cells = pack_cells(prns, code_phase, doppler)
        zb = torch.as_tensor(np.asarray(zbar, dtype=np.complex64), device=self.device)
        return self.vjp_device(n, self._cells_dev(cells), cells.size, zb, interm_freq)


def _autograd_function():
    torch = _torch()

    class CorrelatorPower(torch.autograd.Function):
        """P = |z(code_phase, doppler; x)|^2 per cell. Inputs: samples (complex64 CUDA tensor),
        code_phase and doppler (float64 CUDA tensors of n cells); PRNs are fixed per call."""

        @staticmethod
        def forward(ctx, x, code_phase, doppler, corr, prns, interm_freq):
            cells = pack_cells(np.asarray(prns), code_phase.detach().cpu().numpy(), doppler.detach().cpu().numpy())
            cd = corr._cells_dev(cells)
            raw = corr.eval_device(x.detach(), cd, cells.size, False, interm_freq)
            r = raw.view(torch.float64)[: cells.size * 9].view(cells.size, 9)
            power, grad, z = r[:, 0], r[:, 1:3], torch.complex(r[:, 6], r[:, 7])
            ctx.save_for_backward(grad, z, cd)
            ctx.corr, ctx.n, ctx.ncell, ctx.fi = corr, x.numel(), cells.size, interm_freq
            return power.to(code_phase.dtype).reshape(code_phase.shape)

        @staticmethod
        def backward(ctx, pbar):
            grad, z, cd = ctx.saved_tensors
            pb = pbar.reshape(-1).to(torch.float64)
            gx = gt = gf = None
            if ctx.needs_input_grad[0]:
                zbar = (2.0 * pb * z).to(torch.complex64)
                gx = ctx.corr.vjp_device(ctx.n, cd, ctx.ncell, zbar, ctx.fi)
            if ctx.needs_input_grad[1]:
                gt = (pb * grad[:, 0]).reshape(pbar.shape)
            if ctx.needs_input_grad[2]:
                gf = (pb * grad[:, 1]).reshape(pbar.shape)
            return gx, gt, gf, None, None, None

    return CorrelatorPower


_CP = None


def correlator_power(corr: Correlator, x, prns, code_phase, doppler, interm_freq: float = 0.0):
    """Differentiable P(code_phase, doppler; x) for every cell (torch autograd)."""
    global _CP
    if _CP is None:
        _CP = _autograd_function()
    return _CP.apply(x, code_phase, doppler, corr, list(np.asarray(prns).reshape(-1)), float(interm_freq))
