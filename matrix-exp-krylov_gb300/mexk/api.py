"""Python mirror of the reference's solver interface, over the mexk C ABI.

``Context`` plays the reference's DeviceContext + ArnoldiRunner
(main.cu:747-1125, 1253-2081): upload a CSR matrix once, then call
``expmv`` (host vectors, like ArnoldiRunner::compute_expmv) or
``expmv_device`` (device pointers). Results carry the reference's
``converged`` / ``restarts_done`` / ``last_residual`` fields.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from ._lib import (M_MAX, M_MAX_MIXED, PREC_FP64, PREC_MIXED, Params, Result, Step, Stepping, check,
                   default_stepping, lib)

PRECISIONS = {"fp64": PREC_FP64, "mixed": PREC_MIXED}


def _ptr(a, ct):
    return a.ctypes.data_as(C.POINTER(ct))


CONTROLLERS = {"reference": 0, "search": 1, "learned": 2}


def params(m, t, tol=1e-6, max_restarts=0, reorthogonalize=True, precision="fp64",
           controller="reference", window=0, stepping=None) -> Params:
    """window: 0 = orthogonalise against the whole basis (Arnoldi); W >= 2 =
    against the last W vectors (mixed precision, symmetric A only).
    stepping: None (TimeSteppingParams derived from m, t, tol, max_restarts as
    the reference's constructor does) or a dict overriding some of them
    (dt_init, dt_min, dt_max, tol_step, max_steps, max_rejects, safety, grow,
    shrink, adapt_m, m_max, m_step)."""
    prec = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
    ctrl = CONTROLLERS[controller] if isinstance(controller, str) else int(controller)
    p = Params(int(m), float(t), float(tol), int(max_restarts), int(bool(reorthogonalize)), prec, ctrl,
               int(window), None)
    if stepping is not None:
        ts = default_stepping(int(m), float(t), float(tol), int(max_restarts))
        unknown = set(stepping) - set(ts)
        if unknown:
            raise ValueError(f"unknown time-stepping parameters {sorted(unknown)}")
        ts.update(stepping)
        ints = {f for f, ct in Stepping._fields_ if ct is C.c_int}
        p._stepping = Stepping(**{k: int(v) if k in ints else float(v) for k, v in ts.items()})  # kept alive with p
        p.stepping = C.pointer(p._stepping)
    return p


class Context:
    """One device's copy of A plus basis and work buffers."""

    def __init__(self, A, m_alloc: int = 30, device: int = 0):
        self._h = C.c_void_p()
        self._net_loaded = False
        check(lib().mexk_context_create(device, C.byref(self._h)), "mexk_context_create")
        if A is None:  # filled by from_bincsr
            return
        self.n = int(A.n)
        self.nnz = int(A.nnz)
        self.m_alloc = int(m_alloc)
        rp = np.ascontiguousarray(A.row_ptr, dtype=np.int32)
        ci = np.ascontiguousarray(A.col_idx, dtype=np.int32)
        va = np.ascontiguousarray(A.values, dtype=np.float64)
        try:
            check(lib().mexk_context_upload_csr(self._h, self.n, self.nnz, _ptr(rp, C.c_int), _ptr(ci, C.c_int),
                                                _ptr(va, C.c_double), self.m_alloc), "mexk_context_upload_csr")
        except Exception:
            self.close()
            raise

    @classmethod
    def from_bincsr(cls, path, m_alloc: int = 30, device: int = 0):
        """A context loaded straight from a Binary CSR v1 file
        (mexk_context_load_bincsr); .load_info holds the header fields,
        max |a_ij| and the load's wall time."""
        from ._lib import BincsrInfo

        ctx = cls(None, m_alloc, device)
        info = BincsrInfo()
        try:
            check(lib().mexk_context_load_bincsr(ctx._h, os.fsencode(str(path)), int(m_alloc), C.byref(info)),
                  "mexk_context_load_bincsr")
        except Exception:
            ctx.close()
            raise
        ctx.n, ctx.nnz, ctx.m_alloc = int(info.rows), int(info.nnz), int(m_alloc)
        ctx.load_info = {f: getattr(info, f) for f, _ in info._fields_}
        return ctx

    @property
    def handle(self):
        return self._h

    @property
    def stream(self) -> int:
        return lib().mexk_context_stream(self._h) or 0

    def close(self):
        if self._h:
            lib().mexk_context_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def load_controller(self, path=None, window_path=None):
        """Loads the learned controller's networks (default: the trained files
        shipped with the package): the one for full Gram-Schmidt cycles and,
        when its file exists, the one for solves with a window of 2."""
        from . import controller as K

        w = np.ascontiguousarray(K.load(path or K.WEIGHTS), dtype=np.float32)
        check(lib().mexk_context_set_controller(self._h, w.ctypes.data_as(C.POINTER(C.c_float)), w.size),
              "mexk_context_set_controller")
        wp = window_path or (K.WINDOW_WEIGHTS if path is None else None)
        if wp and os.path.exists(wp):
            ww = np.ascontiguousarray(K.load(wp), dtype=np.float32)
            check(lib().mexk_context_set_window_controller(self._h, ww.ctypes.data_as(C.POINTER(C.c_float)),
                                                           ww.size), "mexk_context_set_window_controller")
        self._net_loaded = True

    def _ensure_net(self, controller):
        if controller in ("learned", 2) and not self._net_loaded:
            self.load_controller()

    def expmv(self, v, t, m, tol=1e-6, max_restarts=0, reorthogonalize=True, precision="fp64",
              controller="reference", window=0, stepping=None):
        """y = exp(t A) v with host vectors. Returns (y, result dict)."""
        self._ensure_net(controller)
        v = np.ascontiguousarray(v, dtype=np.float64)
        if v.shape != (self.n,):
            raise ValueError("v must have length n")
        y = np.zeros(self.n)
        p = params(m, t, tol, max_restarts, reorthogonalize, precision, controller, window, stepping)
        r = Result()
        check(lib().mexk_expmv(self._h, C.byref(p), _ptr(v, C.c_double), _ptr(y, C.c_double), C.byref(r)),
              "mexk_expmv")
        return y, r.as_dict()

    def expmv_device(self, v_ptr: int, y_ptr: int, t, m, tol=1e-6, max_restarts=0, reorthogonalize=True,
                     precision="fp64", stream: int = 0, controller="reference", window=0, stepping=None):
        self._ensure_net(controller)
        p = params(m, t, tol, max_restarts, reorthogonalize, precision, controller, window, stepping)
        r = Result()
        check(lib().mexk_expmv_device(self._h, C.byref(p), C.c_void_p(v_ptr), C.c_void_p(y_ptr),
                                      C.c_void_p(stream), C.byref(r)), "mexk_expmv_device")
        return r.as_dict()

    def steps(self):
        cnt = C.c_int(0)
        check(lib().mexk_get_steps(self._h, None, 0, C.byref(cnt)), "mexk_get_steps")
        n = cnt.value
        buf = (Step * max(n, 1))()
        check(lib().mexk_get_steps(self._h, buf, n, C.byref(cnt)), "mexk_get_steps")
        return [(s.t_done, s.dt, s.err, s.m_used, s.accepts, s.rejects) for s in buf[: min(n, len(buf))]]

    def set_basis(self, V_cols: np.ndarray, precision="fp64"):
        """V_cols: (ncols, n) array, row i = basis column i."""
        V = np.ascontiguousarray(V_cols, dtype=np.float64)
        check(lib().mexk_context_set_basis(self._h, PRECISIONS[precision], _ptr(V, C.c_double), V.shape[0]),
              "mexk_context_set_basis")

    def get_basis(self, ncols: int, precision="fp64") -> np.ndarray:
        V = np.zeros((ncols, self.n))
        check(lib().mexk_context_get_basis(self._h, PRECISIONS[precision], _ptr(V, C.c_double), ncols),
              "mexk_context_get_basis")
        return V

    def profile_kernel(self, kind: str, j: int, iters: int = 3, precision="fp64") -> float:
        """Mean CUDA-event duration (ms) of one solver kernel at Arnoldi step j."""
        from ._lib import KERNELS

        ms = C.c_double(0.0)
        check(lib().mexk_profile_kernel(self._h, KERNELS[kind], PRECISIONS[precision], j, iters, C.byref(ms)),
              "mexk_profile_kernel")
        return ms.value

    SPMV_FORMS = ("staged", "direct", "pattern")

    def spmv_form(self, precision="fp64") -> str:
        """The SpMV form the context runs for a precision: "pattern" (one
        byte per row naming one of <= 256 distinct rows; the default when the
        matrix has that form), "staged" (CSR tiles staged in shared memory;
        the default when every row block's columns span less than 65,536) or
        "direct" (one block per CSR row block)."""
        f = C.c_int(0)
        check(lib().mexk_context_get_spmv_form(self._h, PRECISIONS[precision], C.byref(f)),
              "mexk_context_get_spmv_form")
        return self.SPMV_FORMS[f.value]

    def set_spmv_form(self, form: str, precision="fp64") -> None:
        check(lib().mexk_context_set_spmv_form(self._h, PRECISIONS[precision], self.SPMV_FORMS.index(form)),
              "mexk_context_set_spmv_form")

    LANCZOS_FORMS = ("stepwise", "fused")

    def lanczos_form(self) -> str:
        """How window-2 bases run their steps: "stepwise" (two launches per
        step, the default) or "fused" (one cooperative launch per basis, when
        selected and the basis's rows fit)."""
        f = C.c_int(0)
        check(lib().mexk_context_get_lanczos_form(self._h, C.byref(f)), "mexk_context_get_lanczos_form")
        return self.LANCZOS_FORMS[f.value]

    def set_lanczos_form(self, form: str) -> None:
        check(lib().mexk_context_set_lanczos_form(self._h, self.LANCZOS_FORMS.index(form)),
              "mexk_context_set_lanczos_form")

    def arnoldi_step(self, j: int, reorthogonalize=True, precision="fp64"):
        h = np.zeros(j + 1)
        beta = C.c_double(0.0)
        ok = C.c_int(0)
        check(lib().mexk_arnoldi_step(self._h, j, int(reorthogonalize), PRECISIONS[precision], _ptr(h, C.c_double),
                                      C.byref(beta), C.byref(ok)), "mexk_arnoldi_step")
        return bool(ok.value), h, beta.value


def device_count() -> int:
    c = C.c_int(0)
    check(lib().mexk_device_count(C.byref(c)), "mexk_device_count")
    return c.value


__all__ = ["Context", "params", "device_count", "PRECISIONS", "M_MAX", "M_MAX_MIXED"]
