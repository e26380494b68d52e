"""Batched solves through the C ABI (mexk_batch_*): many independent
problems, each a CSR matrix, a time t and a block of up to 16 right-hand
sides, advanced together in mixed precision.

    with Batch(m=30, tol=1e-6) as b:
        for A, V, t in problems:          # V: (nrhs, n)
            b.add(A, V, t)
        b.upload()
        b.run()
        Y, results = b.result(0)          # Y: (nrhs, n)
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import BATCH_M_MAX, BATCH_RHS, BatchInfo, BatchParams, Result, check, lib


def _ptr(a, ctype):
    return a.ctypes.data_as(C.POINTER(ctype))


class Batch:
    def __init__(self, m: int = 30, tol: float = 1e-6, max_restarts: int = 0, reorthogonalize: bool = True,
                 basis_bytes: int = 0, autotune: bool = True, device: int = 0):
        p = BatchParams(m, tol, max_restarts, 1 if reorthogonalize else 0, int(basis_bytes), 1 if autotune else 0)
        h = C.c_void_p()
        check(lib().mexk_batch_create(device, C.byref(p), C.byref(h)), "mexk_batch_create")
        self._h = h
        self._keep = []  # host arrays read again by upload
        self._shapes = []

    def add(self, A, V, t: float) -> int:
        """A: CSR with row_ptr / col_idx / values; V: (nrhs, n) start vectors."""
        V = np.atleast_2d(np.asarray(V, dtype=np.float64))
        nrhs, n = V.shape
        if n != A.n or not 1 <= nrhs <= BATCH_RHS:
            raise ValueError("V must be (nrhs, n) with 1 <= nrhs <= 16")
        rp = np.ascontiguousarray(A.row_ptr, dtype=np.int32)
        ci = np.ascontiguousarray(A.col_idx, dtype=np.int32)
        va = np.ascontiguousarray(A.values, dtype=np.float64)
        Vr = np.ascontiguousarray(V.T)  # rows x nrhs, row-major
        idx = C.c_int(-1)
        check(lib().mexk_batch_add(self._h, A.n, _ptr(rp, C.c_int), _ptr(ci, C.c_int), _ptr(va, C.c_double),
                                   float(t), nrhs, _ptr(Vr, C.c_double), C.byref(idx)), "mexk_batch_add")
        self._keep.append((rp, ci, va, Vr))
        self._shapes.append((n, nrhs))
        return idx.value

    def upload(self):
        check(lib().mexk_batch_upload(self._h), "mexk_batch_upload")
        self._keep = []

    def run(self):
        check(lib().mexk_batch_run(self._h), "mexk_batch_run")

    def result(self, index: int):
        n, nrhs = self._shapes[index]
        Y = np.zeros((n, nrhs))
        res = (Result * nrhs)()
        check(lib().mexk_batch_result(self._h, index, _ptr(Y, C.c_double), res), "mexk_batch_result")
        return np.ascontiguousarray(Y.T), [r.as_dict() for r in res]

    def info(self) -> dict:
        i = BatchInfo()
        check(lib().mexk_batch_info(self._h, C.byref(i)), "mexk_batch_info")
        return i.as_dict()

    KINDS = {"spmm": 0, "dot": 1, "update": 2}

    def profile(self, kind: str, j: int, iters: int = 3):
        """(ms per launch, wave rows, wave nonzeros) of one per-step kernel
        of the first wave at step j (after a run)."""
        ms, rows, nnz = C.c_double(), C.c_longlong(), C.c_longlong()
        check(lib().mexk_batch_profile(self._h, self.KINDS[kind], j, iters, C.byref(ms), C.byref(rows),
                                       C.byref(nnz)), "mexk_batch_profile")
        return ms.value, rows.value, nnz.value

    def close(self):
        if self._h:
            lib().mexk_batch_destroy(self._h)
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


__all__ = ["Batch", "BATCH_RHS", "BATCH_M_MAX"]
