"""ORACLE -- test infrastructure, not product code.

ctypes access to the CPU restatement (``_build/liboracle.so``) and, when it
was built in a container that has the reference tree, to the reference's own
CPU program compiled against the Eigen-subset shim (``_ref/libref_expmv.so``).
Only tests, ``__graft_entry__.smoke()`` and the benchmark's CPU leg import
this module; the CUDA product path never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libref_expmv.so")
REF_CLI = os.path.join(HERE, "_ref", "matrix_exp_cpu")

_DP = C.POINTER(C.c_double)
_IP = C.POINTER(C.c_int)


class Stepping(C.Structure):
    """TimeSteppingParams (main_cpu.cpp:417-430)."""
    _fields_ = [("dt_init", C.c_double), ("dt_min", C.c_double), ("dt_max", C.c_double), ("tol_step", C.c_double),
                ("max_steps", C.c_int), ("max_rejects", C.c_int), ("safety", C.c_double), ("grow", C.c_double),
                ("shrink", C.c_double), ("adapt_m", C.c_int), ("m_max", C.c_int), ("m_step", C.c_int)]


def stepping_defaults(m, t, tol, max_restarts) -> dict:
    """The constructor's derivation (main_cpu.cpp:453-466)."""
    return dict(dt_init=t / (max_restarts if max_restarts > 0 else 1), dt_min=max(1e-12, t * 1e-6), dt_max=t,
                tol_step=tol, max_steps=max_restarts if max_restarts > 0 else 1000, max_rejects=20, safety=0.8,
                grow=1.5, shrink=0.5, adapt_m=0, m_max=m, m_step=0)


def _stepping(m, t, tol, max_restarts, overrides):
    ts = stepping_defaults(m, t, tol, max_restarts)
    ts.update(overrides or {})
    ints = {f for f, ct in Stepping._fields_ if ct is C.c_int}
    return ts, Stepping(**{k: int(v) if k in ints else float(v) for k, v in ts.items()})


class Params(C.Structure):
    _fields_ = [("m", C.c_int), ("t", C.c_double), ("tol", C.c_double), ("max_restarts", C.c_int),
                ("reorthogonalize", C.c_int), ("max_cycles", C.c_int), ("quiet", C.c_int),
                ("stepping", C.POINTER(Stepping))]


class Stats(C.Structure):
    _fields_ = [("converged", C.c_int), ("restarts_done", C.c_int), ("last_residual", C.c_double),
                ("attempts", C.c_int), ("cycles", C.c_int), ("spmv_count", C.c_longlong),
                ("v_norm_initial", C.c_double)]


class Step(C.Structure):
    _fields_ = [("t_done", C.c_double), ("dt", C.c_double), ("err", C.c_double), ("m_used", C.c_int),
                ("accepts", C.c_int), ("rejects", C.c_int)]


def reference_dir() -> str:
    """The reference source tree: $MEXK_REFERENCE_DIR, else a `reference`
    directory beside the repository."""
    return os.environ.get("MEXK_REFERENCE_DIR") or os.path.normpath(os.path.join(HERE, "..", "..", "reference"))


def build(with_reference: bool | None = None) -> None:
    """make -C oracle (and `ref` when the reference tree is present)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    ref_dir = reference_dir()
    have = os.path.exists(os.path.join(ref_dir, "main_cpu.cpp"))
    if with_reference and not have:
        raise FileNotFoundError(f"reference tree not found at {ref_dir} (set MEXK_REFERENCE_DIR)")
    if with_reference is None:
        with_reference = have
    if with_reference:
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={ref_dir}"], check=True)


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build(with_reference=False)
        L = C.CDLL(LIB_PATH)
        L.oracle_expmv.argtypes = [C.c_int, _IP, _IP, _DP, _DP, _DP, C.POINTER(Params),
                                   C.POINTER(Stats), C.POINTER(Step), C.c_int, _IP]
        L.oracle_expmv.restype = C.c_int
        L.oracle_spmv.argtypes = [C.c_int, _IP, _IP, _DP, _DP, _DP]
        L.oracle_arnoldi_step.argtypes = [C.c_int, _IP, _IP, _DP, _DP, C.c_int, C.c_int, _DP, _DP, _DP]
        L.oracle_arnoldi_step.restype = C.c_int
        L.oracle_small_expm.argtypes = [C.c_int, _DP, C.c_int, C.c_double, C.c_double, _DP, _DP]
        L.oracle_lift.argtypes = [C.c_int, C.c_int, _DP, _DP, C.c_double, _DP]
        L.oracle_expm.argtypes = [C.c_int, _DP, _DP]
        L.oracle_expm.restype = C.c_int
        _lib = L
    return _lib


def have_reference() -> bool:
    return os.path.exists(REF_PATH)


def ref():
    global _ref
    if _ref is None:
        R = C.CDLL(REF_PATH)
        R.ref_expmv.argtypes = [C.c_int, C.c_longlong, _IP, _IP, _DP, _DP, _DP, C.c_int, C.c_double,
                                C.c_double, C.c_int, C.c_int, _IP, _IP, _DP]
        R.ref_expmv_ts.argtypes = [C.c_int, C.c_longlong, _IP, _IP, _DP, _DP, _DP, C.c_int, C.c_double,
                                   C.c_double, C.c_int, C.c_int, _DP, _IP, _IP, _IP, _DP]
        R.ref_load.argtypes = [C.c_char_p, C.c_int, _IP, _IP, C.POINTER(C.c_longlong)]
        R.ref_load.restype = C.c_void_p
        R.ref_copy_csr.argtypes = [C.c_void_p, _IP, _IP, _DP]
        R.ref_free.argtypes = [C.c_void_p]
        _ref = R
    return _ref


def _p(a, ct):
    return a.ctypes.data_as(C.POINTER(ct))


def _csr(A):
    rp = np.ascontiguousarray(A.row_ptr, dtype=np.int32)
    ci = np.ascontiguousarray(A.col_idx, dtype=np.int32)
    va = np.ascontiguousarray(A.values, dtype=np.float64)
    return rp, ci, va


def expmv(A, v, t, m, tol=1e-6, max_restarts=0, reorthogonalize=True, max_cycles=0, log_cap=4096, stepping=None):
    """Oracle y = exp(tA)v; returns (y, stats dict, list of step tuples).
    stepping: a dict of TimeSteppingParams overrides (None: the defaults)."""
    rp, ci, va = _csr(A)
    v = np.ascontiguousarray(v, dtype=np.float64)
    y = np.zeros(A.n)
    p = Params(m, t, tol, max_restarts, int(reorthogonalize), max_cycles, 1, None)
    if stepping is not None:
        _, ts = _stepping(m, t, tol, max_restarts, stepping)
        p.stepping = C.pointer(ts)
    st = Stats()
    log = (Step * log_cap)()
    nlog = C.c_int(0)
    rc = lib().oracle_expmv(A.n, _p(rp, C.c_int), _p(ci, C.c_int), _p(va, C.c_double),
                            _p(v, C.c_double), _p(y, C.c_double), C.byref(p), C.byref(st), log,
                            log_cap, C.byref(nlog))
    if rc != 0:
        raise RuntimeError("oracle_expmv failed")
    steps = [(s.t_done, s.dt, s.err, s.m_used, s.accepts, s.rejects) for s in log[: nlog.value]]
    stats = {k: getattr(st, k) for k, _ in Stats._fields_}
    return y, stats, steps


def spmv(A, x):
    rp, ci, va = _csr(A)
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.zeros(A.n)
    lib().oracle_spmv(A.n, _p(rp, C.c_int), _p(ci, C.c_int), _p(va, C.c_double), _p(x, C.c_double),
                      _p(y, C.c_double))
    return y


def arnoldi_step(A, V, j, reorthogonalize=True):
    """In-place step on a column-major basis V with shape (m+1, n) (row = basis vector)."""
    rp, ci, va = _csr(A)
    assert V.flags.c_contiguous and V.dtype == np.float64
    w = np.zeros(A.n)
    h = np.zeros(j + 1)
    beta = C.c_double(0.0)
    ok = lib().oracle_arnoldi_step(A.n, _p(rp, C.c_int), _p(ci, C.c_int), _p(va, C.c_double),
                                   _p(V, C.c_double), j, int(reorthogonalize), _p(w, C.c_double),
                                   _p(h, C.c_double), C.byref(beta))
    return bool(ok), h, beta.value, w


def expm(M):
    M = np.asfortranarray(M, dtype=np.float64)
    k = M.shape[0]
    E = np.zeros((k, k), order="F")
    lib().oracle_expm(k, M.ctypes.data_as(_DP), E.ctypes.data_as(_DP))
    return E


def small_expm(H, k, dt, v_norm):
    """H: (m+1, m) array (any order). Returns (wH of length k+1, err)."""
    Hf = np.asfortranarray(H, dtype=np.float64)
    wH = np.zeros(k + 1)
    err = C.c_double(0.0)
    lib().oracle_small_expm(k, Hf.ctypes.data_as(_DP), Hf.shape[0], dt, v_norm, _p(wH, C.c_double),
                            C.byref(err))
    return wH, err.value


def lift(V, k, wH, v_norm):
    """V: (m+1, n) C-contiguous rows = basis vectors."""
    n = V.shape[1]
    y = np.zeros(n)
    lib().oracle_lift(n, k, _p(np.ascontiguousarray(V), C.c_double),
                      _p(np.ascontiguousarray(wH, dtype=np.float64), C.c_double), v_norm,
                      _p(y, C.c_double))
    return y


def reference_expmv(A, v, t, m, tol=1e-6, max_restarts=0, reorthogonalize=True, capture=True, stepping=None):
    """The reference's own ArnoldiRunnerCPU (built from main_cpu.cpp). Returns
    (y, stats dict, [STEP] lines). stepping: TimeSteppingParams overrides set
    on the runner before compute_expmv."""
    rp, ci, va = _csr(A)
    v = np.ascontiguousarray(v, dtype=np.float64)
    y = np.zeros(A.n)
    rd, cv = C.c_int(0), C.c_int(0)
    res = C.c_double(0.0)
    import tempfile

    lines = []
    with tempfile.TemporaryFile(mode="w+b") as tmp:
        saved = os.dup(1) if capture else None
        if capture:
            os.dup2(tmp.fileno(), 1)
        try:
            if stepping is None:
                ref().ref_expmv(A.n, A.nnz, _p(rp, C.c_int), _p(ci, C.c_int), _p(va, C.c_double),
                                _p(v, C.c_double), _p(y, C.c_double), m, t, tol, max_restarts,
                                int(reorthogonalize), C.byref(rd), C.byref(cv), C.byref(res))
            else:
                ts, _ = _stepping(m, t, tol, max_restarts, stepping)
                tsd = np.array([ts[k] for k in ("dt_init", "dt_min", "dt_max", "tol_step", "safety", "grow",
                                                "shrink")], dtype=np.float64)
                tsi = np.array([ts[k] for k in ("max_steps", "max_rejects", "adapt_m", "m_max", "m_step")],
                               dtype=np.int32)
                ref().ref_expmv_ts(A.n, A.nnz, _p(rp, C.c_int), _p(ci, C.c_int), _p(va, C.c_double),
                                   _p(v, C.c_double), _p(y, C.c_double), m, t, tol, max_restarts,
                                   int(reorthogonalize), _p(tsd, C.c_double), _p(tsi, C.c_int), C.byref(rd),
                                   C.byref(cv), C.byref(res))
        finally:
            if capture:
                os.dup2(saved, 1)
                os.close(saved)
        if capture:
            tmp.seek(0)
            lines = [ln for ln in tmp.read().decode().splitlines() if ln.startswith("[STEP]")]
    return y, {"restarts_done": rd.value, "converged": cv.value, "last_residual": res.value}, lines
