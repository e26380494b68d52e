"""ctypes binding of the mexk C ABI (include/mexk.h).

Loads ``_build/libmexk.so`` (built in-tree by ``mexk.build`` /
``__graft_entry__.build()``). There is no fallback: if the library is
missing, every call raises.
"""
from __future__ import annotations

import ctypes as C
import os
import re

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ROOT = os.path.dirname(PKG)
BUILD = os.path.join(PKG, "_build")
LIB_PATH = os.path.join(BUILD, "libmexk.so")
HOST_LIB_PATH = os.path.join(BUILD, "libmexk_host.so")
HEADER = os.path.join(ROOT, "include", "mexk.h")

MEXK_OK = 0
PREC_FP64 = 0
PREC_MIXED = 1
M_MAX = 128
M_MAX_MIXED = 64
CTRL_REFERENCE = 0
CTRL_SEARCH = 1
CTRL_LEARNED = 2


class MexkError(RuntimeError):
    pass


class Stepping(C.Structure):
    """mexk_stepping_t: the reference's TimeSteppingParams (main.cu:1237-1250)."""
    _fields_ = [("dt_init", C.c_double), ("dt_min", C.c_double), ("dt_max", C.c_double), ("tol_step", C.c_double),
                ("max_steps", C.c_int), ("max_rejects", C.c_int), ("safety", C.c_double), ("grow", C.c_double),
                ("shrink", C.c_double), ("adapt_m", C.c_int), ("m_max", C.c_int), ("m_step", C.c_int)]


def default_stepping(m, t, tol, max_restarts) -> dict:
    """TimeSteppingParams as the reference's ArnoldiRunner constructor derives
    them from ArnoldiParams (main.cu:1292-1305)."""
    return dict(dt_init=t / (max_restarts if max_restarts > 0 else 1), dt_min=max(1e-12, t * 1e-6), dt_max=t,
                tol_step=tol, max_steps=max_restarts if max_restarts > 0 else 1000, max_rejects=20, safety=0.8,
                grow=1.5, shrink=0.5, adapt_m=0, m_max=m, m_step=0)


class Params(C.Structure):
    _fields_ = [("m", C.c_int), ("t", C.c_double), ("tol", C.c_double), ("max_restarts", C.c_int),
                ("reorthogonalize", C.c_int), ("precision", C.c_int), ("controller", C.c_int),
                ("ortho_window", C.c_int), ("stepping", C.POINTER(Stepping))]


class Result(C.Structure):
    _fields_ = [("converged", C.c_int), ("restarts_done", C.c_int), ("last_residual", C.c_double),
                ("attempts", C.c_int), ("cycles", C.c_int), ("spmv_count", C.c_longlong),
                ("t_done", C.c_double), ("status", C.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Step(C.Structure):
    _fields_ = [("t_done", C.c_double), ("dt", C.c_double), ("err", C.c_double), ("m_used", C.c_int),
                ("accepts", C.c_int), ("rejects", C.c_int), ("m_basis", C.c_int)]


class BincsrInfo(C.Structure):
    _fields_ = [("rows", C.c_longlong), ("cols", C.c_longlong), ("nnz", C.c_longlong), ("index_dtype", C.c_int),
                ("value_dtype", C.c_int), ("flags", C.c_uint), ("checks_passed", C.c_int), ("max_abs", C.c_double),
                ("seconds", C.c_double)]


class BatchParams(C.Structure):
    _fields_ = [("m", C.c_int), ("tol", C.c_double), ("max_restarts", C.c_int), ("reorthogonalize", C.c_int),
                ("basis_bytes", C.c_longlong), ("autotune", C.c_int)]


class BatchInfo(C.Structure):
    _fields_ = [("problems", C.c_int), ("waves", C.c_int), ("tile_rows", C.c_int), ("dot_columns", C.c_int),
                ("spmm_unroll", C.c_int), ("cycles", C.c_int), ("rows", C.c_longlong), ("nnz", C.c_longlong),
                ("tune_ms", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


BATCH_RHS = 16
BATCH_M_MAX = 32

_VP = C.c_void_p
_IP = C.POINTER(C.c_int)
_DP = C.POINTER(C.c_double)

_PROTOS = {
    "mexk_error_string": ([C.c_int], C.c_char_p),
    "mexk_last_error_detail": ([], C.c_char_p),
    "mexk_version": ([], C.c_char_p),
    "mexk_batch_create": ([C.c_int, C.POINTER(BatchParams), C.POINTER(C.c_void_p)], C.c_int),
    "mexk_batch_add": ([C.c_void_p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_double),
                        C.c_double, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_int)], C.c_int),
    "mexk_batch_upload": ([C.c_void_p], C.c_int),
    "mexk_batch_run": ([C.c_void_p], C.c_int),
    "mexk_batch_result": ([C.c_void_p, C.c_int, C.POINTER(C.c_double), C.POINTER(Result)], C.c_int),
    "mexk_batch_info": ([C.c_void_p, C.POINTER(BatchInfo)], C.c_int),
    "mexk_batch_destroy": ([C.c_void_p], C.c_int),
    "mexk_batch_profile": ([C.c_void_p, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_double),
                            C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)], C.c_int),
    "mexk_device_count": ([_IP], C.c_int),
    "mexk_context_create": ([C.c_int, C.POINTER(_VP)], C.c_int),
    "mexk_context_upload_csr": ([_VP, C.c_int, C.c_longlong, _IP, _IP, _DP, C.c_int], C.c_int),
    "mexk_context_destroy": ([_VP], C.c_int),
    "mexk_context_stream": ([_VP], _VP),
    "mexk_expmv": ([_VP, C.POINTER(Params), _DP, _DP, C.POINTER(Result)], C.c_int),
    "mexk_expmv_device": ([_VP, C.POINTER(Params), _VP, _VP, _VP, C.POINTER(Result)], C.c_int),
    "mexk_get_steps": ([_VP, C.POINTER(Step), C.c_int, _IP], C.c_int),
    "mexk_spmv_f64": ([C.c_int, _VP, _VP, _VP, _VP, _VP, _VP], C.c_int),
    "mexk_spmv_f32": ([C.c_int, _VP, _VP, _VP, _VP, _VP, _VP], C.c_int),
    "mexk_arnoldi_step": ([_VP, C.c_int, C.c_int, C.c_int, _DP, _DP, _IP], C.c_int),
    "mexk_context_set_basis": ([_VP, C.c_int, _DP, C.c_int], C.c_int),
    "mexk_context_get_basis": ([_VP, C.c_int, _DP, C.c_int], C.c_int),
    "mexk_expm_f64": ([C.c_int, _VP, C.c_int, _VP, C.c_int, _VP], C.c_int),
    "mexk_profile_kernel": ([_VP, C.c_int, C.c_int, C.c_int, C.c_int, _DP], C.c_int),
    "mexk_context_get_spmv_form": ([_VP, C.c_int, _IP], C.c_int),
    "mexk_context_set_spmv_form": ([_VP, C.c_int, C.c_int], C.c_int),
    "mexk_gram_schmidt_f64_noalloc": ([C.c_int, C.c_int, _VP, C.c_int, _VP, C.c_int, _VP, _VP, _VP, _VP],
                                      C.c_int),
    "mexk_context_set_controller": ([_VP, C.POINTER(C.c_float), C.c_int], C.c_int),
    "mexk_context_set_window_controller": ([_VP, C.POINTER(C.c_float), C.c_int], C.c_int),
    "mexk_krylov_start": ([_VP, C.c_int, _DP, _DP], C.c_int),
    "mexk_krylov_build": ([_VP, C.c_int, C.c_int, C.c_int, _DP, _IP], C.c_int),
    "mexk_krylov_advance": ([_VP, C.c_int, C.c_int, _DP, _DP], C.c_int),
    "mexk_krylov_result": ([_VP, _DP], C.c_int),
    "mexk_mlp_forward": ([_VP, _VP, C.c_int, _VP, _VP], C.c_int),
    "mexk_mlp_gradient": ([_VP, _VP, _VP, _VP, C.c_int, _VP, _VP, _VP, _VP], C.c_int),
    "mexk_mlp_adam_step": ([_VP, _VP, _VP, _VP, _VP, C.c_int, C.c_int, C.c_float, _VP, _VP, _VP], C.c_int),
    "mexk_controller_predict": ([_VP, _VP, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                                 C.c_double, _VP, _VP], C.c_int),
    "mexk_test_force_wait_timeout": ([C.c_int, C.c_int], C.c_int),
    "mexk_context_get_lanczos_form": ([_VP, _IP], C.c_int),
    "mexk_context_set_lanczos_form": ([_VP, C.c_int], C.c_int),
    "mexk_bincsr_probe": ([C.c_char_p, C.POINTER(BincsrInfo)], C.c_int),
    "mexk_context_load_bincsr": ([_VP, C.c_char_p, C.c_int, C.POINTER(BincsrInfo)], C.c_int),
}

KERNELS = {"spmv": 0, "gs_dot": 1, "gs_upd_dot": 2, "gs_upd_norm": 3, "normalize": 4, "lift": 5, "controller": 6,
           "gram_dot": 7, "gram_update": 8, "gram_norm": 9, "spmv_dots": 10, "lanczos_cycle": 11}

_lib = None


def header_functions(path: str = HEADER):
    """Names of the functions declared in a C header."""
    text = open(path).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(mexk_\w+)\s*\(", text, flags=re.M)))


def lib():
    """The loaded libmexk.so; raises MexkError when it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise MexkError(f"CUDA library {LIB_PATH} is not built; run __graft_entry__.build()")
        L = C.CDLL(LIB_PATH)
        for name, (args, res) in _PROTOS.items():
            if hasattr(L, name):
                f = getattr(L, name)
                f.argtypes = args
                f.restype = res
        _lib = L
    return _lib


def check(rc: int, what: str = "mexk call") -> None:
    if rc != MEXK_OK:
        L = lib()
        msg = L.mexk_error_string(rc).decode()
        det = L.mexk_last_error_detail().decode()
        raise MexkError(f"{what}: {msg} (code {rc}){': ' + det if det else ''}")
