"""Host-side checks that need no GPU: the C ABI library loads and exports every
function include/mexk.h declares, argument checking fails cleanly, the
seeded generators produce the workloads' shapes, and the Python mirror's
structs match the C header."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from mexk import _lib
from mexk import synthetic as S


def test_library_exports_every_declared_symbol():
    L = _lib.lib()
    names = _lib.header_functions()
    assert len(names) >= 18
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    assert L.mexk_version().startswith(b"mexk")


def test_host_library_loads():
    C.CDLL(_lib.HOST_LIB_PATH)


def test_sm103a_only():
    """libmexk.so carries sm_103a code (checked through cuobjdump's ELF list only
    is not needed: the build passes one -gencode, asserted here)."""
    from mexk import build

    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_invalid_arguments_without_gpu():
    L = _lib.lib()
    # NULL output, bad k, bad context: argument checks come before any CUDA call
    assert L.mexk_context_create(0, None) == _lib_err("INVALID")
    assert L.mexk_expm_f64(0, None, 0, None, 0, None) == _lib_err("INVALID")
    assert L.mexk_gram_schmidt_f64_noalloc(10, 0, 1, 10, 1, 1, 1, 1, 1, None) == _lib_err("INVALID")
    assert L.mexk_expmv(None, None, None, None, None) == _lib_err("INVALID")
    form = C.c_int(-1)
    assert L.mexk_context_get_spmv_form(None, 0, C.byref(form)) == _lib_err("INVALID")
    assert L.mexk_context_set_spmv_form(None, 0, 2) == _lib_err("INVALID")
    assert L.mexk_profile_kernel(None, 0, 0, 0, 1, None) == _lib_err("INVALID")
    assert L.mexk_error_string(3) == b"allocation failed"


def _lib_err(name):
    return {"INVALID": 1, "CUDA": 2}[name]


def test_struct_layouts_match_header(tmp_path):
    """ctypes mirrors of the header structs: sizes and offsets equal what a C
    compiler sees in include/mexk.h."""
    src = tmp_path / "layout.c"
    fields = {"mexk_params_t": _lib.Params, "mexk_result_t": _lib.Result, "mexk_step_t": _lib.Step,
              "mexk_bincsr_info_t": _lib.BincsrInfo}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "mexk.h"', "int main(void) {"]
    for cname, py in fields.items():
        lines.append(f'printf("%zu\\n", sizeof({cname}));')
        for f, _ in py._fields_:
            lines.append(f'printf("%zu\\n", offsetof({cname}, {f}));')
    lines.append("return 0; }")
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.dirname(_lib.HEADER), str(src), "-o", str(exe)], check=True)
    out = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    want = []
    for py in fields.values():
        want.append(C.sizeof(py))
        want.extend(getattr(py, f).offset for f, _ in py._fields_)
    assert out == want


def test_cli_without_gpu_fails_cleanly():
    """On a machine without a GPU the program reports it and exits 1."""
    exe = os.path.join(_lib.BUILD, "matrix_exp")
    p = subprocess.run([exe, "10"], capture_output=True, text=True, timeout=60)
    try:
        import torch

        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        pytest.skip("GPU present")
    assert p.returncode == 1
    assert "Starting matrix_exp application." in p.stdout


def test_config0_shape():
    P = S.config0()
    A = P.A
    assert A.n == 2000 and A.nnz == 22000
    lens = np.diff(A.row_ptr)
    assert np.all(lens == 11)
    rows = np.repeat(np.arange(A.n), lens)
    diag = A.values[A.col_idx == rows]
    off = np.abs(A.values[A.col_idx != rows]).reshape(A.n, 10).sum(axis=1)
    assert np.allclose(diag, -off - 1.0)
    for r in range(0, A.n, 97):
        c = A.col_idx[A.row_ptr[r]:A.row_ptr[r + 1]]
        assert np.all(np.diff(c) > 0)
    assert np.all(P.v == 0.1) and P.t == 1.0 and P.m == 30


def test_config1_shape():
    A = S.laplacian_2d(2048)
    assert A.n == 4_194_304 and A.nnz == 20_963_328
    h = 1.0 / 2049
    assert A.values.min() == pytest.approx(-4 / h ** 2) and A.values.max() == pytest.approx(1 / h ** 2)


def test_config4_shape():
    A = S.convection_diffusion_3d(128, 10.0)
    assert A.n == 2_097_152 and A.nnz == 14_581_760


def test_power_law_rows():
    A = S.power_law(200_000, seed=2)
    lens = np.diff(A.row_ptr) - 1
    assert lens.min() >= 2 and lens.max() <= 2048
    assert 8 < lens.mean() < 20
    rows = np.repeat(np.arange(A.n), lens + 1)
    key = rows.astype(np.int64) * A.n + A.col_idx
    assert np.all(np.diff(key) > 0)  # sorted, no duplicates


def test_laplacian_mode_is_eigenvector():
    N = 20
    A = S.laplacian_2d(N)
    u, lam = S.laplacian_2d_mode(N, 3, 5)
    rows = np.repeat(np.arange(A.n), np.diff(A.row_ptr))
    Au = np.bincount(rows, weights=A.values * u[A.col_idx], minlength=A.n)
    assert np.allclose(Au, lam * u, atol=1e-9 * abs(lam))


def test_config3_problem_is_seeded():
    a = S.config3_problem(0, n_range=(1e3, 5e3), nrhs=2)
    b = S.config3_problem(0, n_range=(1e3, 5e3), nrhs=2)
    assert a.A.n == b.A.n and np.array_equal(a.A.values, b.A.values) and np.array_equal(a.v, b.v)
    assert a.v.shape == (2, a.A.n) and 0.1 <= a.t <= 2.0
