"""Batched solves (mexk_batch_*): many matrices x 16 right-hand sides in
mixed precision, checked per (problem, rhs) against a dense FP64 oracle
(scipy.linalg.expm for n <= 2000), against wave packing and re-runs, and for
the t = 0 / zero-vector edge cases. Host-side validation runs on CPU.
"""
import ctypes as C

import numpy as np
import pytest

from mexk import synthetic as S


def _problems(specs, seed0=500):
    out = []
    for i, (n, deg, nrhs, t) in enumerate(specs):
        rng = np.random.default_rng(seed0 + i)
        A = S.random_diag_dominant(n, deg, seed0 + i, rng=rng)
        V = rng.standard_normal((nrhs, n))
        out.append((A, V, t))
    return out


SPECS = [(100, 5, 16, 0.3), (257, 12, 16, 1.0), (640, 20, 7, 2.0), (1200, 8, 16, 0.1), (2000, 15, 3, 1.5)]


def _run(problems, **kw):
    from mexk.batch import Batch

    with Batch(m=30, tol=1e-6, **kw) as b:
        for A, V, t in problems:
            b.add(A, V, t)
        b.upload()
        b.run()
        out = [b.result(i) for i in range(len(problems))]
        info = b.info()
    return out, info


# ------------------------------------------------------------------ CPU: validation
def test_batch_add_validation_cpu():
    from mexk._lib import BatchParams, lib

    L = lib()
    h = C.c_void_p()
    assert L.mexk_batch_create(0, C.byref(BatchParams(30, 1e-6, 0, 1, 0, 0)), C.byref(h)) == 0
    try:
        A = S.random_diag_dominant(64, 4, 1)
        rp = np.ascontiguousarray(A.row_ptr, dtype=np.int32)
        ci = np.ascontiguousarray(A.col_idx, dtype=np.int32)
        va = np.ascontiguousarray(A.values)
        V = np.ones((64, 2))
        P = lambda a, t: a.ctypes.data_as(C.POINTER(t))  # noqa: E731
        idx = C.c_int(-1)
        assert L.mexk_batch_add(h, 64, P(rp, C.c_int), P(ci, C.c_int), P(va, C.c_double), 1.0, 2,
                                P(V, C.c_double), C.byref(idx)) == 0 and idx.value == 0
        bad = ci.copy()
        bad[3] = 64  # column out of range
        assert L.mexk_batch_add(h, 64, P(rp, C.c_int), P(bad, C.c_int), P(va, C.c_double), 1.0, 2,
                                P(V, C.c_double), C.byref(idx)) == 1
        assert L.mexk_batch_add(h, 64, P(rp, C.c_int), P(ci, C.c_int), P(va, C.c_double), 1.0, 17,
                                P(V, C.c_double), C.byref(idx)) == 1  # > 16 right-hand sides
        small = S.random_diag_dominant(20, 3, 2)  # m = 30 >= rows
        assert L.mexk_batch_add(h, 20, P(np.ascontiguousarray(small.row_ptr, dtype=np.int32), C.c_int),
                                P(np.ascontiguousarray(small.col_idx, dtype=np.int32), C.c_int),
                                P(np.ascontiguousarray(small.values), C.c_double), 1.0, 1,
                                P(np.ones(20), C.c_double), C.byref(idx)) == 1
    finally:
        L.mexk_batch_destroy(h)
    bad_m = C.c_void_p()
    assert L.mexk_batch_create(0, C.byref(BatchParams(33, 1e-6, 0, 1, 0, 0)), C.byref(bad_m)) == 1


# ------------------------------------------------------------------ GPU
@pytest.mark.gpu
def test_batch_matches_dense_expm():
    import scipy.linalg

    problems = _problems(SPECS)
    out, info = _run(problems, autotune=False)
    assert info["problems"] == len(SPECS) and info["waves"] == 1
    worst = 0.0
    for (A, V, t), (Y, res) in zip(problems, out):
        E = scipy.linalg.expm(t * A.to_dense())
        for r in range(V.shape[0]):
            ref = E @ V[r]
            err = np.linalg.norm(Y[r] - ref) / np.linalg.norm(ref)
            worst = max(worst, err)
            assert res[r]["converged"] == 1 and abs(res[r]["t_done"] - t) <= 1e-12 * max(1.0, t)
    assert worst <= 1e-6, worst


@pytest.mark.gpu
def test_batch_matches_single_vector_fp64_path():
    from mexk.api import Context

    problems = _problems(SPECS[:3])
    out, _ = _run(problems, autotune=False)
    for (A, V, t), (Y, _) in zip(problems, out):
        with Context(A, m_alloc=30) as ctx:
            for r in (0, V.shape[0] - 1):
                y, _ = ctx.expmv(V[r], t, 30, precision="fp64")
                assert np.linalg.norm(Y[r] - y) <= 1e-6 * np.linalg.norm(y)


@pytest.mark.gpu
def test_batch_waves_do_not_change_results():
    problems = _problems(SPECS)
    one, info1 = _run(problems, autotune=False)
    # a budget of 2048 rows per wave (m + 2 = 32 FP32 vectors of 16 RHS per row)
    many, info2 = _run(problems, autotune=False, basis_bytes=2100 * 32 * 16 * 4)
    assert info1["waves"] == 1 and info2["waves"] >= 3
    for (Y1, r1), (Y2, r2) in zip(one, many):
        assert np.array_equal(Y1, Y2)
        assert [x["attempts"] for x in r1] == [x["attempts"] for x in r2]


@pytest.mark.gpu
def test_batch_rerun_and_autotune():
    from mexk.batch import Batch

    problems = _problems(SPECS[:4])
    with Batch(m=30, tol=1e-6, autotune=True) as b:
        for A, V, t in problems:
            b.add(A, V, t)
        b.upload()
        b.run()
        first = [b.result(i)[0] for i in range(len(problems))]
        b.run()
        second = [b.result(i)[0] for i in range(len(problems))]
        info = b.info()
    for a, c in zip(first, second):
        assert np.array_equal(a, c)
    assert info["tile_rows"] in (1024, 4096, 16384)
    assert info["dot_columns"] in (2, 4) and info["spmm_unroll"] in (4, 8)
    assert info["cycles"] >= 1 and info["tune_ms"] > 0.0


@pytest.mark.gpu
def test_batch_zero_vector_and_zero_time():
    problems = _problems([(300, 6, 4, 1.0), (300, 6, 2, 0.0)])
    A0, V0, t0 = problems[0]
    V0 = V0.copy()
    V0[2] = 0.0  # a zero right-hand side
    problems[0] = (A0, V0, t0)
    out, _ = _run(problems, autotune=False)
    (Y0, r0), (Y1, r1) = out
    assert np.all(Y0[2] == 0.0)
    assert np.all(Y1 == 0.0)  # no step runs for t = 0: y stays zero (main_cpu.cpp:467)
    assert all(x["converged"] == 1 for x in r0)
