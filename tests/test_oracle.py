"""The oracle pinned before it is trusted: against the golden fixtures made by
the reference's own CPU program, against dense expm, and against the
analytic diagonal case. CPU only."""
import numpy as np
import pytest
import scipy.linalg as sl

from conftest import GOLDEN_NAMES, format_step, load_golden


@pytest.mark.parametrize("name", GOLDEN_NAMES)
def test_oracle_matches_reference_fixture(oracle_mod, name):
    A, d = load_golden(name)
    y, st, steps = oracle_mod.expmv(A, d["v"], float(d["t"]), int(d["m"]), tol=float(d["tol"]),
                                    max_restarts=int(d["max_restarts"]))
    # Same arithmetic as the reference build: bit-identical output.
    assert np.array_equal(y, d["y"]), np.abs(y - d["y"]).max()
    assert st["restarts_done"] == int(d["restarts_done"])
    assert st["converged"] == int(d["converged"])
    assert st["last_residual"] == float(d["last_residual"])
    assert [format_step(s) for s in steps] == list(d["step_lines"])


def test_diagonal_known_answer(oracle_mod):
    from mexk import synthetic as S

    n = 1000
    A = S.diagonal_test_matrix(n)
    y, st, _ = oracle_mod.expmv(A, np.full(n, 0.1), 1.0, 30, max_restarts=10)
    exact = 0.1 * np.exp(1.0 + np.arange(n) / n)
    assert np.linalg.norm(y - exact) / np.linalg.norm(exact) < 1e-13
    assert st["converged"] == 1


@pytest.mark.parametrize("name", ["cfg0_random_n2000", "powerlaw_n2048", "heat_N32", "convdiff_N8_pe100",
                                  "rejects_skew_n300_t20_m8"])
def test_oracle_vs_dense_expm(oracle_mod, name):
    A, d = load_golden(name)
    exact = sl.expm(float(d["t"]) * A.to_dense()) @ d["v"]
    err = np.linalg.norm(d["y"] - exact) / np.linalg.norm(exact)
    # The controller bounds the per-step residual estimate by tol (absolute).
    assert err < 1e-6, err


@pytest.mark.parametrize("scale", [1e-3, 0.05, 0.3, 1.0, 3.0, 30.0, 300.0])
def test_expm_matches_scipy(oracle_mod, scale):
    rng = np.random.default_rng(int(scale * 1000))
    for k in (1, 2, 7, 30, 64):
        M = rng.standard_normal((k, k)) * scale / max(1.0, np.sqrt(k))
        E = oracle_mod.expm(M)
        Es = sl.expm(M)
        # Scaling and squaring loses about one ulp per squaring: bound by |M|_1.
        tol = 1e-13 * max(10.0, np.abs(M).sum(axis=0).max())
        assert np.abs(E - Es).max() <= tol * max(1.0, np.abs(Es).max()), (k, scale)


def test_pade_coefficients_exact(oracle_mod):
    import ctypes as C
    from math import factorial

    L = oracle_mod.lib()
    L.oracle_pade_coefficients.argtypes = [C.c_int, C.POINTER(C.c_double)]
    for m in (3, 5, 7, 9, 13):
        b = (C.c_double * 14)()
        assert L.oracle_pade_coefficients(m, b) == m + 1
        for j in range(m + 1):
            exact = factorial(2 * m - j) // (factorial(j) * factorial(m - j))
            assert b[j] == float(exact)
    assert L.oracle_pade_coefficients(4, (C.c_double * 14)()) == 0


def test_oracle_arnoldi_relation(oracle_mod):
    """A V_m = V_{m+1} H_m and V orthonormal, from the oracle's step function."""
    from mexk import synthetic as S

    A = S.random_diag_dominant(400, 7, seed=5)
    m = 12
    V = np.zeros((m + 1, A.n))
    v = np.random.default_rng(6).standard_normal(A.n)
    V[0] = v / np.linalg.norm(v)
    H = np.zeros((m + 1, m))
    for j in range(m):
        ok, h, beta, _ = oracle_mod.arnoldi_step(A, V, j)
        assert ok
        H[: j + 1, j] = h
        H[j + 1, j] = beta
    Ad = A.to_dense()
    assert np.abs(Ad @ V[:m].T - V.T @ H).max() < 1e-12 * np.abs(Ad).max()
    assert np.abs(V @ V.T - np.eye(m + 1)).max() < 1e-13


@pytest.mark.parametrize("seed", range(6))
def test_oracle_bitwise_vs_reference_build(oracle_mod, seed):
    """Random small problems: the C restatement and the reference's own
    main_cpu.cpp (built against the shim) agree bit for bit."""
    if not oracle_mod.have_reference():
        pytest.skip("reference build not present in this container")
    from mexk import synthetic as S

    rng = np.random.default_rng(1000 + seed)
    n = int(rng.integers(20, 400))
    A = S.random_diag_dominant(n, int(rng.integers(1, 8)), seed=seed)
    v = rng.standard_normal(n)
    t = float(rng.uniform(0.1, 8.0))
    m = int(rng.integers(1, min(40, n - 1)))
    mr = int(rng.integers(-1, 4))
    y1, st1, steps = oracle_mod.expmv(A, v, t, m, max_restarts=mr)
    y2, st2, lines = oracle_mod.reference_expmv(A, v, t, m, max_restarts=mr)
    assert np.array_equal(y1, y2)
    assert st1["restarts_done"] == st2["restarts_done"] and st1["converged"] == st2["converged"]
    assert [format_step(s) for s in steps] == lines
