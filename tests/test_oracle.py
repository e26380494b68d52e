"""The oracle pinned before it is trusted: against the golden fixtures made by
the reference's own CPU program, against dense expm, and against the
analytic diagonal case. CPU only."""
import numpy as np
import pytest
import scipy.linalg as sl

from conftest import GOLDEN_NAMES, fixture_stepping, format_step, load_golden


@pytest.mark.parametrize("name", GOLDEN_NAMES)
def test_oracle_matches_reference_fixture(oracle_mod, name):
    A, d = load_golden(name)
    y, st, steps = oracle_mod.expmv(A, d["v"], float(d["t"]), int(d["m"]), tol=float(d["tol"]),
                                    max_restarts=int(d["max_restarts"]), stepping=fixture_stepping(d))
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
                                  "rejects_skew_n300_t20_m8", "m100_defaults_cfg0", "stepping_skew_n300",
                                  "adapt_m_skew_n300", "decay_diag_n600", "decay_convdiff16_pe100",
                                  "decay_convdiff16_pe1000", "decay_heat_N64"])
def test_oracle_vs_dense_expm(oracle_mod, name):
    A, d = load_golden(name)
    exact = dense_expmv(A, d)
    err = np.linalg.norm(d["y"] - exact) / np.linalg.norm(exact)
    # The controller bounds the per-step residual estimate by tol (absolute);
    # the decaying fixtures use tol 1e-8, far below their |y|.
    assert err < 1e-6, err


def dense_expmv(A, d):
    if A.n == int(np.count_nonzero(np.diff(A.row_ptr))) and np.array_equal(A.col_idx, np.arange(A.n)):
        return np.exp(float(d["t"]) * A.values) * d["v"]  # diagonal
    return sl.expm(float(d["t"]) * A.to_dense()) @ d["v"]


def test_underflowing_fixture_is_zero(oracle_mod):
    """Convection-diffusion at Pe = 1000 and t = 1 (the config-4 time): every
    mode decays below the double range, and the reference returns y = 0 to
    within its absolute tolerance."""
    A, d = load_golden("convdiff16_pe1000_t1")
    assert np.linalg.norm(d["y"]) <= float(d["tol"])
    y, st, _ = oracle_mod.expmv(A, d["v"], 1.0, 30, tol=float(d["tol"]))
    assert np.array_equal(y, d["y"]) and st["converged"] == 1


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


@pytest.mark.parametrize("seed", range(4))
def test_oracle_stepping_bitwise_vs_reference_build(oracle_mod, seed):
    """Caller-set TimeSteppingParams, adapt_m included: the restatement and
    the reference's own program (ts_params set on its runner) agree bit for bit."""
    if not oracle_mod.have_reference():
        pytest.skip("reference build not present in this container")
    from mexk import synthetic as S

    rng = np.random.default_rng(2000 + seed)
    n = int(rng.integers(60, 300))
    A = S.random_diag_dominant(n, int(rng.integers(2, 8)), seed=seed + 50)
    v = rng.standard_normal(n)
    t = float(rng.uniform(0.5, 6.0))
    m = int(rng.integers(3, 12))
    ts = dict(dt_init=float(rng.uniform(0.05, 2.0)), dt_min=1e-5, dt_max=float(rng.uniform(0.5, 4.0)),
              tol_step=float(10 ** rng.uniform(-10, -5)), safety=float(rng.uniform(0.6, 0.95)),
              grow=float(rng.uniform(1.1, 3.0)), shrink=float(rng.uniform(0.2, 0.7)),
              max_rejects=int(rng.integers(3, 25)), max_steps=int(rng.integers(2, 400)),
              adapt_m=int(seed % 2), m_step=int(rng.integers(1, 5)), m_max=m + int(rng.integers(0, 12)))
    y1, st1, steps = oracle_mod.expmv(A, v, t, m, tol=ts["tol_step"], stepping=ts)
    y2, st2, lines = oracle_mod.reference_expmv(A, v, t, m, tol=ts["tol_step"], stepping=ts)
    assert np.array_equal(y1, y2)
    assert st1["restarts_done"] == st2["restarts_done"] and st1["converged"] == st2["converged"]
    assert [format_step(s) for s in steps] == lines
