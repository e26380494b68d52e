"""Parity of the CUDA path (through the C ABI) with the oracle and the
reference's golden fixtures. Needs a GB300 and the built libmexk.so.

Tolerances: the FP64 path must agree with the reference's FP64 output to a
relative 2-norm error of 1e-12 and take the same accept/reject decisions;
every other form (mixed precision, the candidate-step controllers, the
short-recurrence window) must stay within a relative 2-norm error of 1e-6
of the reference's output.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import GOLDEN_NAMES, fixture_stepping, load_golden

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
MIXED_TOL = 1e-6

# Fixtures whose reference solve converged: the reference's y is within
# 1e-8 (relative) of dense expm on every one of them, so a form that must
# agree with it to 1e-6 is held to its own accuracy.
CONVERGED = ["cfg0_random_n2000", "heat_N32", "powerlaw_n2048", "convdiff_N8_pe100", "diag_n1000_kat",
             "rejects_skew_n300_t20_m8", "breakdown_j2_diag3", "breakdown_j0_2I", "decay_diag_n600",
             "decay_convdiff16_pe100", "decay_convdiff16_pe1000", "decay_heat_N64"]
# Symmetric ones (the short-recurrence window applies).
SYMMETRIC = ["heat_N32", "decay_heat_N64", "decay_diag_n600", "breakdown_j2_diag3", "breakdown_j0_2I",
             "diag_n1000_kat"]


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


@pytest.fixture(scope="module")
def torch_cuda():
    import torch

    assert torch.cuda.is_available(), "GPU tests need CUDA"
    return torch


def _dev(torch, a, dtype):
    return torch.from_numpy(np.ascontiguousarray(a)).to(device="cuda", dtype=dtype)


# ------------------------------------------------------------------ SpMV
@pytest.mark.parametrize("case", ["cfg0_random_n2000", "powerlaw_n2048", "heat_N32", "convdiff_N8_pe100"])
def test_spmv_f64_bitwise(torch_cuda, oracle_mod, case):
    from mexk._lib import check, lib

    torch = torch_cuda
    A, _ = load_golden(case)
    x = np.random.default_rng(7).standard_normal(A.n)
    rp, ci = _dev(torch, A.row_ptr, torch.int32), _dev(torch, A.col_idx, torch.int32)
    va, xd = _dev(torch, A.values, torch.float64), _dev(torch, x, torch.float64)
    yd = torch.empty(A.n, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    check(lib().mexk_spmv_f64(A.n, rp.data_ptr(), ci.data_ptr(), va.data_ptr(), xd.data_ptr(), yd.data_ptr(), None))
    y = yd.cpu().numpy()
    y_ref = oracle_mod.spmv(A, x)
    lens = np.diff(A.row_ptr)
    short = lens <= 64
    # Rows of at most 64 nonzeros: one rounded product per nonzero, summed in
    # order (longer rows are summed by a warp or the block: within rounding).
    assert np.array_equal(y[short], y_ref[short])
    rows = np.repeat(np.arange(A.n), lens)
    absum = np.bincount(rows, weights=np.abs(A.values * x[A.col_idx]), minlength=A.n)
    assert np.all(np.abs(y[~short] - y_ref[~short]) <= 1e-13 * absum[~short])


def test_spmv_long_rows_and_empty_rows(torch_cuda, oracle_mod):
    """Rows longer than a tile (block reduction), empty rows, one huge row."""
    from mexk import synthetic as S
    from mexk._lib import check, lib

    torch = torch_cuda
    n = 6000
    rng = np.random.default_rng(3)
    lens = rng.integers(0, 6, size=n)
    lens[10] = 5000
    lens[11] = 0
    lens[4000] = 2049
    lens[4001] = 2048
    rows = np.repeat(np.arange(n), lens)
    cols = np.concatenate([np.sort(rng.choice(n, size=l, replace=False)) for l in lens])
    rp = np.zeros(n + 1, dtype=np.int32)
    np.cumsum(lens, out=rp[1:])
    A = S.CSR(n, rp, cols.astype(np.int32), rng.standard_normal(rows.size))
    x = rng.standard_normal(n)
    d = [_dev(torch, a, t) for a, t in ((A.row_ptr, torch.int32), (A.col_idx, torch.int32),
                                        (A.values, torch.float64), (x, torch.float64))]
    yd = torch.full((n,), np.nan, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    check(lib().mexk_spmv_f64(n, d[0].data_ptr(), d[1].data_ptr(), d[2].data_ptr(), d[3].data_ptr(),
                              yd.data_ptr(), None))
    y = yd.cpu().numpy()
    y_ref = oracle_mod.spmv(A, x)
    assert np.allclose(y, y_ref, rtol=1e-13, atol=1e-13)
    assert y[11] == 0.0


def test_spmv_f32(torch_cuda):
    from mexk import synthetic as S
    from mexk._lib import check, lib

    torch = torch_cuda
    A = S.power_law(20000, seed=9)
    x = np.random.default_rng(1).standard_normal(A.n).astype(np.float32)
    d = [_dev(torch, a, t) for a, t in ((A.row_ptr, torch.int32), (A.col_idx, torch.int32),
                                        (A.values.astype(np.float32), torch.float32), (x, torch.float32))]
    yd = torch.empty(A.n, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    check(lib().mexk_spmv_f32(A.n, d[0].data_ptr(), d[1].data_ptr(), d[2].data_ptr(), d[3].data_ptr(),
                              yd.data_ptr(), None))
    ref = A.to_dense().astype(np.float64) @ x.astype(np.float64) if A.n <= 4000 else None
    # float64 reference of the float32 data
    rows = np.repeat(np.arange(A.n), np.diff(A.row_ptr))
    prod = A.values.astype(np.float32).astype(np.float64) * x.astype(np.float64)[A.col_idx]
    ref = np.bincount(rows, weights=prod, minlength=A.n)
    assert rel(yd.cpu().numpy().astype(np.float64), ref) < 1e-5


# ------------------------------------------------------------------ expm
@pytest.mark.parametrize("k", [1, 2, 5, 17, 30, 40, 64])
@pytest.mark.parametrize("scale", [1e-3, 0.2, 0.9, 2.0, 8.0, 150.0])
def test_expm_f64_vs_oracle(torch_cuda, oracle_mod, k, scale):
    from mexk._lib import check, lib

    torch = torch_cuda
    rng = np.random.default_rng(k * 1000 + int(scale * 10))
    M = rng.standard_normal((k, k)) * scale / max(1.0, np.sqrt(k))
    E_ref = oracle_mod.expm(M)
    Md = torch.from_numpy(np.asfortranarray(M).ravel(order="F")).cuda()
    Ed = torch.zeros(k * k, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    check(lib().mexk_expm_f64(k, Md.data_ptr(), k, Ed.data_ptr(), k, None))
    E = Ed.cpu().numpy().reshape(k, k, order="F")
    tol = 1e-13 * max(10.0, np.abs(M).sum(axis=0).max())
    assert np.abs(E - E_ref).max() <= tol * max(1.0, np.abs(E_ref).max())


# ------------------------------------------------------------------ Arnoldi step
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_arnoldi_steps_vs_oracle(oracle_mod, precision):
    from mexk import synthetic as S
    from mexk.api import Context

    A = S.power_law(3000, seed=4)
    m = 24
    v = np.random.default_rng(5).standard_normal(A.n)
    V = np.zeros((m + 1, A.n))
    V[0] = v / np.linalg.norm(v)
    ratios = []
    with Context(A, m_alloc=m) as ctx:
        ctx.set_basis(V[:1], precision=precision)
        for j in range(m):
            ok_o, h_o, beta_o, _ = oracle_mod.arnoldi_step(A, V, j)
            ratios.append(np.sqrt(np.sum(np.asarray(h_o) ** 2) + beta_o ** 2) / beta_o)
            ok, h, beta = ctx.arnoldi_step(j, precision=precision)
            assert ok and ok_o
            scale = np.abs(h_o).max()
            # Two independently built bases (CGS2 on the device, MGS2 in the
            # oracle) drift apart by rounding as j grows.
            tol = 1e-12 if precision == "fp64" else 2e-5
            assert np.abs(h - h_o).max() <= tol * scale, (j, np.abs(h - h_o).max() / scale)
            assert abs(beta - beta_o) <= tol * scale
        Vg = ctx.get_basis(m + 1, precision=precision)
    tolv = 1e-12 if precision == "fp64" else 1e-4
    assert np.abs(Vg - V).max() < tolv
    # Orthonormality of the device basis. FP64: CGS2 to rounding. Mixed: the
    # Gram-corrected step measures and removes every earlier loss (no growth
    # from step to step), but the FP32 rounding of its single update stays in
    # the new column: a few u = 2^-24 times |w| / h_{j+1,j} of that step.
    G = Vg @ Vg.T
    bound = 1e-13 if precision == "fp64" else 4 * 2.0 ** -24 * max(ratios)
    assert np.abs(G - np.eye(m + 1)).max() < bound


def test_arnoldi_breakdown_detected():
    from mexk import synthetic as S
    from mexk.api import Context

    n = 90
    A = S.CSR(n, np.arange(n + 1, dtype=np.int32), np.arange(n, dtype=np.int32), np.tile([-1.0, -2.0, -3.0], 30))
    v = np.random.default_rng(1).uniform(0, 1, n)
    V = np.zeros((4, n))
    V[0] = v / np.linalg.norm(v)
    with Context(A, m_alloc=10) as ctx:
        ctx.set_basis(V[:1])
        oks = [ctx.arnoldi_step(j)[0] for j in range(3)]
    assert oks == [True, True, False]


# ------------------------------------------------------------------ full solves
@pytest.mark.parametrize("name", GOLDEN_NAMES)
def test_expmv_fp64_matches_reference(name):
    from mexk.api import Context

    A, d = load_golden(name)
    m = int(d["m"])
    ts = fixture_stepping(d)
    m_alloc = max(m, int(ts["m_max"])) if ts else m
    with Context(A, m_alloc=m_alloc) as ctx:
        y, res = ctx.expmv(d["v"], float(d["t"]), m, tol=float(d["tol"]), max_restarts=int(d["max_restarts"]),
                           stepping=ts)
        steps = ctx.steps()
    assert rel(y, d["y"]) <= FP64_TOL, rel(y, d["y"])
    assert res["restarts_done"] == int(d["restarts_done"])
    assert res["converged"] == int(d["converged"])
    ref_steps = [ln.split() for ln in d["step_lines"]]
    assert len(steps) == len(ref_steps)
    for s, r in zip(steps, ref_steps):
        # m_used / accepts / rejects exact; t, dt and err to printed precision
        assert f"m_used={s[3]}" == r[4] and f"accepts={s[4]}" == r[5] and f"rejects={s[5]}" == r[6]
        assert f"dt={s[1]:g}" == r[2]
        # The estimate h_{k+1,k} |e_k^T exp(dt H) e1| |v| is a product of the
        # basis's smallest quantities: CGS2 on the device and the reference's
        # MGS2 round its late columns differently, so on strongly decaying
        # spectra it agrees to a few percent only; the decisions (checked
        # above) and y are what must match.
        ref_err = float(r[3].split("=")[1])
        floor = 1e-3 * float(d["tol"]) + 1e-12 * np.linalg.norm(d["v"])
        assert abs(s[2] - ref_err) <= 0.1 * abs(ref_err) + floor


@pytest.mark.parametrize("name", CONVERGED)
def test_expmv_mixed_within_tolerance(name):
    from mexk.api import Context

    A, d = load_golden(name)
    m = int(d["m"])
    with Context(A, m_alloc=m) as ctx:
        y, res = ctx.expmv(d["v"], float(d["t"]), m, tol=float(d["tol"]), max_restarts=int(d["max_restarts"]),
                           precision="mixed")
    assert rel(y, d["y"]) <= MIXED_TOL, rel(y, d["y"])


def test_expmv_device_pointers(torch_cuda):
    from mexk import synthetic as S
    from mexk.api import Context

    torch = torch_cuda
    P = S.config0()
    v = torch.from_numpy(P.v).cuda()
    y = torch.zeros(P.A.n, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    with Context(P.A, m_alloc=30) as ctx:
        res = ctx.expmv_device(v.data_ptr(), y.data_ptr(), P.t, P.m)
        y_host, _ = ctx.expmv(P.v, P.t, P.m)
    assert res["converged"] == 1
    assert np.array_equal(y.cpu().numpy(), y_host)


def test_t_zero_and_zero_vector():
    """Edge cases the reference defines: t = 0 runs no step (y = 0); v = 0
    breaks down at once and returns 0."""
    from mexk import synthetic as S
    from mexk.api import Context

    A = S.random_diag_dominant(200, 4, seed=1)
    with Context(A, m_alloc=10) as ctx:
        y, res = ctx.expmv(np.ones(200), 0.0, 10)
        assert not y.any() and res["restarts_done"] == 0 and res["converged"] == 0
        y, res = ctx.expmv(np.zeros(200), 1.0, 10)
        assert not y.any() and res["converged"] == 1


def test_invalid_arguments_rejected():
    from mexk import MexkError
    from mexk import synthetic as S
    from mexk.api import Context

    A = S.random_diag_dominant(50, 3, seed=2)
    with Context(A, m_alloc=10) as ctx:
        with pytest.raises(MexkError):
            ctx.expmv(np.ones(50), 1.0, 11)  # m > m_alloc
        with pytest.raises(MexkError):
            ctx.expmv(np.ones(50), 1.0, 0)
    with pytest.raises(MexkError):
        Context(S.random_diag_dominant(20, 3, seed=2), m_alloc=129)


# ------------------------------------------------------------------ full size
def test_heat2048_modes_known_answer():
    """Full 2048^2 heat workload with v = a combination of three Laplacian
    eigenmodes: exp(tA)v = sum c_i exp(t lambda_i) u_i exactly, and the
    Krylov space closes after three vectors (breakdown at j = 2)."""
    from mexk import synthetic as S
    from mexk.api import Context

    N = 2048
    A = S.laplacian_2d(N)
    modes = [(1, 1, 1.0), (3, 2, 0.5), (40, 7, -0.25)]
    v = np.zeros(A.n)
    exact = np.zeros(A.n)
    t = 1e-5
    for p, q, c in modes:
        u, lam = S.laplacian_2d_mode(N, p, q)
        v += c * u
        exact += c * np.exp(t * lam) * u
    with Context(A, m_alloc=30) as ctx:
        y, res = ctx.expmv(v, t, 30)
        assert res["converged"] == 1
        assert rel(y, exact) < 1e-11, rel(y, exact)
        y32, _ = ctx.expmv(v, t, 30, precision="mixed")
        assert rel(y32, exact) < MIXED_TOL, rel(y32, exact)


def test_cli_diagonal_known_answer(tmp_path):
    """The matrix_exp program on its built-in diagonal matrix (main.cu:2196)."""
    import os
    import subprocess

    from mexk._lib import BUILD

    out = tmp_path / "y.txt"
    env = dict(os.environ, OUTPUT_Y_FILE=str(out))
    p = subprocess.run([os.path.join(BUILD, "matrix_exp"), "1000"], env=env, capture_output=True, text=True,
                       timeout=300)
    assert p.returncode == 0, p.stderr
    assert "converged=yes" in p.stdout
    y = np.loadtxt(out)
    exact = 0.1 * np.exp(1.0 + np.arange(1000) / 1000)
    assert rel(y, exact) < 1e-13


def test_cli_verbose_h_lines():
    """--verbose-h prints the reference's store_H_column line for every
    column of every attempt's basis (main.cu:1951), before its [STEP] line."""
    import os
    import subprocess

    from mexk._lib import BUILD

    p = subprocess.run([os.path.join(BUILD, "matrix_exp"), "1000", "--verbose-h"], capture_output=True, text=True,
                       timeout=300)
    assert p.returncode == 0, p.stderr
    lines = p.stdout.splitlines()
    steps = [i for i, ln in enumerate(lines) if ln.startswith("[STEP]")]
    assert steps
    prev = -1
    for i in steps:
        m_used = int(lines[i].split("m_used=")[1].split()[0])
        hl = [ln for ln in lines[prev + 1:i] if ln.startswith("    H_m column")]
        assert len(hl) == m_used
        assert hl[0] == "    H_m column 0 stored. Current H_m size: 31x30"
        assert hl[-1].startswith(f"    H_m column {m_used - 1} stored.")
        prev = i


def test_heat2048_fp64_matches_reference_run():
    """Full-size workload (n = 4,194,304) against the reference's own run:
    the same accept/reject sequence and y to 1e-12 (norm, sum and entries at
    seeded positions)."""
    import os

    from conftest import GOLDEN
    from mexk import synthetic as S
    from mexk.api import Context

    d = np.load(os.path.join(GOLDEN, "heat2048_reference.npz"))
    P = S.config1()
    assert P.A.nnz == int(d["nnz"])
    with Context(P.A, m_alloc=P.m) as ctx:
        y, res = ctx.expmv(P.v, P.t, P.m)
        steps = ctx.steps()
        y32, res32 = ctx.expmv(P.v, P.t, P.m, precision="mixed")
    ref_steps = [ln.split() for ln in d["step_lines"]]
    assert len(steps) == len(ref_steps)
    for s, r in zip(steps, ref_steps):
        assert f"m_used={s[3]}" == r[4] and f"accepts={s[4]}" == r[5] and f"rejects={s[5]}" == r[6]
        assert f"dt={s[1]:g}" == r[2] and f"t={s[0]:g}" == r[1]
    assert res["restarts_done"] == int(d["restarts_done"]) and res["converged"] == int(d["converged"])
    assert abs(np.linalg.norm(y) - float(d["y_norm"])) <= 1e-12 * float(d["y_norm"])
    assert abs(y.sum() - float(d["y_sum"])) <= 1e-12 * np.abs(y).sum()
    pos = d["positions"]
    assert rel(y[pos], d["y_at"]) <= FP64_TOL and rel(y[:16], d["y_head"]) <= FP64_TOL
    # mixed precision: within 1e-6 of the FP64 result
    assert rel(y32, y) <= MIXED_TOL, rel(y32, y)


def test_powerlaw_fp64_matches_reference_run():
    """Config 2 at full size (n = 8,388,608, 121M nonzeros, m = 40) against
    the reference's own run: the same accept/reject sequence and y to 1e-12
    (norm, sum and entries at seeded positions); the mixed forms within 1e-6
    of that FP64 result."""
    import os

    from conftest import GOLDEN
    from mexk import synthetic as S
    from mexk.api import Context

    d = np.load(os.path.join(GOLDEN, "powerlaw_reference.npz"))
    P = S.config2()
    assert P.A.nnz == int(d["nnz"])
    with Context(P.A, m_alloc=P.m) as ctx:
        y, res = ctx.expmv(P.v, P.t, P.m)
        steps = ctx.steps()
        others = {f: ctx.expmv(P.v, P.t, P.m, precision="mixed", controller=f)[0] for f in ("reference", "search")}
    ref_steps = [ln.split() for ln in d["step_lines"]]
    assert len(steps) == len(ref_steps)
    for s_, r in zip(steps, ref_steps):
        assert f"m_used={s_[3]}" == r[4] and f"accepts={s_[4]}" == r[5] and f"rejects={s_[5]}" == r[6]
        assert f"dt={s_[1]:g}" == r[2] and f"t={s_[0]:g}" == r[1]
    assert res["restarts_done"] == int(d["restarts_done"]) and res["converged"] == int(d["converged"])
    assert abs(np.linalg.norm(y) - float(d["y_norm"])) <= 1e-12 * float(d["y_norm"])
    assert abs(y.sum() - float(d["y_sum"])) <= 1e-12 * np.abs(y).sum()
    pos = d["positions"]
    assert rel(y[pos], d["y_at"]) <= FP64_TOL and rel(y[:16], d["y_head"]) <= FP64_TOL
    for f, y32 in others.items():
        assert rel(y32, y) <= MIXED_TOL, (f, rel(y32, y))


# ------------------------------------------------------------------ step controllers
@pytest.mark.parametrize("name", CONVERGED)
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_search_controller_accuracy(name, precision):
    """Candidate-step control: every accepted step passes the residual test
    (mixed precision: within the FP32 resolution of the iterate while the
    accepted errors stay within 5e-7 of its norm), so the result stays within
    1e-6 (relative) of the reference's."""
    from mexk.api import Context

    A, d = load_golden(name)
    m = int(d["m"])
    with Context(A, m_alloc=m) as ctx:
        y, res = ctx.expmv(d["v"], float(d["t"]), m, tol=float(d["tol"]), max_restarts=int(d["max_restarts"]),
                           precision=precision, controller="search")
    assert res["converged"] == 1
    assert rel(y, d["y"]) <= MIXED_TOL, rel(y, d["y"])


@pytest.mark.parametrize("name", SYMMETRIC)
@pytest.mark.parametrize("controller", ["search", "learned"])
@pytest.mark.parametrize("lanczos", ["stepwise", "fused"])
def test_headline_form_vs_reference_fixtures(name, controller, lanczos):
    """The benchmark's chosen form -- mixed precision, candidate-step
    control, the short-recurrence window of 2, its steps as two launches
    each or as one cooperative launch per basis -- against the reference's
    own output on symmetric problems, decaying ones included."""
    from mexk.api import Context

    A, d = load_golden(name)
    m = int(d["m"])
    with Context(A, m_alloc=m) as ctx:
        ctx.set_lanczos_form(lanczos)
        y, res = ctx.expmv(d["v"], float(d["t"]), m, tol=float(d["tol"]), precision="mixed", controller=controller,
                           window=2)
    assert res["converged"] == 1
    assert rel(y, d["y"]) <= MIXED_TOL, rel(y, d["y"])


FP64_WINDOW_TOL = 1e-9


@pytest.mark.parametrize("name", SYMMETRIC)
def test_fp64_window_vs_reference_fixtures(name):
    """Plain FP64 with the short-recurrence window of 2 (Lanczos: CGS2 over
    the last two basis vectors, the reference's controller) against the
    reference's own full-Arnoldi output on symmetric problems: the same
    accept/reject decisions and y within FP64_WINDOW_TOL (the Krylov
    approximation's own error, not rounding, sets the difference)."""
    from mexk.api import Context

    A, d = load_golden(name)
    m = int(d["m"])
    with Context(A, m_alloc=m) as ctx:
        y, res = ctx.expmv(d["v"], float(d["t"]), m, tol=float(d["tol"]), max_restarts=int(d["max_restarts"]),
                           precision="fp64", window=2)
        steps = ctx.steps()
    ref_steps = [ln.split() for ln in d["step_lines"]]
    print(name, res["restarts_done"], int(d["restarts_done"]), rel(y, d["y"]) if np.linalg.norm(d["y"]) > 0 else 0.0)
    assert res["converged"] == int(d["converged"])
    assert res["restarts_done"] == int(d["restarts_done"])
    assert len(steps) == len(ref_steps)
    for st, r in zip(steps, ref_steps):  # the same attempts, accepts and rejects
        assert f"dt={st[1]:g}" == r[2] and f"accepts={st[4]}" == r[5] and f"rejects={st[5]}" == r[6]
    if np.linalg.norm(d["y"]) > 0:
        assert rel(y, d["y"]) <= FP64_WINDOW_TOL, rel(y, d["y"])


def test_underflowing_config4_time():
    """Convection-diffusion at Pe = 1000 and t = 1, the config-4 time: the
    exact solution underflows to zero; every form returns |y| within the
    absolute tolerance, as the reference does (y = 0)."""
    from mexk.api import Context

    A, d = load_golden("convdiff16_pe1000_t1")
    with Context(A, m_alloc=30) as ctx:
        for prec, ctrl, w in (("fp64", "reference", 0), ("mixed", "search", 0), ("mixed", "learned", 0)):
            y, res = ctx.expmv(d["v"], 1.0, 30, tol=float(d["tol"]), precision=prec, controller=ctrl, window=w)
            assert res["converged"] == 1
            assert np.linalg.norm(y) <= res["restarts_done"] * float(d["tol"]), (prec, ctrl, np.linalg.norm(y))


def test_relaxed_tolerance_budget_holds():
    """Mixed precision with candidate-step control accepts steps above tol
    only while the accepted errors add up to at most 5e-7 of the iterate's
    norm: on the skew problem (|y| = |v| = 17, 60+ reference steps at
    tol 1e-6) the sum of accepted errors stays within tol per step plus
    5e-7 |y|."""
    from mexk.api import Context

    A, d = load_golden("rejects_skew_n300_t20_m8")
    tol = 1e-9
    with Context(A, m_alloc=8) as ctx:
        y, res = ctx.expmv(d["v"], 20.0, 8, tol=tol, precision="mixed", controller="search")
        steps = ctx.steps()
    # an attempt was accepted when the next one counts one more accept (the last one: the solve converged)
    acc = [steps[i] for i in range(len(steps)) if i + 1 == len(steps) or steps[i + 1][4] == steps[i][4] + 1]
    assert len(acc) == res["restarts_done"]
    errs = sum(s[2] for s in acc)
    ny = np.linalg.norm(d["v"])
    assert errs <= len(acc) * tol + 5e-7 * ny * 1.0001, (errs, len(acc))
    assert rel(y, d["y"]) <= MIXED_TOL


def test_search_controller_takes_fewer_cycles():
    from mexk.api import Context

    A, d = load_golden("heat_N32")
    with Context(A, m_alloc=30) as ctx:
        _, r_ref = ctx.expmv(d["v"], float(d["t"]), 30)
        _, r_s = ctx.expmv(d["v"], float(d["t"]), 30, controller="search")
    assert r_s["cycles"] < r_ref["cycles"], (r_s, r_ref)


def test_search_controller_abort_path():
    """m = 1 can never pass the residual test: candidates fail, the
    reference shrink rule takes over and aborts after 20 rejects."""
    from mexk.api import Context

    A, d = load_golden("abort_m1_n100")
    with Context(A, m_alloc=4) as ctx:
        _, res = ctx.expmv(d["v"], float(d["t"]), 1, controller="search")
        steps = ctx.steps()
    assert res["converged"] == 0 and res["restarts_done"] == 0
    assert steps[-1][5] == 19 and len(steps) == 19


# ------------------------------------------------------------------ short-recurrence window
@pytest.mark.gpu
@pytest.mark.parametrize("controller", ["reference", "search"])
def test_window_on_symmetric_matrix(controller):
    """Mixed precision, orthogonalisation against the last 2 basis vectors
    (Lanczos' short recurrence) on symmetric heat matrices: within 1e-6 of
    the full FP64 Arnoldi result."""
    from mexk import synthetic as S
    from mexk.api import Context

    for N, t in ((96, 1e-5), (160, 3e-5)):
        A = S.laplacian_2d(N, h=1.0 / 2049)
        v = np.random.default_rng(N).uniform(0, 1, A.n)
        with Context(A, m_alloc=30) as ctx:
            y64, _ = ctx.expmv(v, t, 30, precision="fp64")
            y, r = ctx.expmv(v, t, 30, precision="mixed", controller=controller, window=2)
            assert r["converged"] == 1
            assert rel(y, y64) <= 1e-6, (N, rel(y, y64))


@pytest.mark.gpu
def test_window_refused_for_nonsymmetric_matrix():
    from mexk import synthetic as S
    from mexk._lib import MexkError
    from mexk.api import Context

    A = S.random_diag_dominant(500, 6, seed=3)
    v = np.ones(A.n)
    with Context(A, m_alloc=30) as ctx:
        with pytest.raises(MexkError, match="symmetric"):
            ctx.expmv(v, 0.5, 30, precision="mixed", window=2)
        with pytest.raises(MexkError, match="symmetric"):
            ctx.expmv(v, 0.5, 30, precision="fp64", window=2)
        with pytest.raises(MexkError):
            ctx.expmv(v, 0.5, 30, precision="mixed", window=1)
        y, r = ctx.expmv(v, 0.5, 30, precision="mixed")  # the context stays usable
        assert r["converged"] == 1


def _long_row_matrix(n=6000, seed=3):
    """Rows longer than a tile (block sum), empty rows, rows at the tile
    boundary, short random rows."""
    from mexk import synthetic as S

    rng = np.random.default_rng(seed)
    lens = rng.integers(0, 6, size=n)
    lens[10], lens[11], lens[4000], lens[4001] = 5000, 0, 2049, 2048
    cols = np.concatenate([np.sort(rng.choice(n, size=l, replace=False)) for l in lens])
    rp = np.zeros(n + 1, dtype=np.int32)
    np.cumsum(lens, out=rp[1:])
    return S.CSR(n, rp, cols.astype(np.int32), rng.standard_normal(int(lens.sum())) * 0.05)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["powerlaw_n2048", "heat_N32", "convdiff_N8_pe100", "long_rows"])
def test_spmv_forms_give_identical_solves(name):
    """Every SpMV form computes the same products and adds each row's in
    column order: FP64 solves are bitwise the same whichever form the context
    runs; mixed ones (whose two-column steps take their dots in a
    form-dependent order) stay within 1e-6 of FP64 under all."""
    from mexk import synthetic as S
    from mexk.api import Context

    if name == "long_rows":
        A, v, t, m = _long_row_matrix(), None, 0.3, 20
    elif name == "heat_N32":
        A, v, t, m = S.laplacian_2d(96, h=1.0 / 2049), None, 1e-5, 30
    else:
        A, d = load_golden(name)
        v, t, m = d["v"], float(d["t"]), int(d["m"])
    if v is None:
        v = np.random.default_rng(7).uniform(0, 1, A.n)
    stencil = name in ("heat_N32", "convdiff_N8_pe100")
    runs = [("mixed", "reference", 0), ("mixed", "search", 0)]
    if name == "heat_N32":
        runs.append(("mixed", "search", 2))
    with Context(A, m_alloc=m) as ctx:
        default = "pattern" if stencil else "staged"  # n < 65,536: every CSR span narrow
        assert ctx.spmv_form("fp64") == ctx.spmv_form("mixed") == default
        forms = ("staged", "direct") + (("pattern",) if stencil else ())
        out = {}
        for form in forms:
            ctx.set_spmv_form(form, precision="fp64")
            assert ctx.spmv_form("fp64") == form
            out[form] = ctx.expmv(v, t, m, precision="fp64")
        y64, r64 = out["staged"]
        for form in forms[1:]:
            y, r = out[form]
            assert np.array_equal(y, y64), form
            assert r["attempts"] == r64["attempts"] and r["cycles"] == r64["cycles"]
        for prec, ctrl, w in runs:
            for form in forms:
                ctx.set_spmv_form(form, precision=prec)
                y, r = ctx.expmv(v, t, m, precision=prec, controller=ctrl, window=w)
                assert r["converged"] == 1
                assert rel(y, y64) <= 1e-6, (prec, ctrl, w, form, rel(y, y64))


@pytest.mark.gpu
def test_scattered_columns_choose_direct_form():
    """A matrix whose row blocks span more than 65,536 columns runs the
    direct SpMV form; its FP64 solve is bitwise that of the staged form."""
    from mexk import synthetic as S
    from mexk._lib import MexkError
    from mexk.api import Context

    A = S.random_diag_dominant(200_000, 6, seed=4)
    v = np.random.default_rng(4).standard_normal(A.n)
    with Context(A, m_alloc=20) as ctx:
        assert ctx.spmv_form("fp64") == ctx.spmv_form("mixed") == "direct"
        with pytest.raises(MexkError, match="row-pattern"):
            ctx.set_spmv_form("pattern", "fp64")
        y_d, r_d = ctx.expmv(v, 0.2, 20, precision="fp64")
        ctx.set_spmv_form("staged", "fp64")
        y_s, r_s = ctx.expmv(v, 0.2, 20, precision="fp64")
        assert np.array_equal(y_d, y_s) and r_d["attempts"] == r_s["attempts"]
        ctx.set_spmv_form("staged", "mixed")
        y_m, _ = ctx.expmv(v, 0.2, 20, precision="mixed")
        assert rel(y_m, y_d) <= 1e-6


def _banded(n, offsets, vals_of_row, drop=()):
    """CSR with entries at row + offset (inside [0, n)), values from
    vals_of_row(r) (one per offset), rows in `drop` empty."""
    from mexk import synthetic as S

    rp, ci, va = [0], [], []
    for r in range(n):
        if r not in drop:
            vr = vals_of_row(r)
            for o, a in zip(offsets, vr):
                if 0 <= r + o < n:
                    ci.append(r + o)
                    va.append(a)
        rp.append(len(ci))
    return S.CSR(n, np.array(rp, np.int32), np.array(ci, np.int32), np.array(va, np.float64))


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["empty_rows", "256_patterns", "257_patterns", "row_of_17", "row_of_16",
                                  "ragged_tail"])
def test_row_pattern_detection(case):
    """The pattern form is taken exactly when every row is one of <= 256
    patterns of <= 16 entries; when taken, FP64 solves are bitwise those of
    the staged CSR form (empty rows, the last partial chunk of rows
    included)."""
    from mexk.api import Context

    offs5 = (-40, -1, 0, 1, 40)
    base = (0.3, 0.2, -1.5, 0.25, 0.1)
    if case == "empty_rows":
        A, want = _banded(5000, offs5, lambda r: base, drop={0, 17, 2500, 4999}), "pattern"
    elif case == "256_patterns":  # 254 diagonal values in the interior + the first and the last row
        A, want = _banded(3000, (-1, 0, 1), lambda r: (0.1, -1.0 - (r % 254) / 1000, 0.2)), "pattern"
    elif case == "257_patterns":
        A, want = _banded(3000, (-1, 0, 1), lambda r: (0.1, -1.0 - (r % 255) / 1000, 0.2)), "staged"
    elif case == "row_of_17":
        offs = tuple(range(-8, 9))
        A, want = _banded(2000, offs, lambda r: [0.01] * 8 + [-1.0] + [0.01] * 8), "staged"
    elif case == "row_of_16":
        offs = tuple(range(-8, 8))
        A, want = _banded(2000, offs, lambda r: [0.01] * 8 + [-1.0] + [0.01] * 7), "pattern"
    else:  # n not a multiple of the 1024-row chunk nor of 4
        A, want = _banded(1024 * 3 + 7, offs5, lambda r: base), "pattern"
    v = np.random.default_rng(2).uniform(-1, 1, A.n)
    with Context(A, m_alloc=20) as ctx:
        assert ctx.spmv_form("fp64") == want
        if want != "pattern":
            return
        y_p, r_p = ctx.expmv(v, 0.4, 20, precision="fp64")
        ctx.set_spmv_form("staged", "fp64")
        y_s, r_s = ctx.expmv(v, 0.4, 20, precision="fp64")
        assert np.array_equal(y_p, y_s) and r_p["attempts"] == r_s["attempts"]
        y_m, _ = ctx.expmv(v, 0.4, 20, precision="mixed")
        assert rel(y_m, y_s) <= 1e-6


# ------------------------------------------------------------------ the C++ drop-in API
def _runner_check(tmp_path):
    """Compiles tests/cpp/runner_check.cpp against the public header and the
    built host library (g++ is on both the build and the GPU machines)."""
    import os
    import subprocess

    from conftest import ROOT
    from mexk._lib import BUILD

    exe = tmp_path / "runner_check"
    src = os.path.join(ROOT, "tests", "cpp", "runner_check.cpp")
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"), "-o", str(exe), src,
                    "-L", BUILD, f"-Wl,-rpath,{BUILD}", "-lmexk_host", "-lmexk"], check=True)
    return str(exe)


@pytest.mark.parametrize("name", ["m100_defaults_cfg0", "stepping_skew_n300", "adapt_m_skew_n300",
                                  "stepping_cap_cfg0", "heat_N32"])
def test_cpp_runner_matches_reference(tmp_path, name):
    """A C++ program using ArnoldiParams (m = 100: the reference's default)
    and an edited runner.ts_params prints the reference's [STEP] lines
    verbatim and returns its y to 1e-12."""
    import subprocess

    from mexk.bincsr import write_bincsr

    exe = _runner_check(tmp_path)
    A, d = load_golden(name)
    write_bincsr(tmp_path / "a.bincsr", A.row_ptr, A.col_idx, A.values)
    np.ascontiguousarray(d["v"], dtype=np.float64).tofile(tmp_path / "v.bin")
    args = [exe, str(tmp_path / "a.bincsr"), str(tmp_path / "v.bin"), str(tmp_path / "y.bin"), str(int(d["m"])),
            repr(float(d["t"])), repr(float(d["tol"])), str(int(d["max_restarts"]))]
    ts = fixture_stepping(d)
    if ts:
        args += [repr(float(ts[k])) for k in ("dt_init", "dt_min", "dt_max", "tol_step")]
        args += [str(int(ts[k])) for k in ("max_steps", "max_rejects")]
        args += [repr(float(ts[k])) for k in ("safety", "grow", "shrink")]
        args += [str(int(ts[k])) for k in ("adapt_m", "m_max", "m_step")]
    p = subprocess.run(args, capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stderr
    lines = [ln.split() for ln in p.stdout.splitlines() if ln.startswith("[STEP]")]
    ref_lines = [ln.split() for ln in d["step_lines"]]
    assert len(lines) == len(ref_lines)
    for s, r in zip(lines, ref_lines):
        # t, dt, m_used, accepts, rejects verbatim; err to its printed digits
        # (its last ones differ where the estimate sits at the rounding floor)
        assert s[:3] + s[4:] == r[:3] + r[4:], (s, r)
        e, re_ = float(s[3].split("=")[1]), float(r[3].split("=")[1])
        floor = 1e-3 * float(d["tol"]) + 1e-12 * np.linalg.norm(d["v"])
        assert abs(e - re_) <= 0.1 * abs(re_) + floor, (s, r)
    y = np.fromfile(tmp_path / "y.bin", dtype=np.float64)
    assert rel(y, d["y"]) <= FP64_TOL, rel(y, d["y"])
    assert f"RESULT restarts_done={int(d['restarts_done'])} converged={int(d['converged'])}" in p.stdout


# ------------------------------------------------------------------ fused Lanczos cycle
@pytest.mark.parametrize("N", [32, 97, 160, 700])
@pytest.mark.parametrize("controller", ["reference", "search"])
def test_lanczos_fused_form_matches_stepwise(N, controller):
    """Window-2 bases in one cooperative launch against the two-kernel
    steps: the same row sums and updates, dot products summed in another
    order -- both within 1e-6 of FP64, and of each other (grids whose row
    count is not a multiple of the blocks' row groups included)."""
    from mexk import synthetic as S
    from mexk.api import Context

    A = S.laplacian_2d(N, h=1.0 / 2049)
    v = np.random.default_rng(N).uniform(0, 1, A.n)
    t = 2e-5
    with Context(A, m_alloc=30) as ctx:
        assert ctx.lanczos_form() == "stepwise"  # the default
        ctx.set_lanczos_form("fused")
        y64, _ = ctx.expmv(v, t, 30, precision="fp64")
        yf, rf = ctx.expmv(v, t, 30, precision="mixed", controller=controller, window=2)
        ctx.set_lanczos_form("stepwise")
        assert ctx.lanczos_form() == "stepwise"
        ys, rs = ctx.expmv(v, t, 30, precision="mixed", controller=controller, window=2)
        ctx.set_lanczos_form("fused")
        yf2, _ = ctx.expmv(v, t, 30, precision="mixed", controller=controller, window=2)
    assert rf["converged"] == rs["converged"] == 1
    assert rel(yf, y64) <= MIXED_TOL and rel(ys, y64) <= MIXED_TOL, (rel(yf, y64), rel(ys, y64))
    assert np.array_equal(yf, yf2)  # deterministic: the same sums in the same order every launch
