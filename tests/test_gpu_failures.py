"""Failure handling on the device, exercised without faulting the GPU:
a bounded wait made to run out through the testing hook, non-finite inputs
(the reference's breakdown path), broken controller networks (the plain
heuristic takes over), and refused time-stepping parameters."""
import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def test_bounded_wait_timeout_reports_and_context_survives(oracle_mod):
    """Block 0 of the staged SpMV waits on a barrier nothing arrives at: its
    1 ms bound runs out, it drains its copies, the solve stops with
    MEXK_ERR_DEVICE (timeout), and the same context then solves normally."""
    from mexk import synthetic as S
    from mexk._lib import MexkError, check, lib
    from mexk.api import Context

    A = S.random_diag_dominant(20000, 6, seed=12)
    v = np.random.default_rng(12).standard_normal(A.n)
    y_ref, st_ref, _ = oracle_mod.expmv(A, v, 0.5, 20)
    with Context(A, m_alloc=20) as ctx:
        assert ctx.spmv_form("fp64") == "staged"
        check(lib().mexk_test_force_wait_timeout(0, 1))
        try:
            with pytest.raises(MexkError, match="device wait gave up"):
                ctx.expmv(v, 0.5, 20)
            with pytest.raises(MexkError, match="device wait gave up"):
                ctx.expmv(v, 0.5, 20, precision="mixed")
        finally:
            check(lib().mexk_test_force_wait_timeout(0, 0))
        y, res = ctx.expmv(v, 0.5, 20)
    assert res["status"] == 0 and res["restarts_done"] == st_ref["restarts_done"]
    assert rel(y, y_ref) <= 1e-12


def test_fused_cycle_barrier_timeout_reports_and_context_survives():
    """Block 0 of the fused Lanczos cycle leaves before its first grid
    barrier: the other blocks' bounded waits run out (about a second), every
    block leaves, the solve stops with MEXK_ERR_DEVICE (timeout), and the
    context then solves normally with the barrier words reset."""
    from mexk import synthetic as S
    from mexk._lib import MexkError, check, lib
    from mexk.api import Context

    A = S.laplacian_2d(300, h=1.0 / 2049)
    v = np.random.default_rng(3).uniform(0, 1, A.n)
    with Context(A, m_alloc=30) as ctx:
        ctx.set_lanczos_form("fused")
        assert ctx.lanczos_form() == "fused"
        y_ok, _ = ctx.expmv(v, 1e-5, 30, precision="mixed", controller="search", window=2)
        check(lib().mexk_test_force_wait_timeout(0, 1))
        try:
            with pytest.raises(MexkError, match="device wait gave up"):
                ctx.expmv(v, 1e-5, 30, precision="mixed", controller="search", window=2)
        finally:
            check(lib().mexk_test_force_wait_timeout(0, 0))
        y, res = ctx.expmv(v, 1e-5, 30, precision="mixed", controller="search", window=2)
    assert res["status"] == 0 and np.array_equal(y, y_ok)


@pytest.mark.parametrize("where", ["nan_in_v", "inf_in_v", "nan_in_A", "inf_in_A"])
@pytest.mark.parametrize("form", [("fp64", "reference"), ("mixed", "reference"), ("mixed", "search")])
def test_non_finite_input_takes_the_breakdown_path(oracle_mod, where, form):
    """A NaN or Inf in v or in A makes |w| non-finite at the first step: the
    breakdown test (main.cu:1911) truncates the basis, the step is accepted
    with err = 0, and the lift drops the non-finite coefficients -- y = 0 and
    one accepted step, as the reference's own program returns."""
    from mexk import synthetic as S
    from mexk.api import Context

    A, d = load_golden("cfg0_random_n2000")
    v = d["v"].copy()
    vals = A.values.copy()
    bad = np.nan if where.startswith("nan") else np.inf
    if where.endswith("_v"):
        v[7] = bad
    else:
        vals[100] = bad
    B = S.CSR(A.n, A.row_ptr, A.col_idx, vals)
    y_ref, st_ref, steps_ref = oracle_mod.expmv(B, v, 1.0, 30)
    assert not y_ref.any() and st_ref["converged"] == 1 and st_ref["restarts_done"] == 1
    prec, ctrl = form
    with Context(B, m_alloc=30) as ctx:
        y, res = ctx.expmv(v, 1.0, 30, precision=prec, controller=ctrl)
        steps = ctx.steps()
        # the context stays usable for finite input
        y2, _ = ctx.expmv(d["v"], 1.0, 30) if where.endswith("_v") else (None, None)
    assert not y.any()
    assert res["converged"] == 1 and res["restarts_done"] == 1 and res["cycles"] == 1
    assert steps[0][2] == 0.0 and steps[0][3] == 1  # err = 0, m_used = 1 (breakdown at the first step)
    if y2 is not None:
        assert rel(y2, d["y"]) <= 1e-12


@pytest.mark.parametrize("net", ["zeros", "scaled_1e30", "nan"])
@pytest.mark.parametrize("name", ["heat_N32", "cfg0_random_n2000", "decay_heat_N64"])
def test_broken_network_falls_back(net, name):
    """A learned controller whose network outputs nothing useful (all-zero
    weights and normalisation, weights scaled by 1e30, NaN weights): its
    step predictions are non-finite or degenerate, the candidate search and
    the reference heuristic still choose every step, and the result stays
    within 1e-6 of the reference's."""
    import ctypes as C

    from mexk import controller as K
    from mexk._lib import MEXK_OK, lib
    from mexk.api import Context

    A, d = load_golden(name)
    w = np.ascontiguousarray(K.load(K.WEIGHTS), dtype=np.float32)
    if net == "zeros":
        w[:] = 0.0
    elif net == "scaled_1e30":
        w[: 4866] *= np.float32(1e30)
    else:
        w[:] = np.nan
    m = int(d["m"])
    with Context(A, m_alloc=m) as ctx:
        assert lib().mexk_context_set_controller(ctx.handle, w.ctypes.data_as(C.POINTER(C.c_float)), w.size) == MEXK_OK
        ctx._net_loaded = True
        for prec, window in (("mixed", 0), ("fp64", 0)) + ((("mixed", 2),) if name != "cfg0_random_n2000" else ()):
            y, res = ctx.expmv(d["v"], float(d["t"]), m, tol=float(d["tol"]), precision=prec, controller="learned",
                               window=window)
            assert res["converged"] == 1, (prec, window)
            assert rel(y, d["y"]) <= 1e-6, (prec, window, rel(y, d["y"]))


def test_invalid_stepping_refused():
    """Time-stepping parameters that would stall or corrupt the controller
    are refused before any device work; adapt_m beyond the allocation too
    (main.cu:1441-1444)."""
    from mexk import synthetic as S
    from mexk._lib import MexkError
    from mexk.api import Context

    A = S.random_diag_dominant(300, 4, seed=3)
    v = np.ones(A.n)
    with Context(A, m_alloc=20) as ctx:
        for bad in (dict(dt_min=0.0), dict(dt_max=1e-9, dt_min=1e-6), dict(dt_init=float("nan")),
                    dict(grow=0.0), dict(shrink=-1.0), dict(max_rejects=0), dict(safety=float("nan")),
                    dict(adapt_m=1, m_step=4, m_max=24)):
            with pytest.raises(MexkError):
                ctx.expmv(v, 1.0, 10, stepping=bad)
        with pytest.raises(MexkError, match="adapt_m"):
            ctx.expmv(v, 1.0, 10, precision="mixed", stepping=dict(adapt_m=1, m_step=2, m_max=14))
        y, res = ctx.expmv(v, 1.0, 10, stepping=dict(adapt_m=1, m_step=2, m_max=14))
        assert res["converged"] == 1
