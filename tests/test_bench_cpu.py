"""bench.py's bookkeeping, without a GPU: the algorithmic bytes per kernel
kind and SpMV form (the roofline's numerator), the kernels of a step as a
solve runs them (the launch count), and the clock samples kept for the timed
region."""
import datetime
import importlib.util
import os
import tempfile
import time

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_spmv_bytes_per_form(bench):
    n, nnz = 4_194_304, 20_963_328
    csr32 = bench.kernel_bytes("spmv", n, nnz, 1, True)
    assert csr32 == nnz * 8 + 4 * (n + 1) + 2 * n * 4
    assert bench.kernel_bytes("spmv", n, nnz, 1, False) == nnz * 12 + 4 * (n + 1) + 2 * n * 8
    assert bench.kernel_bytes("spmv", n, nnz, 1, True, form="pattern") == n + 2 * n * 4
    # with dots: u_{j-1} is read unless a window of 2 takes u_{j-1}.w from the update
    assert bench.kernel_bytes("spmv_dots", n, nnz, 2, True, window=0, form="pattern") == n + 3 * n * 4
    assert bench.kernel_bytes("spmv_dots", n, nnz, 2, True, window=2, form="pattern") == n + 2 * n * 4
    assert bench.kernel_bytes("spmv_dots", n, nnz, 2, True, window=2) == csr32 + n * 4


def test_sweep_bytes_follow_the_window(bench):
    n = 1000
    assert bench.kernel_bytes("gram_update", n, 0, 30, True, window=2) == 2 * n * 4 + 2 * n * 4
    assert bench.kernel_bytes("gram_update", n, 0, 30, True) == 30 * n * 4 + 2 * n * 4
    assert bench.kernel_bytes("lift", n, 0, 30, True) == 30 * n * 4 + 8 * n


def test_step_kernels(bench):
    mixed = bench.STEP_KINDS["mixed"]
    assert bench.step_kinds("mixed", 0, 2) == mixed  # step 0: its own dot sweep
    assert bench.step_kinds("mixed", 5, 2) == ["spmv_dots", "gram_update"]
    assert bench.step_kinds("mixed", 1, 0) == ["spmv_dots", "gram_update"]  # step 1 of full Arnoldi
    assert bench.step_kinds("mixed", 5, 0) == mixed
    assert bench.step_kinds("mixed", 5, 2, dots_in_spmv=False) == mixed  # the direct CSR form
    assert bench.step_kinds("fp64", 5, 0) == bench.STEP_KINDS["fp64"]


def test_clock_samples_kept_for_the_timed_region(bench):
    c = bench.ClockSampler(0)
    c.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
    now = time.time()
    for dt, mhz, cap in ((-0.5, 1000, "Not Active"), (0.01, 2070, "Active"), (0.03, 2070, "Not Active"),
                         (0.9, 1200, "Not Active")):
        ts = datetime.datetime.fromtimestamp(now + dt).strftime("%Y/%m/%d %H:%M:%S.%f")[:-3]
        c.file.write(f"{ts}, 0, {mhz}, 2070, 900.0, 0x0, Not Active, Not Active, Not Active, {cap}\n")
    c.file.flush()
    c.proc = object()  # a sampler that ran
    c.t_begin, c.t_end = now, now + 0.05
    out = c.summary()
    assert out["samples_in_timed_region"] == 2 and out["samples"] == 2
    assert out["sm_mhz"] == 2070.0 and out["sm_max_mhz"] == 2070.0
    assert out["reasons"] == ["sw_power_cap"]
