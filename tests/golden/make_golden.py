"""Generate the golden fixtures in this directory from the reference itself.

Runs the reference's own CPU program (main_cpu.cpp's ArnoldiRunnerCPU,
compiled from the reference tree against the project's Eigen-subset shim by
``make -C oracle ref``) on small seeded cases and stores inputs, y, the
summary fields and the printed [STEP] lines as compressed .npz files.
Needs the reference tree (MEXK_REFERENCE_DIR, or a `reference` directory
beside the repository);
the fixtures it writes are committed so tests run without it.

    python tests/golden/make_golden.py [fixture names...]
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "matrix-exp-krylov_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle as O  # noqa: E402
from mexk import synthetic as S  # noqa: E402


def skew300():
    """Skew-symmetric part of random_diag_dominant(300, 3, seed=21): exp(tA) is
    orthogonal, so no decay hides errors."""
    B = S.random_diag_dominant(300, 3, seed=21).to_dense()
    np.fill_diagonal(B, 0.0)
    Ad = B - B.T
    rows, cols = np.nonzero(Ad)
    rp = np.zeros(301, dtype=np.int32)
    np.cumsum(np.bincount(rows, minlength=300), out=rp[1:])
    return S.CSR(300, rp, cols.astype(np.int32), Ad[rows, cols], "skew300")


def diag_linspace(n, lo, hi):
    """Diagonal matrix with eigenvalues evenly spaced from lo to hi."""
    return S.CSR(n, np.arange(n + 1, dtype=np.int32), np.arange(n, dtype=np.int32), np.linspace(lo, hi, n),
                 f"diag_linspace({n}, {lo}, {hi})")


def cases():
    """(name, CSR, v, t, m, max_restarts, store_matrix, generator description[, tol, stepping])."""
    out = []
    P = S.config0()
    out.append(("cfg0_random_n2000", P.A, P.v, P.t, P.m, 0, True, "config0(n=2000, seed=0)"))
    D = S.diagonal_test_matrix(1000)
    out.append(("diag_n1000_kat", D, np.full(1000, 0.1), 1.0, 30, 10, False, "diagonal_test_matrix(1000)"))
    n = 64
    I2 = S.CSR(n, np.arange(n + 1, dtype=np.int32), np.arange(n, dtype=np.int32), np.full(n, 2.0), "2I")
    v = np.random.default_rng(11).uniform(-1, 1, n)
    out.append(("breakdown_j0_2I", I2, v, 0.7, 10, 0, False, "2*I, n=64"))
    n = 90
    d3 = np.tile([-1.0, -2.0, -3.0], n // 3)
    D3 = S.CSR(n, np.arange(n + 1, dtype=np.int32), np.arange(n, dtype=np.int32), d3, "diag3")
    v = np.random.default_rng(12).uniform(0, 1, n)
    out.append(("breakdown_j2_diag3", D3, v, 1.5, 10, 0, False, "diag(-1,-2,-3 repeated), n=90"))
    R = skew300()
    v = np.random.default_rng(22).standard_normal(300)
    out.append(("rejects_skew_n300_t20_m8", R, v, 20.0, 8, 0, True, "skew part of random_diag_dominant(300, 3, seed=21)"))
    R2 = S.random_diag_dominant(100, 4, seed=31)
    v = np.random.default_rng(32).uniform(0, 1, 100)
    out.append(("abort_m1_n100", R2, v, 1.0, 1, 0, True, "random_diag_dominant(100, 4, seed=31)"))
    R3 = S.random_diag_dominant(300, 6, seed=41)
    v = np.random.default_rng(42).uniform(0, 1, 300)
    out.append(("maxsteps_cap_n300", R3, v, 10.0, 10, 2, True, "random_diag_dominant(300, 6, seed=41)"))
    L = S.laplacian_2d(32)
    v = np.random.default_rng(1).uniform(0, 1, L.n)
    out.append(("heat_N32", L, v, 0.01, 30, 0, False, "laplacian_2d(32)"))
    PL = S.power_law(2048, seed=2)
    v = np.random.default_rng(3).standard_normal(2048)
    out.append(("powerlaw_n2048", PL, v, 0.5, 40, 0, True, "power_law(2048, seed=2)"))
    CD = S.convection_diffusion_3d(8, 100.0)
    v = np.random.default_rng(4).uniform(0, 1, CD.n)
    out.append(("convdiff_N8_pe100", CD, v, 0.01, 30, 0, False, "convection_diffusion_3d(8, 100)"))
    # The reference's ArnoldiParams() defaults: m = 100, tol = 1e-8, max_restarts = 10 (main.cu:1221-1230).
    P0 = S.config0()
    out.append(("m100_defaults_cfg0", P0.A, P0.v, 1.0, 100, 10, False, "config0(n=2000, seed=0)", 1e-8, None))
    # Caller-set TimeSteppingParams (main.cu:1237-1250), with rejects and a step cap.
    SK = skew300()
    vs = np.random.default_rng(22).standard_normal(300)
    out.append(("stepping_skew_n300", SK, vs, 20.0, 8, 0, False, "skew300", 1e-7,
                dict(dt_init=1.0, dt_min=1e-4, dt_max=4.0, tol_step=1e-7, max_rejects=6, safety=0.9, grow=2.0,
                     shrink=0.3, max_steps=500)))
    out.append(("adapt_m_skew_n300", SK, vs, 20.0, 8, 0, False, "skew300", 1e-6,
                dict(adapt_m=1, m_step=6, m_max=26)))
    out.append(("stepping_cap_cfg0", P0.A, P0.v, 1.0, 12, 0, False, "config0(n=2000, seed=0)", 1e-9,
                dict(dt_init=0.05, grow=1.1, max_steps=4)))
    # Decaying solutions (|y| << |v|) at the reference's default tol 1e-8: a
    # diagonal with eigenvalues -1..-60, convection-diffusion on 16^3, and a
    # symmetric heat operator on 64^2.
    DG = diag_linspace(600, -1.0, -60.0)
    out.append(("decay_diag_n600", DG, np.ones(600), 1.0, 30, 0, False, "diag_linspace(600, -1.0, -60.0)", 1e-8,
                None))
    for pe, t in ((100.0, 0.01), (1000.0, 1e-3)):
        CDd = S.convection_diffusion_3d(16, pe)
        vd = np.random.default_rng(4).uniform(0, 1, CDd.n)
        out.append((f"decay_convdiff16_pe{int(pe)}", CDd, vd, t, 30, 0, False,
                    f"convection_diffusion_3d(16, {int(pe)})", 1e-8, None))
    # The 128^3 convection-diffusion workload's time t = 1 at Pe = 1000: the solution underflows to zero.
    CDu = S.convection_diffusion_3d(16, 1000.0)
    vu = np.random.default_rng(4).uniform(0, 1, CDu.n)
    out.append(("convdiff16_pe1000_t1", CDu, vu, 1.0, 30, 0, False, "convection_diffusion_3d(16, 1000)", 1e-6,
                None))
    H64 = S.laplacian_2d(64)
    vh = np.random.default_rng(5).uniform(0, 1, H64.n)
    out.append(("decay_heat_N64", H64, vh, 0.05, 30, 0, False, "laplacian_2d(64)", 1e-8, None))
    return out


def main(only=None):
    O.build(with_reference=True)
    if not O.have_reference():
        raise SystemExit("reference build missing")
    for case in cases():
        name, A, v, t, m, mr, store, desc = case[:8]
        tol, stepping = case[8:10] if len(case) > 8 else (1e-6, None)
        if only and name not in only:
            continue
        y, st, lines = O.reference_expmv(A, v, t, m, tol=tol, max_restarts=mr, stepping=stepping)
        data = dict(v=v, y=y, t=t, m=m, tol=tol, max_restarts=mr,
                    restarts_done=st["restarts_done"], converged=st["converged"],
                    last_residual=st["last_residual"], step_lines=np.array(lines), n=A.n, nnz=A.nnz,
                    generator=desc)
        if stepping:
            ts, _ = O._stepping(m, t, tol, mr, stepping)
            data.update({"ts_" + k: v_ for k, v_ in ts.items()})
        if store:
            data.update(row_ptr=A.row_ptr, col_idx=A.col_idx, values=A.values)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **data)
        print(f"{name}: n={A.n} nnz={A.nnz} restarts_done={st['restarts_done']} "
              f"converged={st['converged']} steps={len(lines)}")


if __name__ == "__main__":
    main(set(sys.argv[1:]) or None)
