"""Generate the golden fixtures in this directory from the reference itself.

Runs the reference's own CPU program (main_cpu.cpp's ArnoldiRunnerCPU,
compiled from the reference tree against the project's Eigen-subset shim by
``make -C oracle ref``) on small seeded cases and stores inputs, y, the
summary fields and the printed [STEP] lines as compressed .npz files.
Needs the reference tree (default /root/reference, or MEXK_REFERENCE_DIR);
the fixtures it writes are committed so tests run without it.

    python tests/golden/make_golden.py
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


def cases():
    """(name, CSR, v, t, m, max_restarts, store_matrix, generator description)."""
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
    B = S.random_diag_dominant(300, 3, seed=21).to_dense()
    np.fill_diagonal(B, 0.0)
    Ad = B - B.T  # skew-symmetric: exp(tA) is orthogonal, no decay to hide errors
    rows, cols = np.nonzero(Ad)
    rp = np.zeros(301, dtype=np.int32)
    np.cumsum(np.bincount(rows, minlength=300), out=rp[1:])
    R = S.CSR(300, rp, cols.astype(np.int32), Ad[rows, cols], "skew300")
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
    return out


def main():
    O.build(with_reference=True)
    if not O.have_reference():
        raise SystemExit("reference build missing")
    for name, A, v, t, m, mr, store, desc in cases():
        y, st, lines = O.reference_expmv(A, v, t, m, max_restarts=mr)
        data = dict(v=v, y=y, t=t, m=m, tol=1e-6, max_restarts=mr,
                    restarts_done=st["restarts_done"], converged=st["converged"],
                    last_residual=st["last_residual"], step_lines=np.array(lines), n=A.n, nnz=A.nnz,
                    generator=desc)
        if store:
            data.update(row_ptr=A.row_ptr, col_idx=A.col_idx, values=A.values)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **data)
        print(f"{name}: n={A.n} nnz={A.nnz} restarts_done={st['restarts_done']} "
              f"converged={st['converged']} steps={len(lines)}")


if __name__ == "__main__":
    main()
