"""Full-size golden record for the heat-equation workload (2048^2 grid).

Runs the reference's own CPU program (main_cpu.cpp via ``make -C oracle
ref``) once on the full workload -- A = 2D Dirichlet Laplacian / h^2,
h = 1/2049, v ~ U[0,1] (seed 1), t = 1e-5, m = 30, tol 1e-6, run to
convergence -- and stores its [STEP] decision sequence, summary fields and
a compact fingerprint of y (norm, sum, leading entries, entries at seeded
positions). Takes tens of minutes single-threaded; the output is committed
as heat2048_reference.npz.

    python tests/golden/make_golden_large.py
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "matrix-exp-krylov_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle as O  # noqa: E402
from mexk import synthetic as S  # noqa: E402


def fingerprint_positions(n, count=64, seed=123):
    return np.sort(np.random.default_rng(seed).choice(n, size=count, replace=False))


def main():
    O.build(with_reference=True)
    P = S.config1()
    t0 = time.time()
    y, st, lines = O.reference_expmv(P.A, P.v, P.t, P.m, tol=P.tol, max_restarts=0)
    wall = time.time() - t0
    pos = fingerprint_positions(P.A.n)
    np.savez_compressed(os.path.join(HERE, "heat2048_reference.npz"), t=P.t, m=P.m, tol=P.tol, max_restarts=0,
                        n=P.A.n, nnz=P.A.nnz, restarts_done=st["restarts_done"], converged=st["converged"],
                        last_residual=st["last_residual"], step_lines=np.array(lines), y_norm=np.linalg.norm(y),
                        y_sum=y.sum(), y_head=y[:16], positions=pos, y_at=y[pos], wall_seconds=wall,
                        generator="config1(N=2048, seed=1)")
    print(f"done in {wall:.0f}s: {st} attempts={len(lines)}")


if __name__ == "__main__":
    main()
