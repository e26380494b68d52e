"""Full-size golden records of the benchmark workloads.

Runs the reference's own CPU program (main_cpu.cpp via ``make -C oracle
ref``) once on a full workload, run to convergence with tol 1e-6, and
stores its [STEP] decision sequence, summary fields and a compact
fingerprint of y (norm, sum, leading entries, entries at seeded positions):

  heat2048  A = 2D Dirichlet Laplacian / h^2 on a 2048^2 grid, h = 1/2049,
            v ~ U[0,1] (seed 1), t = 1e-5, m = 30  -> heat2048_reference.npz
  powerlaw  n = 8,388,608 power-law rows (Zipf 1.8, seed 2), v ~ N(0,1),
            t = 0.5, m = 40                       -> powerlaw_reference.npz

Each takes minutes to an hour single-threaded; the outputs are committed.

    python tests/golden/make_golden_large.py [heat2048|powerlaw]
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


WORKLOADS = {
    "heat2048": (lambda: S.config1(), "config1(N=2048, seed=1)", "heat2048_reference.npz"),
    "powerlaw": (lambda: S.config2(), "config2(n=8388608, seed=2)", "powerlaw_reference.npz"),
}


def main(name: str = "heat2048"):
    make, desc, out = WORKLOADS[name]
    O.build(with_reference=True)
    P = make()
    t0 = time.time()
    y, st, lines = O.reference_expmv(P.A, P.v, P.t, P.m, tol=1e-6, max_restarts=0)
    wall = time.time() - t0
    pos = fingerprint_positions(P.A.n)
    np.savez_compressed(os.path.join(HERE, out), t=P.t, m=P.m, tol=1e-6, max_restarts=0,
                        n=P.A.n, nnz=P.A.nnz, restarts_done=st["restarts_done"], converged=st["converged"],
                        last_residual=st["last_residual"], step_lines=np.array(lines), y_norm=np.linalg.norm(y),
                        y_sum=y.sum(), y_head=y[:16], positions=pos, y_at=y[pos], wall_seconds=wall,
                        generator=desc)
    print(f"{name} done in {wall:.0f}s: {st} attempts={len(lines)}")


if __name__ == "__main__":
    main(*(sys.argv[1:2] or ["heat2048"]))
