import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "matrix-exp-krylov_gb300")
ORACLE = os.path.join(ROOT, "oracle")
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (PKG, ORACLE):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libmexk.so")


def load_golden(name):
    """A golden fixture as (CSR, dict of fields)."""
    from mexk import synthetic as S

    d = dict(np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False))
    if "row_ptr" in d:
        A = S.CSR(int(d["n"]), d["row_ptr"].astype(np.int32), d["col_idx"].astype(np.int32),
                  d["values"].astype(np.float64), name)
    else:
        A = rebuild_matrix(name, str(d["generator"]))
    assert A.nnz == int(d["nnz"])
    return A, d


def rebuild_matrix(name, desc):
    """Matrices whose fixtures store only their generator."""
    from mexk import synthetic as S

    if desc.startswith("diagonal_test_matrix"):
        return S.diagonal_test_matrix(1000)
    if desc == "2*I, n=64":
        n = 64
        return S.CSR(n, np.arange(n + 1, dtype=np.int32), np.arange(n, dtype=np.int32), np.full(n, 2.0))
    if desc.startswith("diag(-1,-2,-3"):
        n = 90
        return S.CSR(n, np.arange(n + 1, dtype=np.int32), np.arange(n, dtype=np.int32),
                     np.tile([-1.0, -2.0, -3.0], n // 3))
    if desc.startswith("laplacian_2d("):
        return S.laplacian_2d(int(desc[len("laplacian_2d("):-1]))
    if desc.startswith("convection_diffusion_3d("):
        N, pe = desc[len("convection_diffusion_3d("):-1].split(",")
        return S.convection_diffusion_3d(int(N), float(pe))
    if desc == "config0(n=2000, seed=0)":
        return S.config0().A
    if desc == "skew300":
        B = S.random_diag_dominant(300, 3, seed=21).to_dense()
        np.fill_diagonal(B, 0.0)
        Ad = B - B.T
        rows, cols = np.nonzero(Ad)
        rp = np.zeros(301, dtype=np.int32)
        np.cumsum(np.bincount(rows, minlength=300), out=rp[1:])
        return S.CSR(300, rp, cols.astype(np.int32), Ad[rows, cols], "skew300")
    if desc.startswith("diag_linspace("):
        n, lo, hi = desc[len("diag_linspace("):-1].split(",")
        n = int(n)
        return S.CSR(n, np.arange(n + 1, dtype=np.int32), np.arange(n, dtype=np.int32),
                     np.linspace(float(lo), float(hi), n))
    raise KeyError(desc)


def fixture_stepping(d):
    """The TimeSteppingParams a fixture was made with (None: the defaults)."""
    ts = {k[3:]: d[k].item() for k in d if k.startswith("ts_")}
    return ts or None


# Small fixtures with stored inputs; the full-size heat2048 record only holds
# a decision sequence and a fingerprint of y.
GOLDEN_NAMES = sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz"))
                      if not os.path.basename(p).endswith("_reference.npz"))


def format_step(s):
    """The reference's [STEP] line (std::cout default float format = %g)."""
    t_done, dt, err, m_used, acc, rej = s
    return f"[STEP] t={t_done:g} dt={dt:g} err={err:g} m_used={m_used} accepts={acc} rejects={rej}"


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle as O

    O.build(with_reference=None)
    return O
