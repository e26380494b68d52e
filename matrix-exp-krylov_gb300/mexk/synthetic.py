"""Seeded synthetic inputs for exp(tA)v workloads.

The reference ships no matrices and its generator
(tools/generate_matrices.py:39-83) draws density-based COO matrices with a
positive diagonal, which cannot produce these workloads, so the generators
here are written for this project. Every matrix is returned as CSR with
int32 row pointers / column indices (sorted, no duplicates) and float64
values, the layout CSRHost holds after loading (main.cu:86-95).

All randomness comes from ``numpy.random.default_rng(seed)`` (PCG64), the
generator family the reference's tool uses (tools/generate_matrices.py:47).
A matrix's draws come first in the stream, the vectors' draws after them.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np


@dataclass
class CSR:
    n: int
    row_ptr: np.ndarray  # int32 (n+1)
    col_idx: np.ndarray  # int32 (nnz)
    values: np.ndarray  # float64 (nnz)
    name: str = ""

    @property
    def nnz(self) -> int:
        return int(self.col_idx.size)

    def to_dense(self) -> np.ndarray:
        d = np.zeros((self.n, self.n))
        rows = np.repeat(np.arange(self.n), np.diff(self.row_ptr))
        np.add.at(d, (rows, self.col_idx), self.values)
        return d

    def max_abs(self) -> float:
        return float(np.abs(self.values).max()) if self.nnz else 0.0


@dataclass
class Problem:
    """One exp(tA)v problem: matrix, start vector(s), and solver settings."""

    A: CSR
    v: np.ndarray  # (n,) or (r, n) for a block of right-hand sides
    t: float
    m: int
    tol: float = 1e-6
    max_restarts: int = 0
    meta: dict = field(default_factory=dict)


# ---------------------------------------------------------------- helpers
def _assemble(n: int, rows: np.ndarray, cols: np.ndarray, vals: np.ndarray, diag: np.ndarray,
              name: str) -> CSR:
    """Off-diagonal entries sorted by (row, col), plus one diagonal per row."""
    rows = rows.astype(np.int64, copy=False)
    cols = cols.astype(np.int64, copy=False)
    off_counts = np.bincount(rows, minlength=n)
    less = np.bincount(rows[cols < rows], minlength=n)  # off-diagonals left of the diagonal
    nnz = rows.size + n
    row_ptr = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(off_counts + 1, out=row_ptr[1:])
    # destination of each off-diagonal: its index + rows inserted before + 1 if right of diag
    dest = np.arange(rows.size, dtype=np.int64) + rows + (cols > rows)
    col_idx = np.empty(nnz, dtype=np.int32)
    values = np.empty(nnz, dtype=np.float64)
    col_idx[dest] = cols
    values[dest] = vals
    dpos = row_ptr[:-1] + less
    col_idx[dpos] = np.arange(n, dtype=np.int32)
    values[dpos] = diag
    if row_ptr[-1] > np.iinfo(np.int32).max:
        raise ValueError("nnz exceeds int32")
    return CSR(n, row_ptr.astype(np.int32), col_idx, values, name)


def _distinct_offdiag_columns(rng: np.random.Generator, n: int, degrees: np.ndarray):
    """For row i draw degrees[i] distinct columns uniformly from [0, n) minus {i}.

    Duplicates are re-drawn (in sorted order of the current draw) until none
    remain; the result is sorted by (row, col).
    """
    degrees = np.asarray(degrees, dtype=np.int64)
    if np.any(degrees > n - 1):
        raise ValueError("row degree exceeds n-1")
    rows = np.repeat(np.arange(n, dtype=np.int64), degrees)
    cols = rng.integers(0, n - 1, size=rows.size, dtype=np.int64)
    cols += cols >= rows  # skip the diagonal
    key = rows * n + cols
    while True:
        key.sort()
        dup = np.zeros(key.size, dtype=bool)
        dup[1:] = key[1:] == key[:-1]
        nd = int(dup.sum())
        if nd == 0:
            break
        r = key[dup] // n
        c = rng.integers(0, n - 1, size=nd, dtype=np.int64)
        c += c >= r
        key[dup] = r * n + c
    return key // n, key % n


# ---------------------------------------------------------------- workloads
def random_diag_dominant(n: int, degree: int | np.ndarray, seed: int, off_scale: float = 0.5,
                         diag_shift: float = 1.0, rng: np.random.Generator | None = None) -> CSR:
    """Rows with ``degree`` distinct uniform off-diagonal columns, values
    U[-off_scale, off_scale], diagonal -(row |off| sum) - diag_shift."""
    rng = np.random.default_rng(seed) if rng is None else rng
    deg = np.full(n, degree, dtype=np.int64) if np.isscalar(degree) else np.asarray(degree)
    rows, cols = _distinct_offdiag_columns(rng, n, deg)
    vals = rng.uniform(-off_scale, off_scale, size=rows.size)
    diag = -np.bincount(rows, weights=np.abs(vals), minlength=n) - diag_shift
    return _assemble(n, rows, cols, vals, diag, f"random_n{n}")


def laplacian_2d(N: int, h: float | None = None) -> CSR:
    """A = Delta_h on an N x N interior grid with Dirichlet boundary:
    diagonal -4/h^2, the four neighbours +1/h^2, natural ordering p = i + N j."""
    h = 1.0 / (N + 1) if h is None else h
    n = N * N
    inv = 1.0 / (h * h)
    p = np.arange(n, dtype=np.int64)
    i = p % N
    j = p // N
    cand = np.stack([p - N, p - 1, p, p + 1, p + N], axis=1)
    ok = np.stack([j > 0, i > 0, np.ones(n, bool), i < N - 1, j < N - 1], axis=1)
    vals = np.where(cand == p[:, None], -4.0 * inv, inv)
    counts = ok.sum(axis=1)
    row_ptr = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(counts, out=row_ptr[1:])
    return CSR(n, row_ptr.astype(np.int32), cand[ok].astype(np.int32), vals[ok].astype(np.float64),
               f"laplacian2d_{N}")


def laplacian_2d_mode(N: int, p: int, q: int, h: float | None = None):
    """Eigenvector sin(p pi x) sin(q pi y) of laplacian_2d and its eigenvalue."""
    h = 1.0 / (N + 1) if h is None else h
    x = np.arange(1, N + 1) * h
    u = np.outer(np.sin(q * np.pi * x), np.sin(p * np.pi * x)).ravel()  # index i + N j
    lam = -(4.0 / (h * h)) * (math.sin(p * math.pi * h / 2) ** 2 + math.sin(q * math.pi * h / 2) ** 2)
    return u, lam


def convection_diffusion_3d(N: int, pe: float, h: float | None = None,
                            velocity=(1.0, 0.5, 0.25)) -> CSR:
    """A = Delta_h - (b . grad)_upwind on an N^3 Dirichlet grid, b = velocity*pe.

    First-order upwinding for b > 0: the backward neighbour in direction d
    gets 1/h^2 + b_d/h, the forward neighbour 1/h^2, the diagonal
    -6/h^2 - sum_d b_d/h. Ordering p = i + N j + N^2 k.
    """
    h = 1.0 / (N + 1) if h is None else h
    n = N ** 3
    inv2 = 1.0 / (h * h)
    b = [vel * pe for vel in velocity]
    p = np.arange(n, dtype=np.int64)
    i = p % N
    j = (p // N) % N
    k = p // (N * N)
    NN = N * N
    cand = np.stack([p - NN, p - N, p - 1, p, p + 1, p + N, p + NN], axis=1)
    ok = np.stack([k > 0, j > 0, i > 0, np.ones(n, bool), i < N - 1, j < N - 1, k < N - 1], axis=1)
    coef = np.array([inv2 + b[2] / h, inv2 + b[1] / h, inv2 + b[0] / h,
                     -6.0 * inv2 - (b[0] + b[1] + b[2]) / h, inv2, inv2, inv2])
    vals = np.broadcast_to(coef, cand.shape)
    counts = ok.sum(axis=1)
    row_ptr = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(counts, out=row_ptr[1:])
    return CSR(n, row_ptr.astype(np.int32), cand[ok].astype(np.int32), vals[ok].astype(np.float64),
               f"convdiff3d_{N}_pe{pe:g}")


def power_law(n: int, seed: int, zipf_a: float = 1.8, min_deg: int = 2, max_deg: int = 2048,
              rng: np.random.Generator | None = None) -> CSR:
    """Row off-diagonal counts ~ Zipf(zipf_a) clipped to [min_deg, max_deg],
    distinct uniform columns, values U[-1,1], diagonal -(row |off| sum) - 0.5."""
    rng = np.random.default_rng(seed) if rng is None else rng
    deg = np.clip(rng.zipf(zipf_a, size=n), min_deg, min(max_deg, n - 1))
    return random_diag_dominant(n, deg, seed, off_scale=1.0, diag_shift=0.5, rng=rng)


def diagonal_test_matrix(n: int) -> CSR:
    """The CLI's built-in matrix A = diag(1 + i/n) (main.cu:2196-2217)."""
    i = np.arange(n)
    return CSR(n, np.arange(n + 1, dtype=np.int32), i.astype(np.int32), 1.0 + i / n,
               f"diag_{n}")


# ---------------------------------------------------------------- configs
def config0(n: int = 2000, seed: int = 0) -> Problem:
    """Random sparse A, 10 distinct off-diagonals per row, v = 0.1, t = 1, m = 30."""
    A = random_diag_dominant(n, 10, seed)
    return Problem(A, np.full(n, 0.1), 1.0, 30, meta={"config": 0, "seed": seed})


def config1(N: int = 2048, seed: int = 1) -> Problem:
    """Heat equation: A = 2D Dirichlet Laplacian / h^2, h = 1/(N+1); v ~ U[0,1]; t = 1e-5."""
    A = laplacian_2d(N)
    v = np.random.default_rng(seed).uniform(0.0, 1.0, size=A.n)
    return Problem(A, v, 1e-5, 30, meta={"config": 1, "seed": seed, "grid": N})


def config2(n: int = 8_388_608, seed: int = 2) -> Problem:
    """Irregular power-law rows; v ~ N(0,1); t = 0.5; m = 40."""
    rng = np.random.default_rng(seed)
    A = power_law(n, seed, rng=rng)
    v = rng.standard_normal(n)
    return Problem(A, v, 0.5, 40, meta={"config": 2, "seed": seed})


def config3_problem(index: int, n_range=(1e4, 2e6), nrhs: int = 16) -> Problem:
    """Problem ``index`` (seed 100+index) of the batched uneven workload."""
    seed = 100 + index
    rng = np.random.default_rng(seed)
    n = int(round(10 ** rng.uniform(math.log10(n_range[0]), math.log10(n_range[1]))))
    deg = int(rng.integers(5, 21))
    A = random_diag_dominant(n, deg, seed, rng=rng)
    V = rng.standard_normal((nrhs, n))
    t = float(rng.uniform(0.1, 2.0))
    return Problem(A, V, t, 30, meta={"config": 3, "seed": seed, "degree": deg})


def config3_sizes(index: int):
    """(n, degree, t) of problem ``index`` of the batched workload, drawn
    from numpy's generator seeded 100 + index: n log-uniform in [1e4, 2e6],
    degree uniform in {5..20}, t uniform in [0.1, 2]."""
    rng = np.random.default_rng(100 + index)
    n = int(round(10 ** rng.uniform(4.0, math.log10(2e6))))
    deg = int(rng.integers(5, 21))
    t = float(rng.uniform(0.1, 2.0))
    return n, deg, t


def config3_generated(index: int, nrhs: int = 16, device: str = "cuda") -> Problem:
    """Problem ``index`` of the batched workload generated on the GPU (torch's
    seeded Philox generator, seed 100 + index): config 0's structure -- each
    row has ``degree`` distinct off-diagonal columns uniform over the other
    columns, values U[-0.5, 0.5], diagonal -(row |off| sum) - 1 -- with the
    sizes of config3_sizes and nrhs N(0,1) start vectors. Much faster than
    the numpy generator at the workload's 1.5e9 nonzeros; not bit-identical
    to it."""
    import torch

    n, deg, t = config3_sizes(index)
    g = torch.Generator(device=device)
    g.manual_seed(100 + index)
    rows = torch.arange(n, device=device, dtype=torch.int64).unsqueeze(1)

    def draw(r):
        c = torch.randint(0, n - 1, (r.shape[0], deg), generator=g, device=device, dtype=torch.int64)
        return c + (c >= r).to(torch.int64)  # skip the diagonal

    cols, _ = torch.sort(draw(rows), dim=1)
    for _ in range(64):
        dup = (cols[:, 1:] == cols[:, :-1]).any(dim=1)
        idx = dup.nonzero().squeeze(1)
        if idx.numel() == 0:
            break
        fresh, _ = torch.sort(draw(rows[idx]), dim=1)
        cols[idx] = fresh
    else:
        raise RuntimeError("duplicate columns left after 64 redraws")
    vals = torch.rand((n, deg), generator=g, device=device, dtype=torch.float64) - 0.5
    diag = -vals.abs().sum(dim=1, keepdim=True) - 1.0
    allc = torch.cat([cols, rows], dim=1)
    allv = torch.cat([vals, diag], dim=1)
    order = torch.argsort(allc, dim=1)
    allc = torch.gather(allc, 1, order).to(torch.int32).reshape(-1).cpu().numpy()
    allv = torch.gather(allv, 1, order).reshape(-1).cpu().numpy()
    V = torch.randn((nrhs, n), generator=g, device=device, dtype=torch.float64).cpu().numpy()
    row_ptr = np.arange(0, (n + 1) * (deg + 1), deg + 1, dtype=np.int32)
    A = CSR(n, row_ptr, allc, allv, f"config3_{index}")
    return Problem(A, V, t, 30, meta={"config": 3, "seed": 100 + index, "degree": deg, "generator": "torch"})


def config4(N: int = 128, pe: float = 10.0, seed: int = 4) -> Problem:
    """3D convection-diffusion, upwinded velocity (1,0.5,0.25)*pe, h = 1/(N+1); v ~ U[0,1]; t = 1."""
    A = convection_diffusion_3d(N, pe)
    v = np.random.default_rng(seed).uniform(0.0, 1.0, size=A.n)
    return Problem(A, v, 1.0, 30, meta={"config": 4, "seed": seed, "pe": pe, "grid": N})
