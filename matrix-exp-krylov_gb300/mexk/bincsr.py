"""Binary CSR v1 (``.bincsr``) and MatrixMarket writers for synthetic inputs.

Layout as specified by the reference's docs/binary_csr_v1.md: a 64-byte
little-endian header (magic ``CSR\\0\\0\\0\\0\\1``, version, flags, nrows,
ncols, nnz, index dtype 1=u32/2=u64, value dtype 1=f32/2=f64, two reserved
zero u64) followed by indptr, indices and data with no padding. The header
packing follows the format table, the same one tools/generate_matrices.py:143-156
writes. Reading is done by the C++ loader (CSRHost::from_binary_csr); the
numpy reader here only serves tests and scripts.
"""
from __future__ import annotations

import struct

import numpy as np

MAGIC = b"CSR\x00\x00\x00\x00\x01"
HEADER = struct.Struct("<8sIIQQQIIQQ")
FLAG_SORTED = 1 << 0
FLAG_NO_DUP = 1 << 1
FLAG_SYM_UPPER = 1 << 2


def write_bincsr(path, row_ptr, col_idx, values, ncols=None, index_dtype="u32", value_dtype="f64",
                 flags=FLAG_SORTED | FLAG_NO_DUP, version=1, reserved=(0, 0)):
    n = int(len(row_ptr) - 1)
    ncols = n if ncols is None else int(ncols)
    nnz = int(len(col_idx))
    it = {"u32": (np.uint32, 1), "u64": (np.uint64, 2)}[index_dtype]
    vt = {"f32": (np.float32, 1), "f64": (np.float64, 2)}[value_dtype]
    with open(path, "wb") as f:
        f.write(HEADER.pack(MAGIC, version, flags, n, ncols, nnz, it[1], vt[1], reserved[0], reserved[1]))
        np.asarray(row_ptr).astype(it[0]).tofile(f)
        np.asarray(col_idx).astype(it[0]).tofile(f)
        np.asarray(values).astype(vt[0]).tofile(f)


def read_bincsr(path):
    """Returns (n, ncols, row_ptr int64, col_idx int64, values float64, flags)."""
    with open(path, "rb") as f:
        hdr = HEADER.unpack(f.read(64))
        magic, version, flags, n, ncols, nnz, idt, vdt, _, _ = hdr
        if magic != MAGIC or version != 1:
            raise ValueError("not a Binary CSR v1 file")
        it = {1: np.uint32, 2: np.uint64}[idt]
        vt = {1: np.float32, 2: np.float64}[vdt]
        rp = np.fromfile(f, dtype=it, count=n + 1).astype(np.int64)
        ci = np.fromfile(f, dtype=it, count=nnz).astype(np.int64)
        va = np.fromfile(f, dtype=vt, count=nnz).astype(np.float64)
    return n, ncols, rp, ci, va, flags


def write_matrix_market(path, n, rows, cols, vals, symmetric=False, pattern=False, ncols=None):
    """Coordinate MatrixMarket text (1-based indices)."""
    ncols = n if ncols is None else ncols
    field = "pattern" if pattern else "real"
    sym = "symmetric" if symmetric else "general"
    with open(path, "w") as f:
        f.write(f"%%MatrixMarket matrix coordinate {field} {sym}\n")
        f.write(f"{n} {ncols} {len(rows)}\n")
        for r, c, v in zip(rows, cols, vals):
            if pattern:
                f.write(f"{r + 1} {c + 1}\n")
            else:
                f.write(f"{r + 1} {c + 1} {float(v):.17g}\n")
