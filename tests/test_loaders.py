"""CSRHost loaders (host/csr_host.cpp) through the csr_tool program: valid
Binary CSR v1 and MatrixMarket inputs give the expected CSR (and the same CSR
as the reference's own loader when its build is present); malformed inputs
exit with status 1 and the reference's message. CPU only."""
import gzip
import os
import struct
import subprocess

import numpy as np
import pytest

from mexk import bincsr as B
from mexk import synthetic as S

TOOL = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "matrix-exp-krylov_gb300",
                    "_build", "csr_tool")


@pytest.fixture(scope="module", autouse=True)
def built():
    if not os.path.exists(TOOL):
        from mexk import build

        build.build_host()
    assert os.path.exists(TOOL)


def load(path, tmp_path):
    out = str(tmp_path / "out")
    p = subprocess.run([TOOL, str(path), out], capture_output=True, text=True, timeout=120)
    if p.returncode != 0:
        return p.returncode, p.stderr, None
    rp = np.fromfile(out + ".rowptr", dtype=np.int32)
    ci = np.fromfile(out + ".col", dtype=np.int32)
    va = np.fromfile(out + ".val", dtype=np.float64)
    return 0, p.stdout, (rp, ci, va)


def small_matrix():
    return S.random_diag_dominant(50, 4, seed=3)


@pytest.mark.parametrize("idt", ["u32", "u64"])
@pytest.mark.parametrize("vdt", ["f32", "f64"])
def test_bincsr_roundtrip(tmp_path, idt, vdt):
    A = small_matrix()
    path = tmp_path / "a.bincsr"
    B.write_bincsr(path, A.row_ptr, A.col_idx, A.values, index_dtype=idt, value_dtype=vdt)
    rc, out, csr = load(path, tmp_path)
    assert rc == 0, out
    rp, ci, va = csr
    assert np.array_equal(rp, A.row_ptr) and np.array_equal(ci, A.col_idx)
    want = A.values.astype(np.float32).astype(np.float64) if vdt == "f32" else A.values
    assert np.array_equal(va, want)
    assert f"index_dtype={idt} value_dtype={vdt} symmetric_upper=no" in out


def test_bincsr_symmetric_upper_expands(tmp_path):
    rng = np.random.default_rng(5)
    n = 30
    D = np.triu(rng.standard_normal((n, n)) * (rng.random((n, n)) < 0.2)) + np.eye(n)
    rows, cols = np.nonzero(D)
    rp = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(np.bincount(rows, minlength=n), out=rp[1:])
    path = tmp_path / "s.bincsr"
    B.write_bincsr(path, rp, cols, D[rows, cols], flags=B.FLAG_SORTED | B.FLAG_NO_DUP | B.FLAG_SYM_UPPER)
    rc, out, csr = load(path, tmp_path)
    assert rc == 0, out
    full = D + np.triu(D, 1).T
    r2, c2 = np.nonzero(full)
    assert np.array_equal(csr[1], c2) and np.allclose(csr[2], full[r2, c2])


def test_matrix_market_general_symmetric_pattern_duplicates(tmp_path):
    p = tmp_path / "g.mtx"
    p.write_text("%%MatrixMarket matrix coordinate real general\n% comment\n3 3 5\n"
                 "1 1 2.0\n3 2 -1.5\n1 1 0.5\n2 3 4\n3 3 1\n")
    rc, out, csr = load(p, tmp_path)
    assert rc == 0, out
    assert list(csr[0]) == [0, 1, 2, 4] and list(csr[1]) == [0, 2, 1, 2]
    assert np.allclose(csr[2], [2.5, 4.0, -1.5, 1.0])
    p = tmp_path / "s.mtx"
    p.write_text("%%MatrixMarket matrix coordinate pattern symmetric\n3 3 2\n2 1\n3 3\n")
    rc, out, csr = load(p, tmp_path)
    assert rc == 0
    assert list(csr[0]) == [0, 1, 2, 3] and list(csr[1]) == [1, 0, 2] and np.allclose(csr[2], 1.0)


def test_matrix_market_gz(tmp_path):
    p = tmp_path / "g.mtx.gz"
    with gzip.open(p, "wt") as f:
        f.write("%%MatrixMarket matrix coordinate real general\n2 2 2\n1 2 3.5\n2 1 -1\n")
    rc, out, csr = load(p, tmp_path)
    assert rc == 0, out
    assert list(csr[1]) == [1, 0] and np.allclose(csr[2], [3.5, -1.0])


def _hdr(**kw):
    d = dict(magic=B.MAGIC, version=1, flags=3, n=2, ncols=2, nnz=2, idt=1, vdt=2, r0=0, r1=0)
    d.update(kw)
    return B.HEADER.pack(d["magic"], d["version"], d["flags"], d["n"], d["ncols"], d["nnz"], d["idt"], d["vdt"],
                         d["r0"], d["r1"])


def _payload(rp=(0, 1, 2), ci=(0, 1), va=(1.0, 2.0)):
    return np.array(rp, np.uint32).tobytes() + np.array(ci, np.uint32).tobytes() + np.array(va).tobytes()


BAD = [
    ("too small", b"CSR", "Binary CSR file too small"),
    ("magic", _hdr(magic=b"CSR\x00\x00\x00\x00\x02") + _payload(), "Invalid Binary CSR magic"),
    ("version", _hdr(version=2) + _payload(), "Unsupported Binary CSR version 2"),
    ("index dtype", _hdr(idt=3) + _payload(), "Unsupported index_dtype=3"),
    ("value dtype", _hdr(vdt=7) + _payload(), "Unsupported value_dtype=7"),
    ("reserved", _hdr(r1=5) + _payload(), "Reserved header fields must be zero"),
    ("int32", _hdr(n=2 ** 31) + _payload(), "exceed int32 limits"),
    ("size", _hdr() + _payload() + b"x", "Binary CSR size mismatch"),
    ("indptr0", _hdr() + _payload(rp=(1, 1, 2)), "indptr[0] must be 0"),
    ("monotone", _hdr() + _payload(rp=(0, 2, 1)), "indptr is not non-decreasing at row 1"),
    ("indptr end", _hdr() + _payload(rp=(0, 1, 1)), "indptr[nrows] != nnz"),
    ("column", _hdr() + _payload(ci=(0, 2)), "Column index out of range at k=1"),
    ("sorted", _hdr(n=1, nnz=2) + np.array((0, 2), np.uint32).tobytes() + np.array((1, 0), np.uint32).tobytes()
     + np.array((1.0, 2.0)).tobytes(), "Row 0 is not sorted"),
    ("dup", _hdr(n=1, nnz=2, flags=2) + np.array((0, 2), np.uint32).tobytes()
     + np.array((1, 1), np.uint32).tobytes() + np.array((1.0, 2.0)).tobytes(), "Row 0 has duplicates"),
    ("sym square", _hdr(flags=4, ncols=3) + _payload(), "symmetric_upper requires square matrix"),
]


@pytest.mark.parametrize("name,data,msg", BAD, ids=[b[0] for b in BAD])
def test_bincsr_rejects(tmp_path, name, data, msg):
    p = tmp_path / "bad.bincsr"
    p.write_bytes(data)
    rc, err, _ = load(p, tmp_path)
    assert rc == 1 and msg in err, (rc, err)


MTX_BAD = [
    ("object", "%%MatrixMarket vector coordinate real general\n", "object must be 'matrix'"),
    ("format", "%%MatrixMarket matrix array real general\n", "Only 'coordinate' format"),
    ("field", "%%MatrixMarket matrix coordinate complex general\n", "Only 'real' or 'pattern'"),
    ("symmetry", "%%MatrixMarket matrix coordinate real hermitian\n", "Only 'general' or 'symmetric'"),
    ("no header", "1 1 1\n", "Failed to parse MatrixMarket header"),
    ("bounds", "%%MatrixMarket matrix coordinate real general\n2 2 1\n3 1 1.0\n", "index out of bounds r=3 c=1"),
    ("count", "%%MatrixMarket matrix coordinate real general\n2 2 3\n1 1 1.0\n", "Expected 3 entries but read 1"),
    ("value", "%%MatrixMarket matrix coordinate real general\n2 2 1\n1 1\n", "Failed to read value for entry 0"),
]


@pytest.mark.parametrize("name,text,msg", MTX_BAD, ids=[b[0] for b in MTX_BAD])
def test_matrix_market_rejects(tmp_path, name, text, msg):
    p = tmp_path / "bad.mtx"
    p.write_text(text)
    rc, err, _ = load(p, tmp_path)
    assert rc == 1 and msg in err, (rc, err)


def test_loader_matches_reference_loader(tmp_path, oracle_mod):
    """Same CSR as the reference's own CSRHost loader (main_cpu.cpp build)."""
    if not oracle_mod.have_reference():
        pytest.skip("reference build not present")
    import ctypes as C

    R = oracle_mod.ref()
    A = S.power_law(3000, seed=12)
    cases = []
    p1 = tmp_path / "a.bincsr"
    B.write_bincsr(p1, A.row_ptr, A.col_idx, A.values)
    cases.append((p1, 1))
    rows = np.repeat(np.arange(A.n), np.diff(A.row_ptr))
    p2 = tmp_path / "a.mtx"
    B.write_matrix_market(p2, A.n, rows[:4000], A.col_idx[:4000], A.values[:4000])
    cases.append((p2, 0))
    for path, binary in cases:
        r, c, z = C.c_int(), C.c_int(), C.c_longlong()
        h = R.ref_load(str(path).encode(), binary, C.byref(r), C.byref(c), C.byref(z))
        rp = np.zeros(r.value + 1, np.int32)
        ci = np.zeros(z.value, np.int32)
        va = np.zeros(z.value)
        R.ref_copy_csr(h, rp.ctypes.data_as(C.POINTER(C.c_int)), ci.ctypes.data_as(C.POINTER(C.c_int)),
                       va.ctypes.data_as(C.POINTER(C.c_double)))
        R.ref_free(h)
        rc, out, csr = load(path, tmp_path)
        assert rc == 0
        assert np.array_equal(csr[0], rp) and np.array_equal(csr[1], ci) and np.array_equal(csr[2], va)


# ------------------------------------------------------------------ header probe (C ABI, no GPU)
HEADER_BAD = [b for b in BAD if b[0] in ("too small", "magic", "version", "index dtype", "value dtype", "reserved",
                                         "int32", "size")]


@pytest.mark.parametrize("name,data,msg", HEADER_BAD, ids=[b[0] for b in HEADER_BAD])
def test_bincsr_probe_rejects(tmp_path, name, data, msg):
    """mexk_bincsr_probe: the header checks of the host loader, its messages."""
    import ctypes as C

    from mexk._lib import BincsrInfo, lib

    p = tmp_path / "bad.bincsr"
    p.write_bytes(data)
    info = BincsrInfo()
    assert lib().mexk_bincsr_probe(str(p).encode(), C.byref(info)) == 1
    assert msg in lib().mexk_last_error_detail().decode()


def test_bincsr_probe_reads_header(tmp_path):
    import ctypes as C

    from mexk._lib import BincsrInfo, lib

    A = small_matrix()
    p = tmp_path / "a.bincsr"
    B.write_bincsr(p, A.row_ptr, A.col_idx, A.values, index_dtype="u64", value_dtype="f32", flags=B.FLAG_SORTED)
    info = BincsrInfo()
    assert lib().mexk_bincsr_probe(str(p).encode(), C.byref(info)) == 0
    assert (info.rows, info.cols, info.nnz) == (A.n, A.n, A.nnz)
    assert (info.index_dtype, info.value_dtype, info.flags, info.checks_passed) == (2, 1, 1, 1)
    assert lib().mexk_bincsr_probe(str(tmp_path / "missing.bincsr").encode(), C.byref(info)) == 1
    assert "Could not open binary CSR file" in lib().mexk_last_error_detail().decode()
