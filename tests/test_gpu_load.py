"""Binary CSR straight into a context (mexk_context_load_bincsr): the same
matrix as the host upload of the file's CSR (solves bitwise equal), every
rejection of the host loader with its message, chunk-crossing sizes, and the
matrix_exp program with and without --host-load."""
import os
import subprocess

import numpy as np
import pytest

from mexk import bincsr as B
from mexk import synthetic as S

pytestmark = pytest.mark.gpu


def _csr_of_file(path):
    n, _, rp, ci, va, _ = B.read_bincsr(path)
    return S.CSR(n, rp.astype(np.int32), ci.astype(np.int32), va)


def _same_solves(path, window_ok, m=20, t=0.3):
    from mexk.api import Context

    A = _csr_of_file(path)
    v = np.random.default_rng(5).uniform(0, 1, A.n)
    forms = [("fp64", 0), ("mixed", 0)] + ([("mixed", 2)] if window_ok else [])
    with Context.from_bincsr(path, m_alloc=m) as ca, Context(A, m_alloc=m) as cb:
        assert (ca.n, ca.nnz) == (A.n, A.nnz)
        assert ca.load_info["max_abs"] == np.abs(A.values).max()
        assert ca.load_info["checks_passed"] == 4
        for prec, w in forms:
            ya, ra = ca.expmv(v, t, m, precision=prec, controller="search" if w else "reference", window=w)
            yb, rb = cb.expmv(v, t, m, precision=prec, controller="search" if w else "reference", window=w)
            assert np.array_equal(ya, yb), (prec, w)
            assert ra["attempts"] == rb["attempts"]


@pytest.mark.parametrize("idt", ["u32", "u64"])
@pytest.mark.parametrize("vdt", ["f32", "f64"])
def test_load_matches_host_upload(tmp_path, idt, vdt):
    A = S.random_diag_dominant(3000, 8, seed=11)
    p = tmp_path / "a.bincsr"
    B.write_bincsr(p, A.row_ptr, A.col_idx, A.values, index_dtype=idt, value_dtype=vdt)
    _same_solves(p, window_ok=False)
    H = S.laplacian_2d(150, h=1.0 / 151)
    q = tmp_path / "h.bincsr"
    B.write_bincsr(q, H.row_ptr, H.col_idx, H.values, index_dtype=idt, value_dtype=vdt)
    _same_solves(q, window_ok=True, t=1e-3)


def test_load_crosses_chunks(tmp_path):
    """u64 indices (168 MB) and f32 values (84 MB) cross the 64 MB staging
    chunks; the heat2048 matrix."""
    from mexk.api import Context

    H = S.laplacian_2d(2048)
    p = tmp_path / "heat2048.bincsr"
    B.write_bincsr(p, H.row_ptr, H.col_idx, H.values, index_dtype="u64", value_dtype="f32")
    A = _csr_of_file(p)
    v = np.random.default_rng(1).uniform(0, 1, A.n)
    with Context.from_bincsr(p, m_alloc=30) as ca:
        ya, _ = ca.expmv(v, 1e-5, 30, precision="mixed", controller="search", window=2)
    with Context(A, m_alloc=30) as cb:
        yb, _ = cb.expmv(v, 1e-5, 30, precision="mixed", controller="search", window=2)
    assert np.array_equal(ya, yb)


def _bad_cases():
    from test_loaders import BAD

    return BAD


@pytest.mark.parametrize("case", _bad_cases(), ids=[b[0] for b in _bad_cases()])
def test_load_rejects_like_host_loader(tmp_path, case):
    from mexk._lib import MexkError
    from mexk.api import Context

    name, data, msg = case
    p = tmp_path / "bad.bincsr"
    p.write_bytes(data)
    with pytest.raises(MexkError) as e:
        Context.from_bincsr(p, m_alloc=1)
    if name == "sym square":  # symmetric_upper files are left to the host loader
        assert "symmetric_upper" in str(e.value)
    else:
        assert msg in str(e.value), str(e.value)


def _run_cli(args, out):
    from mexk._lib import BUILD

    env = dict(os.environ, OUTPUT_Y_FILE=str(out))
    p = subprocess.run([os.path.join(BUILD, "matrix_exp")] + args, env=env, capture_output=True, text=True,
                       timeout=600)
    keep = [l for l in p.stdout.splitlines() if not l.startswith(("METRIC", "Saved y to"))]
    return p.returncode, keep, p.stderr


def test_cli_direct_load_matches_host_load(tmp_path):
    A = S.random_diag_dominant(4000, 6, seed=21)
    p = tmp_path / "a.bincsr"
    B.write_bincsr(p, A.row_ptr, A.col_idx, A.values, index_dtype="u64", value_dtype="f32")
    rc1, out1, err1 = _run_cli([str(p), "--m", "20", "--t", "0.5"], tmp_path / "y1.txt")
    rc2, out2, err2 = _run_cli([str(p), "--m", "20", "--t", "0.5", "--host-load"], tmp_path / "y2.txt")
    assert rc1 == 0 and rc2 == 0, (err1, err2)
    assert out1 == out2
    assert np.array_equal(np.loadtxt(tmp_path / "y1.txt"), np.loadtxt(tmp_path / "y2.txt"))
    # a row-check failure: the header line, then the host loader's message
    bad = tmp_path / "bad.bincsr"
    bad.write_bytes(B.HEADER.pack(B.MAGIC, 1, 1, 2, 2, 2, 1, 2, 0, 0) + np.array((0, 2, 2), np.uint32).tobytes()
                    + np.array((1, 0), np.uint32).tobytes() + np.array((1.0, 2.0)).tobytes())
    r1 = _run_cli([str(bad)], tmp_path / "z1.txt")
    r2 = _run_cli([str(bad), "--host-load"], tmp_path / "z2.txt")
    assert r1[0] == r2[0] == 1 and r1[1] == r2[1] and r1[2] == r2[2], (r1, r2)
