"""The allocation-free Gram-Schmidt entry point against the allocating one.

mexk_gram_schmidt_f64_noalloc serves callers that may not allocate device
memory (their own pool or arena owns it all, or they bind the C ABI over FFI
and only pass buffers). It must give the same h, beta and next basis vector
as mexk_arnoldi_step, whose context allocated its scratch, on two calls in a
row (the second reuses the shared scratch array left by the first).
This file is collected last.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12


def test_noalloc_gram_schmidt_matches_context_step():
    import torch

    from mexk import synthetic as S
    from mexk._lib import check, lib
    from mexk.api import Context

    A = S.power_law(5000, seed=8)
    n = A.n
    m = 6
    v = np.random.default_rng(9).standard_normal(n)
    V0 = (v / np.linalg.norm(v))[None, :]
    with Context(A, m_alloc=m) as ctx:
        ctx.set_basis(V0)
        ref = [ctx.arnoldi_step(j) for j in range(2)]
        Vref = ctx.get_basis(3)
    rp = torch.from_numpy(A.row_ptr).cuda()
    ci = torch.from_numpy(A.col_idx).cuda()
    va = torch.from_numpy(A.values).cuda()
    Vd = torch.zeros((3, n), dtype=torch.float64, device="cuda")
    Vd[0] = torch.from_numpy(V0[0]).cuda()
    w = torch.empty(n, dtype=torch.float64, device="cuda")
    h = torch.empty(4, dtype=torch.float64, device="cuda")
    beta = torch.empty(1, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    for j in range(2):  # two calls in a row through the shared scratch
        check(lib().mexk_spmv_f64(n, rp.data_ptr(), ci.data_ptr(), va.data_ptr(), Vd[j].data_ptr(),
                                  w.data_ptr(), None))
        check(lib().mexk_gram_schmidt_f64_noalloc(n, j + 1, Vd.data_ptr(), n, w.data_ptr(), 1, h.data_ptr(),
                                                   beta.data_ptr(), Vd[j + 1].data_ptr(), None))
        torch.cuda.synchronize()
        ok_ref, h_ref, beta_ref = ref[j]
        assert ok_ref
        hj = h.cpu().numpy()[: j + 1]
        scale = np.abs(h_ref).max()
        assert np.abs(hj - h_ref).max() <= FP64_TOL * scale
        assert abs(beta.item() - beta_ref) <= FP64_TOL * beta_ref
        q = Vd[j + 1].cpu().numpy()
        assert np.linalg.norm(q - Vref[j + 1]) <= FP64_TOL * np.linalg.norm(Vref[j + 1])


def test_noalloc_full_width_and_breakdown():
    """k = 64 (the largest basis it takes) against the context step, then a
    vector inside the span of V: beta = 0 and q left untouched."""
    import torch

    from mexk import synthetic as S
    from mexk._lib import check, lib
    from mexk.api import Context

    A = S.random_diag_dominant(20000, 8, seed=21)
    n, k = A.n, 64
    v = np.random.default_rng(22).standard_normal(n)
    with Context(A, m_alloc=k) as ctx:
        ctx.set_basis((v / np.linalg.norm(v))[None, :])
        for j in range(k - 1):
            assert ctx.arnoldi_step(j)[0]
        Vk = ctx.get_basis(k)
        ok_ref, h_ref, beta_ref = ctx.arnoldi_step(k - 1)
        q_ref = ctx.get_basis(k + 1)[k]
    assert ok_ref
    Vd = torch.from_numpy(np.ascontiguousarray(Vk)).cuda()
    rp = torch.from_numpy(A.row_ptr).cuda()
    ci = torch.from_numpy(A.col_idx).cuda()
    va = torch.from_numpy(A.values).cuda()
    w = torch.empty(n, dtype=torch.float64, device="cuda")
    h = torch.empty(k, dtype=torch.float64, device="cuda")
    beta = torch.empty(1, dtype=torch.float64, device="cuda")
    q = torch.full((n,), 7.0, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    check(lib().mexk_spmv_f64(n, rp.data_ptr(), ci.data_ptr(), va.data_ptr(), Vd[k - 1].data_ptr(), w.data_ptr(),
                              None))
    check(lib().mexk_gram_schmidt_f64_noalloc(n, k, Vd.data_ptr(), n, w.data_ptr(), 1, h.data_ptr(),
                                               beta.data_ptr(), q.data_ptr(), None))
    torch.cuda.synchronize()
    scale = np.abs(h_ref).max()
    assert np.abs(h.cpu().numpy() - h_ref).max() <= FP64_TOL * scale
    assert abs(beta.item() - beta_ref) <= FP64_TOL * beta_ref
    assert np.linalg.norm(q.cpu().numpy() - q_ref) <= FP64_TOL * np.linalg.norm(q_ref)
    # breakdown: w = a combination of the columns of V leaves nothing after the projection
    # (small coefficients: the rounding left over stays far below the 1e-14 breakdown threshold)
    coeffs = torch.from_numpy(1e-3 * np.random.default_rng(23).standard_normal(k)).cuda()
    w2 = (coeffs[:, None] * Vd).sum(0).contiguous()
    q2 = torch.full((n,), 7.0, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    check(lib().mexk_gram_schmidt_f64_noalloc(n, k, Vd.data_ptr(), n, w2.data_ptr(), 1, h.data_ptr(),
                                               beta.data_ptr(), q2.data_ptr(), None))
    torch.cuda.synchronize()
    assert beta.item() == 0.0
    assert torch.all(q2 == 7.0).item()
    assert np.abs(h.cpu().numpy() - coeffs.cpu().numpy()).max() <= 1e-12 * np.abs(coeffs.cpu().numpy()).max()


def test_noalloc_rejects_oversized_k():
    from mexk._lib import lib

    assert lib().mexk_gram_schmidt_f64_noalloc(100, 65, 1, 100, 1, 1, 1, 1, 1, None) != 0
    assert b"k must be" in lib().mexk_last_error_detail()
