"""mexk_profile_kernel, the source of the bench's per-kernel table: every
kernel kind of a solve times as a positive duration, and the kinds that
update w in place (timed from a fresh state per launch) imply rates a GB300
can deliver -- a launch that skipped its work would read as tens of TB/s."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FP64_KINDS = ["spmv", "gs_dot", "gs_upd_dot", "gs_upd_norm", "normalize", "lift", "controller"]
MIXED_KINDS = ["spmv", "gram_dot", "gram_update", "gram_norm", "lift", "controller"]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_every_kind_times(precision):
    from mexk import synthetic as S
    from mexk.api import Context

    A = S.laplacian_2d(256, h=1.0 / 2049)  # 65,536 rows: the pattern form
    v = np.random.default_rng(3).uniform(0, 1, A.n)
    n = A.n
    s = 8 if precision == "fp64" else 4
    with Context(A, m_alloc=30) as ctx:
        ctx.expmv(v, 1e-5, 30, precision=precision, controller="search")
        for kind in FP64_KINDS if precision == "fp64" else MIXED_KINDS:
            ms = ctx.profile_kernel(kind, 12, 3, precision)
            assert 0.0 < ms < 50.0, (kind, ms)
            if kind in ("gs_upd_dot", "gs_upd_norm", "normalize"):
                # at least two vectors of n move per launch: far below 20 TB/s
                assert 2 * n * s / (ms * 1e-3) < 20e12, (kind, ms)
        if precision == "mixed":
            ctx.expmv(v, 1e-5, 30, precision="mixed", controller="search", window=2)
            for j in (1, 12):
                for kind in ("spmv_dots", "gram_update"):
                    ms = ctx.profile_kernel(kind, j, 3, "mixed")
                    assert 0.0 < ms < 50.0, (kind, j, ms)
            # the fused form of the window-2 steps: one launch for steps 1..j
            ctx.set_lanczos_form("fused")
            assert ctx.lanczos_form() == "fused"
            ctx.expmv(v, 1e-5, 30, precision="mixed", controller="search", window=2)
            t29 = ctx.profile_kernel("lanczos_cycle", 29, 3, "mixed")
            t5 = ctx.profile_kernel("lanczos_cycle", 5, 3, "mixed")
            assert 0.0 < t5 < t29 < 50.0, (t5, t29)
            # a step writes one FP32 vector at least: far below 20 TB/s
            assert 28 * n * 4 / (t29 * 1e-3) < 20e12
