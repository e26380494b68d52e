"""Row sharding on CPU ranks (gloo): the partition and halo plans of
mexk.sharding against the drop-in C++ API's partition_rows /
build_owner_ghost_maps / validate_ghost_maps (the reference's rules,
main.cu:526-744), and a sharded restarted-Arnoldi solve over world sizes 2
and 3 -- halo exchange of q_j before each SpMV, one all-reduce per
Gram-Schmidt pass -- that reproduces the single-partition solve of the
oracle to 1e-12 with the same accept/reject decisions. No GPU."""
import os
import socket
import subprocess

import numpy as np
import pytest

from conftest import ROOT

FP64_TOL = 1e-12


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


@pytest.fixture(scope="module")
def ghost_check(tmp_path_factory):
    from mexk._lib import BUILD

    exe = tmp_path_factory.mktemp("cpp") / "ghost_check"
    if not os.path.exists(os.path.join(BUILD, "libmexk_host.so")):
        pytest.skip("host library not built")
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"), "-o", str(exe),
                    os.path.join(ROOT, "tests", "cpp", "ghost_check.cpp"), "-L", BUILD, f"-Wl,-rpath,{BUILD}",
                    "-lmexk_host", "-lmexk"], check=True)
    return str(exe)


def _matrices():
    from mexk import synthetic as S

    yield "random500", S.random_diag_dominant(500, 6, seed=3)
    yield "powerlaw2000", S.power_law(2000, seed=5)
    yield "heat20", S.laplacian_2d(20)
    yield "tiny3", S.random_diag_dominant(3, 1, seed=1)  # fewer rows than partitions: empty blocks


@pytest.mark.parametrize("parts", [2, 3, 4])
def test_plans_match_cpp_ghost_maps(ghost_check, tmp_path, parts):
    from mexk import sharding as SH
    from mexk.bincsr import write_bincsr

    for name, A in _matrices():
        path = tmp_path / f"{name}.bincsr"
        write_bincsr(path, A.row_ptr, A.col_idx, A.values)
        p = subprocess.run([ghost_check, str(path), str(parts)], capture_output=True, text=True, timeout=120)
        assert p.returncode == 0 and p.stdout.strip().endswith("VALID"), (name, p.stderr)
        plans = [SH.build_halo_plan(A.row_ptr, A.col_idx, A.values, r, parts) for r in range(parts)]
        SH.validate_plans(plans)
        got = {"PART": {}, "RECV": {}, "SEND": {}, "OFFS": {}}
        for ln in p.stdout.splitlines():
            f = ln.split()
            if f[0] == "PART":
                got["PART"][int(f[1])] = (int(f[2]), int(f[3]))
            elif f[0] in ("RECV", "SEND"):
                got[f[0]][(int(f[1]), int(f[2]))] = [int(c) for c in f[3:]]
            elif f[0] == "OFFS":
                bar = f.index("|")
                got["OFFS"][int(f[1])] = (int(f[2]), int(f[3]), [int(c) for c in f[4:bar]],
                                          [int(c) for c in f[bar + 1:]])
        for r, pl in enumerate(plans):
            assert got["PART"][r] == (pl.n_local, len(pl.values)), (name, r)
            assert {o: got["RECV"][(r, o)] for (rr, o) in got["RECV"] if rr == r} == \
                {o: list(v) for o, v in pl.recv.items()}, (name, r)
            assert {c: got["SEND"][(r, c)] for (rr, c) in got["SEND"] if rr == r} == \
                {c: list(v) for c, v in pl.send.items()}, (name, r)
            tot_r, tot_s, roff, soff = got["OFFS"][r]
            assert tot_r == pl.n_ghost and tot_s == sum(len(v) for v in pl.send.values())
            # the reference's offsets count only peers with entries before them, in rank order
            assert [roff[o] for o in pl.recv] == [pl.recv_offsets[o] for o in pl.recv]
            assert [soff[c] for c in pl.send] == [pl.send_offsets[c] for c in pl.send]


def test_cpp_validate_rejects_mismatch(ghost_check, tmp_path):
    from mexk import sharding as SH
    from mexk import synthetic as S
    from mexk.bincsr import write_bincsr

    A = S.random_diag_dominant(400, 5, seed=9)
    path = tmp_path / "a.bincsr"
    write_bincsr(path, A.row_ptr, A.col_idx, A.values)
    p = subprocess.run([ghost_check, str(path), "3", "corrupt"], capture_output=True, text=True, timeout=120)
    assert p.returncode == 1 and "Ghost map mismatch between owner" in p.stderr
    plans = [SH.build_halo_plan(A.row_ptr, A.col_idx, A.values, r, 3) for r in range(3)]
    c = next(iter(plans[0].send))
    plans[0].send[c] = plans[0].send[c][:-1]
    with pytest.raises(ValueError, match="Ghost map mismatch"):
        SH.validate_plans(plans)


def test_local_renumbering_reproduces_the_product():
    """Each rank's renumbered row block times [x_owned | x_ghost] equals its
    rows of A x."""
    import scipy.sparse as sp

    from mexk import sharding as SH
    from mexk import synthetic as S

    A = S.power_law(3000, seed=7)
    x = np.random.default_rng(1).standard_normal(A.n)
    full = sp.csr_matrix((A.values, A.col_idx, A.row_ptr), shape=(A.n, A.n)) @ x
    for parts in (2, 5):
        for r in range(parts):
            pl = SH.build_halo_plan(A.row_ptr, A.col_idx, A.values, r, parts)
            ext = np.concatenate([x[pl.row_start:pl.row_end], x[pl.incoming()]])
            loc = sp.csr_matrix((pl.values, pl.col_idx, pl.row_ptr), shape=(pl.n_local, len(ext))) @ ext
            assert np.array_equal(loc, full[pl.row_start:pl.row_end])


# ---------------------------------------------------------------- sharded solve
def _sharded_expmv(plan, v_loc, t, m, tol, oracle_mod):
    """The reference's time-stepping solve (main.cu:1411-1571) on this rank's
    rows: q_j's halo exchange before each SpMV, CGS2 with one all-reduce of
    the (j+1)-vector of dots per pass and one of |w|^2, the small exponential
    replicated on every rank, the lift on local rows. Returns (y_loc, steps)."""
    import scipy.sparse as sp
    import torch

    from mexk import sharding as SH

    n_loc = plan.n_local
    A_loc = sp.csr_matrix((plan.values, plan.col_idx, plan.row_ptr), shape=(n_loc, n_loc + plan.n_ghost))

    def allreduce(vec):
        return SH.allreduce_sum(torch.from_numpy(np.ascontiguousarray(vec, dtype=np.float64))).numpy()

    def start(x):
        nrm = float(np.sqrt(allreduce(np.array([x @ x]))[0]))
        return nrm, x * ((1.0 / nrm) if nrm > 1e-14 else 1.0)

    dt_max, dt_min, dt = t, max(1e-12, t * 1e-6), t
    v_norm, q = start(v_loc)
    V = np.zeros((m + 1, n_loc))
    V[0] = q
    t_done, accepted, steps = 0.0, 0, []
    y = np.zeros(n_loc)
    while t_done < t and accepted < 1000:
        dt = min(dt, t - t_done)
        rejects = 0
        H = np.zeros((m + 1, m))
        k_used, breakdown = 0, False
        for j in range(m):
            x_ext = SH.halo_exchange(plan, torch.from_numpy(V[j].copy())).numpy()
            w = A_loc @ x_ext
            h1 = allreduce(V[: j + 1] @ w)
            w = w - V[: j + 1].T @ h1
            h2 = allreduce(V[: j + 1] @ w)
            w = w - V[: j + 1].T @ h2
            H[: j + 1, j] = h1 + h2
            beta = float(np.sqrt(allreduce(np.array([w @ w]))[0]))
            k_used = j + 1
            if not (beta >= 1e-14) or np.isinf(beta):
                breakdown = True
                break
            H[j + 1, j] = beta
            V[j + 1] = w * (1.0 / beta)
        while True:
            wH, err = oracle_mod.small_expm(H, k_used, dt, v_norm)
            if breakdown:
                err = 0.0
            steps.append((dt, err, k_used, accepted, rejects))
            if err <= tol or breakdown:
                y = oracle_mod.lift(V, k_used, wH, v_norm)
                t_done += dt
                accepted += 1
                if t_done >= t:
                    return y, steps
                v_norm, V[0] = start(y)
                if err < 0.1 * tol:
                    dt = min(dt * 1.5 * 0.8, dt_max)
                break
            rejects += 1
            if rejects >= 20:
                return y, steps
            dt = max(dt * 0.5 * 0.8, dt_min)
    return y, steps


def _rank_main(rank, world, port, case, out_dir):
    import sys

    for p in (os.path.join(ROOT, "matrix-exp-krylov_gb300"), os.path.join(ROOT, "oracle"),
              os.path.join(ROOT, "tests")):
        if p not in sys.path:
            sys.path.insert(0, p)
    import torch.distributed as dist

    import oracle as O
    from mexk import sharding as SH

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        A, v, t, m = _case(case)
        plan = SH.build_halo_plan(A.row_ptr, A.col_idx, A.values, rank, world)
        y_loc, steps = _sharded_expmv(plan, v[plan.row_start:plan.row_end], t, m, 1e-6, O)
        np.savez(os.path.join(out_dir, f"rank{rank}.npz"), y=y_loc, steps=np.array(steps), r0=plan.row_start)
        dist.barrier()
    finally:
        dist.destroy_process_group()


def _case(case):
    from mexk import synthetic as S

    if case == "cfg0":
        P = S.config0()
        return P.A, P.v, P.t, P.m
    if case == "heat":
        A = S.laplacian_2d(40)
        return A, np.random.default_rng(1).uniform(0, 1, A.n), 0.01, 30
    A = S.power_law(3000, seed=11)
    return A, np.random.default_rng(12).standard_normal(A.n), 0.3, 20


@pytest.mark.parametrize("world", [2, 3])
@pytest.mark.parametrize("case", ["cfg0", "heat", "powerlaw"])
def test_sharded_solve_matches_single_partition(tmp_path, oracle_mod, world, case):
    import torch.multiprocessing as mp

    mp.start_processes(_rank_main, args=(world, _free_port(), case, str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    parts = sorted((np.load(tmp_path / f"rank{r}.npz") for r in range(world)), key=lambda d: int(d["r0"]))
    y = np.concatenate([d["y"] for d in parts])
    steps = parts[0]["steps"]
    for d in parts[1:]:
        assert np.array_equal(d["steps"], steps)  # every rank took the same decisions
    A, v, t, m = _case(case)
    y_ref, st, ref_steps = oracle_mod.expmv(A, v, t, m)
    assert np.linalg.norm(y - y_ref) <= FP64_TOL * np.linalg.norm(y_ref)
    assert len(steps) == len(ref_steps)
    for s, r in zip(steps, ref_steps):
        # dt, m_used, accepts, rejects equal; err to its leading digits (near
        # the rounding floor its last ones differ: the decisions must not)
        assert s[0] == r[1] and int(s[2]) == r[3] and int(s[3]) == r[4] and int(s[4]) == r[5]
        assert abs(s[1] - r[2]) <= 1e-5 * abs(r[2]) + 1e-3 * 1e-6
