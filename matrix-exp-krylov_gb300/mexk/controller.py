"""Learned step-size / Krylov-dimension controller: data, training, weights.

Training data come from the method itself. For a solve state (start vector
q1 = y/|y| at time t_done) and each Krylov dimension m in M_SET, the GPU
builds the Arnoldi basis (mexk_krylov_build); the host then evaluates the
residual estimate |H(k,k-1) [exp(tau H_k) e1]_{k-1}| |v| on a 1/8-octave
grid of steps tau and keeps the largest passing step tau_max(m). Every grid
point is one (tau, m, cost, error) tuple. The state's best dimension m* maximises
tau_max(m) / cost(m) under the measured cycle-cost model below; the trajectory
advances with (m*, tau_max(m*)) so the states seen are those the learned
policy visits. Two networks: one priced for full Gram-Schmidt cycles, one for
the window-2 short recurrence of a symmetric A (cycles linear in m).

Network (8 -> 64 -> 64 -> 2, GELU, FP32; mexk_mlp_* kernels):
  inputs  the basis features of csrc/controller_net.cuh (same formulas here)
  output0 log2(tau_max(m) * |H_k|_1) for the basis just built
  output1 (m* - 10) / 50, the dimension for the next cycle
Weights are stored as a raw little-endian float32 file of MEXK_NET_TOTAL
values (controller_net.f32) with a JSON description beside it.
"""
from __future__ import annotations

import ctypes as C
import json
import math
import os
import time

import numpy as np

from ._lib import PREC_FP64, PREC_MIXED, check, lib

NET_IN, NET_HID, NET_OUT = 8, 64, 2
NET_PARAMS = 4866
NET_TOTAL = 4886
M_SET = (10, 20, 30, 40, 50, 60)
FP32_FLOOR = 2.0 ** -24
ERR_BUDGET_REL = 5e-7  # accepted errors, relative to |y|, the relaxed tolerance may spend
HERE = os.path.dirname(os.path.abspath(__file__))
WEIGHTS = os.path.join(HERE, "controller_net.f32")
META = os.path.join(HERE, "controller_net.json")
# the network for solves with a window of 2 (symmetric A), trained on that cycle's cost
WINDOW_WEIGHTS = os.path.join(HERE, "controller_net_window.f32")


# ------------------------------------------------------------------ features
def features(H, k, rem, tol, vnorm, tau_prev, err_prev):
    """Host copy of net::basis_features (controller_net.cuh). H: (m+1, m)."""
    Hk = np.triu(H[:k, :k], -1)
    n1 = max(np.abs(Hk).sum(axis=0).max(), 1e-300)
    fro = float((Hk ** 2).sum())
    upper = float((np.triu(Hk, 2) ** 2).sum())
    hk = abs(H[k, k - 1])
    jm = k // 2
    hm = abs(H[jm + 1, jm])
    span = max(k - 1 - jm, 1)
    f = np.array([
        math.log2(n1 * max(rem, 1e-300)),
        math.log2(hk / n1 + 1e-30),
        (math.log2(hk + 1e-300) - math.log2(hm + 1e-300)) / span,
        math.log2(tol / max(vnorm, 1e-300)),
        k / 64.0,
        math.sqrt(upper / fro) if fro > 0 else 0.0,
        math.log2(tau_prev * n1) if tau_prev > 0 else math.log2(n1 * max(rem, 1e-300)),
        math.log2(err_prev / tol) if err_prev > 0 else 0.0,
    ], dtype=np.float64)
    f[~np.isfinite(f)] = 0.0
    return np.clip(f, -200, 200).astype(np.float32), n1


# ------------------------------------------------------------------ cost model
# Cycles are priced by their measured time on GB300 (mixed precision, the
# candidate-step search, one cycle per graph launch), fitted as
# F + C m + D m^2 milliseconds. The network sees no problem size, so the
# labels come from one consistent price per kind of cycle:
#   "arnoldi"  full Gram-Schmidt (any A): the 128^3 convection-diffusion
#              workload, 2,097,152 rows; m = 10..60 -> 0.54, 1.27, 2.28,
#              3.56, 5.18, 7.00 ms per cycle (the sweeps grow with k);
#   "window2"  the short recurrence of a symmetric A (ortho_window = 2):
#              heat 2048^2, 4,194,304 rows; m = 10..60 -> 0.38, 0.65, 0.93,
#              1.23, 1.59, 1.94 ms per cycle (every step reads four vectors).
CYCLE_COST_MS = {
    "arnoldi": (0.0924, 0.030694, 0.0014114),
    "window2": (0.14639, 0.022511, 0.00012409),
}


def cycle_cost(m, kind="arnoldi"):
    """Seconds per Krylov cycle of dimension m under the measured model."""
    F, C_, D = CYCLE_COST_MS[kind]
    return (F + C_ * m + D * m * m) * 1e-3


# ------------------------------------------------------------------ step search
def residual(H, k, tau, beta):
    from scipy.linalg import expm

    E = expm(tau * H[:k, :k])
    return abs(H[k, k - 1] * E[k - 1, 0]) * beta, E[:k, 0]


def largest_tau(H, k, beta, tol, rem, start, breakdown=False):
    """Largest step on a 1/8-octave grid (capped at rem) whose estimate passes.
    Returns (tau, wH, err, tuples[(tau, err)])."""
    tuples = []
    if breakdown:
        err, w = residual(H, k, rem, beta)
        return rem, w, 0.0, [(rem, 0.0)]
    tau = min(max(start, 1e-300), rem)
    err, w = residual(H, k, tau, beta)
    tuples.append((tau, err))
    if err <= tol:
        best = (tau, w, err)
        while tau < rem:
            tau = min(tau * 2 ** 0.125, rem)
            err, w = residual(H, k, tau, beta)
            tuples.append((tau, err))
            if err > tol:
                break
            best = (tau, w, err)
    else:
        best = None
        for _ in range(400):
            tau *= 2 ** -0.125
            err, w = residual(H, k, tau, beta)
            tuples.append((tau, err))
            if err <= tol:
                best = (tau, w, err)
                break
        if best is None:
            return None, None, None, tuples
    return best[0], best[1], best[2], tuples


# ------------------------------------------------------------------ data
def sweep_problem(ctx, A, v, t, precision="mixed", tol=1e-6, max_states=60, m_set=M_SET, log=None,
                  kind="arnoldi"):
    """Walk one solve with per-state sweeps over m. Returns (X, T, tuples)."""
    L = lib()
    prec = PREC_MIXED if precision == "mixed" else PREC_FP64
    floor = FP32_FLOOR if precision == "mixed" else 0.0
    budget = ERR_BUDGET_REL if precision == "mixed" else 0.0
    v = np.ascontiguousarray(v, dtype=np.float64)
    beta = C.c_double(0.0)
    check(L.mexk_krylov_start(ctx.handle, prec, v.ctypes.data_as(C.POINTER(C.c_double)), C.byref(beta)))
    beta = beta.value
    t_done, tau_prev, err_prev = 0.0, 0.0, 0.0
    err_acc = 0.0  # the errors accepted so far (the relaxed tolerance's budget)
    X, T, tuples = [], [], []
    mmax = min(max(m_set), ctx.m_alloc, A.n - 1)
    for _ in range(max_states):
        rem = t - t_done
        if rem <= 0 or beta <= 1e-300:
            break
        # the device's rule for a mixed-precision solve under the candidate
        # search: max(tol, min(2^-24 |y|, 5e-7 |y| - accepted errors))
        tol_eff = max(tol, min(floor * beta, budget * beta - err_acc))
        per_m = []
        for m in m_set:
            if m > mmax:
                continue
            H = np.zeros((m + 1, m), order="F")
            k = C.c_int(0)
            check(L.mexk_krylov_build(ctx.handle, prec, m, 1, H.ctypes.data_as(C.POINTER(C.c_double)),
                                      C.byref(k)), "mexk_krylov_build")
            k = k.value
            f, n1 = features(H, k, rem, tol_eff, beta, tau_prev, err_prev)
            start = tau_prev * 2 if tau_prev > 0 else rem
            tau, w, err, tp = largest_tau(H, k, beta, tol_eff, rem, start, breakdown=k < m)
            cost = cycle_cost(m, kind)
            tuples.extend((tt, m, cost, ee) for tt, ee in tp)
            if tau is None:
                continue
            per_m.append((m, k, tau, w, err, f, n1, cost))
        if not per_m:
            break
        best = max(per_m, key=lambda r: r[2] / r[7])
        m_star = best[0]
        for (m, k, tau, w, err, f, n1, cost) in per_m:
            X.append(f)
            T.append([math.log2(tau * n1), (m_star - 10) / 50.0])
        # advance with the best (m*, tau_max(m*)): rebuild its basis, lift, restart
        m, k, tau, w, err = best[0], best[1], best[2], best[3], best[4]
        H = np.zeros((m + 1, m), order="F")
        kk = C.c_int(0)
        check(L.mexk_krylov_build(ctx.handle, prec, m, 1, H.ctypes.data_as(C.POINTER(C.c_double)), C.byref(kk)))
        coef = np.ascontiguousarray(beta * w[:k], dtype=np.float64)
        nb = C.c_double(0.0)
        check(L.mexk_krylov_advance(ctx.handle, prec, k, coef.ctypes.data_as(C.POINTER(C.c_double)), C.byref(nb)))
        beta = nb.value
        t_done += tau
        err_acc += err
        tau_prev, err_prev = tau, err
        if log:
            log(f"  t={t_done:.3e} m*={m_star} tau={tau:.3e} beta={beta:.3e}")
    return np.array(X, np.float32).reshape(-1, NET_IN), np.array(T, np.float32).reshape(-1, NET_OUT), tuples


def skew_problem(n, degree, seed, shift=0.1):
    """Oscillatory test matrix: random sparse S, A = S - S^T - shift*I."""
    from . import synthetic as S

    B = S.random_diag_dominant(n, degree, seed=seed)
    rows = np.repeat(np.arange(n), np.diff(B.row_ptr))
    off = B.col_idx != rows
    r, c, x = rows[off], B.col_idx[off].astype(np.int64), B.values[off]
    rr = np.concatenate([r, c, np.arange(n)])
    cc = np.concatenate([c, r, np.arange(n)])
    xx = np.concatenate([x, -x, np.full(n, -shift)])
    key = rr * n + cc
    order = np.argsort(key, kind="stable")
    key, xx = key[order], xx[order]
    uk, first = np.unique(key, return_index=True)
    sums = np.add.reduceat(xx, first)
    rows_u = (uk // n).astype(np.int64)
    rp = np.zeros(n + 1, np.int64)
    np.cumsum(np.bincount(rows_u, minlength=n), out=rp[1:])
    return S.CSR(n, rp.astype(np.int32), (uk % n).astype(np.int32), sums, f"skew{n}")


# Times for the 3D convection-diffusion sweeps (h = 1/129): the solution
# decays by a moderate factor while t*|A| stays in the hundreds.
CONVDIFF_T = {1.0: 2e-3, 10.0: 2e-3, 100.0: 1e-3, 1000.0: 1e-4}


def training_problems(scale="small", kind="arnoldi"):
    """Seeded problems for the sweeps. "arnoldi": 3D convection-diffusion at
    the four Peclet numbers of the learned-controller workload (coarser
    grids, times from CONVDIFF_T), 2D heat at the heat2048 stiffness, and
    oscillatory skew-symmetric-plus-shift matrices. "window2" (symmetric A
    only): 2D heat over grids and horizons around the heat2048 workload's
    stiffness and 3D diffusion (the convection-diffusion operator at Pe = 0)."""
    from . import synthetic as S

    probs = []
    if kind == "window2":
        for N in (64, 128, 256, 384, 512, 768, 1024, 1536):
            A = S.laplacian_2d(N, h=1.0 / 2049)
            v = np.random.default_rng(N).uniform(0, 1, A.n)
            for f in (1, 3):
                probs.append((f"heat{N}_{f}t", A, v, f * 1e-5))
        for N in (20, 28, 40):
            A = S.convection_diffusion_3d(N, 0.0, h=1.0 / 129)
            v = np.random.default_rng(100 + N).uniform(0, 1, A.n)
            for t in (2e-3, 6e-3):
                probs.append((f"diffusion{N}_t{t:g}", A, v, t))
        return probs
    wide = scale == "wide"
    grids = (20, 28, 40, 52) if wide else ((20, 28, 40) if scale == "small" else (48, 64))
    for N in grids:
        for pe, t in CONVDIFF_T.items():
            A = S.convection_diffusion_3d(N, pe, h=1.0 / 129)
            v = np.random.default_rng(int(pe) + N).uniform(0, 1, A.n)
            probs.append((f"convdiff{N}_pe{pe:g}", A, v, t))
            if wide:  # the same operator over a twice longer horizon
                probs.append((f"convdiff{N}_pe{pe:g}_2t", A, v, 2 * t))
    for N in ((64, 128, 192, 256, 320, 384) if wide else (64, 128, 192, 256)):
        A = S.laplacian_2d(N, h=1.0 / 2049)
        v = np.random.default_rng(N).uniform(0, 1, A.n)
        probs.append((f"heat{N}", A, v, 1e-5))
        if wide:
            probs.append((f"heat{N}_3t", A, v, 3e-5))
    for seed in range(6 if wide else 3):
        A = skew_problem(20000, 6, seed=50 + seed)
        v = np.random.default_rng(60 + seed).standard_normal(A.n)
        probs.append((f"skew20k_{seed}", A, v, 15.0))
    return probs


# ------------------------------------------------------------------ training
def init_weights(X, T, seed=0):
    rng = np.random.default_rng(seed)
    w = np.zeros(NET_TOTAL, np.float32)
    o = 0

    def take(shape, fan_in):
        nonlocal o
        size = int(np.prod(shape))
        w[o:o + size] = (rng.standard_normal(size) * math.sqrt(2.0 / fan_in)).astype(np.float32)
        o += size

    take((NET_IN, NET_HID), NET_IN)
    o += NET_HID
    take((NET_HID, NET_HID), NET_HID)
    o += NET_HID
    take((NET_HID, NET_OUT), NET_HID)
    o += NET_OUT
    assert o == NET_PARAMS
    w[NET_PARAMS:NET_PARAMS + NET_IN] = X.mean(axis=0)
    w[NET_PARAMS + NET_IN:NET_PARAMS + 2 * NET_IN] = np.maximum(X.std(axis=0), 1e-3)
    w[NET_PARAMS + 2 * NET_IN:NET_PARAMS + 2 * NET_IN + NET_OUT] = T.mean(axis=0)
    w[NET_PARAMS + 2 * NET_IN + NET_OUT:] = np.maximum(T.std(axis=0), 1e-3)
    return w


def train(X, T, epochs=400, batch=256, lr=2e-3, seed=0, log=None):
    """Adam on the GPU through mexk_mlp_adam_step. Returns (weights, losses)."""
    import torch

    L = lib()
    dev = "cuda"
    w = torch.from_numpy(init_weights(X, T, seed)).to(dev)
    adam = torch.zeros(2 * NET_PARAMS, dtype=torch.float32, device=dev)
    Xd = torch.from_numpy(np.ascontiguousarray(X, np.float32)).to(dev)
    Td = torch.from_numpy(np.ascontiguousarray(T, np.float32)).to(dev)
    scratch = torch.zeros(64 * NET_PARAMS, dtype=torch.float32, device=dev)
    parts = torch.zeros(64, dtype=torch.float32, device=dev)
    N = X.shape[0]
    rng = np.random.default_rng(seed)
    step = 0
    losses = []
    for ep in range(epochs):
        perm = torch.from_numpy(rng.permutation(N).astype(np.int32)).to(dev)
        lr_ep = lr * 0.5 * (1 + math.cos(math.pi * ep / epochs))
        tot = 0.0
        for b0 in range(0, N, batch):
            cnt = min(batch, N - b0)
            step += 1
            check(L.mexk_mlp_adam_step(w.data_ptr(), adam.data_ptr(), Xd.data_ptr(), Td.data_ptr(),
                                       perm.data_ptr() + 4 * b0, cnt, step, lr_ep, parts.data_ptr(),
                                       scratch.data_ptr(), None), "mexk_mlp_adam_step")
            tot += float(parts.sum()) if (b0 + batch >= N) else 0.0
        losses.append(evaluate_loss(w, Xd, Td))
        if log and (ep % 50 == 0 or ep == epochs - 1):
            log(f"epoch {ep}: loss {losses[-1]:.4f}")
    return w.cpu().numpy(), losses


def forward(weights, X):
    """Network outputs for rows X (GPU kernel)."""
    import torch

    w = torch.as_tensor(weights, dtype=torch.float32).cuda() if not torch.is_tensor(weights) else weights
    Xd = torch.as_tensor(np.ascontiguousarray(X, np.float32)).cuda()
    Y = torch.zeros((X.shape[0], NET_OUT), dtype=torch.float32, device="cuda")
    check(lib().mexk_mlp_forward(w.data_ptr(), Xd.data_ptr(), X.shape[0], Y.data_ptr(), None))
    torch.cuda.synchronize()
    return Y.cpu().numpy()


def evaluate_loss(w, Xd, Td):
    import torch

    Y = torch.zeros((Xd.shape[0], NET_OUT), dtype=torch.float32, device="cuda")
    check(lib().mexk_mlp_forward(w.data_ptr(), Xd.data_ptr(), Xd.shape[0], Y.data_ptr(), None))
    om = w[NET_PARAMS + 2 * NET_IN:NET_PARAMS + 2 * NET_IN + NET_OUT]
    osd = w[NET_PARAMS + 2 * NET_IN + NET_OUT:]
    return float((((Y - Td) / osd) ** 2).mean())


def save(weights, meta, path=WEIGHTS):
    """Weights as raw little-endian float32 at `path`, description beside it (.json)."""
    np.asarray(weights, dtype="<f4").tofile(path)
    with open(os.path.splitext(path)[0] + ".json", "w") as f:
        json.dump(meta, f, indent=1)


def load(path=WEIGHTS):
    w = np.fromfile(path, dtype="<f4")
    if w.size != NET_TOTAL:
        raise ValueError(f"{path}: expected {NET_TOTAL} floats, found {w.size}")
    return w


def main(argv=None):
    """python -m mexk.controller [--out DIR]: sweeps + training on the GPU."""
    import argparse

    from .api import Context

    ap = argparse.ArgumentParser()
    ap.add_argument("--epochs", type=int, default=400)
    ap.add_argument("--states", type=int, default=40)
    ap.add_argument("--data-out", default=None, help="also save the raw sweep data (.npz)")
    ap.add_argument("--scale", default="small", choices=["small", "wide", "large"], help="training problem set")
    ap.add_argument("--out", default=None, help="directory for the weights and their .json (default: the package)")
    ap.add_argument("--kind", default="arnoldi", choices=sorted(CYCLE_COST_MS),
                    help="cycle cost model: full Gram-Schmidt, or the window-2 short recurrence (symmetric A)")
    ap.add_argument("--m-set", default=",".join(str(m) for m in M_SET),
                    help="Krylov dimensions swept per state (the labels' m* is one of them)")
    args = ap.parse_args(argv)
    m_set = tuple(int(x) for x in args.m_set.split(","))
    t0 = time.time()
    Xs, Ts, ntuples, names = [], [], 0, []
    for name, A, v, t in training_problems(args.scale, args.kind):
        with Context(A, m_alloc=max(M_SET)) as ctx:
            X, T, tup = sweep_problem(ctx, A, v, t, max_states=args.states, kind=args.kind, m_set=m_set)
        Xs.append(X)
        Ts.append(T)
        ntuples += len(tup)
        names.append(name)
        print(f"{name}: n={A.n} samples={len(X)} tuples={len(tup)} ({time.time() - t0:.0f}s)", flush=True)
    X = np.concatenate(Xs)
    T = np.concatenate(Ts)
    if args.data_out:
        np.savez_compressed(args.data_out, X=X, T=T)
    w, losses = train(X, T, epochs=args.epochs, log=print)
    meta = {"inputs": NET_IN, "hidden": NET_HID, "outputs": NET_OUT, "samples": int(len(X)),
            "tuples": int(ntuples), "problems": names, "epochs": args.epochs, "final_loss": losses[-1],
            "initial_loss": losses[0], "m_set": list(m_set), "precision": "mixed",
            "cost_model": {"kind": args.kind, "cycle_ms_F_C_D": list(CYCLE_COST_MS[args.kind])},
            "scale": args.scale, "seconds": round(time.time() - t0, 1)}
    fname = os.path.basename(WEIGHTS if args.kind == "arnoldi" else WINDOW_WEIGHTS)
    save(w, meta, os.path.join(args.out, fname) if args.out else os.path.join(HERE, fname))
    print(json.dumps(meta))


if __name__ == "__main__":
    main()
