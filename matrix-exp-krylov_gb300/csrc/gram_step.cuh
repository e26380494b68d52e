// Device pieces of a mixed-precision Arnoldi step over at most two basis
// columns (j - 1 and j), shared by the dot sweep (gram_mixed.cu) and the
// SpMV that accumulates the same dot products in its row sums (spmv.cu).
//
// Partial sums live in GramArgs::part, slot-major: slot v of row block b at
// v * GRAM_MAX_ROW_BLOCKS + b; slots: a = U^T w at the column, b = U^T u_j at
// GRAM_BOFF + column, |w|^2 at GRAM_NWOFF.
#pragma once

#include "mexk_internal.cuh"

namespace mexk {
namespace {

constexpr unsigned kStepFull = 0xffffffffu;

// Sum over row blocks b < nrb(v) of the partials of nv values, value v in
// slot slot(v), into out[v]; every thread of the block calls it. FP64 adds
// and shuffles take about 64 and 100 cycles of latency on this GPU (FP32: 4),
// so the sum is shaped for depth: g2 adjacent lanes share a value, each loads
// PR partials per round and adds them as a tree, then the lanes combine by an
// xor butterfly (every lane ends with the same bits). The order depends only
// on nrb and nv.
template <int PR, typename SlotFn, typename NrbFn>
__device__ __forceinline__ void step_sum_partials(const double* part, int nv, SlotFn slot, NrbFn nrbf, double* out) {
    const int nt = static_cast<int>(blockDim.x);
    int g2 = 32;
    while (g2 > 1 && g2 * nv > nt) g2 >>= 1;
    const int t = threadIdx.x;
    const int vi = t / g2, sub = t % g2;
    double sum = 0.0;
    if (vi < nv) {
        const int nrb = nrbf(vi);
        const double* P = part + static_cast<size_t>(slot(vi)) * GRAM_MAX_ROW_BLOCKS;
        for (int b0 = sub; b0 < nrb; b0 += PR * g2) {
            double v[PR];
#pragma unroll
            for (int u = 0; u < PR; ++u) {
                const int b = b0 + u * g2;
                v[u] = b < nrb ? __ldcg(P + b) : 0.0;
            }
#pragma unroll
            for (int h = 1; h < PR; h <<= 1)
#pragma unroll
                for (int u = 0; u + h < PR; u += 2 * h) v[u] += v[u + h];
            sum += v[0];
        }
    }
    for (int o = 1; o < g2; o <<= 1) sum += __shfl_xor_sync(kStepFull, sum, o);
    if (vi < nv && sub == 0) out[vi] = sum;
}

// Block stage of a dot sweep: the warps' FP32 totals of NV values (lane l of
// warp q holds value l in s_red[q][l]) summed over the eight warps as an FP64
// tree, then written by thread v to the row block's slot slot(v) (skipped
// when slot(v) < 0).
template <int NV, typename SlotFn>
__device__ __forceinline__ void step_write_partials(double (&s_red)[8][NV], double* part, int rb, SlotFn slot) {
    __syncthreads();
    const int q = threadIdx.x;
    if (q < NV) {
        const double t = ((s_red[0][q] + s_red[1][q]) + (s_red[2][q] + s_red[3][q])) +
                         ((s_red[4][q] + s_red[5][q]) + (s_red[6][q] + s_red[7][q]));
        const int sl = slot(q);
        if (sl >= 0) part[static_cast<size_t>(sl) * GRAM_MAX_ROW_BLOCKS + rb] = t;
    }
}

__device__ __forceinline__ int step2_slot(int v, int kw, int lo) {
    return v < kw ? lo + v : (v < 2 * kw ? GRAM_BOFF + lo + (v - kw) : GRAM_NWOFF);
}

struct Step2Out {
    double sj, beta, hp, hj, g01, p, ip;
    bool bad;
};

// The part of the chain that needs only b_{j-1} = u_{j-1}.u_j, b_j = |u_j|^2
// and a_{j-1} (kw = 2; zeros for kw = 1) with s0 and ip_j: s_j, H(j, j-1)
// and the breakdown test of main.cu:1911 (the square root runs beside the
// chain, whose results are used only once the test has passed), s_j^2,
// G(j-1, j) and c_{j-1}.
struct Step2Pre {
    double sj, sj2, beta, g01, cp;
    bool bad;
};
__device__ __forceinline__ Step2Pre step2_chain_pre(double bjm1, double bj, double a0, int j, double s0, double ip_j) {
    Step2Pre o;
    o.sj = (bj > 0.0 && !isinf(bj)) ? rsqrt(bj) : 0.0;
    o.beta = j >= 1 ? sqrt(bj) * ip_j : 1.0;
    o.bad = !(o.beta >= 1e-14) || isinf(o.beta);
    o.sj2 = o.sj * o.sj;
    o.g01 = (s0 * bjm1) * o.sj;  // G(j-1, j)
    o.cp = (s0 * a0) * o.sj;     // c_{j-1}
    return o;
}

// The rest, from a_j, |w|^2 and c_{j-1}: c = s s_j a, h = c - (G - I) c, the
// update coefficients and the pre-scale p of the next column.
__device__ __forceinline__ Step2Out step2_chain_rest(const Step2Pre& pr, int kw, double aj, double nw, double cp,
                                                     int reortho) {
    Step2Out o;
    o.bad = pr.bad;
    const double sj2 = pr.sj2;
    const double cj = sj2 * aj;
    double hj = cj, hp = 0.0, g01 = 0.0, part;
    if (kw == 2) {
        g01 = pr.g01;
        hp = cp;
        if (reortho) {
            hp = cp - __dmul_rn(g01, cj);
            hj = cj - __dmul_rn(g01, cp);
        }
        const double gh0 = fma(g01, hj, hp), gh1 = hj + __dmul_rn(g01, hp);
        part = hp * (gh0 - 2.0 * cp) + hj * (gh1 - 2.0 * cj);
    } else {
        part = hj * (hj - 2.0 * cj);
    }
    const double w2 = sj2 * nw;
    const double u2 = w2 + part;
    double p = 1.0, ip = 1.0;
    if (u2 > 1e-8 * w2 && !isinf(u2)) {
        p = rsqrt(u2);
        ip = u2 * p;
    } else if (w2 > 0.0 && !isinf(w2)) {
        p = rsqrt(w2);
        ip = w2 * p;
    }
    o.sj = pr.sj;
    o.beta = pr.beta;
    o.hp = hp;
    o.hj = hj;
    o.g01 = g01;
    o.p = p;
    o.ip = ip;
    return o;
}

// The scalar chain of a step over at most two columns (kw = 1 or 2; lo =
// j + 1 - kw) from its sums tot = {a (kw), b (kw), |w|^2}: s_j = 1/|u_j|,
// H(j, j-1) = |u_j| / p_j with the breakdown test, the Gram entry G(j-1, j),
// c = s s_j a, h = c - (G - I) c, the update coefficients and the pre-scale
// p of the next column (one rsqrt, a few products, one rsqrt). s0 = s_{lo}
// (kw = 2), ip_j = 1 / (pre-scale of column j).
__device__ __forceinline__ Step2Out step2_chain(const double* tot, int kw, int j, int reortho, double s0,
                                                double ip_j) {
    const Step2Pre pr = step2_chain_pre(kw == 2 ? tot[kw] : 0.0, tot[2 * kw - 1], kw == 2 ? tot[0] : 0.0, j, s0, ip_j);
    return step2_chain_rest(pr, kw, tot[kw - 1], tot[2 * kw], pr.cp, reortho);
}

// Writes a step's results (step2_chain) into H, the Gram state and the
// solver state: H(j, j-1) (0 on breakdown, which also sets the breakdown
// flag and writes nothing else), s_j, G(j, j) and G(j-1, j), H(lo:j, j),
// the update coefficients, the next column's inverse pre-scale and the
// update scales. One thread.
__device__ __forceinline__ void step2_store(const GramArgs& g, int kw, const Step2Out& o, double s0) {
    const int j = g.j;
    const int lo = j + 1 - kw;
    GramState* gs = g.gs;
    double* G = gs->G;
    const size_t ldh = static_cast<size_t>(g.ldh);
    if (j >= 1) g.H[j + static_cast<size_t>(j - 1) * ldh] = o.bad ? 0.0 : o.beta;
    if (j >= 1 && o.bad) {
        g.st->breakdown = 1;
        g.st->k_used = j;
        return;
    }
    gs->s[j] = o.sj;
    G[j + static_cast<size_t>(j) * GRAM_LD] = 1.0;
    if (kw == 2) {
        G[lo + static_cast<size_t>(j) * GRAM_LD] = o.g01;
        G[j + static_cast<size_t>(lo) * GRAM_LD] = o.g01;
        g.H[lo + static_cast<size_t>(j) * ldh] = o.hp;
        gs->coef[lo] = static_cast<float>(s0 * o.hp);
    }
    g.H[j + static_cast<size_t>(j) * ldh] = o.hj;
    gs->coef[j] = static_cast<float>(o.sj * o.hj);
    gs->ip[j + 1] = o.ip;
    gs->wsc = static_cast<float>(o.sj);
    gs->psc = static_cast<float>(o.p);
}

// The finish of a step over at most two columns, in the last block of the
// sweep that wrote the a and |w|^2 partials (over nrb_a row blocks; the b
// partials over nrb_b row blocks, possibly written by the previous step's
// update): the partial sums, then one thread runs step2_chain and
// step2_store.
// PR: partials loaded per lane and round (20: one round for up to 640 row
// blocks, where the caller's registers allow).
template <int PR = 16>
__device__ __forceinline__ void step2_finish(const GramArgs& g, int nrb_a, int nrb_b) {
    const int j = g.j;
    const int lo = g.lo;
    const int kw = j + 1 - lo;
    __shared__ double s_tot[5];  // a (kw), b (kw), |w|^2
    const int t = threadIdx.x;
    GramState* gs = g.gs;
    const size_t ldh = static_cast<size_t>(g.ldh);
    for (int r = t; r < lo; r += blockDim.x) g.H[r + static_cast<size_t>(j) * ldh] = 0.0;  // outside the window
    const double s0 = kw == 2 ? gs->s[lo] : 0.0;
    const double ip_j = gs->ip[j];
    // b (and, for a symmetric A, a_{j-1}) come from the previous update
    const bool a0_from_update = g.sym && kw == 2;
    step_sum_partials<PR>(
        g.part, 2 * kw + 1, [&](int v) { return step2_slot(v, kw, lo); },
        [&](int v) { return ((v >= kw && v < 2 * kw) || (v == 0 && a0_from_update)) ? nrb_b : nrb_a; }, s_tot);
    __syncthreads();
    if (t != 0) return;
    const Step2Out o = step2_chain(s_tot, kw, j, g.reortho, s0, ip_j);
    step2_store(g, kw, o, s0);
}

// For a step over two columns whose dots the SpMV takes (kw = 2): the
// chain's first part (step2_chain_pre) from the previous update's partials,
// which exist before the SpMV starts -- b_{j-1}, b_j and, with g.sym, a_{j-1}
// over nrb_b row blocks -- summed as step2_finish<PR> sums them and stored in
// g.gs->pre. One block calls it (every thread) after its own rows and before
// it arrives, so that the last block's finish only runs the rest.
template <int PR>
__device__ __forceinline__ void step2_precompute(const GramArgs& g, int nrb_b) {
    const int j = g.j;
    const int lo = g.lo;  // j - 1
    __shared__ double s_pb[3];
    const bool sym = g.sym != 0;
    step_sum_partials<PR>(
        g.part, sym ? 3 : 2, [&](int v) { return v == 0 ? GRAM_BOFF + lo : (v == 1 ? GRAM_BOFF + j : lo); },
        [&](int) { return nrb_b; }, s_pb);
    __syncthreads();
    if (threadIdx.x == 0) {
        GramState* gs = g.gs;
        const Step2Pre pr = step2_chain_pre(s_pb[0], s_pb[1], sym ? s_pb[2] : 0.0, j, __ldcg(&gs->s[lo]),
                                            __ldcg(&gs->ip[j]));
        gs->pre[0] = pr.sj;
        gs->pre[1] = pr.sj2;
        gs->pre[2] = pr.beta;
        gs->pre[3] = pr.g01;
        gs->pre[4] = pr.cp;
        gs->pre[5] = pr.bad ? 1.0 : 0.0;
    }
}

// The finish of such a step in the last block: the SpMV's partials (a_j,
// |w|^2 and, without g.sym, a_{j-1}), the chain's first part from
// g.gs->pre, the rest of the chain and the stores. Bit for bit the result of
// step2_finish<PR>: the same sums and the same operations.
template <int PR>
__device__ __forceinline__ void step2_finish_pre(const GramArgs& g, int nrb_a) {
    const int j = g.j;
    const int lo = g.lo;
    __shared__ double s_ta[3];  // a_j, |w|^2, a_{j-1}
    const int t = threadIdx.x;
    GramState* gs = g.gs;
    const size_t ldh = static_cast<size_t>(g.ldh);
    for (int r = t; r < lo; r += blockDim.x) g.H[r + static_cast<size_t>(j) * ldh] = 0.0;  // outside the window
    const bool sym = g.sym != 0;
    // the block's last warp (idle during the sums, which need at most three)
    // fetches the first part meanwhile, so the two round trips overlap
    __shared__ double s_pre[7];
    const int tl = t - (static_cast<int>(blockDim.x) - 32);
    if (tl >= 0 && tl < 6) s_pre[tl] = __ldcg(&gs->pre[tl]);
    if (tl == 6) s_pre[6] = __ldcg(&gs->s[lo]);
    step_sum_partials<PR>(
        g.part, sym ? 2 : 3, [&](int v) { return v == 0 ? j : (v == 1 ? GRAM_NWOFF : lo); },
        [&](int) { return nrb_a; }, s_ta);
    __syncthreads();
    if (t != 0) return;
    Step2Pre pr;
    pr.sj = s_pre[0];
    pr.sj2 = s_pre[1];
    pr.beta = s_pre[2];
    pr.g01 = s_pre[3];
    pr.cp = s_pre[4];
    pr.bad = s_pre[5] != 0.0;
    const double s0 = s_pre[6];
    const double cp = sym ? pr.cp : (s0 * s_ta[2]) * pr.sj;
    const Step2Out o = step2_chain_rest(pr, 2, s_ta[0], s_ta[1], cp, g.reortho);
    step2_store(g, 2, o, s0);
}

}  // namespace
}  // namespace mexk
