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

// The finish of a step over at most two columns, in the last block of the
// sweep that wrote the a and |w|^2 partials (over nrb_a row blocks; the b
// partials over nrb_b row blocks, possibly written by the previous step's
// update). After the sums one thread runs the whole chain: s_j = 1/|u_j|,
// H(j, j-1) = |u_j| / p_j with the breakdown test of main.cu:1911, the Gram
// entry G(j-1, j), c = s s_j a, h = c - (G - I) c, H(:, j), the update
// coefficients and the pre-scale p of the next column (one rsqrt, a few
// products, one rsqrt).
// PR: partials loaded per lane and round (20: one round for up to 640 row
// blocks, where the caller's registers allow).
template <int PR = 16>
__device__ __forceinline__ void step2_finish(const GramArgs& g, int nrb_a, int nrb_b) {
    DevState* st = g.st;
    const int j = g.j;
    const int lo = g.lo;
    const int kw = j + 1 - lo;
    __shared__ double s_tot[5];  // a (kw), b (kw), |w|^2
    const int t = threadIdx.x;
    GramState* gs = g.gs;
    double* G = gs->G;
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
    const double bj = s_tot[2 * kw - 1];
    const double sj = (bj > 0.0 && !isinf(bj)) ? rsqrt(bj) : 0.0;
    // H(j, j-1) and the breakdown test: the square root runs beside the
    // chain below, which writes nothing until the test has passed
    const double beta = j >= 1 ? sqrt(bj) * ip_j : 1.0;
    const bool bad = !(beta >= 1e-14) || isinf(beta);
    const double sj2 = sj * sj;
    const double cj = sj2 * s_tot[kw - 1];
    double hj = cj, hp = 0.0, g01 = 0.0, part;
    if (kw == 2) {
        g01 = (s0 * s_tot[kw]) * sj;              // G(j-1, j)
        const double cp = (s0 * s_tot[0]) * sj;  // c_{j-1}
        hp = cp;
        if (g.reortho) {
            hp = cp - __dmul_rn(g01, cj);
            hj = cj - __dmul_rn(g01, cp);
        }
        const double gh0 = fma(g01, hj, hp), gh1 = hj + __dmul_rn(g01, hp);
        part = hp * (gh0 - 2.0 * cp) + hj * (gh1 - 2.0 * cj);
    } else {
        part = hj * (hj - 2.0 * cj);
    }
    const double w2 = sj2 * s_tot[2 * kw];
    const double u2 = w2 + part;
    double p = 1.0, ip = 1.0;
    if (u2 > 1e-8 * w2 && !isinf(u2)) {
        p = rsqrt(u2);
        ip = u2 * p;
    } else if (w2 > 0.0 && !isinf(w2)) {
        p = rsqrt(w2);
        ip = w2 * p;
    }
    if (j >= 1) g.H[j + static_cast<size_t>(j - 1) * ldh] = bad ? 0.0 : beta;
    if (j >= 1 && bad) {
        st->breakdown = 1;
        st->k_used = j;
        return;
    }
    gs->s[j] = sj;
    G[j + static_cast<size_t>(j) * GRAM_LD] = 1.0;
    if (kw == 2) {
        G[lo + static_cast<size_t>(j) * GRAM_LD] = g01;
        G[j + static_cast<size_t>(lo) * GRAM_LD] = g01;
        g.H[lo + static_cast<size_t>(j) * ldh] = hp;
        gs->coef[lo] = static_cast<float>(s0 * hp);
    }
    g.H[j + static_cast<size_t>(j) * ldh] = hj;
    gs->coef[j] = static_cast<float>(sj * hj);
    gs->ip[j + 1] = ip;
    gs->wsc = static_cast<float>(sj);
    gs->psc = static_cast<float>(p);
}

}  // namespace
}  // namespace mexk
