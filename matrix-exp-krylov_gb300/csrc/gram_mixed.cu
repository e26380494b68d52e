// K2, mixed precision: Gram-Schmidt over an FP32 basis with one reducing
// sweep and one streaming sweep per Arnoldi step.
//
// The reference orthogonalises with two MGS passes and normalises with a
// separate norm (main.cu:1769-1942): on one GPU that is five passes over the
// basis per step. Here column c of the FP32 basis stores u_c and the basis
// vector is v_c = s_c u_c, with s_c = 1/|u_c| kept in FP64; G = V^T V (unit
// diagonal) is kept in FP64 as the basis grows. Step j, k = j+1 columns:
//
//   gram_dot     one pass over u_0..u_j and w = A u_j:
//                  a = U^T w,  b = U^T u_j,  |w|^2
//                then, in the last block to finish:
//                  s_j = 1/sqrt(b_j)             the exact norm of the column
//                                                written by the previous step,
//                  H(j, j-1) = |u_j| / p_j       so its subdiagonal entry,
//                  G(:, j) = s s_j b             the Gram row of the new vector,
//                  c = s s_j a                   = V^T (A v_j),
//                  h = c - (G - I) c             (reorthogonalised),
//                  H(0:j, j) = h.
//   gram_update  u_{j+1} = p (s_j w - sum_c (s_c h_c) u_c) into column j+1,
//                a pure streaming pass (no reduction).
//   gram_norm    after the last step: |u_m| -> H(m, m-1).
//
// Classical Gram-Schmidt with one reorthogonalisation (CGS2) computes
// h1 = V^T w, then h2 = V^T (w - V h1) = c - G c, and uses h1 + h2 = c - (G-I) c:
// the coefficients here are CGS2's to first order in G - I, with the second
// pass evaluated from the Gram matrix instead of a second sweep (the
// one-reduction CGS2 formulations of Swirydowicz, Langou, Ananthan, Yang and
// Thomas, Numer. Linear Algebra Appl. 28(2), 2021, follow the same idea).
// The residual orthogonality of u_{j+1} is then set by the rounding of the
// FP32 update alone and does not grow from step to step. The pre-scale p
// comes from |w - V h|^2 = |w|^2 - 2 h.c + h^T G h and only keeps the stored
// column near unit length: the next step measures its norm exactly.
//
// With a window of W columns (symmetric A only: the short recurrence of
// Lanczos) both sweeps use columns j+1-W..j and H(0:j-W, j) = 0; the Gram
// correction then re-orthogonalises against the window.
//
// Dots multiply and accumulate in FP32 per thread (a few dozen terms), then
// sum across warps, blocks and the grid in FP64 in a fixed order, so every
// result is deterministic. The FP64 path keeps explicit CGS2 sweeps
// (gram_schmidt.cu), whose rounding follows the reference's passes.
#include "gram_step.cuh"

#include <math.h>

#include <algorithm>

namespace mexk {

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int GT = 256;          // threads per block
constexpr int GW = GT / 32;      // warps per block
constexpr int GG = 8;            // basis columns per block of the dot sweep
constexpr int UCH = 8;           // columns loaded together by the update

__device__ __forceinline__ float dot4(const float4& a, const float4& b) {
    return fmaf(a.w, b.w, fmaf(a.z, b.z, fmaf(a.y, b.y, a.x * b.x)));
}

// Butterfly transpose-reduction over the warp (K power of two <= 32):
// afterwards lane l holds the warp total of a[l % K].
template <int K>
__device__ __forceinline__ float transpose_reduce(float (&a)[K], int lane) {
#pragma unroll
    for (int s = K / 2; s >= 1; s >>= 1) {
        const bool upper = (lane & s) != 0;
#pragma unroll
        for (int i = 0; i < s; ++i) {
            const float send = upper ? a[i] : a[i + s];
            const float keep = upper ? a[i + s] : a[i];
            a[i] = keep + __shfl_xor_sync(FULL, send, s);
        }
    }
    float v = a[0];
#pragma unroll
    for (int s = K; s < 32; s <<= 1) v += __shfl_xor_sync(FULL, v, s);
    return v;
}

__device__ __forceinline__ const float4* col4(const float* V, size_t ldv, int c) {
    return reinterpret_cast<const float4*>(V + static_cast<size_t>(c) * ldv);
}

// Last block of a grid whose nrb row blocks each wrote their partials of
// step j (slots: a at column, b at GRAM_BOFF + column, |w|^2 at GRAM_NWOFF):
// sums them and finishes the step (Gram row, h, H, coefficients, pre-scale).
// All threads of the block call it. CAP: most columns the step may involve
// (the staged Gram block is CAP x CAP). Column lo + i is handled by thread i
// (warp 0, and warp 1 past 32 columns); the scalar chain of the new column
// runs in warp 7, which has nothing else to do, so that no warp carries two
// dependent FP64 chains.
template <int CAP>
__device__ __noinline__ void gram_finish(const GramArgs& g, int nrb) {
    static_assert(GW == 8, "the scalar chain runs in warp 7");
    DevState* st = g.st;
    const int j = g.j;
    const int k = j + 1;
    const int lo = g.lo;
    const int kw = k - lo;
    const int jw = j - lo;  // previous columns inside the window
    __shared__ double s_tot[2 * GRAM_M + 1];  // a (kw), b (kw), |w|^2
    __shared__ double s_c[CAP], s_h[CAP], s_sc[CAP], s_y[CAP];
    __shared__ double s_G[CAP][CAP + 1];  // G(lo:k, lo:k), row-major, padded, indexed from lo
    __shared__ double s_sj, s_w2s;
    __shared__ int s_bad;
    const int t = threadIdx.x;
    GramState* gs = g.gs;
    double* G = gs->G;
    const size_t ldh = static_cast<size_t>(g.ldh);
    // Stage 1: the previous columns' Gram block and scales, and the partial sums.
    for (int e = t; e < jw * jw; e += GT) {
        const int r = e % jw, c = e / jw;
        s_G[r][c] = G[(lo + r) + static_cast<size_t>(lo + c) * GRAM_LD];
    }
    double sc_t = 0.0;
    if (t < jw) sc_t = gs->s[lo + t];
    const double ip_j = gs->ip[j];
    step_sum_partials<12>(g.part, 2 * kw + 1, [&](int v) { return step2_slot(v, kw, lo); },
                          [&](int) { return nrb; }, s_tot);
    __syncthreads();
    // Stage 2: warp 7 lane 0: s_j = 1/|u_j| and H(j, j-1) = |u_j| / p_j (the
    // breakdown test of main.cu:1911); threads i < jw meanwhile scale their
    // column's b and a by s_i.
    if (t == GT - 32) {
        const double bj = s_tot[2 * kw - 1];
        const bool ok = bj > 0.0 && !isinf(bj);
        const double sj = ok ? rsqrt(bj) : 0.0;
        int bad = 0;
        if (j >= 1) {
            const double beta = sqrt(bj) * ip_j;
            bad = !(beta >= 1e-14) || isinf(beta);
            g.H[j + static_cast<size_t>(j - 1) * ldh] = bad ? 0.0 : beta;
            if (bad) {
                st->breakdown = 1;
                st->k_used = j;
            }
        }
        const double sj2 = sj * sj;
        gs->s[j] = sj;
        s_sj = sj;
        s_w2s = sj2 * s_tot[2 * kw];
        s_c[jw] = sj2 * s_tot[jw];  // c_j = s_j s_j a_j
        s_sc[jw] = sj;
        s_bad = bad;
    } else if (t < jw) {
        s_sc[t] = sc_t;
        s_y[t] = sc_t * s_tot[t];
        s_tot[kw + t] *= sc_t;  // s_i b_i
    }
    __syncthreads();
    if (s_bad) return;
    const double sj = s_sj;
    // Stage 3: the Gram row of column j and c = s s_j a.
    if (t < jw) {
        const double gv = s_tot[kw + t] * sj;
        G[(lo + t) + static_cast<size_t>(j) * GRAM_LD] = gv;
        G[j + static_cast<size_t>(lo + t) * GRAM_LD] = gv;
        s_G[t][jw] = gv;
        s_G[jw][t] = gv;
        s_c[t] = s_y[t] * sj;
    } else if (t == jw) {
        G[j + static_cast<size_t>(j) * GRAM_LD] = 1.0;
        s_G[jw][jw] = 1.0;
    }
    __syncthreads();
    // Stage 4: h = c - (G - I) c over the window (four running sums), H(:, j)
    // with zeros outside the window, coefficients s h.
    if (t < kw) {
        double hv = s_c[t];
        if (g.reortho) {
            double e0 = 0.0, e1 = 0.0, e2 = 0.0, e3 = 0.0;
            int q = 0;
            for (; q + 3 < kw; q += 4) {
                e0 = fma(q == t ? 0.0 : s_G[t][q], s_c[q], e0);
                e1 = fma(q + 1 == t ? 0.0 : s_G[t][q + 1], s_c[q + 1], e1);
                e2 = fma(q + 2 == t ? 0.0 : s_G[t][q + 2], s_c[q + 2], e2);
                e3 = fma(q + 3 == t ? 0.0 : s_G[t][q + 3], s_c[q + 3], e3);
            }
            for (; q < kw; ++q) e0 = fma(q == t ? 0.0 : s_G[t][q], s_c[q], e0);
            hv -= (e0 + e1) + (e2 + e3);
        }
        s_h[t] = hv;
        g.H[(lo + t) + static_cast<size_t>(j) * ldh] = hv;
        gs->coef[lo + t] = static_cast<float>(s_sc[t] * hv);
    }
    for (int r = t; r < lo; r += GT) g.H[r + static_cast<size_t>(j) * ldh] = 0.0;  // outside the window
    __syncthreads();
    // Stage 5 (warp 0): |w - V h|^2 = |w|^2 - 2 h.c + h^T G h, the pre-scale p
    // of the new column and its inverse.
    if (t < 32) {
        double part = 0.0;
        for (int i = t; i < kw; i += 32) {
            double g0 = 0.0, g1 = 0.0, g2 = 0.0, g3 = 0.0;
            int q = 0;
            for (; q + 3 < kw; q += 4) {
                g0 = fma(s_G[i][q], s_h[q], g0);
                g1 = fma(s_G[i][q + 1], s_h[q + 1], g1);
                g2 = fma(s_G[i][q + 2], s_h[q + 2], g2);
                g3 = fma(s_G[i][q + 3], s_h[q + 3], g3);
            }
            for (; q < kw; ++q) g0 = fma(s_G[i][q], s_h[q], g0);
            part += s_h[i] * (((g0 + g1) + (g2 + g3)) - 2.0 * s_c[i]);
        }
        for (int o = 1; o < 32 && o < kw; o <<= 1) part += __shfl_xor_sync(FULL, part, o);
        if (t == 0) {
            const double w2 = s_w2s;
            const double u2 = w2 + part;
            double p = 1.0, ip = 1.0;
            if (u2 > 1e-8 * w2 && !isinf(u2)) {
                p = rsqrt(u2);
                ip = u2 * p;
            } else if (w2 > 0.0 && !isinf(w2)) {
                p = rsqrt(w2);
                ip = w2 * p;
            }
            gs->ip[j + 1] = ip;
            gs->wsc = static_cast<float>(sj);
            gs->psc = static_cast<float>(p);
        }
    }
}

// Sweep 1. Block b handles column group b % ngroups (GG columns) over the rows
// of row block b / ngroups; the groups of one row block are adjacent in launch
// order, so w and u_j are fetched from DRAM once and re-read from L2.
__global__ void __launch_bounds__(GT, 4) gram_dot_kernel(GramArgs g) {
    pdl_wait();
    DevState* st = g.st;
    if (st->breakdown || st->done) return;
    const int j = g.j;
    const int k = j + 1;
    const int lo = g.lo;      // columns lo..j take part (lo = 0: all)
    const int kw = k - lo;
    const int ngroups = (kw + GG - 1) / GG;
    const int grp = blockIdx.x % ngroups;
    const int rb = blockIdx.x / ngroups;
    const int nrb = gridDim.x / ngroups;
    const int c0 = lo + grp * GG;
    const size_t ldv = static_cast<size_t>(g.ldv);
    const float4* __restrict__ w4 = reinterpret_cast<const float4*>(g.w);
    const float4* __restrict__ u4 = col4(g.V, ldv, j);

    float acc_a[GG], acc_b[GG], acc_w = 0.f;
#pragma unroll
    for (int c = 0; c < GG; ++c) {
        acc_a[c] = 0.f;
        acc_b[c] = 0.f;
    }
    const int n4 = (g.n + 3) / 4;
    for (int i = rb * GT + threadIdx.x; i < n4; i += nrb * GT) {
        const float4 x = __ldg(w4 + i);
        const float4 u = __ldg(u4 + i);
        float4 v[GG];
#pragma unroll
        for (int c = 0; c < GG; ++c)
            v[c] = (c0 + c < k) ? __ldcs(col4(g.V, ldv, c0 + c) + i) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int c = 0; c < GG; ++c) {
            acc_a[c] += dot4(v[c], x);
            acc_b[c] += dot4(v[c], u);
        }
        if (grp == 0) acc_w += dot4(x, x);
    }
    pdl_trigger();

    // block stage: warp butterflies in FP32, then the warps in FP64
    __shared__ double s_red[GW][2 * GG + 1];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const float ra = transpose_reduce<GG>(acc_a, lane);
    const float rbv = transpose_reduce<GG>(acc_b, lane);
    const float rw = warp_sum(acc_w);
    if (lane < GG) {
        s_red[warp][lane] = ra;
        s_red[warp][GG + lane] = rbv;
    }
    if (lane == 0) s_red[warp][2 * GG] = rw;
    step_write_partials(s_red, g.part, rb, [&](int q) {
        if (q < GG) return c0 + q < k ? c0 + q : -1;
        if (q < 2 * GG) return c0 + q - GG < k ? GRAM_BOFF + c0 + q - GG : -1;
        return grp == 0 ? GRAM_NWOFF : -1;
    });

    // grid stage: the last block sums the row blocks and finishes the step
    __shared__ int s_flag;
    if (!grid_last_block(g.counter, &s_flag)) return;
    gram_finish<GRAM_M>(g, nrb);
}

// Sweep 1 for a step over at most two columns (the first two Arnoldi steps,
// every step of a window of 2): w, u_j and u_{j-1} are each read once, two
// rows per thread per iteration, one column group. The loads keep their L2
// lines (default policy): the update reads the same three vectors next, and
// with the matrix streamed evict-first they are still in L2.
__global__ void __launch_bounds__(GT, 4) gram_dot2_kernel(GramArgs g) {
    pdl_wait();
    DevState* st = g.st;
    if (st->breakdown || st->done) return;
    const int j = g.j;
    const int lo = g.lo;  // j - 1 or j
    const bool two = lo < j;
    const size_t ldv = static_cast<size_t>(g.ldv);
    const float4* __restrict__ w4 = reinterpret_cast<const float4*>(g.w);
    const float4* __restrict__ u4 = col4(g.V, ldv, j);
    const float4* __restrict__ p4 = col4(g.V, ldv, two ? j - 1 : j);
    // acc: a_{j-1}, a_j, b_{j-1}, b_j, |w|^2
    float acc[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
    const int n4 = (g.n + 3) / 4;
    const int stride = gridDim.x * GT;
    int i = blockIdx.x * GT + threadIdx.x;
    for (; i + stride < n4; i += 2 * stride) {
        const float4 x0 = __ldg(w4 + i), x1 = __ldg(w4 + i + stride);
        const float4 u0 = __ldg(u4 + i), u1 = __ldg(u4 + i + stride);
        float4 v0 = make_float4(0.f, 0.f, 0.f, 0.f), v1 = v0;
        if (two) {
            v0 = __ldg(p4 + i);
            v1 = __ldg(p4 + i + stride);
        }
        acc[0] += dot4(v0, x0) + dot4(v1, x1);
        acc[1] += dot4(u0, x0) + dot4(u1, x1);
        acc[2] += dot4(v0, u0) + dot4(v1, u1);
        acc[3] += dot4(u0, u0) + dot4(u1, u1);
        acc[4] += dot4(x0, x0) + dot4(x1, x1);
    }
    if (i < n4) {
        const float4 x0 = __ldg(w4 + i);
        const float4 u0 = __ldg(u4 + i);
        const float4 v0 = two ? __ldg(p4 + i) : make_float4(0.f, 0.f, 0.f, 0.f);
        acc[0] += dot4(v0, x0);
        acc[1] += dot4(u0, x0);
        acc[2] += dot4(v0, u0);
        acc[3] += dot4(u0, u0);
        acc[4] += dot4(x0, x0);
    }
    pdl_trigger();

    __shared__ double s_red[GW][5];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < 5; ++q) {
        const float r = warp_sum(acc[q]);
        if (lane == 0) s_red[warp][q] = r;
    }
    step_write_partials(s_red, g.part, blockIdx.x, [&](int q) {
        switch (q) {
            case 0: return two ? j - 1 : -1;
            case 1: return j;
            case 2: return two ? GRAM_BOFF + j - 1 : -1;
            case 3: return GRAM_BOFF + j;
            default: return GRAM_NWOFF;
        }
    });
    __shared__ int s_flag;
    if (!grid_last_block(g.counter, &s_flag)) return;
    step2_finish(g, gridDim.x, gridDim.x);
}

// Sweep 2: u_{j+1} = psc * (wsc * w - sum_c coef_c u_c), written to column
// j+1 with a default (L2-allocating) store: the next SpMV gathers from it.
__global__ void __launch_bounds__(GT, 4) gram_update_kernel(GramArgs g) {
    pdl_wait();
    DevState* st = g.st;
    if (st->breakdown || st->done) return;
    __shared__ float s_coef[GRAM_M + UCH];
    __shared__ float s_sc[2];
    const int k = g.j + 1;
    const int lo = g.lo;
    // a short window's columns were just read by the dot sweep and are still
    // in L2 (default loads); a long basis is streamed (evict-first)
    const bool keep = k - lo <= 4;
    const GramState* gs = g.gs;
    if (threadIdx.x < GRAM_M + UCH) s_coef[threadIdx.x] = threadIdx.x < k ? gs->coef[threadIdx.x] : 0.f;
    if (threadIdx.x == 0) {
        s_sc[0] = gs->wsc;
        s_sc[1] = gs->psc;
    }
    __syncthreads();
    const float wsc = s_sc[0];
    const float psc = s_sc[1];
    const size_t ldv = static_cast<size_t>(g.ldv);
    const float4* __restrict__ w4 = reinterpret_cast<const float4*>(g.w);
    float4* __restrict__ out = reinterpret_cast<float4*>(g.V + static_cast<size_t>(g.j + 1) * ldv);
    const int n4 = (g.n + 3) / 4;
    for (int i = blockIdx.x * GT + threadIdx.x; i < n4; i += gridDim.x * GT) {
        const float4 x = __ldg(w4 + i);
        float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int cbi = 0; cbi < GRAM_M; cbi += UCH) {
            const int cb = lo + cbi;
            if (cb < k) {
                float4 v[UCH];
#pragma unroll
                for (int c = 0; c < UCH; ++c)
                    v[c] = (cb + c < k) ? (keep ? __ldg(col4(g.V, ldv, cb + c) + i) : __ldcs(col4(g.V, ldv, cb + c) + i))
                                        : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
                for (int c = 0; c < UCH; ++c) {
                    const float h = s_coef[cb + c];
                    s.x = fmaf(v[c].x, h, s.x);
                    s.y = fmaf(v[c].y, h, s.y);
                    s.z = fmaf(v[c].z, h, s.z);
                    s.w = fmaf(v[c].w, h, s.w);
                }
            }
        }
        float4 r;
        r.x = fmaf(x.x, wsc, -s.x) * psc;
        r.y = fmaf(x.y, wsc, -s.y) * psc;
        r.z = fmaf(x.z, wsc, -s.z) * psc;
        r.w = fmaf(x.w, wsc, -s.w) * psc;
        out[i] = r;
    }
    pdl_trigger();
}

// Sweep 2 of a step over at most two columns: u_{j+1} = psc * (wsc * w -
// (cp u_{j-1} + cj u_j)), the products summed in the order of
// gram_update_kernel (bit-identical), two rows per thread per iteration for
// more loads in flight (the three vectors come from L2).
__global__ void __launch_bounds__(GT, 4) gram_update2_kernel(GramArgs g) {
    pdl_wait();
    DevState* st = g.st;
    if (st->breakdown || st->done) return;
    const int j = g.j;
    const bool two = g.lo < j;
    const GramState* gs = g.gs;
    const float cp = two ? gs->coef[g.lo] : 0.f, cj = gs->coef[j];
    const float wsc = gs->wsc, psc = gs->psc;
    const size_t ldv = static_cast<size_t>(g.ldv);
    const float4* __restrict__ w4 = reinterpret_cast<const float4*>(g.w);
    const float4* __restrict__ u4 = col4(g.V, ldv, j);
    const float4* __restrict__ p4 = col4(g.V, ldv, two ? j - 1 : j);
    float4* __restrict__ out = reinterpret_cast<float4*>(g.V + static_cast<size_t>(j + 1) * ldv);
    const int n4 = (g.n + 3) / 4;
    const int stride = gridDim.x * GT;
    auto one = [&](const float4& x, const float4& u, const float4& v) {
        float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
        if (two) {
            s.x = fmaf(v.x, cp, s.x);
            s.y = fmaf(v.y, cp, s.y);
            s.z = fmaf(v.z, cp, s.z);
            s.w = fmaf(v.w, cp, s.w);
        }
        s.x = fmaf(u.x, cj, s.x);
        s.y = fmaf(u.y, cj, s.y);
        s.z = fmaf(u.z, cj, s.z);
        s.w = fmaf(u.w, cj, s.w);
        float4 r;
        r.x = fmaf(x.x, wsc, -s.x) * psc;
        r.y = fmaf(x.y, wsc, -s.y) * psc;
        r.z = fmaf(x.z, wsc, -s.z) * psc;
        r.w = fmaf(x.w, wsc, -s.w) * psc;
        return r;
    };
    // step j+1's b: u_j . u_{j+1} and |u_{j+1}|^2; with g.sym its a_j = w_j . u_{j+1}
    // (FP32 per thread)
    float bu = 0.f, bb = 0.f, ba = 0.f;
    int i = blockIdx.x * GT + threadIdx.x;
    for (; i + stride < n4; i += 2 * stride) {
        const float4 x0 = __ldg(w4 + i), x1 = __ldg(w4 + i + stride);
        const float4 u0 = __ldg(u4 + i), u1 = __ldg(u4 + i + stride);
        const float4 v0 = two ? __ldg(p4 + i) : u0, v1 = two ? __ldg(p4 + i + stride) : u1;
        const float4 r0 = one(x0, u0, v0), r1 = one(x1, u1, v1);
        out[i] = r0;
        out[i + stride] = r1;
        bu += dot4(u0, r0) + dot4(u1, r1);
        bb += dot4(r0, r0) + dot4(r1, r1);
        ba += dot4(x0, r0) + dot4(x1, r1);
    }
    if (i < n4) {
        const float4 x0 = __ldg(w4 + i), u0 = __ldg(u4 + i);
        const float4 v0 = two ? __ldg(p4 + i) : u0;
        const float4 r0 = one(x0, u0, v0);
        out[i] = r0;
        bu += dot4(u0, r0);
        bb += dot4(r0, r0);
        ba += dot4(x0, r0);
    }
    pdl_trigger();
    if (g.write_b) {
        __shared__ double s_red[GW][3];
        const float ru = warp_sum(bu), rb = warp_sum(bb), ra = warp_sum(ba);
        if ((threadIdx.x & 31) == 0) {
            s_red[threadIdx.x >> 5][0] = ru;
            s_red[threadIdx.x >> 5][1] = rb;
            s_red[threadIdx.x >> 5][2] = ra;
        }
        const bool sym = g.sym != 0;
        step_write_partials(s_red, g.part, blockIdx.x, [&](int q) { return q < 2 ? GRAM_BOFF + j + q : (sym ? j : -1); });
    }
}

// From b = |u_{j+1}|^2 (one thread): H(j+1, j), s_{j+1} and the breakdown
// flag (main.cu:1911).
__device__ __forceinline__ void last_norm_store(const GramArgs& g, double b) {
    DevState* st = g.st;
    GramState* gs = g.gs;
    const int jn = g.j + 1;
    const double beta = sqrt(b) * gs->ip[jn];
    const bool bad = !(beta >= 1e-14) || isinf(beta);
    if (jn < g.ldh) g.H[jn + static_cast<size_t>(g.j) * g.ldh] = bad ? 0.0 : beta;
    gs->s[jn] = (b > 0.0 && !isinf(b)) ? rsqrt(b) : 0.0;
    gs->G[jn + static_cast<size_t>(jn) * GRAM_LD] = 1.0;
    if (bad) {
        st->breakdown = 1;
        st->k_used = jn;
    }
}

// |u_{j+1}|^2 by grid reduction; the last block sets H(j+1, j), s_{j+1} and
// the breakdown flag (main.cu:1911).
__global__ void __launch_bounds__(GT) gram_norm_kernel(GramArgs g) {
    pdl_wait();
    pdl_trigger();
    DevState* st = g.st;
    if (st->breakdown || st->done) return;
    const int jn = g.j + 1;
    const float4* __restrict__ u4 = col4(g.V, static_cast<size_t>(g.ldv), jn);
    const int n4 = (g.n + 3) / 4;
    float acc = 0.f;
    for (int i = blockIdx.x * GT + threadIdx.x; i < n4; i += gridDim.x * GT) {
        const float4 u = __ldg(u4 + i);
        acc += dot4(u, u);
    }
    __shared__ double s_red[GW][1];
    const float r = warp_sum(acc);
    if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5][0] = r;
    step_write_partials(s_red, g.part, blockIdx.x, [](int) { return 0; });
    __shared__ int s_flag;
    if (!grid_last_block(g.counter, &s_flag)) return;
    __shared__ double s_tot[1];
    step_sum_partials<20>(g.part, 1, [](int) { return 0; }, [&](int) { return static_cast<int>(gridDim.x); }, s_tot);
    __syncthreads();
    if (threadIdx.x == 0) last_norm_store(g, s_tot[0]);
}

// The same from the |u_{j+1}|^2 partials the last two-column update wrote
// into column j+1's b slot (over g.b_blocks row blocks): one block sums
// them, no sweep of u_{j+1}.
__global__ void __launch_bounds__(GT) gram_norm_partials_kernel(GramArgs g) {
    pdl_wait();
    pdl_trigger();  // the controller may take the idle SMs meanwhile
    DevState* st = g.st;
    if (st->breakdown || st->done) return;
    const int jn = g.j + 1;
    __shared__ double s_tot[1];
    step_sum_partials<20>(g.part, 1, [&](int) { return GRAM_BOFF + jn; }, [&](int) { return g.b_blocks; }, s_tot);
    __syncthreads();
    if (threadIdx.x == 0) last_norm_store(g, s_tot[0]);
}

int row_blocks(int n, int per_sm) {
    const long long n4 = (static_cast<long long>(n) + 3) / 4;
    long long rb = static_cast<long long>(device_sm_count()) * per_sm;
    const long long need = (n4 + GT - 1) / GT;
    if (need < rb) rb = need;
    if (rb > GRAM_MAX_ROW_BLOCKS) rb = GRAM_MAX_ROW_BLOCKS;
    return rb < 1 ? 1 : static_cast<int>(rb);
}

}  // namespace

int device_sm_count() {
    static int sms = 0;
    if (sms == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    }
    return sms;
}

int launch_gram_dot(const GramArgs& a, cudaStream_t s) {
    if (a.j < 0 || a.j >= GRAM_M) return MEXK_ERR_INVALID;
    if (a.lo < 0 || a.lo > a.j) return MEXK_ERR_INVALID;
    const int kw = a.j + 1 - a.lo;
    cudaError_t e;
    if (kw <= 2) {
        // two rows per thread per iteration, 3 row blocks per SM (measured
        // best of 2-6); the finish sums their partials in one round of loads
        e = launch_dependent(gram_dot2_kernel, row_blocks((a.n + 1) / 2, 3), GT, 0, s, a);
    } else {
        const int ngroups = (kw + GG - 1) / GG;
        // One wave of 4 resident blocks per SM over all column groups (a partial
        // second wave would run at half occupancy); 2 row blocks per SM at most.
        int nrb = row_blocks(a.n, 2);
        if (ngroups > 2) nrb = std::min(nrb, std::max(1, 4 * device_sm_count() / ngroups));
        e = launch_dependent(gram_dot_kernel, nrb * ngroups, GT, 0, s, a);
    }
    if (e != cudaSuccess) {
        set_cuda_error(e, "gram_dot_kernel", __FILE__, __LINE__);
        return MEXK_ERR_CUDA;
    }
    return MEXK_OK;
}

int gram_update2_blocks(int n) { return row_blocks((n + 1) / 2, 4); }

int launch_gram_update(const GramArgs& a, cudaStream_t s) {
    if (a.j < 0 || a.j >= GRAM_M || a.lo < 0 || a.lo > a.j) return MEXK_ERR_INVALID;
    const cudaError_t e = a.j + 1 - a.lo <= 2
                              ? launch_dependent(gram_update2_kernel, gram_update2_blocks(a.n), GT, 0, s, a)
                              : launch_dependent(gram_update_kernel, row_blocks(a.n, 4), GT, 0, s, a);
    if (e != cudaSuccess) {
        set_cuda_error(e, "gram_update_kernel", __FILE__, __LINE__);
        return MEXK_ERR_CUDA;
    }
    return MEXK_OK;
}

int launch_gram_norm(const GramArgs& a, cudaStream_t s) {
    if (a.j < 0 || a.j >= GRAM_M) return MEXK_ERR_INVALID;
    const cudaError_t e = launch_dependent(gram_norm_kernel, row_blocks(a.n, 4), GT, 0, s, a);
    if (e != cudaSuccess) {
        set_cuda_error(e, "gram_norm_kernel", __FILE__, __LINE__);
        return MEXK_ERR_CUDA;
    }
    return MEXK_OK;
}

int launch_gram_norm_partials(const GramArgs& a, cudaStream_t s) {
    if (a.j < 0 || a.j + 1 >= GRAM_M || a.b_blocks < 1 || a.b_blocks > GRAM_MAX_ROW_BLOCKS) return MEXK_ERR_INVALID;
    const cudaError_t e = launch_dependent(gram_norm_partials_kernel, 1, GT, 0, s, a);
    if (e != cudaSuccess) {
        set_cuda_error(e, "gram_norm_partials_kernel", __FILE__, __LINE__);
        return MEXK_ERR_CUDA;
    }
    return MEXK_OK;
}

}  // namespace mexk
