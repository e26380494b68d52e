// Kernels of the batched solver (layout in batch.cuh).
//
// Per Arnoldi step j every active state of a wave advances through:
//   spmm    W = A_p U_j for every problem p, all 16 right-hand sides of a row
//           at once: one read of the matrix row, 16-wide x gathers;
//   dot     per problem and RHS: a = U^T W, b = U^T u_j, |W|^2 (the same
//           one-reduction Gram-corrected step as the single-vector FP32
//           path), partials per tile, then the last tile of each problem
//           finishes its 16 states;
//   update  u_{j+1} = psc (wsc W - sum_c coef_c u_c), streaming.
// After the last step: the last column's norms (H(m, m-1)); then the
// controllers (one block per state, controller_kernel), the lift y = U
// (s * coef), the restart u_0 = y / |y| and the per-problem status.
//
// Reductions run per problem in a fixed order (per-thread FP32 over the rows
// of a tile, then lanes, warps in FP64, then tiles in order), so a
// problem's results do not depend on which other problems share its wave.
#include "batch.cuh"

#include <math.h>

namespace mexk {
namespace batch {

namespace {

constexpr unsigned FULL = 0xffffffffu;

__device__ __forceinline__ float4 zero4() { return make_float4(0.f, 0.f, 0.f, 0.f); }

__device__ __forceinline__ void fma4(float4& acc, const float4& a, const float4& b) {
    acc.x = fmaf(a.x, b.x, acc.x);
    acc.y = fmaf(a.y, b.y, acc.y);
    acc.z = fmaf(a.z, b.z, acc.z);
    acc.w = fmaf(a.w, b.w, acc.w);
}

// Sum over the 8 lanes of a warp that own the same row quarter (lane % 4).
__device__ __forceinline__ float quad_sum(float v) {
    v += __shfl_xor_sync(FULL, v, 4);
    v += __shfl_xor_sync(FULL, v, 8);
    v += __shfl_xor_sync(FULL, v, 16);
    return v;
}
__device__ __forceinline__ double quad_sum(double v) {
    v += __shfl_xor_sync(FULL, v, 4);
    v += __shfl_xor_sync(FULL, v, 8);
    v += __shfl_xor_sync(FULL, v, 16);
    return v;
}
__device__ __forceinline__ float4 quad_sum(float4 v) {
    return make_float4(quad_sum(v.x), quad_sum(v.y), quad_sum(v.z), quad_sum(v.w));
}

__device__ __forceinline__ const float4* col4(const Layout& L, int c) {
    return reinterpret_cast<const float4*>(L.U + static_cast<size_t>(c) * L.ldu);
}

// Arrival of one block of problem p; true in the last of `expected` blocks.
// One fence per block, by the arriving thread (as in grid_last_block).
__device__ __forceinline__ bool problem_last(unsigned int* counter, unsigned int expected, int* s_flag) {
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const bool last = atomicAdd(counter, 1u) == expected - 1u;
        if (last) {
            __threadfence();
            *counter = 0u;
        }
        *s_flag = last ? 1 : 0;
    }
    __syncthreads();
    return *s_flag != 0;
}

// Sum of slot `slot` over the tiles of problem p.
__device__ __forceinline__ double tiles_sum(const Layout& L, int p, int slot) {
    const int t0 = L.ptile0[p];
    const int nt = L.ptiles[p];
    double t = 0.0;
    for (int tt = 0; tt < nt; ++tt) t += __ldcg(&L.part[static_cast<size_t>(t0 + tt) * BPS + slot]);
    return t;
}

// ---------------------------------------------------------------- SpMM
// One 64-row chunk per block iteration: the chunk's nonzeros (contiguous in
// CSR) are staged in shared memory with coalesced loads, then each row
// quarter issues its row's x gathers U at a time from the staged columns.
// Chunks with more than SP_STAGE nonzeros read their columns directly.
constexpr int SP_STAGE = 2048;

template <int U>
__global__ void __launch_bounds__(BT) spmm_kernel(Layout L, int j) {
    __shared__ int s_col[SP_STAGE];
    __shared__ float s_val[SP_STAGE];
    const int q = threadIdx.x & 3;
    const int rl = threadIdx.x >> 2;
    const float4* __restrict__ X4 = col4(L, j);
    float4* __restrict__ Y4 = reinterpret_cast<float4*>(L.W);
    for (int ch = L.C0 + blockIdx.x; ch < L.C1; ch += gridDim.x) {
        const int p = L.chunk_prob[ch];
        if (L.pdone[p]) continue;
        const long long r0 = static_cast<long long>(ch) * BROWS;
        const long long row = r0 + rl;
        const long long c0 = L.row_ptr[r0];
        const long long c1 = L.row_ptr[r0 + BROWS];
        const long long e0 = L.row_ptr[row];
        const long long e1 = L.row_ptr[row + 1];
        const long long xoff = L.prow0[p] - L.R0;
        float4 acc = zero4();
        if (c1 - c0 <= SP_STAGE) {
            const int cnt = static_cast<int>(c1 - c0);
            __syncthreads();
            for (int e = threadIdx.x; e < cnt; e += BT) {
                s_col[e] = __ldcs(&L.col[c0 + e]);
                s_val[e] = __ldcs(&L.val[c0 + e]);
            }
            __syncthreads();
            int e = static_cast<int>(e0 - c0);
            const int z = static_cast<int>(e1 - c0);
            for (; e + U <= z; e += U) {
                float4 xv[U];
#pragma unroll
                for (int u = 0; u < U; ++u) xv[u] = __ldg(X4 + (xoff + s_col[e + u]) * 4 + q);
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    const float a = s_val[e + u];
                    fma4(acc, make_float4(a, a, a, a), xv[u]);
                }
            }
            for (; e < z; ++e) {
                const float a = s_val[e];
                fma4(acc, make_float4(a, a, a, a), __ldg(X4 + (xoff + s_col[e]) * 4 + q));
            }
        } else {
            long long e = e0;
            for (; e + 4 <= e1; e += 4) {
                int c[4];
                float a[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    c[u] = __ldg(&L.col[e + u]);
                    a[u] = __ldg(&L.val[e + u]);
                }
                float4 xv[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) xv[u] = __ldg(X4 + (xoff + c[u]) * 4 + q);
#pragma unroll
                for (int u = 0; u < 4; ++u) fma4(acc, make_float4(a[u], a[u], a[u], a[u]), xv[u]);
            }
            for (; e < e1; ++e) {
                const float a = __ldg(&L.val[e]);
                fma4(acc, make_float4(a, a, a, a), __ldg(X4 + (xoff + __ldg(&L.col[e])) * 4 + q));
            }
        }
        Y4[(row - L.R0) * 4 + q] = acc;
    }
}

// ---------------------------------------------------------------- dot sweep
// Finishes step j of the 16 states of problem p (one warp per state at a
// time, lane t = basis index t): the same arithmetic as gram_mixed.cu.
__device__ void finish_dot(const Layout& L, int p, int j, int k, int reortho) {
    __shared__ double sa[BM_MAX][BR], sb[BM_MAX][BR], sw[BR];
    const int nv = (2 * k + 1) * BR;
    for (int v = threadIdx.x; v < nv; v += BT) {
        if (v < k * BR) (&sa[0][0])[v] = tiles_sum(L, p, A_OFF + v);
        else if (v < 2 * k * BR) (&sb[0][0])[v - k * BR] = tiles_sum(L, p, B_OFF + (v - k * BR));
        else sw[v - 2 * k * BR] = tiles_sum(L, p, W_OFF + (v - 2 * k * BR));
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    for (int r = warp; r < BR; r += BT / 32) {
        const int b = p * BR + r;
        DevState* st = L.st + b;
        float* coef = L.coef + static_cast<size_t>(b) * BLD;
        const bool inactive = st->done || st->breakdown;
        double* H = L.H + static_cast<size_t>(b) * BLD * BM_MAX;
        double* sv = L.s + static_cast<size_t>(b) * (BLD + 1);
        double* pv = L.pre + static_cast<size_t>(b) * (BLD + 1);
        bool bad = inactive;
        const double bj = sb[j][r];
        if (!inactive && j >= 1) {
            // h_{j,j-1} = |u_j| / p_j; breakdown test as main.cu:1911
            const double beta = sqrt(bj) / pv[j];
            bad = !(beta >= 1e-14) || isinf(beta);
            if (lane == 0) {
                H[j + static_cast<size_t>(j - 1) * BLD] = bad ? 0.0 : beta;
                if (bad) {
                    st->breakdown = 1;
                    st->k_used = j;
                }
            }
        }
        if (bad) {
            coef[lane] = 0.f;
            if (lane == 0) {
                L.wsc[b] = 0.f;
                L.psc[b] = 0.f;
            }
            continue;
        }
        const double sj = (bj > 0.0 && !isinf(bj)) ? 1.0 / sqrt(bj) : 0.0;
        if (lane == 0) sv[j] = sj;
        double* G = L.G + static_cast<size_t>(b) * BLD * BLD;
        double cval = 0.0, sc = 0.0;
        if (lane < k) {
            sc = (lane == j) ? sj : sv[lane];
            const double gv = (lane == j) ? 1.0 : sc * sj * sb[lane][r];
            G[lane + static_cast<size_t>(j) * BLD] = gv;
            G[j + static_cast<size_t>(lane) * BLD] = gv;
            cval = sc * sj * sa[lane][r];
        }
        __syncwarp();
        double e = 0.0;
        for (int qq = 0; qq < k; ++qq) {
            const double cq = __shfl_sync(FULL, cval, qq);
            if (lane < k && qq != lane) e = fma(G[lane + static_cast<size_t>(qq) * BLD], cq, e);
        }
        const double hv = reortho ? cval - e : cval;
        if (lane < k) {
            H[lane + static_cast<size_t>(j) * BLD] = hv;
            coef[lane] = static_cast<float>(sc * hv);
        }
        double gh = 0.0;
        for (int qq = 0; qq < k; ++qq) {
            const double hq = __shfl_sync(FULL, hv, qq);
            if (lane < k) gh = fma(G[lane + static_cast<size_t>(qq) * BLD], hq, gh);
        }
        double part = (lane < k) ? hv * gh - 2.0 * hv * cval : 0.0;
        part = warp_sum(part);
        if (lane == 0) {
            const double w2 = sj * sj * sw[r];
            const double u2 = w2 + part;
            double pn = 1.0;
            if (u2 > 1e-8 * w2 && !isinf(u2)) pn = 1.0 / sqrt(u2);
            else if (w2 > 0.0 && !isinf(w2)) pn = 1.0 / sqrt(w2);
            pv[j + 1] = pn;
            L.wsc[b] = static_cast<float>(sj);
            L.psc[b] = static_cast<float>(pn);
        }
    }
}

template <int GG>
__global__ void __launch_bounds__(BT, 3) dot_kernel(Layout L, int j, int reortho, int tune) {
    const int k = j + 1;
    const int ngroups = (k + GG - 1) / GG;
    const int tile = blockIdx.x / ngroups;
    const int grp = blockIdx.x - tile * ngroups;
    const int p = L.tile_prob[tile];
    if (L.pdone[p]) return;
    const int c0 = grp * GG;
    const int q = threadIdx.x & 3;
    const int rl = threadIdx.x >> 2;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const long long base = L.tile_row0[tile] - L.R0;
    const int nr = L.tile_nrows[tile];
    const float4* __restrict__ W4 = reinterpret_cast<const float4*>(L.W);
    const float4* __restrict__ Uj = col4(L, j);
    float4 aa[GG], bb[GG], ww = zero4();
#pragma unroll
    for (int c = 0; c < GG; ++c) {
        aa[c] = zero4();
        bb[c] = zero4();
    }
    for (int r = rl; r < nr; r += BROWS) {
        const size_t i = static_cast<size_t>(base + r) * 4 + q;
        const float4 x = __ldg(W4 + i);
        const float4 u = __ldg(Uj + i);
        float4 v[GG];
#pragma unroll
        for (int c = 0; c < GG; ++c) v[c] = (c0 + c < k) ? __ldcs(col4(L, c0 + c) + i) : zero4();
#pragma unroll
        for (int c = 0; c < GG; ++c) {
            fma4(aa[c], v[c], x);
            fma4(bb[c], v[c], u);
        }
        if (grp == 0) fma4(ww, x, x);
    }
    __shared__ __align__(16) float red[BT / 32][2 * GG + 1][BR];
#pragma unroll
    for (int c = 0; c < GG; ++c) {
        aa[c] = quad_sum(aa[c]);
        bb[c] = quad_sum(bb[c]);
    }
    ww = quad_sum(ww);
    if (lane < 4) {
#pragma unroll
        for (int c = 0; c < GG; ++c) {
            *reinterpret_cast<float4*>(&red[warp][c][4 * lane]) = aa[c];
            *reinterpret_cast<float4*>(&red[warp][GG + c][4 * lane]) = bb[c];
        }
        *reinterpret_cast<float4*>(&red[warp][2 * GG][4 * lane]) = ww;
    }
    __syncthreads();
    double* P = L.part + static_cast<size_t>(tile) * BPS;
    for (int v = threadIdx.x; v < (2 * GG + 1) * BR; v += BT) {
        const int val = v / BR;
        const int r = v - val * BR;
        double t = 0.0;
#pragma unroll
        for (int w = 0; w < BT / 32; ++w) t += red[w][val][r];
        if (val < GG) {
            if (c0 + val < k) P[A_OFF + (c0 + val) * BR + r] = t;
        } else if (val < 2 * GG) {
            if (c0 + val - GG < k) P[B_OFF + (c0 + val - GG) * BR + r] = t;
        } else if (grp == 0) {
            P[W_OFF + r] = t;
        }
    }
    __shared__ int s_flag;
    if (!problem_last(L.pcount + p, static_cast<unsigned>(L.ptiles[p] * ngroups), &s_flag)) return;
    if (tune) return;
    finish_dot(L, p, j, k, reortho);
}

// ---------------------------------------------------------------- update sweep
constexpr int UCH = 8;

__global__ void __launch_bounds__(BT) update_kernel(Layout L, int j) {
    const int k = j + 1;
    const int q = threadIdx.x & 3;
    const int rl = threadIdx.x >> 2;
    __shared__ float4 sco[BM_MAX][4];
    __shared__ float4 ssc[2][4];
    const float4* __restrict__ W4 = reinterpret_cast<const float4*>(L.W);
    float4* __restrict__ Out = reinterpret_cast<float4*>(L.U + static_cast<size_t>(j + 1) * L.ldu);
    for (int tile = blockIdx.x; tile < L.T; tile += gridDim.x) {
        const int p = L.tile_prob[tile];
        if (L.pdone[p]) continue;
        __syncthreads();
        for (int v = threadIdx.x; v < BM_MAX * BR; v += BT) {
            const int c = v / BR;
            const int r = v - c * BR;
            reinterpret_cast<float*>(sco)[v] = (c < k) ? L.coef[static_cast<size_t>(p * BR + r) * BLD + c] : 0.f;
        }
        if (threadIdx.x < BR) {
            reinterpret_cast<float*>(ssc)[threadIdx.x] = L.wsc[p * BR + threadIdx.x];
            reinterpret_cast<float*>(ssc)[BR + threadIdx.x] = L.psc[p * BR + threadIdx.x];
        }
        __syncthreads();
        const float4 wsc = ssc[0][q];
        const float4 psc = ssc[1][q];
        const long long base = L.tile_row0[tile] - L.R0;
        const int nr = L.tile_nrows[tile];
        for (int r = rl; r < nr; r += BROWS) {
            const size_t i = static_cast<size_t>(base + r) * 4 + q;
            const float4 x = __ldg(W4 + i);
            float4 s = zero4();
#pragma unroll
            for (int cb = 0; cb < BM_MAX; cb += UCH) {
                if (cb < k) {
                    float4 v[UCH];
#pragma unroll
                    for (int c = 0; c < UCH; ++c) v[c] = (cb + c < k) ? __ldcs(col4(L, cb + c) + i) : zero4();
#pragma unroll
                    for (int c = 0; c < UCH; ++c) fma4(s, v[c], sco[cb + c][q]);
                }
            }
            float4 o;
            o.x = fmaf(x.x, wsc.x, -s.x) * psc.x;
            o.y = fmaf(x.y, wsc.y, -s.y) * psc.y;
            o.z = fmaf(x.z, wsc.z, -s.z) * psc.z;
            o.w = fmaf(x.w, wsc.w, -s.w) * psc.w;
            Out[i] = o;
        }
    }
}

// ---------------------------------------------------------------- per-RHS norms
// Writes the 16 per-RHS sums of a block (acc per thread, FP64) to slot
// W_OFF of the tile partial.
__device__ __forceinline__ void tile_rhs_partial(const Layout& L, int tile, const double (&acc)[4]) {
    __shared__ double red[BT / 32][BR];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    double t[4];
#pragma unroll
    for (int d = 0; d < 4; ++d) t[d] = quad_sum(acc[d]);
    if (lane < 4) {
#pragma unroll
        for (int d = 0; d < 4; ++d) red[warp][4 * lane + d] = t[d];
    }
    __syncthreads();
    if (threadIdx.x < BR) {
        double s = 0.0;
#pragma unroll
        for (int w = 0; w < BT / 32; ++w) s += red[w][threadIdx.x];
        L.part[static_cast<size_t>(tile) * BPS + W_OFF + threadIdx.x] = s;
    }
}

// |u_{j+1}|^2 per state after the last step: H(j+1, j), s_{j+1}, breakdown.
__global__ void __launch_bounds__(BT) norm_last_kernel(Layout L, int j) {
    const int tile = blockIdx.x;
    const int p = L.tile_prob[tile];
    if (L.pdone[p]) return;
    const int q = threadIdx.x & 3;
    const int rl = threadIdx.x >> 2;
    const long long base = L.tile_row0[tile] - L.R0;
    const int nr = L.tile_nrows[tile];
    const float4* __restrict__ Un = col4(L, j + 1);
    float4 a = zero4();
    for (int r = rl; r < nr; r += BROWS) {
        const float4 u = __ldg(Un + static_cast<size_t>(base + r) * 4 + q);
        fma4(a, u, u);
    }
    const double acc[4] = {a.x, a.y, a.z, a.w};
    tile_rhs_partial(L, tile, acc);
    __shared__ int s_flag;
    if (!problem_last(L.pcount + p, static_cast<unsigned>(L.ptiles[p]), &s_flag)) return;
    if (threadIdx.x < BR) {
        const int b = p * BR + threadIdx.x;
        DevState* st = L.st + b;
        if (st->done || st->breakdown) return;
        const double nb = tiles_sum(L, p, W_OFF + threadIdx.x);
        double* pv = L.pre + static_cast<size_t>(b) * (BLD + 1);
        const double beta = sqrt(nb) / pv[j + 1];
        const bool bad = !(beta >= 1e-14) || isinf(beta);
        L.H[static_cast<size_t>(b) * BLD * BM_MAX + (j + 1) + static_cast<size_t>(j) * BLD] = bad ? 0.0 : beta;
        L.s[static_cast<size_t>(b) * (BLD + 1) + j + 1] = (nb > 0.0 && !isinf(nb)) ? 1.0 / sqrt(nb) : 0.0;
        if (bad) {
            st->breakdown = 1;
            st->k_used = j + 1;
        }
    }
}

// ---------------------------------------------------------------- lift / start
// start = 1: |v| of the start vectors V0 (every unfinished state).
// start = 0: y = sum_c (coef_c s_c) u_c for states with a pending lift (FP32
// products, compensated FP32 sums, FP64 result), and |y|.
// Then, per state, the restart scale 1/|y| (main.cu:2023-2073).
__global__ void __launch_bounds__(BT) lift_kernel(Layout L, int kmax, int start) {
    const int tile = blockIdx.x;
    const int p = L.tile_prob[tile];
    if (L.pdone[p]) return;
    __shared__ float4 scl[BM_MAX][4];
    __shared__ int smask[BR];
    if (!start) {
        for (int v = threadIdx.x; v < BM_MAX * BR; v += BT) {
            const int c = v / BR;
            const int r = v - c * BR;
            const int b = p * BR + r;
            const DevState* st = L.st + b;
            float cv = 0.f;
            if (st->lift && c < st->k_lift)
                cv = static_cast<float>(L.coefl[static_cast<size_t>(b) * BLD + c] *
                                        L.s[static_cast<size_t>(b) * (BLD + 1) + c]);
            reinterpret_cast<float*>(scl)[v] = cv;
        }
    }
    if (threadIdx.x < BR) {
        const DevState* st = L.st + p * BR + threadIdx.x;
        smask[threadIdx.x] = start ? (st->done ? 0 : 1) : st->lift;
    }
    __syncthreads();
    const int q = threadIdx.x & 3;
    const int rl = threadIdx.x >> 2;
    const bool m0 = smask[4 * q] != 0, m1 = smask[4 * q + 1] != 0, m2 = smask[4 * q + 2] != 0,
               m3 = smask[4 * q + 3] != 0;
    const long long grow = L.tile_row0[tile];
    const long long base = grow - L.R0;
    const int nr = L.tile_nrows[tile];
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    for (int r = rl; r < nr; r += BROWS) {
        double2* y2 = reinterpret_cast<double2*>(L.Y + static_cast<size_t>(grow + r) * BR + 4 * q);
        double y[4];
        if (start) {
            const double2* v2 = reinterpret_cast<const double2*>(L.V0 + static_cast<size_t>(grow + r) * BR + 4 * q);
            const double2 y01 = v2[0];
            const double2 y23 = v2[1];
            y[0] = y01.x;
            y[1] = y01.y;
            y[2] = y23.x;
            y[3] = y23.y;
        } else {
            if (!(m0 || m1 || m2 || m3)) continue;
            const size_t i = static_cast<size_t>(base + r) * 4 + q;
            float4 s = zero4(), comp = zero4();
            for (int c = 0; c < kmax; ++c) {
                const float4 u = __ldcs(col4(L, c) + i);
                const float4 cf = scl[c][q];
                float yv, t;
                yv = __fmaf_rn(cf.x, u.x, -comp.x); t = __fadd_rn(s.x, yv); comp.x = __fsub_rn(__fsub_rn(t, s.x), yv); s.x = t;
                yv = __fmaf_rn(cf.y, u.y, -comp.y); t = __fadd_rn(s.y, yv); comp.y = __fsub_rn(__fsub_rn(t, s.y), yv); s.y = t;
                yv = __fmaf_rn(cf.z, u.z, -comp.z); t = __fadd_rn(s.z, yv); comp.z = __fsub_rn(__fsub_rn(t, s.z), yv); s.z = t;
                yv = __fmaf_rn(cf.w, u.w, -comp.w); t = __fadd_rn(s.w, yv); comp.w = __fsub_rn(__fsub_rn(t, s.w), yv); s.w = t;
            }
            y[0] = static_cast<double>(s.x) - static_cast<double>(comp.x);
            y[1] = static_cast<double>(s.y) - static_cast<double>(comp.y);
            y[2] = static_cast<double>(s.z) - static_cast<double>(comp.z);
            y[3] = static_cast<double>(s.w) - static_cast<double>(comp.w);
            if (m0 && m1 && m2 && m3) {
                y2[0] = make_double2(y[0], y[1]);
                y2[1] = make_double2(y[2], y[3]);
            } else {
                double* yd = reinterpret_cast<double*>(y2);
                if (m0) yd[0] = y[0];
                if (m1) yd[1] = y[1];
                if (m2) yd[2] = y[2];
                if (m3) yd[3] = y[3];
            }
        }
        if (m0) acc[0] = fma(y[0], y[0], acc[0]);
        if (m1) acc[1] = fma(y[1], y[1], acc[1]);
        if (m2) acc[2] = fma(y[2], y[2], acc[2]);
        if (m3) acc[3] = fma(y[3], y[3], acc[3]);
    }
    tile_rhs_partial(L, tile, acc);
    __shared__ int s_flag;
    if (!problem_last(L.pcount + p, static_cast<unsigned>(L.ptiles[p]), &s_flag)) return;
    if (threadIdx.x < BR && smask[threadIdx.x]) {
        DevState* st = L.st + p * BR + threadIdx.x;
        const double nrm = sqrt(tiles_sum(L, p, W_OFF + threadIdx.x));
        st->restart_scale = nrm > 1e-14 ? 1.0 / nrm : 1.0;
        // FP32 bases do not resolve errors below their rounding of the iterate:
        // a step also passes below it while the accepted errors stay within
        // err_budget_rel of the iterate's norm.
        if (start) {
            st->v_norm = nrm;
            st->restart = 1;
        } else {
            if (st->restart) st->v_norm = nrm;
            st->lift = 0;
        }
        if (start || st->restart)
            st->tol = fmax(st->tol_base, fmin(st->tol_floor_rel * nrm, st->err_budget_rel * nrm - st->err_acc));
    }
}

// u_0 = y * restart_scale (or v * 1/|v| at the start) for states that
// restart (FP32); zero otherwise.
__global__ void __launch_bounds__(BT) restart_kernel(Layout L, int from_start) {
    __shared__ __align__(16) float ssc[BR];
    const int q = threadIdx.x & 3;
    const int rl = threadIdx.x >> 2;
    float4* __restrict__ U0 = reinterpret_cast<float4*>(L.U);
    for (int tile = blockIdx.x; tile < L.T; tile += gridDim.x) {
        const int p = L.tile_prob[tile];
        if (L.pdone[p]) continue;
        __syncthreads();
        if (threadIdx.x < BR) {
            const DevState* st = L.st + p * BR + threadIdx.x;
            ssc[threadIdx.x] = (st->restart && !st->done) ? static_cast<float>(st->restart_scale) : 0.f;
        }
        __syncthreads();
        const float4 sc = *reinterpret_cast<const float4*>(&ssc[4 * q]);
        const long long grow = L.tile_row0[tile];
        const long long base = grow - L.R0;
        const int nr = L.tile_nrows[tile];
        for (int r = rl; r < nr; r += BROWS) {
            const double* src = from_start ? L.V0 : L.Y;
            const double2* y2 = reinterpret_cast<const double2*>(src + static_cast<size_t>(grow + r) * BR + 4 * q);
            const double2 y01 = y2[0];
            const double2 y23 = y2[1];
            U0[static_cast<size_t>(base + r) * 4 + q] =
                make_float4(static_cast<float>(y01.x) * sc.x, static_cast<float>(y01.y) * sc.y,
                            static_cast<float>(y23.x) * sc.z, static_cast<float>(y23.y) * sc.w);
        }
    }
}

// Per problem: every state done? Counts the states still running.
__global__ void status_kernel(Layout L, int p0, int p1) {
    const int p = p0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= p1) return;
    int running = 0;
    for (int r = 0; r < BR; ++r) running += L.st[p * BR + r].done ? 0 : 1;
    L.pdone[p] = running == 0 ? 1 : 0;
    if (running) atomicAdd(L.active, running);
}

int sm_blocks(int per_sm) { return device_sm_count() * per_sm; }

}  // namespace

int launch_spmm(const Layout& L, int j, int unroll, cudaStream_t s) {
    const int chunks = L.C1 - L.C0;
    if (chunks <= 0) return MEXK_OK;
    const int grid = chunks < sm_blocks(8) ? chunks : sm_blocks(8);
    if (unroll >= 8) spmm_kernel<8><<<grid, BT, 0, s>>>(L, j);
    else spmm_kernel<4><<<grid, BT, 0, s>>>(L, j);
    MEXK_CK_LAUNCH("batch spmm_kernel");
    return MEXK_OK;
}

int launch_dot(const Layout& L, int j, int reortho, int gg, int tune, cudaStream_t s) {
    if (j < 0 || j >= BM_MAX || L.T <= 0) return L.T <= 0 ? MEXK_OK : MEXK_ERR_INVALID;
    const int k = j + 1;
    if (gg == 2) dot_kernel<2><<<L.T * ((k + 1) / 2), BT, 0, s>>>(L, j, reortho, tune);
    else dot_kernel<4><<<L.T * ((k + 3) / 4), BT, 0, s>>>(L, j, reortho, tune);
    MEXK_CK_LAUNCH("batch dot_kernel");
    return MEXK_OK;
}

int launch_update(const Layout& L, int j, cudaStream_t s) {
    if (j < 0 || j >= BM_MAX || L.T <= 0) return L.T <= 0 ? MEXK_OK : MEXK_ERR_INVALID;
    const int grid = L.T < sm_blocks(4) ? L.T : sm_blocks(4);
    update_kernel<<<grid, BT, 0, s>>>(L, j);
    MEXK_CK_LAUNCH("batch update_kernel");
    return MEXK_OK;
}

int launch_norm_last(const Layout& L, int j, cudaStream_t s) {
    if (j < 0 || j >= BM_MAX || L.T <= 0) return L.T <= 0 ? MEXK_OK : MEXK_ERR_INVALID;
    norm_last_kernel<<<L.T, BT, 0, s>>>(L, j);
    MEXK_CK_LAUNCH("batch norm_last_kernel");
    return MEXK_OK;
}

int launch_lift(const Layout& L, int k_max, int start, cudaStream_t s) {
    if (L.T <= 0) return MEXK_OK;
    if (k_max < 0 || k_max > BM_MAX) return MEXK_ERR_INVALID;
    lift_kernel<<<L.T, BT, 0, s>>>(L, k_max, start);
    MEXK_CK_LAUNCH("batch lift_kernel");
    return MEXK_OK;
}

int launch_restart(const Layout& L, int from_start, cudaStream_t s) {
    if (L.T <= 0) return MEXK_OK;
    const int grid = L.T < sm_blocks(4) ? L.T : sm_blocks(4);
    restart_kernel<<<grid, BT, 0, s>>>(L, from_start);
    MEXK_CK_LAUNCH("batch restart_kernel");
    return MEXK_OK;
}

int launch_status(const Layout& L, int p0, int p1, cudaStream_t s) {
    if (p1 <= p0) return MEXK_OK;
    status_kernel<<<(p1 - p0 + 255) / 256, 256, 0, s>>>(L, p0, p1);
    MEXK_CK_LAUNCH("batch status_kernel");
    return MEXK_OK;
}

}  // namespace batch
}  // namespace mexk
