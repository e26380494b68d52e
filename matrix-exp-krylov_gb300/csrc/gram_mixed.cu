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
#include "mexk_internal.cuh"

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

    // block stage: warp butterflies, then the warps in order, in FP64
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
    __syncthreads();
    if (threadIdx.x < 2 * GG + 1) {
        double t = 0.0;
#pragma unroll
        for (int q = 0; q < GW; ++q) t += s_red[q][threadIdx.x];
        double* P = g.part + static_cast<size_t>(rb) * GRAM_STRIDE;
        const int q = threadIdx.x;
        if (q < GG) {
            if (c0 + q < k) P[c0 + q] = t;
        } else if (q < 2 * GG) {
            if (c0 + q - GG < k) P[GRAM_BOFF + c0 + q - GG] = t;
        } else if (grp == 0) {
            P[GRAM_NWOFF] = t;
        }
    }

    // grid stage: the last block sums the row blocks in order and finishes the step
    __shared__ int s_flag;
    if (!grid_last_block(g.counter, &s_flag)) return;
    __shared__ double s_a[MEXK_M_MAX + 1], s_b[MEXK_M_MAX + 1], s_c[MEXK_M_MAX + 1], s_h[MEXK_M_MAX + 1];
    __shared__ double s_sc[MEXK_M_MAX + 1];
    __shared__ double s_G[MEXK_M_MAX][MEXK_M_MAX + 1];  // G(0:k, 0:k), row-major, padded
    __shared__ double s_scr[GT];
    __shared__ double s_w2, s_sj;
    __shared__ int s_bad;
    const int t = threadIdx.x;
    GramState* gs = g.gs;
    double* G = gs->G;
    {
        // Every load of this stage is independent: the row-block partials
        // (four running sums per thread, combined in a fixed order), the
        // previous columns' Gram block and scales.
        const int nv = 2 * kw + 1;
        const int groups = GT / nv;
        const int vi = t % nv;
        const int gi = t / nv;
        double sum = 0.0;
        if (gi < groups) {
            const int off = vi < kw ? lo + vi : (vi < 2 * kw ? GRAM_BOFF + lo + (vi - kw) : GRAM_NWOFF);
            const double* P = g.part + off;
            double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
            int b = gi;
            for (; b + 3 * groups < nrb; b += 4 * groups) {
                a0 += __ldcg(P + static_cast<size_t>(b) * GRAM_STRIDE);
                a1 += __ldcg(P + static_cast<size_t>(b + groups) * GRAM_STRIDE);
                a2 += __ldcg(P + static_cast<size_t>(b + 2 * groups) * GRAM_STRIDE);
                a3 += __ldcg(P + static_cast<size_t>(b + 3 * groups) * GRAM_STRIDE);
            }
            for (; b < nrb; b += groups) a0 += __ldcg(P + static_cast<size_t>(b) * GRAM_STRIDE);
            sum = (a0 + a1) + (a2 + a3);
        }
        const int jw = j - lo;  // previous columns inside the window
        for (int e = t; e < jw * jw; e += GT) {
            const int r = lo + e % jw, c = lo + e / jw;
            s_G[r][c] = G[r + static_cast<size_t>(c) * GRAM_LD];
        }
        if (t >= lo && t < j) s_sc[t] = gs->s[t];
        s_scr[t] = sum;
        __syncthreads();
        if (t < nv) {
            double tot = 0.0;
            for (int q = 0; q < groups; ++q) tot += s_scr[q * nv + t];
            if (t < kw) s_a[lo + t] = tot;
            else if (t < 2 * kw) s_b[lo + t - kw] = tot;
            else s_w2 = tot;
        }
        __syncthreads();
    }
    const size_t ldh = static_cast<size_t>(g.ldh);
    if (t == 0) {
        const double bj = s_b[j];
        int bad = 0;
        if (j >= 1) {
            // the previous step's h_{j,j-1} = |u_j| / p_j; breakdown test as main.cu:1911
            const double beta = sqrt(bj) / gs->p[j];
            bad = !(beta >= 1e-14) || isinf(beta);
            g.H[j + static_cast<size_t>(j - 1) * ldh] = bad ? 0.0 : beta;
            if (bad) {
                st->breakdown = 1;
                st->k_used = j;
            }
        }
        const double sj = (bj > 0.0 && !isinf(bj)) ? 1.0 / sqrt(bj) : 0.0;
        gs->s[j] = sj;
        s_sc[j] = sj;
        s_sj = sj;
        s_bad = bad;
    }
    __syncthreads();
    if (s_bad) return;
    const double sj = s_sj;
    if (t >= lo && t < k) {
        const double sc = s_sc[t];
        const double gv = (t == j) ? 1.0 : sc * sj * s_b[t];
        G[t + static_cast<size_t>(j) * GRAM_LD] = gv;
        G[j + static_cast<size_t>(t) * GRAM_LD] = gv;
        s_G[t][j] = gv;
        s_G[j][t] = gv;
        s_c[t] = sc * sj * s_a[t];
    }
    __syncthreads();
    if (t < lo) {
        g.H[t + static_cast<size_t>(j) * ldh] = 0.0;  // outside the window
    } else if (t < k) {
        double hv = s_c[t];
        if (g.reortho) {
            double e = 0.0;
            for (int q = lo; q < k; ++q)
                if (q != t) e = fma(s_G[t][q], s_c[q], e);
            hv -= e;
        }
        s_h[t] = hv;
        g.H[t + static_cast<size_t>(j) * ldh] = hv;
        gs->coef[t] = static_cast<float>(s_sc[t] * hv);
    }
    __syncthreads();
    // |w - V h|^2 = |w|^2 - 2 h.c + h^T G h  (pre-scale of the new column)
    double part = 0.0;
    if (t >= lo && t < k) {
        double gh = 0.0;
        for (int q = lo; q < k; ++q) gh = fma(s_G[t][q], s_h[q], gh);
        part = s_h[t] * gh - 2.0 * s_h[t] * s_c[t];
    }
    part = block_sum(part, s_scr);
    if (t == 0) {
        const double w2 = sj * sj * s_w2;
        const double u2 = w2 + part;
        double p = 1.0;
        if (u2 > 1e-8 * w2 && !isinf(u2)) p = 1.0 / sqrt(u2);
        else if (w2 > 0.0 && !isinf(w2)) p = 1.0 / sqrt(w2);
        gs->p[j + 1] = p;
        gs->wsc = static_cast<float>(sj);
        gs->psc = static_cast<float>(p);
    }
}

// Sweep 2: u_{j+1} = psc * (wsc * w - sum_c coef_c u_c), written to column
// j+1 with a default (L2-allocating) store: the next SpMV gathers from it.
__global__ void __launch_bounds__(GT, 4) gram_update_kernel(GramArgs g) {
    pdl_wait();
    DevState* st = g.st;
    if (st->breakdown || st->done) return;
    __shared__ float s_coef[MEXK_M_MAX + UCH];
    __shared__ float s_sc[2];
    const int k = g.j + 1;
    const int lo = g.lo;
    const GramState* gs = g.gs;
    if (threadIdx.x < MEXK_M_MAX + UCH) s_coef[threadIdx.x] = threadIdx.x < k ? gs->coef[threadIdx.x] : 0.f;
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
        for (int cbi = 0; cbi < MEXK_M_MAX; cbi += UCH) {
            const int cb = lo + cbi;
            if (cb < k) {
                float4 v[UCH];
#pragma unroll
                for (int c = 0; c < UCH; ++c)
                    v[c] = (cb + c < k) ? __ldcs(col4(g.V, ldv, cb + c) + i) : make_float4(0.f, 0.f, 0.f, 0.f);
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

// |u_{j+1}|^2 by grid reduction; the last block sets H(j+1, j), s_{j+1} and
// the breakdown flag (main.cu:1911).
__global__ void __launch_bounds__(GT) gram_norm_kernel(GramArgs g) {
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
    __shared__ double s_scr[GT];
    const double bsum = block_sum(static_cast<double>(acc), s_scr);
    if (threadIdx.x == 0) g.part[static_cast<size_t>(blockIdx.x) * GRAM_STRIDE] = bsum;
    __shared__ int s_flag;
    if (!grid_last_block(g.counter, &s_flag)) return;
    double tsum = 0.0;
    for (int b = threadIdx.x; b < static_cast<int>(gridDim.x); b += GT)
        tsum += __ldcg(&g.part[static_cast<size_t>(b) * GRAM_STRIDE]);
    const double total = block_sum(tsum, s_scr);
    if (threadIdx.x == 0) {
        GramState* gs = g.gs;
        const double b = total;
        const double beta = sqrt(b) / gs->p[jn];
        const bool bad = !(beta >= 1e-14) || isinf(beta);
        if (jn < g.ldh) g.H[jn + static_cast<size_t>(g.j) * g.ldh] = bad ? 0.0 : beta;
        gs->s[jn] = (b > 0.0 && !isinf(b)) ? 1.0 / sqrt(b) : 0.0;
        gs->G[jn + static_cast<size_t>(jn) * GRAM_LD] = 1.0;
        if (bad) {
            st->breakdown = 1;
            st->k_used = jn;
        }
    }
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
    if (a.j < 0 || a.j >= MEXK_M_MAX) return MEXK_ERR_INVALID;
    if (a.lo < 0 || a.lo > a.j) return MEXK_ERR_INVALID;
    const int ngroups = (a.j + 1 - a.lo + GG - 1) / GG;
    // One wave of 4 resident blocks per SM over all column groups (a partial
    // second wave would run at half occupancy); 2 row blocks per SM at most.
    int nrb = row_blocks(a.n, 2);
    if (ngroups > 2) nrb = std::min(nrb, std::max(1, 4 * device_sm_count() / ngroups));
    const cudaError_t e = launch_dependent(gram_dot_kernel, nrb * ngroups, GT, 0, s, a);
    if (e != cudaSuccess) {
        set_cuda_error(e, "gram_dot_kernel", __FILE__, __LINE__);
        return MEXK_ERR_CUDA;
    }
    return MEXK_OK;
}

int launch_gram_update(const GramArgs& a, cudaStream_t s) {
    if (a.j < 0 || a.j >= MEXK_M_MAX || a.lo < 0 || a.lo > a.j) return MEXK_ERR_INVALID;
    const cudaError_t e = launch_dependent(gram_update_kernel, row_blocks(a.n, 4), GT, 0, s, a);
    if (e != cudaSuccess) {
        set_cuda_error(e, "gram_update_kernel", __FILE__, __LINE__);
        return MEXK_ERR_CUDA;
    }
    return MEXK_OK;
}

int launch_gram_norm(const GramArgs& a, cudaStream_t s) {
    if (a.j < 0 || a.j >= MEXK_M_MAX) return MEXK_ERR_INVALID;
    gram_norm_kernel<<<row_blocks(a.n, 4), GT, 0, s>>>(a);
    MEXK_CK_LAUNCH("gram_norm_kernel");
    return MEXK_OK;
}

}  // namespace mexk
