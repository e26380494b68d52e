// K3: exp(dt*H_k) on the device plus the accept/reject step controller.
//
// The reference computes the small exponential on the host with Eigen
// (matrix_exp_stable, main.cu:33-36), twice per attempt (small_expm_and_lift
// main.cu:1954-1978 and residual_estimate main.cu:2004-2020), after copying
// every H entry to the host. Here one thread block holds the k-by-k matrices
// in shared memory and evaluates the Pade scaling-and-squaring method of
// N. J. Higham, SIAM J. Matrix Anal. Appl. 26(4), 2005 (the method Eigen
// 3.4's MatrixExponential implements): degree 3/5/7/9/13 from the 1-norm,
// 2^-s scaling before degree 13, an LU solve with partial pivoting for
// (V-U)^{-1}(V+U), then s squarings. The same exponential feeds the lift
// coefficients and the residual estimate |H(k,k-1) [exp(dt H_k) e1]_{k-1}| |v|.
//
// The controller (ArnoldiRunner::compute_expmv, main.cu:1431-1518) runs in
// the same block with the reference's arithmetic: accept if err <= tol or
// breakdown; grow dt by 1.5*0.8 when err < 0.1*tol (capped at dt_max);
// otherwise shrink by 0.5*0.8 (floored at dt_min) and retry, aborting after
// 20 rejects. The reference rebuilds the whole Arnoldi basis on every retry;
// the basis depends only on A and the start vector, never on dt, so the
// retry here reuses it and re-evaluates only the exponential: same decisions
// and results, m SpMVs and Gram-Schmidt sweeps fewer per reject.
#include "controller_net.cuh"
#include "mexk_internal.cuh"

#include <math.h>

#include <cooperative_groups.h>

namespace mexk {

namespace {

constexpr int EXPM_THREADS = 512;
constexpr int SEARCH_CLUSTER = 8;  // thread blocks (SMs) per chain of candidate exponentials
// chains of candidates one octave apart: 12 with a network (96 SMs), 8 without (64)
constexpr int SEARCH_CHAINS_NET = 12;
constexpr int SEARCH_CHAINS = 8;

// FP64 adds and FMAs take about 64 cycles of latency on this GPU (FP32: 4),
// and these k <= 64 matrices leave most of the block idle, so every dot
// product runs as four independent chains combined at the end.
__device__ __forceinline__ double dot_k(int k, const double* X, int ldx, const double* Y) {
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
    int l = 0;
    for (; l + 3 < k; l += 4) {
        s0 = fma(X[l * ldx], Y[l], s0);
        s1 = fma(X[(l + 1) * ldx], Y[l + 1], s1);
        s2 = fma(X[(l + 2) * ldx], Y[l + 2], s2);
        s3 = fma(X[(l + 3) * ldx], Y[l + 3], s3);
    }
    for (; l < k; ++l) s0 = fma(X[l * ldx], Y[l], s0);
    return (s0 + s1) + (s2 + s3);
}

// Band of a k x k matrix: entry (r, c) may be nonzero only if r - c <= lb
// and c - r <= ub. A product's band is the sum of its factors' (capped at
// k - 1); a tridiagonal Lanczos H gives banded powers, and a Hessenberg H a
// lower bandwidth that grows by one per factor.
struct Band {
    int lb, ub;
};
__device__ __forceinline__ Band band_mul(Band x, Band y, int k) {
    return {min(x.lb + y.lb, k - 1), min(x.ub + y.ub, k - 1)};
}
__device__ __forceinline__ Band band_max(Band x, Band y) { return {max(x.lb, y.lb), max(x.ub, y.ub)}; }

// dot_k over the terms l in [lo, hi] only (every other product has an exact
// zero factor): the loop keeps dot_k's groups of four and its tail, so each
// nonzero product lands in the same accumulation in the same order and the
// sum is dot_k's.
__device__ __forceinline__ double dot_k_band(int k, int lo, int hi, const double* X, int ldx, const double* Y) {
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
    int l = lo & ~3;
    const int end = min(k, (hi + 4) & ~3);  // past hi, at a group boundary (or k)
    for (; l + 3 < end; l += 4) {
        s0 = fma(X[l * ldx], Y[l], s0);
        s1 = fma(X[(l + 1) * ldx], Y[l + 1], s1);
        s2 = fma(X[(l + 2) * ldx], Y[l + 2], s2);
        s3 = fma(X[(l + 3) * ldx], Y[l + 3], s3);
    }
    for (; l < end; ++l) s0 = fma(X[l * ldx], Y[l], s0);
    return (s0 + s1) + (s2 + s3);
}

// (X Y)_ij = dot over the l both bands allow.
__device__ __forceinline__ double dot_banded(int k, int i, int j, const double* X, Band bx, const double* Y, Band by) {
    const int lo = max(max(i - bx.lb, j - by.ub), 0);
    const int hi = min(min(i + bx.ub, j + by.lb), k - 1);
    return dot_k_band(k, lo, hi, X + i, k, Y + j * k);
}

__device__ void mm(int k, const double* X, const double* Y, double* Z) {
    const int kk = k * k;
    for (int e = threadIdx.x; e < kk; e += blockDim.x) {
        const int i = e % k, j = e / k;
        Z[e] = dot_k(k, X + i, k, Y + j * k);
    }
    __syncthreads();
}

// Z = c0*M0 + c1*M1 + c2*M2 + c3*M3 + cid*I, terms left to right (nt <= 4).
__device__ void lincomb(int k, int nt, const double* c, const double* const* M, double cid, double* Z) {
    const int kk = k * k;
    for (int e = threadIdx.x; e < kk; e += blockDim.x) {
        double s = c[0] * M[0][e];
        for (int t = 1; t < nt; ++t) s = s + c[t] * M[t][e];
        if (cid != 0.0 && (e % k) == (e / k)) s = s + cid;
        Z[e] = s;
    }
    __syncthreads();
}

__device__ void lu_factor(int k, double* D, int* piv, int* status) {
    for (int c = 0; c < k; ++c) {
        if (threadIdx.x < 32) {
            double best = -1.0;
            int bi = k;
            for (int i = c + threadIdx.x; i < k; i += 32) {
                const double v = fabs(D[i + c * k]);
                if (v > best) {
                    best = v;
                    bi = i;
                }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const double ob = __shfl_xor_sync(0xffffffffu, best, o);
                const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
                if (ob > best || (ob == best && oi < bi)) {
                    best = ob;
                    bi = oi;
                }
            }
            if (threadIdx.x == 0) piv[c] = (bi < k) ? bi : c;
        }
        __syncthreads();
        const int p = piv[c];
        if (p != c) {
            for (int j = threadIdx.x; j < k; j += blockDim.x) {
                const double t = D[c + j * k];
                D[c + j * k] = D[p + j * k];
                D[p + j * k] = t;
            }
            __syncthreads();
        }
        const double d = D[c + c * k];
        if (d != 0.0) {
            for (int i = c + 1 + threadIdx.x; i < k; i += blockDim.x) D[i + c * k] /= d;
            __syncthreads();
            const int r = k - c - 1;
            for (int e = threadIdx.x; e < r * r; e += blockDim.x) {
                const int i = c + 1 + e % r, j = c + 1 + e / r;
                D[i + j * k] -= D[i + c * k] * D[c + j * k];
            }
        } else if (threadIdx.x == 0) {
            *status |= ST_LU_SINGULAR;
        }
        __syncthreads();
    }
}

__device__ void lu_solve(int k, const double* LU, const int* piv, double* B) {
    for (int i = 0; i < k; ++i) {
        const int p = piv[i];
        if (p != i) {
            for (int c = threadIdx.x; c < k; c += blockDim.x) {
                const double t = B[i + c * k];
                B[i + c * k] = B[p + c * k];
                B[p + c * k] = t;
            }
            __syncthreads();
        }
    }
    for (int i = 0; i < k - 1; ++i) {
        const int r = k - i - 1;
        for (int e = threadIdx.x; e < r * k; e += blockDim.x) {
            const int l = i + 1 + e % r, c = e / r;
            B[l + c * k] -= LU[l + i * k] * B[i + c * k];
        }
        __syncthreads();
    }
    for (int i = k - 1; i >= 0; --i) {
        for (int c = threadIdx.x; c < k; c += blockDim.x) B[i + c * k] /= LU[i + i * k];
        __syncthreads();
        for (int e = threadIdx.x; e < i * k; e += blockDim.x) {
            const int l = e % i, c = e / i;
            B[l + c * k] -= LU[l + i * k] * B[i + c * k];
        }
        __syncthreads();
    }
}

// Pade [m/m] coefficients b_j = (2m-j)! / (j! (m-j)!), exact integers.
__device__ void pade_coefficients(int m, double* b) {
    for (int j = 0; j <= m; ++j) {
        unsigned long long num = 1ull, den = 1ull;
        for (int i = m - j + 1; i <= 2 * m - j; ++i) num *= static_cast<unsigned long long>(i);
        for (int i = 2; i <= j; ++i) den *= static_cast<unsigned long long>(i);
        b[j] = static_cast<double>(num / den);
    }
}

struct ExpmBuf {
    double *A, *A2, *A4, *A6, *U, *T;
    int* piv;
    double* red;  // >= k doubles
};

// 1-norm column sums of the k-by-k matrix in A (thread j < k: column j).
__device__ __forceinline__ double col_abs_sum(int k, const double* A, int j) {
    double c0 = 0.0, c1 = 0.0, c2 = 0.0, c3 = 0.0;
    int i = 0;
    for (; i + 3 < k; i += 4) {
        c0 += fabs(A[i + j * k]);
        c1 += fabs(A[i + 1 + j * k]);
        c2 += fabs(A[i + 2 + j * k]);
        c3 += fabs(A[i + 3 + j * k]);
    }
    for (; i < k; ++i) c0 += fabs(A[i + j * k]);
    return (c0 + c1) + (c2 + c3);
}

// exp of the k-by-k matrix in B.A (ld k) by Pade scaling and squaring;
// returns the buffer holding the result. All threads of the block must call it.
__device__ double* expm_block(const ExpmBuf& B, int k, int* status) {
    __shared__ int s_deg, s_sq;
    __shared__ double s_b[14];
    if (threadIdx.x < k) B.red[threadIdx.x] = col_abs_sum(k, B.A, threadIdx.x);
    __syncthreads();
    if (threadIdx.x == 0) {
        double l1 = 0.0;
        for (int j = 0; j < k; ++j)
            if (B.red[j] > l1) l1 = B.red[j];
        int sq = 0, deg;
        // A non-finite norm (Inf or NaN entries) keeps degree 13 without
        // scaling: frexp's exponent is unspecified there, and the squaring
        // loop must stay bounded; the result is then non-finite as well.
        if (!(l1 <= 1.7976931348623157e308)) {
            deg = 13;
            *status |= ST_NONFINITE;
        } else if (l1 < 1.495585217958292e-002) deg = 3;
        else if (l1 < 2.539398330063230e-001) deg = 5;
        else if (l1 < 9.504178996162932e-001) deg = 7;
        else if (l1 < 2.097847961257068e+000) deg = 9;
        else {
            deg = 13;
            (void)frexp(l1 / 5.371920351148152, &sq);
            if (sq < 0) sq = 0;
            if (sq > 1100) sq = 1100;  // beyond the double range: l1 is finite here
        }
        s_deg = deg;
        s_sq = sq;
        pade_coefficients(deg, s_b);
    }
    __syncthreads();
    const int deg = s_deg, sq = s_sq;
    const int kk = k * k;
    if (sq > 0) {
        for (int e = threadIdx.x; e < kk; e += blockDim.x) B.A[e] = ldexp(B.A[e], -sq);
        __syncthreads();
    }
    const double* b = s_b;
    mm(k, B.A, B.A, B.A2);
    if (deg >= 5) mm(k, B.A2, B.A2, B.A4);
    if (deg >= 7) mm(k, B.A4, B.A2, B.A6);
    double *pU, *pV;
    if (deg <= 7) {
        const double* M[3] = {deg == 3 ? B.A2 : (deg == 5 ? B.A4 : B.A6), deg == 7 ? B.A4 : B.A2, B.A2};
        const int nt = deg == 3 ? 1 : (deg == 5 ? 2 : 3);
        double cu[3], cv[3];
        if (deg == 3) { cu[0] = b[3]; cv[0] = b[2]; }
        if (deg == 5) { cu[0] = b[5]; cu[1] = b[3]; cv[0] = b[4]; cv[1] = b[2]; }
        if (deg == 7) { cu[0] = b[7]; cu[1] = b[5]; cu[2] = b[3]; cv[0] = b[6]; cv[1] = b[4]; cv[2] = b[2]; }
        lincomb(k, nt, cu, M, b[1], B.T);
        mm(k, B.A, B.T, B.U);
        lincomb(k, nt, cv, M, b[0], B.T);
        pU = B.U;
        pV = B.T;
    } else if (deg == 9) {
        mm(k, B.A6, B.A2, B.U);  // A8 in U
        for (int e = threadIdx.x; e < kk; e += blockDim.x) {
            const double a8 = B.U[e], a6 = B.A6[e], a4 = B.A4[e], a2 = B.A2[e];
            const bool dg = (e % k) == (e / k);
            double u = b[9] * a8 + b[7] * a6 + b[5] * a4 + b[3] * a2;
            double v = b[8] * a8 + b[6] * a6 + b[4] * a4 + b[2] * a2;
            if (dg) { u = u + b[1]; v = v + b[0]; }
            B.T[e] = u;
            B.U[e] = v;
        }
        __syncthreads();
        mm(k, B.A, B.T, B.A2);
        pU = B.A2;
        pV = B.U;
    } else {
        const double* M[3] = {B.A6, B.A4, B.A2};
        const double c1[3] = {b[13], b[11], b[9]};
        lincomb(k, 3, c1, M, 0.0, B.T);
        mm(k, B.A6, B.T, B.U);
        for (int e = threadIdx.x; e < kk; e += blockDim.x) {
            double s = b[7] * B.A6[e] + b[5] * B.A4[e] + b[3] * B.A2[e];
            if ((e % k) == (e / k)) s = s + b[1];
            B.U[e] = B.U[e] + s;
        }
        __syncthreads();
        mm(k, B.A, B.U, B.T);  // U final in T
        const double c3[3] = {b[12], b[10], b[8]};
        lincomb(k, 3, c3, M, 0.0, B.U);
        mm(k, B.A6, B.U, B.A);  // V in A
        for (int e = threadIdx.x; e < kk; e += blockDim.x) {
            double s = b[6] * B.A6[e] + b[4] * B.A4[e] + b[2] * B.A2[e];
            if ((e % k) == (e / k)) s = s + b[0];
            B.A[e] = B.A[e] + s;
        }
        __syncthreads();
        pU = B.T;
        pV = B.A;
    }
    // numer = U + V (into pU), denom = -U + V (into pV)
    for (int e = threadIdx.x; e < kk; e += blockDim.x) {
        const double u = pU[e], v = pV[e];
        pU[e] = u + v;
        pV[e] = -u + v;
    }
    __syncthreads();
    lu_factor(k, pV, B.piv, status);
    lu_solve(k, pV, B.piv, pU);
    double* R = pU;
    double* F = pV;
    for (int s = 0; s < sq; ++s) {
        mm(k, R, R, F);
        double* t = R;
        R = F;
        F = t;
    }
    return R;
}

// 1/i!, i = 0..18: the factorials are exact in double, one rounding each.
constexpr double fact_d(int n) { return n <= 1 ? 1.0 : n * fact_d(n - 1); }
__constant__ double kInvFact[19] = {
    1.0 / fact_d(0),  1.0 / fact_d(1),  1.0 / fact_d(2),  1.0 / fact_d(3),  1.0 / fact_d(4),
    1.0 / fact_d(5),  1.0 / fact_d(6),  1.0 / fact_d(7),  1.0 / fact_d(8),  1.0 / fact_d(9),
    1.0 / fact_d(10), 1.0 / fact_d(11), 1.0 / fact_d(12), 1.0 / fact_d(13), 1.0 / fact_d(14),
    1.0 / fact_d(15), 1.0 / fact_d(16), 1.0 / fact_d(17), 1.0 / fact_d(18)};

// Who computes the k x k products of the Taylor chain. BlockProducts: this
// thread block, all columns. ClusterProducts: the thread blocks of a cluster,
// each holding full copies of the matrices, compute a share of every
// product's columns and write it into every block's copy (distributed shared
// memory), then a cluster barrier. GB300 executes about 2 FP64 FMAs per clock
// per SM, so a 31 x 31 product takes ~7 us on one SM; a cluster of 4 spreads
// it over 4 SMs with the same arithmetic (each element one dot_k).
struct BlockProducts {
    int k;
    __device__ void cols(int* j0, int* j1) const {
        *j0 = 0;
        *j1 = k;
    }
    __device__ void put(double* Z, int idx, double v) const { Z[idx] = v; }
    __device__ void sync() const { __syncthreads(); }
};
struct ClusterProducts {
    int k;
    __device__ void cols(int* j0, int* j1) const {
        const cooperative_groups::cluster_group cl = cooperative_groups::this_cluster();
        const int r = static_cast<int>(cl.block_rank()), c = static_cast<int>(cl.num_blocks());
        *j0 = r * k / c;
        *j1 = (r + 1) * k / c;
    }
    __device__ void put(double* Z, int idx, double v) const {
        const cooperative_groups::cluster_group cl = cooperative_groups::this_cluster();
        const unsigned c = cl.num_blocks();
        for (unsigned p = 0; p < c; ++p) cl.map_shared_rank(Z, p)[idx] = v;
    }
    __device__ void sync() const { cooperative_groups::this_cluster().sync(); }
};

// Z = X Y (k x k) for factors within bands bx, by; columns shared out as P
// says. Returns Z's band.
template <typename P>
__device__ Band mm_p(const P& pr, int k, const double* X, Band bx, const double* Y, Band by, double* Z) {
    int j0, j1;
    pr.cols(&j0, &j1);
    const int cnt = k * (j1 - j0);
    for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
        const int i = e % k, j = j0 + e / k;
        pr.put(Z, i + j * k, dot_banded(k, i, j, X, bx, Y, by));
    }
    pr.sync();
    return band_mul(bx, by, k);
}

// The band of the k x k matrix in A (every thread of the block calls it).
__device__ Band band_of(int k, const double* A) {
    __shared__ int s_lb, s_ub;
    if (threadIdx.x == 0) {
        s_lb = 0;
        s_ub = 0;
    }
    __syncthreads();
    int lb = 0, ub = 0;
    for (int e = threadIdx.x; e < k * k; e += blockDim.x) {
        if (A[e] != 0.0) {
            const int r = e % k, c = e / k;
            lb = max(lb, r - c);
            ub = max(ub, c - r);
        }
    }
    if (lb > 0) atomicMax(&s_lb, lb);
    if (ub > 0) atomicMax(&s_ub, ub);
    __syncthreads();
    return {s_lb, s_ub};
}

// exp of the k-by-k matrix in B.A (ld k) by the degree-18 Taylor polynomial
// with scaling and squaring: X = A / 2^s with |X|_1 <= 1, so the truncated
// terms sum to at most sum_{i>18} 1/i! < 8.5e-18 (below double rounding);
// T_18(X) by Paterson-Stockmeyer with X^2, X^3, X^4 and a Horner recurrence
// in X^4 (7 products, no linear solve), then s squarings. A product-only
// chain suits this GPU's FP64 latency far better than the Pade solve; the
// candidate-step controller uses it (the reference controller keeps Pade,
// as the reference does). Returns the buffer holding the result; every
// thread of the block (of every block of the cluster) must call it, with
// the same B.A.
template <typename P>
__device__ __noinline__ double* expm_taylor(const ExpmBuf& B, int k, const P& pr, Band* band_out) {
    __shared__ int s_sq;
    if (threadIdx.x < k) B.red[threadIdx.x] = col_abs_sum(k, B.A, threadIdx.x);
    __syncthreads();
    if (threadIdx.x < 32) {
        double l1 = 0.0;
        for (int j = threadIdx.x; j < k; j += 32) l1 = fmax(l1, B.red[j]);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) l1 = fmax(l1, __shfl_xor_sync(0xffffffffu, l1, o));
        if (threadIdx.x == 0) {
            int sq = 0;
            if (l1 > 1.0 && !isinf(l1)) {
                (void)frexp(l1, &sq);  // l1 / 2^sq in [0.5, 1)
            }
            s_sq = sq;
        }
    }
    __syncthreads();
    const int sq = s_sq;
    const int kk = k * k;
    if (sq > 0) {
        for (int e = threadIdx.x; e < kk; e += blockDim.x) B.A[e] = ldexp(B.A[e], -sq);
    }
    // the band of X (scaling keeps every zero); the products below skip the
    // terms outside their factors' bands
    const Band b1 = band_of(k, B.A);
    // every block's copy of X must be final before a product writes into it
    pr.sync();
    const double* X = B.A;
    double* X2 = B.A2;
    double* X3 = B.A4;
    double* X4 = B.A6;
    const Band b2 = mm_p(pr, k, X, b1, X, b1, X2);
    const Band b3 = mm_p(pr, k, X2, b2, X, b1, X3);
    const Band b4 = mm_p(pr, k, X2, b2, X2, b2, X4);
    const double* c = kInvFact;
    // Z = c16 I + c17 X + c18 X^2 (every block its full copy)
    double* Z = B.T;
    double* W = B.U;
    for (int e = threadIdx.x; e < kk; e += blockDim.x) {
        double z = c[17] * X[e] + c[18] * X2[e];
        if ((e % k) == (e / k)) z = z + c[16];
        Z[e] = z;
    }
    pr.sync();
    // Z = B_q + X^4 Z, B_q = c_{4q} I + c_{4q+1} X + c_{4q+2} X^2 + c_{4q+3} X^3
    int j0, j1;
    pr.cols(&j0, &j1);
    const int cnt = k * (j1 - j0);
    Band bz = b2;
    for (int q = 3; q >= 0; --q) {
        for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
            const int i = e % k, j = j0 + e / k;
            const int idx = i + j * k;
            double b = c[4 * q + 1] * X[idx] + c[4 * q + 2] * X2[idx] + c[4 * q + 3] * X3[idx];
            if (i == j) b = b + c[4 * q];
            pr.put(W, idx, dot_banded(k, i, j, X4, b4, Z, bz) + b);
        }
        pr.sync();
        bz = band_max(band_mul(b4, bz, k), b3);
        double* t = Z;
        Z = W;
        W = t;
    }
    for (int r = 0; r < sq; ++r) {
        bz = mm_p(pr, k, Z, bz, Z, bz, W);
        double* t = Z;
        Z = W;
        W = t;
    }
    *band_out = bz;
    return Z;
}

__device__ double* expm_taylor_block(const ExpmBuf& B, int k) {
    Band b;
    return expm_taylor(B, k, BlockProducts{k}, &b);
}

__device__ ExpmBuf carve(double* smem, int k) {
    ExpmBuf B;
    const size_t kk = static_cast<size_t>(k) * k;
    B.A = smem;
    B.A2 = B.A + kk;
    B.A4 = B.A2 + kk;
    B.A6 = B.A4 + kk;
    B.U = B.A6 + kk;
    B.T = B.U + kk;
    B.red = B.T + kk;
    B.piv = reinterpret_cast<int*>(B.red + MEXK_M_MAX);
    return B;
}

size_t expm_smem_bytes(int k) {
    return sizeof(double) * (6 * static_cast<size_t>(k) * k + MEXK_M_MAX) + sizeof(int) * MEXK_M_MAX;
}

// Dynamic shared memory of an exponential kernel for dimensions up to m:
// none when the matrices live in the global workspace.
size_t expm_launch_smem(int m) { return m > EXPM_SMEM_K ? 0 : expm_smem_bytes(m); }

__global__ void __launch_bounds__(EXPM_THREADS)
    expm_standalone_kernel(int k, const double* __restrict__ A, int lda, double* __restrict__ E, int lde,
                           int* status, double* ws) {
    extern __shared__ double smem[];
    ExpmBuf B = carve(k > EXPM_SMEM_K ? ws : smem, k);
    for (int e = threadIdx.x; e < k * k; e += blockDim.x) B.A[e] = A[(e % k) + static_cast<size_t>(e / k) * lda];
    __syncthreads();
    double* R = expm_block(B, k, status);
    for (int e = threadIdx.x; e < k * k; e += blockDim.x) E[(e % k) + static_cast<size_t>(e / k) * lde] = R[e];
}

enum : int { DEC_REJECT = 0, DEC_ACCEPT = 1, DEC_ABORT = 2, DEC_REBUILD = 3 };

__global__ void __launch_bounds__(EXPM_THREADS) controller_kernel(ControlArgs a, int m) {
    extern __shared__ double smem[];
    __shared__ int s_k, s_bd, s_dec, s_mcur, s_cyc_bd, s_cyc_k;
    __shared__ double s_dt;
    pdl_wait();  // launched as a dependent of the basis's last kernel
    pdl_trigger();
    // One block per state: block b drives state b (a batch), or the only one.
    DevState* st = a.st + blockIdx.x;
    const double* Hb = a.H + blockIdx.x * a.h_stride;
    double* coef = a.coef + blockIdx.x * a.coef_stride;
    if (st->done) return;
    if (threadIdx.x == 0) {
        const int bd = st->breakdown;
        int k = bd ? st->k_used : m;
        if (k < 1 || k > m) {
            st->status |= ST_BAD_K;
            k = k < 1 ? 1 : m;
        }
        s_k = k;
        s_bd = bd;
        s_dt = st->dt;
        s_mcur = m;
        s_cyc_bd = bd;  // the basis built this cycle: m columns, or k_used up to a breakdown
        s_cyc_k = k;
    }
    __syncthreads();
    const size_t ldh = static_cast<size_t>(a.ldh);
    // The matrices in shared memory, or (m > EXPM_SMEM_K) in the workspace.
    double* const base = m > EXPM_SMEM_K ? a.ws : smem;
    int rejects = st->rejects;
    double err = 0.0;
    double* R = nullptr;
    while (true) {
        const int k = s_k;
        const bool bd = s_bd != 0;
        ExpmBuf B = carve(base, k);
        const double dt = s_dt;
        for (int e = threadIdx.x; e < k * k; e += blockDim.x) B.A[e] = dt * Hb[(e % k) + (e / k) * ldh];
        __syncthreads();
        R = expm_block(B, k, &st->status);
        if (threadIdx.x == 0) {
            err = bd ? 0.0 : fabs(Hb[k + (k - 1) * ldh] * R[k - 1]) * st->v_norm;
            if (st->nlog < st->log_cap && a.log != nullptr) {
                mexk_step_t& L = a.log[st->nlog];
                L.t_done = st->t_done;
                L.dt = dt;
                L.err = err;
                L.m_used = k;
                L.accepts = st->accepted;
                L.rejects = rejects;
                L.m_basis = s_mcur;
            }
            st->nlog += 1;
            st->attempts += 1;
            int dec;
            if (err <= st->tol || bd) {
                dec = DEC_ACCEPT;
            } else {
                ++rejects;
                if (rejects >= st->max_rejects) {
                    dec = DEC_ABORT;
                } else {
                    // main.cu:1507-1513: retry the same dt with a basis m_step
                    // larger (adapt_m, up to m_max), else a shrunk dt with the
                    // base dimension. The reference rebuilds the basis; a basis
                    // of m' columns is the first m' of this cycle's (up to its
                    // breakdown, where a larger one breaks down too), so only a
                    // larger basis than this cycle built needs the next cycle.
                    int mc = s_mcur + st->m_step;
                    const bool grow_m = st->adapt_m && st->m_step > 0 && mc <= st->m_max;
                    if (grow_m) {
                        dec = (mc > m && !s_cyc_bd) ? DEC_REBUILD : DEC_REJECT;
                    } else {
                        dec = DEC_REJECT;
                        const double dt_new = (dt * st->shrink) * st->safety;
                        s_dt = dt_new > st->dt_min ? dt_new : st->dt_min;
                        mc = st->m_base;
                    }
                    s_mcur = mc;
                    if (dec == DEC_REJECT) {
                        const bool bd2 = s_cyc_bd && s_cyc_k <= mc;
                        s_k = bd2 ? s_cyc_k : mc;
                        s_bd = bd2 ? 1 : 0;
                    }
                }
            }
            s_dec = dec;
        }
        __syncthreads();
        if (s_dec != DEC_REJECT) break;
    }
    const int k = s_k;
    if (s_dec == DEC_REBUILD) {
        if (threadIdx.x == 0) {
            st->rejects = rejects;
            st->m_next = s_mcur;
            st->k_used = st->m_next;
            st->breakdown = 0;
            st->cycles += 1;
            st->spmv_count += k;
            st->lift = 0;
            st->restart = 0;
        }
        return;
    }
    // Lift coefficients |v| * wH_i, zero where |wH_i| <= 1e-15 (main.cu:1993).
    const double vn = st->v_norm;
    for (int i = threadIdx.x; i <= k; i += blockDim.x) {
        const double wi = (i < k) ? R[i] : 0.0;
        coef[i] = (fabs(wi) > 1e-15 && isfinite(wi)) ? vn * wi : 0.0;
    }
    if (threadIdx.x == 0) {
        double dt = s_dt;
        st->rejects = 0;
        st->m_next = st->m_base;
        if (s_dec == DEC_ACCEPT) {
            st->t_done += dt;
            st->accepted += 1;
            st->last_residual = err;
            st->err_acc += err;
            if (st->t_done >= st->total_t) {
                st->converged = 1;
                st->done = 1;
                st->restart = 0;
            } else {
                if (err < 0.1 * st->tol) {
                    const double dt_new = (dt * st->grow) * st->safety;
                    dt = dt_new < st->dt_max ? dt_new : st->dt_max;
                }
                if (st->accepted >= st->max_steps) {
                    st->done = 1;
                    st->restart = 0;
                } else {
                    st->restart = 1;
                }
            }
        } else {
            st->converged = 0;
            st->last_residual = err;
            st->t_done = st->total_t;
            st->done = 1;
            st->restart = 0;
        }
        st->k_lift = k;
        st->cycles += 1;
        st->spmv_count += k;
        st->lift = 1;
        if (!st->done) {
            st->breakdown = 0;
            st->k_used = st->m_base;
            const double rem = st->total_t - st->t_done;
            dt = dt < rem ? dt : rem;
        }
        st->dt = dt;
    }
}

// Shared accept bookkeeping of both controllers (main.cu:1476-1516): accepted
// step tau with estimate err, or an abort after too many rejects.
__device__ void finish_cycle(DevState* st, bool accept, double tau, double err, int k, int m_next,
                             double next_center, bool grow_reference) {
    double dt = tau;
    if (accept) {
        st->t_done += tau;
        st->accepted += 1;
        st->last_residual = err;
        st->err_acc += err;
        if (st->t_done >= st->total_t) {
            st->converged = 1;
            st->done = 1;
            st->restart = 0;
        } else {
            if (grow_reference) {
                if (err < 0.1 * st->tol) {
                    const double dt_new = (dt * st->grow) * st->safety;
                    dt = dt_new < st->dt_max ? dt_new : st->dt_max;
                }
            } else {
                dt = next_center < st->dt_max ? next_center : st->dt_max;
            }
            if (st->accepted >= st->max_steps) {
                st->done = 1;
                st->restart = 0;
            } else {
                st->restart = 1;
            }
        }
    } else {
        st->converged = 0;
        st->last_residual = err;
        st->t_done = st->total_t;
        st->done = 1;
        st->restart = 0;
    }
    st->k_lift = k;
    st->cycles += 1;
    st->spmv_count += k;
    st->lift = 1;
    st->tau_prev = tau;
    st->err_prev = err;
    if (!st->done) {
        st->breakdown = 0;
        st->m_next = m_next;
        st->k_used = m_next;
        const double rem = st->total_t - st->t_done;
        dt = dt < rem ? dt : rem;
    }
    st->dt = dt;
}

__device__ void write_log(DevState* st, mexk_step_t* log, double dt, double err, int k, int rejects, int m) {
    if (log != nullptr && st->nlog < st->log_cap) {
        mexk_step_t& L = log[st->nlog];
        L.t_done = st->t_done;
        L.dt = dt;
        L.err = err;
        L.m_used = k;
        L.accepts = st->accepted;
        L.rejects = rejects;
        L.m_basis = m;
    }
    st->nlog += 1;
    st->attempts += 1;
}

// Candidate steps tau_g = center * 2^((g - 24)/4), g = 0..31 (1/64 .. 3.4 x the
// centre), each clamped to the remaining time. Every cluster of
// SEARCH_CLUSTER blocks evaluates a chain of candidates an octave apart
// (their exponentials and residual estimates; the products shared out over
// its SMs); the last block to finish
// takes the largest passing step (its exponential is reused for the lift),
// or, if none passes, continues below the smallest candidate with the
// reference's shrink rule (on its own).
__global__ void __launch_bounds__(EXPM_THREADS, 1) controller_search_kernel(SearchArgs a, int m) {
    extern __shared__ double smem[];
    __shared__ int s_k, s_bd, s_flag, s_best, s_dec, s_mnext;
    __shared__ double s_tau, s_center, s_n1;
    __shared__ float s_f[net::IN], s_a1[net::HID], s_a2[net::HID], s_o[net::OUT];
    // a programmatic dependent of the basis's last kernel: the state and H
    // are read after the wait; the lift may then launch onto the SMs the
    // clusters leave idle (it waits for this grid before reading)
    pdl_wait();
    pdl_trigger();
    DevState* st = a.st;
    if (st->done) return;
    if (threadIdx.x == 0) {
        const int bd = st->breakdown;
        int k = bd ? st->k_used : m;
        if (k < 1 || k > m) k = k < 1 ? 1 : m;
        s_k = k;
        s_bd = bd;
        s_center = st->dt;
        s_mnext = m;
    }
    __syncthreads();
    const int k = s_k;
    const bool bd = s_bd != 0;
    const size_t ldh = static_cast<size_t>(a.ldh);
    const double rem = st->total_t - st->t_done;
    // Mixed precision: a step may also pass below the FP32 resolution of the
    // iterate, while the errors accepted so far stay within err_budget_rel of
    // its norm (both zero for FP64).
    const double relax = fmin(st->tol_floor_rel * st->v_norm, st->err_budget_rel * st->v_norm - st->err_acc);
    const double tol_eff = fmax(st->tol, relax);
    // Learned centre and next dimension: every block evaluates the network on
    // the same inputs, so all agree on the candidate grid.
    double spacing = 0.25;
    int offset = 24;
    if (a.mlp != nullptr) {
        __shared__ double s_col[192];
        net::basis_features(a.H, a.ldh, k, rem, tol_eff, st->v_norm, st->tau_prev, st->err_prev, s_f, s_col, &s_n1);
        net::mlp_forward_block(a.mlp, s_f, s_a1, s_a2, s_o);
        if (threadIdx.x == 0) {
            double c = exp2(static_cast<double>(s_o[0])) / s_n1;
            c = c > st->dt_min ? c : st->dt_min;
            s_center = c < rem ? c : rem;
            // the next basis keeps at least half of this one's columns (the
            // way the step size shrinks by a bounded factor): a network that
            // asks for a much smaller basis near the end of a solve would
            // otherwise trade one cycle for several short ones
            const int m_floor = min((m / 2 + net::M_STEP - 1) / net::M_STEP * net::M_STEP, a.m_cap);
            s_mnext = max(net::next_m_from(s_o[1], a.m_cap), m_floor);
        }
        __syncthreads();
    }
    ExpmBuf B = carve(smem, k);
    {
        // Candidates one octave apart differ by a squaring: exp(2 tau H) =
        // exp(tau H)^2, and as |2 tau H|_1 = 2 |tau H|_1 takes one more
        // halving, both steps reduce to the same scaled matrix whenever
        // |2 tau H|_1 > 1: the squared result is then bit for bit the
        // directly computed one (below that, equal to rounding). So each cluster takes
        // a chain of candidates g0, g0 + P, ... whose steps double, computes
        // the first exponential and squares its way up; a member clamped to
        // the remaining time is computed directly, once (later clamped
        // members are the same step).
        //   network: candidates 0..15 on a 1/8-octave grid around its
        //     prediction (2^-1 .. 2^0.875), chains (c, c+8) for c < 8;
        //     16..31 on the quarter-octave grid the search uses around twice
        //     the previous step (2^-4 .. 2^-0.25 of it), chains (c, c+4,
        //     c+8, c+12) for c = 16..19, so a poor prediction degrades to a
        //     coarser search;
        //   no network: 0..31 on the quarter-octave grid (2^-6 .. 2^1.75 of
        //     the centre), chains (c, .., c+12) for c = 0..3 and 16..19.
        const int chain = static_cast<int>(blockIdx.x) / SEARCH_CLUSTER;
        const bool lead = blockIdx.x % SEARCH_CLUSTER == 0;
        const int nch = a.mlp != nullptr ? SEARCH_CHAINS_NET : SEARCH_CHAINS;
        // chain c: candidates g0, g0 + period, ... (len of them), the first at tau0
        auto chain_of = [&](int c, int* g0, int* period, int* len) {
            if (a.mlp != nullptr && c < 8) {
                *g0 = c;
                *period = 8;
                *len = 2;
            } else if (a.mlp != nullptr) {
                *g0 = SEARCH_CAND / 2 + (c - 8);
                *period = 4;
                *len = 4;
            } else {
                *g0 = c < 4 ? c : SEARCH_CAND / 2 + (c - 4);
                *period = 4;
                *len = 4;
            }
        };
        __shared__ double s_tau0[SEARCH_CHAINS_NET];
        __shared__ int s_grem;
        if (static_cast<int>(threadIdx.x) < nch) {
            int g0, period, len;
            chain_of(threadIdx.x, &g0, &period, &len);
            double t0;
            if (a.mlp != nullptr && static_cast<int>(threadIdx.x) < 8) {
                t0 = s_center * exp2(0.125 * (g0 - 8));
            } else if (a.mlp != nullptr) {
                const double base = st->tau_prev > 0.0 ? 2.0 * st->tau_prev : st->dt;
                t0 = base * exp2(0.25 * (g0 - SEARCH_CAND / 2 - 15));
            } else {
                t0 = s_center * exp2(spacing * (g0 - offset));
            }
            s_tau0[threadIdx.x] = t0;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            // The lowest candidate clamped to the remaining time: the extra
            // cluster evaluates that step once; the other clamped candidates
            // are the same step at a higher index, which the choice below
            // never takes, and are marked as failing.
            int gr = SEARCH_CAND;
            for (int c = 0; c < nch; ++c) {
                int g0, period, len;
                chain_of(c, &g0, &period, &len);
                double t = s_tau0[c];
                for (int i = 0; i < len; ++i, t *= 2.0)
                    if (!(t < rem)) {
                        gr = g0 + i * period < gr ? g0 + i * period : gr;
                        break;
                    }
            }
            s_grem = gr;
        }
        __syncthreads();
        const int g_rem = s_grem;
        const ClusterProducts pr{k};
        auto write_cand = [&](int g, const double* E, double tau) {
            double* c = a.cand + static_cast<size_t>(g) * CAND_STRIDE;
            if (lead)
                for (int r = threadIdx.x; r < k; r += blockDim.x) c[2 + r] = E[r];
            if (lead && threadIdx.x == 0) {
                c[0] = bd ? 0.0 : fabs(a.H[k + (k - 1) * ldh] * E[k - 1]) * st->v_norm;
                c[1] = tau;
            }
            pr.sync();  // the lead has read E before the next product writes into the buffers
        };
        if (chain < nch) {
            int g0, period, len;
            chain_of(chain, &g0, &period, &len);
            double* E = nullptr;
            Band eb{0, 0};
            double t_i = s_tau0[chain];
            for (int i = 0; i < len; ++i, t_i *= 2.0) {
                const int g = g0 + i * period;
                if (!(t_i < rem)) {  // clamped, as every later member
                    if (g != g_rem && lead && threadIdx.x == 0) {
                        double* c = a.cand + static_cast<size_t>(g) * CAND_STRIDE;
                        c[0] = INFINITY;
                        c[1] = rem;
                    }
                    continue;
                }
                if (i == 0) {
                    for (int e = threadIdx.x; e < k * k; e += blockDim.x) B.A[e] = t_i * a.H[(e % k) + (e / k) * ldh];
                    __syncthreads();
                    E = expm_taylor(B, k, pr, &eb);
                } else {
                    double* W = E == B.T ? B.U : B.T;
                    eb = mm_p(pr, k, E, eb, E, eb, W);
                    E = W;
                }
                write_cand(g, E, t_i);
            }
        } else if (g_rem < SEARCH_CAND) {
            // the extra cluster: the remaining time as a step
            for (int e = threadIdx.x; e < k * k; e += blockDim.x) B.A[e] = rem * a.H[(e % k) + (e / k) * ldh];
            __syncthreads();
            Band eb;
            double* E = expm_taylor(B, k, pr, &eb);
            write_cand(g_rem, E, rem);
        }
    }
    if (!grid_last_block(a.counter, &s_flag)) return;
    static_assert(SEARCH_CAND <= 32, "one lane per candidate");
    if (threadIdx.x < 32) {
        // The largest passing step, the lowest index among equal steps (the
        // serial scan's choice), one lane per candidate and a butterfly.
        const int ncand = SEARCH_CAND;
        int g = static_cast<int>(threadIdx.x);
        double tau = -1.0;
        if (g < ncand) {
            const double* c = a.cand + static_cast<size_t>(g) * CAND_STRIDE;
            if (__ldcg(&c[0]) <= tol_eff) tau = __ldcg(&c[1]);
        }
        if (tau < 0.0) g = 32;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const double ot = __shfl_xor_sync(0xffffffffu, tau, o);
            const int og = __shfl_xor_sync(0xffffffffu, g, o);
            if (ot > tau || (ot == tau && og < g)) {
                tau = ot;
                g = og;
            }
        }
        if (threadIdx.x == 0) s_best = g < 32 ? g : -1;
    }
    __syncthreads();
    const double vn = st->v_norm;
    if (s_best >= 0) {
        const double* c = a.cand + static_cast<size_t>(s_best) * CAND_STRIDE;
        for (int i = threadIdx.x; i <= k; i += blockDim.x) {
            const double wi = (i < k) ? __ldcg(&c[2 + i]) : 0.0;
            a.coef[i] = (fabs(wi) > 1e-15 && isfinite(wi)) ? vn * wi : 0.0;
        }
        if (threadIdx.x == 0) {
            const double tau = __ldcg(&c[1]), err = __ldcg(&c[0]);
            write_log(st, a.log, tau, err, k, 0, m);
            // next centre without a network: double the step (the grid reaches 1/64 of it)
            finish_cycle(st, true, tau, err, k, s_mnext, 2.0 * tau, false);
        }
        return;
    }
    // No candidate passed: the reference heuristic below the smallest one.
    if (threadIdx.x == 0) s_tau = __ldcg(&a.cand[1]);
    __syncthreads();
    int rejects = 1;  // the failed candidate round counts as one reject
    double err = 0.0;
    double* R = nullptr;
    while (true) {
        if (threadIdx.x == 0) {
            const double dt_new = (s_tau * st->shrink) * st->safety;
            s_tau = dt_new > st->dt_min ? dt_new : st->dt_min;
        }
        __syncthreads();
        const double dt = s_tau;
        for (int e = threadIdx.x; e < k * k; e += blockDim.x) B.A[e] = dt * a.H[(e % k) + (e / k) * ldh];
        __syncthreads();
        R = expm_taylor_block(B, k);
        if (threadIdx.x == 0) {
            err = bd ? 0.0 : fabs(a.H[k + (k - 1) * ldh] * R[k - 1]) * st->v_norm;
            write_log(st, a.log, dt, err, k, rejects, m);
            if (err <= tol_eff || bd) {
                s_dec = DEC_ACCEPT;
            } else {
                ++rejects;
                s_dec = rejects >= st->max_rejects ? DEC_ABORT : DEC_REJECT;
            }
        }
        __syncthreads();
        if (s_dec != DEC_REJECT) break;
    }
    for (int i = threadIdx.x; i <= k; i += blockDim.x) {
        const double wi = (i < k) ? R[i] : 0.0;
        a.coef[i] = (fabs(wi) > 1e-15 && isfinite(wi)) ? vn * wi : 0.0;
    }
    if (threadIdx.x == 0) finish_cycle(st, s_dec == DEC_ACCEPT, s_tau, err, k, s_mnext, 2.0 * s_tau, false);
}

}  // namespace

int launch_controller_search(const SearchArgs& a, int m, cudaStream_t s) {
    if (m > EXPM_SMEM_K) return MEXK_ERR_UNSUPPORTED;
    cudaLaunchConfig_t cfg = {};
    // the chains and one cluster for the remaining time as a step
    cfg.gridDim = dim3(((a.mlp != nullptr ? SEARCH_CHAINS_NET : SEARCH_CHAINS) + 1) * SEARCH_CLUSTER);
    cfg.blockDim = dim3(EXPM_THREADS);
    cfg.dynamicSmemBytes = expm_smem_bytes(m);
    cfg.stream = s;
    cudaLaunchAttribute attr[2];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = SEARCH_CLUSTER;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    attr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[1].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 2;
    const cudaError_t e = cudaLaunchKernelEx(&cfg, controller_search_kernel, a, m);
    if (e != cudaSuccess) {
        set_cuda_error(e, "controller_search_kernel", __FILE__, __LINE__);
        return MEXK_ERR_CUDA;
    }
    return MEXK_OK;
}

size_t expm_ws_doubles(int k) {
    return 6 * static_cast<size_t>(k) * k + MEXK_M_MAX + (sizeof(int) * MEXK_M_MAX + sizeof(double) - 1) / sizeof(double);
}

int expm_init_attributes() {
    const int bytes = static_cast<int>(expm_smem_bytes(EXPM_SMEM_K));
    MEXK_CK(cudaFuncSetAttribute(expm_standalone_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    MEXK_CK(cudaFuncSetAttribute(controller_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    MEXK_CK(cudaFuncSetAttribute(controller_search_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    return MEXK_OK;
}

int launch_expm_standalone(int k, const double* A, int lda, double* E, int lde, int* status, double* ws,
                           cudaStream_t s) {
    if (k > EXPM_SMEM_K && ws == nullptr) return MEXK_ERR_INVALID;
    const size_t smem = expm_launch_smem(k);
    expm_standalone_kernel<<<1, EXPM_THREADS, smem, s>>>(k, A, lda, E, lde, status, ws);
    MEXK_CK_LAUNCH("expm_standalone_kernel");
    return MEXK_OK;
}

int launch_controller(const ControlArgs& a, int m, cudaStream_t s, int nstates) {
    if (m > EXPM_SMEM_K && (a.ws == nullptr || nstates != 1)) return MEXK_ERR_INVALID;
    const size_t smem = expm_launch_smem(m);
    const cudaError_t e = launch_dependent(controller_kernel, nstates, EXPM_THREADS, smem, s, a, m);
    if (e != cudaSuccess) {
        set_cuda_error(e, "controller_kernel", __FILE__, __LINE__);
        return MEXK_ERR_CUDA;
    }
    return MEXK_OK;
}

}  // namespace mexk

extern "C" int mexk_expm_f64(int k, const double* A, int lda, double* E, int lde, void* stream) {
    if (k < 1 || k > MEXK_M_MAX || !A || !E || lda < k || lde < k) return MEXK_ERR_INVALID;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    int rc0 = mexk::expm_init_attributes();
    if (rc0 != MEXK_OK) return rc0;
    int* d_status = nullptr;
    double* d_ws = nullptr;
    MEXK_CK(cudaMallocAsync(reinterpret_cast<void**>(&d_status), sizeof(int), s));
    if (k > mexk::EXPM_SMEM_K) {
        const cudaError_t e = cudaMallocAsync(reinterpret_cast<void**>(&d_ws), sizeof(double) * mexk::expm_ws_doubles(k), s);
        if (e != cudaSuccess) {
            cudaFreeAsync(d_status, s);
            mexk::set_cuda_error(e, "cudaMallocAsync", __FILE__, __LINE__);
            return MEXK_ERR_ALLOC;
        }
    }
    MEXK_CK(cudaMemsetAsync(d_status, 0, sizeof(int), s));
    int rc = mexk::launch_expm_standalone(k, A, lda, E, lde, d_status, d_ws, s);
    int h_status = 0;
    if (rc == MEXK_OK) {
        cudaError_t e = cudaMemcpyAsync(&h_status, d_status, sizeof(int), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            mexk::set_cuda_error(e, "expm status copy", __FILE__, __LINE__);
            rc = MEXK_ERR_CUDA;
        }
    }
    cudaFreeAsync(d_status, s);
    if (d_ws) cudaFreeAsync(d_ws, s);
    cudaStreamSynchronize(s);
    if (rc == MEXK_OK && (h_status & mexk::ST_LU_SINGULAR)) rc = MEXK_ERR_DEVICE;
    return rc;
}
