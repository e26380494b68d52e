/*
 * Oracle (test infrastructure): dense FP64 Pade scaling-and-squaring
 * exponential. Restates Higham (2005), the method behind the Eigen 3.4.0
 * MatrixExponential that the reference calls at main_cpu.cpp:20-22 and
 * main.cu:33-36. Only tests, the smoke check and the CPU baseline use it.
 */
#include "expm_pade.h"

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

int oracle_pade_coefficients(int m, double* b) {
    if (m != 3 && m != 5 && m != 7 && m != 9 && m != 13) return 0;
    for (int j = 0; j <= m; ++j) {
        /* b_j = (2m-j)! / (j! (m-j)!) = prod_{i=m-j+1}^{2m-j} i / j!  (exact) */
        uint64_t num = 1;
        for (int i = m - j + 1; i <= 2 * m - j; ++i) num *= (uint64_t)i;
        uint64_t den = 1;
        for (int i = 2; i <= j; ++i) den *= (uint64_t)i;
        b[j] = (double)(num / den);
    }
    return m + 1;
}

/* C = A * B, all k-by-k column-major. */
static void matmul(int k, const double* A, const double* B, double* C) {
    for (int j = 0; j < k; ++j) {
        for (int i = 0; i < k; ++i) {
            double s = 0.0;
            for (int l = 0; l < k; ++l) s += A[i + (size_t)l * k] * B[l + (size_t)j * k];
            C[i + (size_t)j * k] = s;
        }
    }
}

/* Dst = sum_t coef[t] * Mat[t] (left to right) + c_id * I. */
static void lincomb(int k, int terms, const double* coef, const double* const* mats,
                    double c_id, double* dst) {
    for (int j = 0; j < k; ++j) {
        for (int i = 0; i < k; ++i) {
            size_t p = i + (size_t)j * k;
            double s = coef[0] * mats[0][p];
            for (int t = 1; t < terms; ++t) s = s + coef[t] * mats[t][p];
            if (c_id != 0.0 && i == j) s = s + c_id;
            dst[p] = s;
        }
    }
}

/* Solve (LU with row pivots piv) X = B in place on B (k columns). */
static void lu_solve(int k, const double* LU, const int* piv, double* B) {
    for (int c = 0; c < k; ++c) {
        double* x = B + (size_t)c * k;
        for (int i = 0; i < k; ++i) {
            int p = piv[i];
            if (p != i) { double t = x[i]; x[i] = x[p]; x[p] = t; }
        }
        for (int i = 0; i < k; ++i) {
            double s = x[i];
            for (int l = 0; l < i; ++l) s -= LU[i + (size_t)l * k] * x[l];
            x[i] = s;
        }
        for (int i = k - 1; i >= 0; --i) {
            double s = x[i];
            for (int l = i + 1; l < k; ++l) s -= LU[i + (size_t)l * k] * x[l];
            x[i] = s / LU[i + (size_t)i * k];
        }
    }
}

/* In-place LU with partial pivoting (first maximum wins). Returns 0, or 1 if
 * an exactly zero pivot column was met (that column is left unscaled). */
static int lu_factor(int k, double* A, int* piv) {
    int singular = 0;
    for (int c = 0; c < k; ++c) {
        int p = c;
        double best = fabs(A[c + (size_t)c * k]);
        for (int i = c + 1; i < k; ++i) {
            double a = fabs(A[i + (size_t)c * k]);
            if (a > best) { best = a; p = i; }
        }
        piv[c] = p;
        if (p != c) {
            for (int j = 0; j < k; ++j) {
                double t = A[c + (size_t)j * k];
                A[c + (size_t)j * k] = A[p + (size_t)j * k];
                A[p + (size_t)j * k] = t;
            }
        }
        double d = A[c + (size_t)c * k];
        if (d == 0.0) { singular = 1; continue; }
        for (int i = c + 1; i < k; ++i) A[i + (size_t)c * k] /= d;
        for (int j = c + 1; j < k; ++j) {
            double u = A[c + (size_t)j * k];
            for (int i = c + 1; i < k; ++i) A[i + (size_t)j * k] -= A[i + (size_t)c * k] * u;
        }
    }
    return singular;
}

int oracle_expm(int k, const double* A_in, double* E) {
    if (k <= 0) return -1;
    size_t kk = (size_t)k * k;
    double* buf = (double*)malloc(sizeof(double) * kk * 8);
    int* piv = (int*)malloc(sizeof(int) * (size_t)k);
    if (!buf || !piv) { free(buf); free(piv); return -1; }
    double* A = buf;
    double* A2 = buf + kk;
    double* A4 = buf + 2 * kk;
    double* A6 = buf + 3 * kk;
    double* A8 = buf + 4 * kk;
    double* U = buf + 5 * kk;
    double* V = buf + 6 * kk;
    double* T = buf + 7 * kk;

    double l1 = 0.0;
    for (int j = 0; j < k; ++j) {
        double s = 0.0;
        for (int i = 0; i < k; ++i) s += fabs(A_in[i + (size_t)j * k]);
        if (s > l1) l1 = s;
    }
    int squarings = 0;
    int degree;
    if (l1 < 1.495585217958292e-002) degree = 3;
    else if (l1 < 2.539398330063230e-001) degree = 5;
    else if (l1 < 9.504178996162932e-001) degree = 7;
    else if (l1 < 2.097847961257068e+000) degree = 9;
    else {
        degree = 13;
        const double maxnorm = 5.371920351148152;
        (void)frexp(l1 / maxnorm, &squarings);
        if (squarings < 0) squarings = 0;
    }
    for (size_t p = 0; p < kk; ++p) A[p] = ldexp(A_in[p], -squarings);

    double b[14];
    oracle_pade_coefficients(degree, b);
    matmul(k, A, A, A2);
    if (degree >= 5) matmul(k, A2, A2, A4);
    if (degree >= 7) matmul(k, A4, A2, A6);
    if (degree == 3) {
        const double cu[1] = {b[3]};
        const double* mu[1] = {A2};
        lincomb(k, 1, cu, mu, b[1], T);
        matmul(k, A, T, U);
        const double cv[1] = {b[2]};
        lincomb(k, 1, cv, mu, b[0], V);
    } else if (degree == 5) {
        const double cu[2] = {b[5], b[3]};
        const double* mu[2] = {A4, A2};
        lincomb(k, 2, cu, mu, b[1], T);
        matmul(k, A, T, U);
        const double cv[2] = {b[4], b[2]};
        lincomb(k, 2, cv, mu, b[0], V);
    } else if (degree == 7) {
        const double cu[3] = {b[7], b[5], b[3]};
        const double* mu[3] = {A6, A4, A2};
        lincomb(k, 3, cu, mu, b[1], T);
        matmul(k, A, T, U);
        const double cv[3] = {b[6], b[4], b[2]};
        lincomb(k, 3, cv, mu, b[0], V);
    } else if (degree == 9) {
        matmul(k, A6, A2, A8);
        const double cu[4] = {b[9], b[7], b[5], b[3]};
        const double* mu[4] = {A8, A6, A4, A2};
        lincomb(k, 4, cu, mu, b[1], T);
        matmul(k, A, T, U);
        const double cv[4] = {b[8], b[6], b[4], b[2]};
        lincomb(k, 4, cv, mu, b[0], V);
    } else {
        /* U = A [A6 (b13 A6 + b11 A4 + b9 A2) + b7 A6 + b5 A4 + b3 A2 + b1 I]
         * V =    A6 (b12 A6 + b10 A4 + b8 A2) + b6 A6 + b4 A4 + b2 A2 + b0 I */
        const double* mu[3] = {A6, A4, A2};
        const double c1[3] = {b[13], b[11], b[9]};
        lincomb(k, 3, c1, mu, 0.0, V);
        matmul(k, A6, V, T);
        const double c2[3] = {b[7], b[5], b[3]};
        lincomb(k, 3, c2, mu, b[1], A8);
        for (size_t p = 0; p < kk; ++p) T[p] = T[p] + A8[p];
        matmul(k, A, T, U);
        const double c3[3] = {b[12], b[10], b[8]};
        lincomb(k, 3, c3, mu, 0.0, T);
        matmul(k, A6, T, V);
        const double c4[3] = {b[6], b[4], b[2]};
        lincomb(k, 3, c4, mu, b[0], A8);
        for (size_t p = 0; p < kk; ++p) V[p] = V[p] + A8[p];
    }
    /* numer = U + V (into E), denom = -U + V (into T) */
    for (size_t p = 0; p < kk; ++p) {
        E[p] = U[p] + V[p];
        T[p] = -U[p] + V[p];
    }
    int singular = lu_factor(k, T, piv);
    lu_solve(k, T, piv, E);
    for (int s = 0; s < squarings; ++s) {
        memcpy(A2, E, sizeof(double) * kk);
        matmul(k, A2, A2, E);
    }
    free(buf);
    free(piv);
    return singular ? -1 : squarings;
}
