/*
 * Dense FP64 matrix exponential for the oracle (test infrastructure only).
 *
 * The reference computes exp(dt*H_k) with Eigen 3.4.0's MatrixFunctions
 * module (main_cpu.cpp:20-22, main.cu:33-36; Eigen is a third-party
 * dependency pinned by build.bash:8 and absent from the reference tree).
 * This file restates the published method that module implements:
 * N. J. Higham, "The scaling and squaring method for the matrix exponential
 * revisited", SIAM J. Matrix Anal. Appl. 26(4):1179-1193, 2005 -- Pade
 * degree 3/5/7/9/13 chosen from the 1-norm with the theta_m bounds of that
 * paper, scaling by 2^-s before the degree-13 approximant, an LU solve with
 * partial pivoting for (V-U)^{-1}(V+U), then s squarings.
 */
#ifndef MEXK_ORACLE_EXPM_PADE_H
#define MEXK_ORACLE_EXPM_PADE_H

#ifdef __cplusplus
extern "C" {
#endif

/* E = exp(A); A and E are k-by-k, column-major, leading dimension k.
 * A and E may not alias. Returns the number of squarings applied, or -1 if
 * k <= 0 or the LU factor is exactly singular. */
int oracle_expm(int k, const double* A, double* E);

/* Integer Pade [m/m] numerator coefficients b_0..b_m for m in {3,5,7,9,13},
 * b_j = (2m-j)! m! / (j! (m-j)!) scaled so that b_m = 1 (exact integers,
 * converted to the nearest double). Returns m+1 or 0 for an unsupported m. */
int oracle_pade_coefficients(int m, double* b);

#ifdef __cplusplus
}
#endif

#endif
