/*
 * ORACLE -- test infrastructure, not product code.
 *
 * A plain-C, single-threaded restatement of the reference's CPU solver
 * ArnoldiRunnerCPU (main_cpu.cpp:388-700): CSR SpMV, modified Gram-Schmidt
 * with a second (re-orthogonalisation) pass, normalisation with the
 * breakdown test, the k-by-k Pade exponential, the lift y = |v| V_k w_H,
 * the residual estimate and the adaptive time-step controller. It is the
 * checker for the CUDA path and the CPU baseline of the benchmark; only
 * tests, the smoke check and the benchmark's CPU leg may call it.
 */
#ifndef MEXK_ORACLE_EXPMV_H
#define MEXK_ORACLE_EXPMV_H

#ifdef __cplusplus
extern "C" {
#endif

/* TimeSteppingParams (main_cpu.cpp:417-430) as a caller may set them. */
typedef struct {
    double dt_init, dt_min, dt_max, tol_step;
    int max_steps, max_rejects;
    double safety, grow, shrink;
    int adapt_m, m_max, m_step;
} oracle_stepping;

typedef struct {
    int m;               /* Krylov dimension (ArnoldiParams::m) */
    double t;            /* total time (ArnoldiParams::t) */
    double tol;          /* per-step tolerance (ArnoldiParams::tol) */
    int max_restarts;    /* <= 0: run until convergence (max_steps = 1000) */
    int reorthogonalize; /* 1: second Gram-Schmidt pass (CLI always sets it) */
    int max_cycles;      /* 0: unlimited. >0: stop after this many Arnoldi
                            basis builds (bounded timing samples only) */
    int quiet;           /* 0: print the reference's [STEP] lines to stdout */
    const oracle_stepping* stepping; /* NULL: derived from m, t, tol, max_restarts
                            as the constructor does (main_cpu.cpp:453-466) */
} oracle_params;

typedef struct {
    int converged;
    int restarts_done;     /* accepted steps (main_cpu.cpp:664) */
    double last_residual;
    int attempts;          /* accepted + rejected attempts */
    int cycles;            /* Arnoldi basis builds performed */
    long long spmv_count;
    double v_norm_initial;
} oracle_stats;

typedef struct {
    double t_done, dt, err;
    int m_used, accepts, rejects;
} oracle_step;

/* y = exp(t A) v following main_cpu.cpp:602-700. A is n-by-n CSR with int32
 * indices and FP64 values. log (may be NULL) receives up to log_cap attempt
 * records, *log_len (may be NULL) the number written. Returns 0, or -1 on
 * bad arguments / allocation failure. */
int oracle_expmv(int n, const int* row_ptr, const int* col_idx, const double* values,
                 const double* v, double* y, const oracle_params* p, oracle_stats* stats,
                 oracle_step* log, int log_cap, int* log_len);

/* y = A x, one row at a time (main_cpu.cpp:388-397). */
void oracle_spmv(int n, const int* row_ptr, const int* col_idx, const double* values,
                 const double* x, double* y);

/* One Arnoldi step j on a column-major basis V (ld = n, columns 0..j valid):
 * w = A V[:,j]; two MGS passes write h[0..j] (= H(0..j, j)); beta = |w|;
 * on success V[:,j+1] = w / beta. Returns 1 on success, 0 on breakdown
 * (beta < 1e-14, NaN or Inf). w is scratch of length n. */
int oracle_arnoldi_step(int n, const int* row_ptr, const int* col_idx, const double* values,
                        double* V, int j, int reorthogonalize, double* w, double* h,
                        double* beta);

/* w_H = first column of exp(dt H_k) (H is (ldh)-by-k column-major, the
 * leading k-by-k block is used) and the residual estimate
 * |H(k,k-1) * w_H[k-1]| * v_norm (main_cpu.cpp:548-587). */
int oracle_small_expm(int k, const double* H, int ldh, double dt, double v_norm, double* wH,
                      double* err);

/* y = sum_{i<=k} (v_norm * wH[i]) V[:,i], skipping |wH[i]| <= 1e-15, with
 * wH[k] = 0 (main_cpu.cpp:562-571). */
void oracle_lift(int n, int k, const double* V, const double* wH, double v_norm, double* y);

#ifdef __cplusplus
}
#endif

#endif
