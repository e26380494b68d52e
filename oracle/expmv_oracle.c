/*
 * ORACLE -- test infrastructure, not product code. See expmv_oracle.h.
 * Every function restates the reference's CPU twin ArnoldiRunnerCPU in
 * main_cpu.cpp, with the same loop orders, so that (built without FP
 * contraction) it reproduces that program's arithmetic.
 */
#include "expmv_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "expm_pade.h"

/* main_cpu.cpp:388-397 */
void oracle_spmv(int n, const int* row_ptr, const int* col_idx, const double* values,
                 const double* x, double* y) {
    for (int r = 0; r < n; ++r) {
        double acc = 0.0;
        for (int k = row_ptr[r]; k < row_ptr[r + 1]; ++k) acc += values[k] * x[col_idx[k]];
        y[r] = acc;
    }
}

/* main_cpu.cpp:493-520 (orthogonalize_mgs) on column j, writing h[0..j]. */
static void mgs2(int n, const double* V, int j, int reortho, double* w, double* h) {
    for (int i = 0; i <= j; ++i) {
        const double* qi = V + (size_t)i * n;
        double hij = 0.0;
        for (int k = 0; k < n; ++k) hij += w[k] * qi[k];
        h[i] = hij;
        for (int k = 0; k < n; ++k) w[k] -= hij * qi[k];
    }
    if (reortho) {
        for (int i = 0; i <= j; ++i) {
            const double* qi = V + (size_t)i * n;
            double corr = 0.0;
            for (int k = 0; k < n; ++k) corr += w[k] * qi[k];
            h[i] += corr;
            for (int k = 0; k < n; ++k) w[k] -= corr * qi[k];
        }
    }
}

/* main_cpu.cpp:522-546 (normalize_new_vector). */
static int normalize(int n, double* V, int j, const double* w, double* beta) {
    double norm_sq = 0.0;
    for (int i = 0; i < n; ++i) norm_sq += w[i] * w[i];
    double g = sqrt(norm_sq);
    *beta = g;
    if (g < 1e-14 || isnan(g) || isinf(g)) return 0;
    double scale = 1.0 / g;
    double* q = V + (size_t)(j + 1) * n;
    for (int i = 0; i < n; ++i) q[i] = w[i] * scale;
    return 1;
}

int oracle_arnoldi_step(int n, const int* row_ptr, const int* col_idx, const double* values,
                        double* V, int j, int reortho, double* w, double* h, double* beta) {
    memset(w, 0, sizeof(double) * (size_t)n);
    oracle_spmv(n, row_ptr, col_idx, values, V + (size_t)j * n, w);
    mgs2(n, V, j, reortho, w, h);
    return normalize(n, V, j, w, beta);
}

int oracle_small_expm(int k, const double* H, int ldh, double dt, double v_norm, double* wH,
                      double* err) {
    if (k <= 0) {
        *err = 0.0;
        return 0;
    }
    size_t kk = (size_t)k * k;
    double* S = (double*)malloc(sizeof(double) * kk);
    double* E = (double*)malloc(sizeof(double) * kk);
    if (!S || !E) {
        free(S);
        free(E);
        return -1;
    }
    /* segment_t * H_m.block(0,0,k,k) (main_cpu.cpp:554-555) */
    for (int c = 0; c < k; ++c)
        for (int r = 0; r < k; ++r) S[r + (size_t)c * k] = dt * H[r + (size_t)c * ldh];
    oracle_expm(k, S, E);
    for (int i = 0; i < k; ++i) wH[i] = E[i];
    wH[k] = 0.0;
    /* main_cpu.cpp:574-587 */
    double e_k = E[k - 1];
    double h_k1 = H[k + (size_t)(k - 1) * ldh];
    *err = fabs(h_k1 * e_k) * v_norm;
    free(S);
    free(E);
    return 0;
}

/* main_cpu.cpp:560-571 */
void oracle_lift(int n, int k, const double* V, const double* wH, double v_norm, double* y) {
    memset(y, 0, sizeof(double) * (size_t)n);
    for (int i = 0; i <= k; ++i) {
        if (fabs(wH[i]) > 1e-15) {
            const double alpha = v_norm * wH[i];
            const double* Vi = V + (size_t)i * n;
            for (int r = 0; r < n; ++r) y[r] += alpha * Vi[r];
        }
    }
}

/* norm, then V[:,0] = x * (1/norm) (or x if norm <= 1e-14); main_cpu.cpp:469-481, 589-600 */
static double set_start_vector(int n, const double* x, double* V) {
    double norm_sq = 0.0;
    for (int i = 0; i < n; ++i) norm_sq += x[i] * x[i];
    double nrm = sqrt(norm_sq);
    double scale = (nrm > 1e-14) ? (1.0 / nrm) : 1.0;
    for (int i = 0; i < n; ++i) V[i] = x[i] * scale;
    return nrm;
}

int oracle_expmv(int n, const int* row_ptr, const int* col_idx, const double* values,
                 const double* v, double* y_out, const oracle_params* p, oracle_stats* stats,
                 oracle_step* log, int log_cap, int* log_len) {
    if (n <= 0 || !p || p->m <= 0) return -1;
    const int m_base = p->m;
    /* ArnoldiRunnerCPU constructor, main_cpu.cpp:453-466, or the caller's
     * TimeSteppingParams as compute_expmv reads them (main_cpu.cpp:608-676) */
    oracle_stepping ts;
    if (p->stepping) {
        ts = *p->stepping;
    } else {
        ts.dt_max = p->t;
        ts.dt_min = (1e-12 > p->t * 1e-6) ? 1e-12 : p->t * 1e-6;
        const double denom = (p->max_restarts > 0) ? p->max_restarts : 1;
        ts.dt_init = p->t / denom;
        ts.tol_step = p->tol;
        ts.max_steps = (p->max_restarts > 0) ? p->max_restarts : 1000;
        ts.max_rejects = 20;
        ts.safety = 0.8;
        ts.grow = 1.5;
        ts.shrink = 0.5;
        ts.adapt_m = 0;
        ts.m_max = p->m;
        ts.m_step = 0;
    }
    const double dt_max = ts.dt_max, dt_min = ts.dt_min, dt_init = ts.dt_init, tol_step = ts.tol_step;
    const int max_steps = ts.max_steps, max_rejects = ts.max_rejects;
    const double safety = ts.safety, grow = ts.grow, shrink = ts.shrink;
    /* storage for the largest basis adapt_m may build (the GPU runner
     * allocates max(m, m_max), main.cu:1343) */
    const int m = (ts.adapt_m && ts.m_max > m_base) ? ts.m_max : m_base;

    size_t ldh = (size_t)m + 1;
    double* V = (double*)calloc((size_t)n * (size_t)(m + 1), sizeof(double));
    double* w = (double*)calloc((size_t)n, sizeof(double));
    double* y = (double*)calloc((size_t)n, sizeof(double));
    double* H = (double*)calloc(ldh * (size_t)m, sizeof(double));
    double* wH = (double*)calloc((size_t)m + 2, sizeof(double));
    double* hcol = (double*)calloc((size_t)m + 1, sizeof(double));
    if (!V || !w || !y || !H || !wH || !hcol) {
        free(V); free(w); free(y); free(H); free(wH); free(hcol);
        return -1;
    }
    oracle_stats st;
    memset(&st, 0, sizeof(st));
    int nlog = 0;

    double v_norm = set_start_vector(n, v, V); /* init_q1 */
    st.v_norm_initial = v_norm;

    const double total_t = p->t;
    double dt = dt_init > dt_min ? dt_init : dt_min;
    dt = dt < dt_max ? dt : dt_max;
    double t_done = 0.0;
    int accepted = 0;
    int converged = 0;
    double last_residual = 0.0;
    int stop = 0;

    while (t_done < total_t && accepted < max_steps && !stop) {
        dt = (dt < total_t - t_done) ? dt : (total_t - t_done);
        int rejects = 0;
        int m_current = m_base;
        while (1) {
            if (p->max_cycles > 0 && st.cycles >= p->max_cycles) { stop = 1; break; }
            memset(H, 0, sizeof(double) * ldh * (size_t)m);
            int k_used = 0;
            int breakdown = 0;
            for (int j = 0; j < m_current; ++j) {
                double beta = 0.0;
                int ok = oracle_arnoldi_step(n, row_ptr, col_idx, values, V, j, p->reorthogonalize,
                                             w, hcol, &beta);
                ++st.spmv_count;
                for (int i = 0; i <= j; ++i) H[i + (size_t)j * ldh] = hcol[i];
                H[(j + 1) + (size_t)j * ldh] = ok ? beta : 0.0;
                k_used = j + 1;
                if (!ok) { breakdown = 1; break; }
            }
            ++st.cycles;
            double err = 0.0;
            oracle_small_expm(k_used, H, (int)ldh, dt, v_norm, wH, &err);
            oracle_lift(n, k_used, V, wH, v_norm, y);
            if (breakdown) err = 0.0;
            ++st.attempts;
            if (!p->quiet)
                printf("[STEP] t=%g dt=%g err=%g m_used=%d accepts=%d rejects=%d\n", t_done, dt, err,
                       k_used, accepted, rejects);
            if (log && nlog < log_cap) {
                oracle_step* s = &log[nlog];
                s->t_done = t_done; s->dt = dt; s->err = err;
                s->m_used = k_used; s->accepts = accepted; s->rejects = rejects;
            }
            ++nlog;
            if (err <= tol_step || breakdown) {
                t_done += dt;
                accepted++;
                last_residual = err;
                if (t_done >= total_t) { converged = 1; break; }
                v_norm = set_start_vector(n, y, V); /* restart_from_y */
                if (err < 0.1 * tol_step) {
                    double dt_new = dt * grow * safety;
                    dt = dt_new < dt_max ? dt_new : dt_max;
                }
                break;
            } else {
                rejects++;
                if (rejects >= max_rejects) {
                    if (!p->quiet) fprintf(stderr, "[STEP] rejected too many times, aborting\n");
                    converged = 0;
                    last_residual = err;
                    t_done = total_t;
                    break;
                }
                if (ts.adapt_m && (m_current + ts.m_step) <= ts.m_max && ts.m_step > 0) {
                    m_current += ts.m_step;
                } else {
                    double dt_new = dt * shrink * safety;
                    dt = dt_new > dt_min ? dt_new : dt_min;
                    m_current = m_base;
                }
                continue;
            }
        }
    }
    for (int i = 0; i < n; ++i) y_out[i] = y[i];
    st.converged = converged;
    st.restarts_done = accepted;
    st.last_residual = last_residual;
    if (stats) *stats = st;
    if (log_len) *log_len = nlog < log_cap ? nlog : log_cap;
    free(V); free(w); free(y); free(H); free(wH); free(hcol);
    return 0;
}
