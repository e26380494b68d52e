// ORACLE -- test infrastructure, not product code.
//
// Compiles the reference's own CPU program (main_cpu.cpp, taken from the
// reference tree through the include path, never copied) against the
// project's Eigen-subset shim and exposes its ArnoldiRunnerCPU and CSRHost
// through a C ABI, so tests can pin the oracle restatement against the
// reference's actual code and generate golden vectors. The program's own
// main() is renamed and left unused.
#define main mexk_reference_cpu_main
#include "main_cpu.cpp"
#undef main

#include <algorithm>
#include <cstdio>

extern "C" {

// ArnoldiRunnerCPU::compute_expmv on caller-provided CSR (main_cpu.cpp:602).
int ref_expmv(int n, long long nnz, const int* row_ptr, const int* col_idx, const double* values,
              const double* v, double* y, int m, double t, double tol, int max_restarts,
              int reortho, int* restarts_done, int* converged, double* last_residual) {
    CSRHost A;
    A.rows = n;
    A.cols = n;
    A.nnz = nnz;
    A.row_ptr.assign(row_ptr, row_ptr + n + 1);
    A.col_idx.assign(col_idx, col_idx + nnz);
    A.values.assign(values, values + nnz);
    ArnoldiParams params(m, t, tol, max_restarts, reortho != 0);
    ArnoldiRunnerCPU runner(A, params);
    std::vector<double> vh(v, v + n);
    std::vector<double> yh(static_cast<size_t>(n), 0.0);
    runner.compute_expmv(vh, yh);
    std::fflush(stdout);
    for (int i = 0; i < n; ++i) y[i] = yh[i];
    *restarts_done = runner.restarts_done;
    *converged = runner.converged ? 1 : 0;
    *last_residual = runner.last_residual;
    return 0;
}

// The same with caller-set TimeSteppingParams (main_cpu.cpp:417-430), which
// compute_expmv reads (main_cpu.cpp:608-676). The basis storage is sized for
// max(m, m_max), as the GPU runner allocates it (main.cu:1343), so that
// adapt_m may grow the basis up to m_max.
int ref_expmv_ts(int n, long long nnz, const int* row_ptr, const int* col_idx, const double* values,
                 const double* v, double* y, int m, double t, double tol, int max_restarts, int reortho,
                 const double* ts_d, const int* ts_i, int* restarts_done, int* converged, double* last_residual) {
    CSRHost A;
    A.rows = n;
    A.cols = n;
    A.nnz = nnz;
    A.row_ptr.assign(row_ptr, row_ptr + n + 1);
    A.col_idx.assign(col_idx, col_idx + nnz);
    A.values.assign(values, values + nnz);
    ArnoldiParams params(m, t, tol, max_restarts, reortho != 0);
    ArnoldiRunnerCPU runner(A, params);
    // ts_d: dt_init, dt_min, dt_max, tol_step, safety, grow, shrink;
    // ts_i: max_steps, max_rejects, adapt_m, m_max, m_step
    runner.ts_params.dt_init = ts_d[0];
    runner.ts_params.dt_min = ts_d[1];
    runner.ts_params.dt_max = ts_d[2];
    runner.ts_params.tol_step = ts_d[3];
    runner.ts_params.safety = ts_d[4];
    runner.ts_params.grow = ts_d[5];
    runner.ts_params.shrink = ts_d[6];
    runner.ts_params.max_steps = ts_i[0];
    runner.ts_params.max_rejects = ts_i[1];
    runner.ts_params.adapt_m = ts_i[2] != 0;
    runner.ts_params.m_max = ts_i[3];
    runner.ts_params.m_step = ts_i[4];
    const int alloc_m = std::max(m, ts_i[3] > 0 ? ts_i[3] : m);
    runner.allocated_m_max = alloc_m;
    runner.V_m.assign(static_cast<size_t>(n) * (alloc_m + 1), 0.0);
    std::vector<double> vh(v, v + n);
    std::vector<double> yh(static_cast<size_t>(n), 0.0);
    runner.compute_expmv(vh, yh);
    std::fflush(stdout);
    for (int i = 0; i < n; ++i) y[i] = yh[i];
    *restarts_done = runner.restarts_done;
    *converged = runner.converged ? 1 : 0;
    *last_residual = runner.last_residual;
    return 0;
}

// CSRHost::from_binary_csr / from_matrix_market (main_cpu.cpp:56, 198).
// Returns a heap CSRHost; these exit the process on malformed input, as the
// reference does.
void* ref_load(const char* path, int binary, int* rows, int* cols, long long* nnz) {
    CSRHost* A = new CSRHost();
    if (binary) A->from_binary_csr(path);
    else A->from_matrix_market(path);
    *rows = A->rows;
    *cols = A->cols;
    *nnz = A->nnz;
    return A;
}

void ref_copy_csr(void* h, int* row_ptr, int* col_idx, double* values) {
    CSRHost* A = static_cast<CSRHost*>(h);
    std::copy(A->row_ptr.begin(), A->row_ptr.end(), row_ptr);
    std::copy(A->col_idx.begin(), A->col_idx.end(), col_idx);
    std::copy(A->values.begin(), A->values.end(), values);
}

void ref_free(void* h) { delete static_cast<CSRHost*>(h); }

}  // extern "C"
