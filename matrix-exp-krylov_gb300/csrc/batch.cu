// Host side of the batched solver: upload, row-space layout, waves, the
// schedule autotuner, one captured graph per wave, results.
//
// HBM layout (whole batch, resident after upload):
//   row_ptr int64[rows+1] (global nonzero offsets), col int32[nnz] (columns
//   local to the problem), val f32[nnz], V and Y f64[rows][16] (start
//   vectors, results), per-problem first row, per-chunk problem, per-state
//   DevState / H / Gram matrix / scales / coefficients.
// Per wave (sized for the largest): U f32[(m+1)][wave rows][16], W f32
// [wave rows][16], tile table and tile partials.
#include "batch.cuh"

#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <string>
#include <vector>

using namespace mexk;
using namespace mexk::batch;

namespace {

struct HostProblem {
    int rows;
    long long nnz;
    const int* row_ptr;
    const int* col;
    const double* val;
    double t;
    int nrhs;
    const double* V;
};

struct Wave {
    int p0 = 0, p1 = 0;      // problems [p0, p1)
    long long R0 = 0, R1 = 0; // global rows
    int C0 = 0, C1 = 0;      // 64-row chunks
    int t0 = 0, T = 0;       // tiles in the global tile table
    cudaGraphExec_t exec = nullptr;
};

template <typename T>
int dalloc(T** p, size_t count) {
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), sizeof(T) * count);
    if (e != cudaSuccess) {
        set_cuda_error(e, "cudaMalloc (batch)", __FILE__, __LINE__);
        return MEXK_ERR_ALLOC;
    }
    return MEXK_OK;
}
template <typename T>
void dfree(T*& p) {
    if (p) cudaFree(p);
    p = nullptr;
}

constexpr int TILE_CANDIDATES[] = {1024, 4096, 16384};
constexpr int DEFAULT_TILE_ROWS = 4096;

}  // namespace

struct mexk_batch_s {
    int device = 0;
    mexk_batch_params_t prm{};
    std::vector<HostProblem> probs;
    cudaStream_t stream = nullptr;
    bool uploaded = false;
    long long rows = 0, nnz = 0;
    int nchunks = 0;
    std::vector<long long> prow0;  // P + 1
    long long* d_row_ptr = nullptr;
    int* d_col = nullptr;
    float* d_val = nullptr;
    long long* d_prow0 = nullptr;
    int* d_chunk_prob = nullptr;
    double* d_V = nullptr;  // start vectors [rows][16]
    double* d_Y = nullptr;  // results [rows][16]
    DevState* d_st = nullptr;
    double* d_H = nullptr;
    double* d_G = nullptr;
    double* d_s = nullptr;
    double* d_pre = nullptr;
    double* d_coefl = nullptr;
    float* d_coef = nullptr;
    float* d_wsc = nullptr;
    float* d_psc = nullptr;
    unsigned int* d_pcount = nullptr;
    int* d_pdone = nullptr;
    int* d_active = nullptr;
    int* h_active = nullptr;
    float* d_U = nullptr;
    float* d_W = nullptr;
    long long wave_rows_cap = 0;
    double* d_part = nullptr;
    int tiles_cap = 0;  // per wave
    int* d_tile_prob = nullptr;
    long long* d_tile_row0 = nullptr;
    int* d_tile_nrows = nullptr;
    int* d_ptile0 = nullptr;
    int* d_ptiles = nullptr;
    int tiles_total_cap = 0;
    std::vector<Wave> waves;
    std::vector<DevState> h_init;  // initial states
    int tile_rows = DEFAULT_TILE_ROWS, gg = 4, unroll = 4;
    bool tuned = false;
    double tune_ms = 0.0;
    int cycles = 0;
    std::vector<DevState> h_final;
    bool have_final = false;
};

namespace {

int P_of(mexk_batch_t b) { return static_cast<int>(b->probs.size()); }

// Tile table of every wave for tile_rows; fills the device arrays.
int build_tiles(mexk_batch_t b, int tile_rows) {
    std::vector<int> tprob, tnr, pt0(P_of(b)), ptn(P_of(b));
    std::vector<long long> trow0;
    for (auto& w : b->waves) {
        w.t0 = static_cast<int>(tprob.size());
        for (int p = w.p0; p < w.p1; ++p) {
            pt0[p] = static_cast<int>(tprob.size()) - w.t0;
            const long long r0 = b->prow0[p];
            const long long rp = b->prow0[p + 1] - r0;
            int cnt = 0;
            for (long long r = 0; r < rp; r += tile_rows) {
                tprob.push_back(p);
                trow0.push_back(r0 + r);
                tnr.push_back(static_cast<int>(std::min<long long>(tile_rows, rp - r)));
                ++cnt;
            }
            ptn[p] = cnt;
        }
        w.T = static_cast<int>(tprob.size()) - w.t0;
    }
    if (static_cast<int>(tprob.size()) > b->tiles_total_cap) return MEXK_ERR_DEVICE;
    for (auto& w : b->waves)
        if (w.T > b->tiles_cap) return MEXK_ERR_DEVICE;
    MEXK_CK(cudaMemcpy(b->d_tile_prob, tprob.data(), sizeof(int) * tprob.size(), cudaMemcpyHostToDevice));
    MEXK_CK(cudaMemcpy(b->d_tile_row0, trow0.data(), sizeof(long long) * trow0.size(), cudaMemcpyHostToDevice));
    MEXK_CK(cudaMemcpy(b->d_tile_nrows, tnr.data(), sizeof(int) * tnr.size(), cudaMemcpyHostToDevice));
    MEXK_CK(cudaMemcpy(b->d_ptile0, pt0.data(), sizeof(int) * pt0.size(), cudaMemcpyHostToDevice));
    MEXK_CK(cudaMemcpy(b->d_ptiles, ptn.data(), sizeof(int) * ptn.size(), cudaMemcpyHostToDevice));
    b->tile_rows = tile_rows;
    return MEXK_OK;
}

Layout layout(mexk_batch_t b, const Wave& w) {
    Layout L;
    L.P = w.p1 - w.p0;
    L.T = w.T;
    L.C0 = w.C0;
    L.C1 = w.C1;
    L.R0 = w.R0;
    L.tile_prob = b->d_tile_prob + w.t0;
    L.tile_row0 = b->d_tile_row0 + w.t0;
    L.tile_nrows = b->d_tile_nrows + w.t0;
    L.ptile0 = b->d_ptile0;
    L.ptiles = b->d_ptiles;
    L.chunk_prob = b->d_chunk_prob;
    L.prow0 = b->d_prow0;
    L.row_ptr = b->d_row_ptr;
    L.col = b->d_col;
    L.val = b->d_val;
    L.U = b->d_U;
    L.ldu = static_cast<size_t>(w.R1 - w.R0) * BR;
    L.W = b->d_W;
    L.V0 = b->d_V;
    L.Y = b->d_Y;
    L.st = b->d_st;
    L.H = b->d_H;
    L.G = b->d_G;
    L.s = b->d_s;
    L.pre = b->d_pre;
    L.coef = b->d_coef;
    L.wsc = b->d_wsc;
    L.psc = b->d_psc;
    L.coefl = b->d_coefl;
    L.part = b->d_part;
    L.pcount = b->d_pcount;
    L.pdone = b->d_pdone;
    L.active = b->d_active;
    return L;
}

// The wave's cycle loop runs on the device: a conditional while node whose
// body is one cycle followed by wave_loop_next. active[0] = states still
// stepping (the status kernel's count), active[1] = cycles run.
__global__ void wave_loop_start(cudaGraphConditionalHandle h, int* active) {
    active[1] = 0;
    cudaGraphSetConditional(h, active[0] > 0 ? 1u : 0u);
}
__global__ void wave_loop_next(cudaGraphConditionalHandle h, int* active, int limit) {
    const int c = active[1] + 1;
    active[1] = c;
    cudaGraphSetConditional(h, (active[0] > 0 && c < limit) ? 1u : 0u);
}

// Start of a wave: |v| per state, u_0 = v / |v|, problem status.
int enqueue_wave_start(mexk_batch_t b, const Wave& w, cudaStream_t s) {
    const Layout L = layout(b, w);
    int rc;
    if ((rc = launch_lift(L, 0, 1, s))) return rc;
    if ((rc = launch_restart(L, 1, s))) return rc;
    MEXK_CK(cudaMemsetAsync(b->d_active, 0, sizeof(int), s));
    return launch_status(L, w.p0, w.p1, s);
}

// One cycle of a wave (captured into its graph).
int enqueue_wave_cycle(mexk_batch_t b, const Wave& w, cudaStream_t s) {
    const Layout L = layout(b, w);
    const int m = b->prm.m;
    int rc;
    MEXK_CK(cudaMemsetAsync(b->d_active, 0, sizeof(int), s));
    for (int j = 0; j < m; ++j) {
        if ((rc = launch_spmm(L, j, b->unroll, s))) return rc;
        if ((rc = launch_dot(L, j, b->prm.reorthogonalize, b->gg, 0, s))) return rc;
        if ((rc = launch_update(L, j, s))) return rc;
    }
    if ((rc = launch_norm_last(L, m - 1, s))) return rc;
    ControlArgs c;
    const size_t s0 = static_cast<size_t>(w.p0) * BR;
    c.st = b->d_st + s0;
    c.H = b->d_H + s0 * BLD * BM_MAX;
    c.ldh = BLD;
    c.coef = b->d_coefl + s0 * BLD;
    c.log = nullptr;
    c.h_stride = static_cast<size_t>(BLD) * BM_MAX;
    c.coef_stride = BLD;
    if ((rc = launch_controller(c, m, s, (w.p1 - w.p0) * BR))) return rc;
    if ((rc = launch_lift(L, m, 0, s))) return rc;
    if ((rc = launch_restart(L, 0, s))) return rc;
    return launch_status(L, w.p0, w.p1, s);
}

// Every state accepts or finishes once per cycle: at most max_steps cycles.
int wave_cycle_limit(mexk_batch_t b) { return (b->prm.max_restarts > 0 ? b->prm.max_restarts : 1000) + 2; }

// The whole wave as one graph: its start, then the cycles in a device-side
// while loop (one launch per wave; the host reads the outcome afterwards).
int capture_wave(mexk_batch_t b, Wave& w) {
    if (w.exec) {
        cudaGraphExecDestroy(w.exec);
        w.exec = nullptr;
    }
    cudaStream_t s = b->stream;
    cudaGraph_t g = nullptr, body = nullptr;
    MEXK_CK(cudaGraphCreate(&g, 0));
    int rc = MEXK_OK;
    cudaError_t e = cudaSuccess;
    std::vector<cudaGraphNode_t> deps;
    cudaGraphConditionalHandle h = 0;
    auto fail = [&](cudaError_t err, const char* what) {
        set_cuda_error(err, what, __FILE__, __LINE__);
        return MEXK_ERR_CUDA;
    };
    if ((e = cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault)) != cudaSuccess) {
        cudaGraphDestroy(g);
        return fail(e, "cudaGraphConditionalHandleCreate (batch)");
    }
    // the start and the loop's first condition, captured into g
    if ((e = cudaStreamBeginCaptureToGraph(s, g, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal)) !=
        cudaSuccess) {
        cudaGraphDestroy(g);
        return fail(e, "cudaStreamBeginCaptureToGraph (batch)");
    }
    rc = enqueue_wave_start(b, w, s);
    if (rc == MEXK_OK) {
        wave_loop_start<<<1, 1, 0, s>>>(h, b->d_active);
        cudaStreamCaptureStatus cs;
        const cudaGraphNode_t* d = nullptr;
        size_t nd = 0;
        e = cudaStreamGetCaptureInfo(s, &cs, nullptr, nullptr, &d, nullptr, &nd);
        if (e == cudaSuccess) deps.assign(d, d + nd);
    }
    cudaGraph_t got = nullptr;
    const cudaError_t e2 = cudaStreamEndCapture(s, &got);
    if (rc != MEXK_OK || e != cudaSuccess || e2 != cudaSuccess) {
        cudaGraphDestroy(g);
        return rc != MEXK_OK ? rc : fail(e != cudaSuccess ? e : e2, "wave start capture (batch)");
    }
    // the while node after it, its body one cycle and the next condition
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t node = nullptr;
    if ((e = cudaGraphAddNode(&node, g, deps.data(), nullptr, deps.size(), &cp)) != cudaSuccess) {
        cudaGraphDestroy(g);
        return fail(e, "cudaGraphAddNode (batch while)");
    }
    body = cp.conditional.phGraph_out[0];
    if ((e = cudaStreamBeginCaptureToGraph(s, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal)) !=
        cudaSuccess) {
        cudaGraphDestroy(g);
        return fail(e, "cudaStreamBeginCaptureToGraph (batch body)");
    }
    rc = enqueue_wave_cycle(b, w, s);
    if (rc == MEXK_OK) wave_loop_next<<<1, 1, 0, s>>>(h, b->d_active, wave_cycle_limit(b));
    const cudaError_t e3 = cudaStreamEndCapture(s, &got);
    if (rc != MEXK_OK || e3 != cudaSuccess) {
        cudaGraphDestroy(g);
        return rc != MEXK_OK ? rc : fail(e3, "wave body capture (batch)");
    }
    e = cudaGraphInstantiate(&w.exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(e, "cudaGraphInstantiate (batch)");
    return MEXK_OK;
}

// Times `reps` launches of `fn` on the batch stream (after one warm-up).
template <typename F>
int time_ms(mexk_batch_t b, F fn, int reps, double* ms) {
    cudaEvent_t e0, e1;
    MEXK_CK(cudaEventCreate(&e0));
    MEXK_CK(cudaEventCreate(&e1));
    int rc = fn();
    if (rc == MEXK_OK) {
        cudaEventRecord(e0, b->stream);
        for (int r = 0; r < reps && rc == MEXK_OK; ++r) rc = fn();
        cudaEventRecord(e1, b->stream);
        cudaEventSynchronize(e1);
        float f = 0.f;
        cudaEventElapsedTime(&f, e0, e1);
        *ms = f / reps;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return rc;
}

// Autotuner: on the first wave, times the dot sweep at step m/2 for every
// (tile rows, columns per block) candidate and the SpMM for each unroll
// depth; keeps the fastest. Timing-only launches leave every state as it is.
int autotune(mexk_batch_t b) {
    const auto t0 = std::chrono::steady_clock::now();
    int rc;
    double best = 1e300;
    int best_tr = DEFAULT_TILE_ROWS, best_gg = 4;
    const int jt = b->prm.m / 2;
    for (int tr : TILE_CANDIDATES) {
        if ((rc = build_tiles(b, tr))) return rc;
        const Layout L = layout(b, b->waves[0]);
        for (int gg : {2, 4}) {
            double ms = 0.0;
            if ((rc = time_ms(b, [&] { return launch_dot(L, jt, 1, gg, 1, b->stream); }, 3, &ms))) return rc;
            if (ms < best) {
                best = ms;
                best_tr = tr;
                best_gg = gg;
            }
        }
    }
    if ((rc = build_tiles(b, best_tr))) return rc;
    b->gg = best_gg;
    const Layout L = layout(b, b->waves[0]);
    double ms4 = 0.0, ms8 = 0.0;
    if ((rc = time_ms(b, [&] { return launch_spmm(L, 0, 4, b->stream); }, 3, &ms4))) return rc;
    if ((rc = time_ms(b, [&] { return launch_spmm(L, 0, 8, b->stream); }, 3, &ms8))) return rc;
    b->unroll = ms8 < ms4 ? 8 : 4;
    MEXK_CK(cudaStreamSynchronize(b->stream));
    b->tune_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    b->tuned = true;
    return MEXK_OK;
}

void init_state(DevState* st, const mexk_batch_params_t& p, double t, bool used) {
    memset(st, 0, sizeof(*st));
    // ArnoldiRunner constructor (main.cu:1292-1305) and the first step size
    // of compute_expmv (main.cu:1426-1434), per right-hand side.
    st->total_t = t;
    st->dt_max = t;
    st->dt_min = std::max(1e-12, t * 1e-6);
    const double dt_init = (p.max_restarts > 0) ? t / p.max_restarts : t;
    st->tol = p.tol;
    st->tol_base = p.tol;
    st->max_steps = (p.max_restarts > 0) ? p.max_restarts : 1000;
    st->max_rejects = 20;
    st->safety = 0.8;
    st->grow = 1.5;
    st->shrink = 0.5;
    st->m = p.m;
    st->m_base = p.m;
    double dt = std::min(std::max(dt_init, st->dt_min), st->dt_max);
    st->done = !(0.0 < st->total_t && 0 < st->max_steps);
    dt = std::min(dt, st->total_t);
    st->dt = dt;
    st->k_used = p.m;
    st->m_next = p.m;
    st->ctrl = MEXK_CTRL_REFERENCE;
    st->tol_floor_rel = 5.9604644775390625e-08;  // 2^-24
    st->err_budget_rel = 5e-7;
    if (!used) {
        st->done = 1;
        st->converged = 1;
    }
}

}  // namespace

extern "C" {

int mexk_batch_create(int device, const mexk_batch_params_t* p, mexk_batch_t* out) {
    if (!p || !out) return MEXK_ERR_INVALID;
    if (p->m < 1 || p->m > MEXK_BATCH_M_MAX || !(p->tol > 0.0) || p->max_restarts < 0 || p->basis_bytes < 0) {
        set_error_text("batch parameters out of range (m 1..32, tol > 0)");
        return MEXK_ERR_INVALID;
    }
    mexk_batch_t b = new mexk_batch_s();
    b->device = device;
    b->prm = *p;
    *out = b;
    return MEXK_OK;
}

int mexk_batch_add(mexk_batch_t b, int rows, const int* row_ptr, const int* col_idx, const double* values, double t,
                   int nrhs, const double* V, int* index) {
    if (!b || b->uploaded || rows < 1 || !row_ptr || !V || nrhs < 1 || nrhs > MEXK_BATCH_RHS || !std::isfinite(t))
        return MEXK_ERR_INVALID;
    if (b->prm.m >= rows) {
        set_error_text("Requested Arnoldi m must be less than the number of rows");
        return MEXK_ERR_INVALID;
    }
    const long long nnz = row_ptr[rows];
    if (row_ptr[0] != 0 || nnz < 0 || (nnz > 0 && (!col_idx || !values))) {
        set_error_text("row_ptr must start at 0 and end at nnz");
        return MEXK_ERR_INVALID;
    }
    for (int r = 0; r < rows; ++r)
        if (row_ptr[r] > row_ptr[r + 1]) {
            set_error_text("row_ptr must be non-decreasing");
            return MEXK_ERR_INVALID;
        }
    for (long long e = 0; e < nnz; ++e)
        if (col_idx[e] < 0 || col_idx[e] >= rows) {
            set_error_text("column index out of range");
            return MEXK_ERR_INVALID;
        }
    b->probs.push_back({rows, nnz, row_ptr, col_idx, values, t, nrhs, V});
    if (index) *index = static_cast<int>(b->probs.size()) - 1;
    return MEXK_OK;
}

int mexk_batch_upload(mexk_batch_t b) {
    if (!b || b->uploaded || b->probs.empty()) return MEXK_ERR_INVALID;
    MEXK_CK(cudaSetDevice(b->device));
    MEXK_CK(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
    int rc;
    if ((rc = expm_init_attributes())) return rc;
    const int P = P_of(b);
    const int m = b->prm.m;
    // row space
    b->prow0.assign(P + 1, 0);
    long long maxrows = 0, maxnnz = 0;
    for (int p = 0; p < P; ++p) {
        const long long rp = (b->probs[p].rows + BROWS - 1) / BROWS * BROWS;
        b->prow0[p + 1] = b->prow0[p] + rp;
        maxrows = std::max(maxrows, rp);
        maxnnz = std::max(maxnnz, b->probs[p].nnz);
        b->nnz += b->probs[p].nnz;
    }
    b->rows = b->prow0[P];
    if (b->rows / BROWS > 2147483647LL) {
        set_error_text("batch row space too large");
        return MEXK_ERR_INVALID;
    }
    b->nchunks = static_cast<int>(b->rows / BROWS);
    const size_t S = static_cast<size_t>(P) * BR;
    if ((rc = dalloc(&b->d_row_ptr, b->rows + 1)) || (rc = dalloc(&b->d_col, b->nnz)) ||
        (rc = dalloc(&b->d_val, b->nnz)) || (rc = dalloc(&b->d_prow0, P + 1)) ||
        (rc = dalloc(&b->d_chunk_prob, b->nchunks)) || (rc = dalloc(&b->d_V, static_cast<size_t>(b->rows) * BR)) ||
        (rc = dalloc(&b->d_Y, static_cast<size_t>(b->rows) * BR)) ||
        (rc = dalloc(&b->d_st, S)) || (rc = dalloc(&b->d_H, S * BLD * BM_MAX)) || (rc = dalloc(&b->d_G, S * BLD * BLD)) ||
        (rc = dalloc(&b->d_s, S * (BLD + 1))) || (rc = dalloc(&b->d_pre, S * (BLD + 1))) ||
        (rc = dalloc(&b->d_coefl, S * BLD)) || (rc = dalloc(&b->d_coef, S * BLD)) || (rc = dalloc(&b->d_wsc, S)) ||
        (rc = dalloc(&b->d_psc, S)) || (rc = dalloc(&b->d_pcount, P)) || (rc = dalloc(&b->d_pdone, P)) ||
        (rc = dalloc(&b->d_active, 2)) || (rc = dalloc(&b->d_ptile0, P)) || (rc = dalloc(&b->d_ptiles, P)))
        return rc;
    MEXK_CK(cudaMemset(b->d_H, 0, sizeof(double) * S * BLD * BM_MAX));
    MEXK_CK(cudaMemset(b->d_pcount, 0, sizeof(unsigned int) * P));
    MEXK_CK(cudaMemset(b->d_pdone, 0, sizeof(int) * P));
    MEXK_CK(cudaMemcpy(b->d_prow0, b->prow0.data(), sizeof(long long) * (P + 1), cudaMemcpyHostToDevice));
    {
        cudaError_t e = cudaMallocHost(reinterpret_cast<void**>(&b->h_active), 2 * sizeof(int));
        if (e != cudaSuccess) {
            set_cuda_error(e, "cudaMallocHost (batch)", __FILE__, __LINE__);
            return MEXK_ERR_ALLOC;
        }
    }
    // CSR, start vectors, chunk owners
    std::vector<long long> rp64(static_cast<size_t>(b->rows) + 1);
    std::vector<int> chunk(b->nchunks);
    double* d_stage = nullptr;
    if ((rc = dalloc(&d_stage, std::max<long long>(maxnnz, 1)))) return rc;
    std::vector<double> ytmp(static_cast<size_t>(maxrows) * BR);
    b->h_init.assign(S, DevState{});
    long long nb = 0;
    for (int p = 0; p < P; ++p) {
        const HostProblem& q = b->probs[p];
        const long long r0 = b->prow0[p];
        const long long rpad = b->prow0[p + 1] - r0;
        for (long long r = 0; r < rpad; ++r) rp64[r0 + r] = nb + q.row_ptr[r < q.rows ? r : q.rows];
        for (long long c = r0 / BROWS; c < (r0 + rpad) / BROWS; ++c) chunk[c] = p;
        if (q.nnz > 0) {
            MEXK_CK(cudaMemcpy(b->d_col + nb, q.col, sizeof(int) * q.nnz, cudaMemcpyHostToDevice));
            MEXK_CK(cudaMemcpy(d_stage, q.val, sizeof(double) * q.nnz, cudaMemcpyHostToDevice));
            if ((rc = launch_narrow_values(d_stage, b->d_val + nb, static_cast<size_t>(q.nnz), nullptr))) return rc;
        }
        for (int r = 0; r < BR; ++r) init_state(&b->h_init[static_cast<size_t>(p) * BR + r], b->prm, q.t, r < q.nrhs);
        const bool live = !b->h_init[static_cast<size_t>(p) * BR].done;
        std::fill(ytmp.begin(), ytmp.begin() + rpad * BR, 0.0);
        if (live)
            for (int i = 0; i < q.rows; ++i)
                for (int r = 0; r < q.nrhs; ++r) ytmp[static_cast<size_t>(i) * BR + r] = q.V[static_cast<size_t>(i) * q.nrhs + r];
        MEXK_CK(cudaMemcpy(b->d_V + r0 * BR, ytmp.data(), sizeof(double) * rpad * BR, cudaMemcpyHostToDevice));
        nb += q.nnz;
    }
    rp64[b->rows] = nb;
    MEXK_CK(cudaDeviceSynchronize());
    dfree(d_stage);
    MEXK_CK(cudaMemcpy(b->d_row_ptr, rp64.data(), sizeof(long long) * rp64.size(), cudaMemcpyHostToDevice));
    MEXK_CK(cudaMemcpy(b->d_chunk_prob, chunk.data(), sizeof(int) * chunk.size(), cudaMemcpyHostToDevice));
    // waves: contiguous problems whose bases fit the budget
    long long budget = b->prm.basis_bytes;
    if (budget <= 0) {
        size_t fr = 0, tot = 0;
        MEXK_CK(cudaMemGetInfo(&fr, &tot));
        budget = static_cast<long long>(0.6 * static_cast<double>(fr));
    }
    const long long per_row = static_cast<long long>(m + 2) * BR * sizeof(float);
    long long cap = budget / per_row / BROWS * BROWS;
    if (cap < maxrows) {
        set_error_text("basis budget too small for the largest problem of the batch");
        return MEXK_ERR_ALLOC;
    }
    b->waves.clear();
    Wave w;
    for (int p = 0; p < P; ++p) {
        if (p > w.p0 && b->prow0[p + 1] - b->prow0[w.p0] > cap) {
            w.p1 = p;
            b->waves.push_back(w);
            w = Wave();
            w.p0 = p;
        }
    }
    w.p1 = P;
    b->waves.push_back(w);
    long long wave_rows = 0;
    int tiles_cap = 0, tiles_total = 0;
    for (auto& x : b->waves) {
        x.R0 = b->prow0[x.p0];
        x.R1 = b->prow0[x.p1];
        x.C0 = static_cast<int>(x.R0 / BROWS);
        x.C1 = static_cast<int>(x.R1 / BROWS);
        wave_rows = std::max(wave_rows, x.R1 - x.R0);
        int tw = 0;  // tiles at the smallest candidate tile size
        for (int p = x.p0; p < x.p1; ++p)
            tw += static_cast<int>((b->prow0[p + 1] - b->prow0[p] + TILE_CANDIDATES[0] - 1) / TILE_CANDIDATES[0]);
        tiles_cap = std::max(tiles_cap, tw);
        tiles_total += tw;
    }
    b->wave_rows_cap = wave_rows;
    b->tiles_cap = tiles_cap;
    b->tiles_total_cap = tiles_total;
    if ((rc = dalloc(&b->d_U, static_cast<size_t>(m + 1) * wave_rows * BR)) ||
        (rc = dalloc(&b->d_W, static_cast<size_t>(wave_rows) * BR)) ||
        (rc = dalloc(&b->d_part, static_cast<size_t>(tiles_cap) * BPS)) ||
        (rc = dalloc(&b->d_tile_prob, tiles_total)) || (rc = dalloc(&b->d_tile_row0, tiles_total)) ||
        (rc = dalloc(&b->d_tile_nrows, tiles_total)))
        return rc;
    MEXK_CK(cudaMemset(b->d_U, 0, sizeof(float) * static_cast<size_t>(m + 1) * wave_rows * BR));
    MEXK_CK(cudaMemset(b->d_W, 0, sizeof(float) * static_cast<size_t>(wave_rows) * BR));
    if ((rc = build_tiles(b, DEFAULT_TILE_ROWS))) return rc;
    b->uploaded = true;
    return MEXK_OK;
}

int mexk_batch_run(mexk_batch_t b) {
    if (!b || !b->uploaded) return MEXK_ERR_NOT_READY;
    MEXK_CK(cudaSetDevice(b->device));
    int rc;
    if (b->prm.autotune && !b->tuned) {
        if ((rc = autotune(b))) return rc;
        for (auto& w : b->waves)
            if (w.exec) {
                cudaGraphExecDestroy(w.exec);
                w.exec = nullptr;
            }
    }
    const int P = P_of(b);
    const size_t S = static_cast<size_t>(P) * BR;
    MEXK_CK(cudaMemcpyAsync(b->d_st, b->h_init.data(), sizeof(DevState) * S, cudaMemcpyHostToDevice, b->stream));
    MEXK_CK(cudaMemsetAsync(b->d_pdone, 0, sizeof(int) * P, b->stream));
    // states that never step keep y = 0 (main_cpu.cpp:467)
    MEXK_CK(cudaMemsetAsync(b->d_Y, 0, sizeof(double) * static_cast<size_t>(b->rows) * BR, b->stream));
    b->cycles = 0;
    b->have_final = false;
    for (auto& w : b->waves) {
        if (!w.exec && (rc = capture_wave(b, w))) return rc;
        // one launch: start vectors, then the cycles until every state is done
        MEXK_CK(cudaGraphLaunch(w.exec, b->stream));
        MEXK_CK(cudaMemcpyAsync(b->h_active, b->d_active, 2 * sizeof(int), cudaMemcpyDeviceToHost, b->stream));
        MEXK_CK(cudaStreamSynchronize(b->stream));
        b->cycles += b->h_active[1];
        if (b->h_active[0] > 0) {
            set_error_text("batch wave did not finish within the step limit");
            return MEXK_ERR_DEVICE;
        }
    }
    // per-state status bits (singular Pade systems, bad k) surface as errors
    b->h_final.resize(S);
    MEXK_CK(cudaMemcpy(b->h_final.data(), b->d_st, sizeof(DevState) * S, cudaMemcpyDeviceToHost));
    b->have_final = true;
    for (const DevState& st : b->h_final)
        if (st.status & (ST_LU_SINGULAR | ST_SMEM | ST_BAD_K | ST_TIMEOUT)) {
            set_error_text("batch: a state reported a device status error");
            return MEXK_ERR_DEVICE;
        }
    return MEXK_OK;
}

int mexk_batch_result(mexk_batch_t b, int problem, double* Y, mexk_result_t* results) {
    if (!b || !b->uploaded || problem < 0 || problem >= P_of(b) || !Y) return MEXK_ERR_INVALID;
    if (!b->have_final) return MEXK_ERR_NOT_READY;
    MEXK_CK(cudaSetDevice(b->device));
    const HostProblem& q = b->probs[problem];
    std::vector<double> tmp(static_cast<size_t>(q.rows) * BR);
    MEXK_CK(cudaMemcpy(tmp.data(), b->d_Y + b->prow0[problem] * BR, sizeof(double) * tmp.size(),
                       cudaMemcpyDeviceToHost));
    for (int i = 0; i < q.rows; ++i)
        for (int r = 0; r < q.nrhs; ++r) Y[static_cast<size_t>(i) * q.nrhs + r] = tmp[static_cast<size_t>(i) * BR + r];
    if (results) {
        for (int r = 0; r < q.nrhs; ++r) {
            const DevState& st = b->h_final[static_cast<size_t>(problem) * BR + r];
            mexk_result_t& o = results[r];
            o.converged = st.converged;
            o.restarts_done = st.accepted;
            o.last_residual = st.last_residual;
            o.attempts = st.attempts;
            o.cycles = st.cycles;
            o.spmv_count = st.spmv_count;
            o.t_done = st.t_done;
            o.status = st.status;
        }
    }
    return MEXK_OK;
}

int mexk_batch_info(mexk_batch_t b, mexk_batch_info_t* info) {
    if (!b || !info) return MEXK_ERR_INVALID;
    info->problems = P_of(b);
    info->waves = static_cast<int>(b->waves.size());
    info->tile_rows = b->tile_rows;
    info->dot_columns = b->gg;
    info->spmm_unroll = b->unroll;
    info->cycles = b->cycles;
    info->rows = b->rows;
    info->nnz = b->nnz;
    info->tune_ms = b->tune_ms;
    return MEXK_OK;
}

int mexk_batch_profile(mexk_batch_t b, int kind, int j, int iters, double* ms_per_launch, long long* wave_rows,
                       long long* wave_nnz) {
    if (!b || !b->uploaded || !ms_per_launch || iters < 1 || j < 0 || j >= b->prm.m || kind < 0 || kind > 2)
        return MEXK_ERR_INVALID;
    if (!b->have_final) return MEXK_ERR_NOT_READY;
    MEXK_CK(cudaSetDevice(b->device));
    const Wave& w = b->waves[0];
    const Layout L = layout(b, w);
    // Finished problems skip every kernel: time the wave as if all were running.
    std::vector<int> saved(w.p1 - w.p0);
    MEXK_CK(cudaMemcpy(saved.data(), b->d_pdone + w.p0, sizeof(int) * saved.size(), cudaMemcpyDeviceToHost));
    MEXK_CK(cudaMemset(b->d_pdone + w.p0, 0, sizeof(int) * saved.size()));
    int rc;
    if (kind == 0) rc = time_ms(b, [&] { return launch_spmm(L, j, b->unroll, b->stream); }, iters, ms_per_launch);
    else if (kind == 1)
        rc = time_ms(b, [&] { return launch_dot(L, j, 1, b->gg, 1, b->stream); }, iters, ms_per_launch);
    else rc = time_ms(b, [&] { return launch_update(L, j, b->stream); }, iters, ms_per_launch);
    MEXK_CK(cudaMemcpy(b->d_pdone + w.p0, saved.data(), sizeof(int) * saved.size(), cudaMemcpyHostToDevice));
    if (rc) return rc;
    if (wave_rows) *wave_rows = w.R1 - w.R0;
    if (wave_nnz) {
        long long nz = 0;
        for (int p = w.p0; p < w.p1; ++p) nz += b->probs[p].nnz;
        *wave_nnz = nz;
    }
    return MEXK_OK;
}

int mexk_batch_destroy(mexk_batch_t b) {
    if (!b) return MEXK_OK;
    if (b->uploaded || b->stream) {
        cudaSetDevice(b->device);
        if (b->stream) cudaStreamSynchronize(b->stream);
    }
    for (auto& w : b->waves)
        if (w.exec) cudaGraphExecDestroy(w.exec);
    dfree(b->d_row_ptr);
    dfree(b->d_col);
    dfree(b->d_val);
    dfree(b->d_prow0);
    dfree(b->d_chunk_prob);
    dfree(b->d_V);
    dfree(b->d_Y);
    dfree(b->d_st);
    dfree(b->d_H);
    dfree(b->d_G);
    dfree(b->d_s);
    dfree(b->d_pre);
    dfree(b->d_coefl);
    dfree(b->d_coef);
    dfree(b->d_wsc);
    dfree(b->d_psc);
    dfree(b->d_pcount);
    dfree(b->d_pdone);
    dfree(b->d_active);
    dfree(b->d_U);
    dfree(b->d_W);
    dfree(b->d_part);
    dfree(b->d_tile_prob);
    dfree(b->d_tile_row0);
    dfree(b->d_tile_nrows);
    dfree(b->d_ptile0);
    dfree(b->d_ptiles);
    if (b->h_active) cudaFreeHost(b->h_active);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return MEXK_OK;
}

}  // extern "C"
