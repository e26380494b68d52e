// Device context and the restarted-Arnoldi driver behind the C ABI.
//
// Replaces DeviceContext (reference main.cu:747-1125) and
// ArnoldiRunner::compute_expmv (main.cu:1411-1571) for one device. The
// reference drives every Arnoldi step from the host (about 10(j+1)+12
// launches and 3 blocking syncs per step, H held on the host). Here a whole
// Krylov cycle -- m x (SpMV, three Gram-Schmidt sweeps, normalise), the
// exponential + controller, the lift and the restart -- is one CUDA graph
// whose kernels read and write a device-resident state block, so the host
// launches one graph per accepted step and syncs once to read `done`.
// The FP64 form runs three CGS2 sweeps and a normalisation per step
// (gram_schmidt.cu); the mixed form one reducing and one streaming sweep
// over an FP32 basis with a device-resident Gram matrix (gram_mixed.cu).
//
// HBM layout per context (n rows, m_alloc maximum Krylov dimension):
//   CSR        row_ptr int32[n+1], col_idx int32[nnz], values f64[nnz]
//              (+ f32 copy of values for the mixed-precision form)
//   row blocks int4[nblocks+1] SpMV schedule {first row, first nonzero, 16-bit column offset, base}
//   col16      uint16 columns of the row blocks whose columns span <= 65536
//   basis V    column-major, leading dimension ldv = n rounded up to 64,
//              m_alloc+1 columns, f64 (+ f32 basis for the mixed form, whose
//              columns carry f64 scales, with the Gram matrix, in GramState)
//   w, y       work vector (basis precision) and result (f64)
//   H          f64 (m_alloc+1) x m_alloc column-major; h1, h2, coef f64
//   partials   f64[4096 x RED_STRIDE] grid-reduction scratch + counter
//   state      DevState (device) mirrored into pinned host memory
#include "mexk_internal.cuh"

#include <nvtx3/nvToolsExt.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

namespace mexk {

static thread_local std::string g_err;

void set_cuda_error(cudaError_t e, const char* what, const char* file, int line) {
    char buf[512];
    snprintf(buf, sizeof(buf), "%s failed: %s (%s:%d)", what, cudaGetErrorString(e), file, line);
    g_err = buf;
}

void set_error_text(const std::string& s) { g_err = s; }

// NVTX range over a host-side phase, named as the reference's ranges
// (NvtxRange, main.cu:38-41): a profiler shows the solve, the start vector
// and each Krylov cycle (whose basis build, exponential, lift and restart run
// as one graph on the device).
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
};

constexpr int PARTIAL_BLOCKS = 4096;
constexpr int LOG_CAP = 8192;

}  // namespace mexk

using namespace mexk;

struct GraphEntry {
    int m, prec, reortho, ctrl, window;
    cudaGraphExec_t exec;
};

struct mexk_context_s {
    int device = 0;
    int sms = 1;
    cudaStream_t stream = nullptr;
    int n = 0;
    long long nnz = 0;
    int m_alloc = 0;
    int ldv = 0;
    int ldh = 0;
    int nblocks = 0;
    int symmetric = -1;  // A == A^T exactly: -1 not yet checked
    int last_window = 0; // ortho_window of the last solve (kernel profiling follows it)
    int last_controller = MEXK_CTRL_REFERENCE;  // controller of the last solve (likewise)
    int* d_row_ptr = nullptr;
    int* d_col = nullptr;
    double* d_val = nullptr;
    float* d_val32 = nullptr;
    int4* d_tiles = nullptr;
    uint16_t* d_col16 = nullptr;
    bool spmv_narrow = false;  // every staged SpMV row block has 16-bit columns
    // The SpMV form per precision (MEXK_SPMV_*): the row-pattern form when
    // every row is one of at most PAT_MAX patterns, else direct (one block per
    // row block) when some row block's columns span 65,536 or more, else staged.
    int spmv_form64 = MEXK_SPMV_STAGED;
    int spmv_form32 = MEXK_SPMV_STAGED;
    RowPatterns* d_pat = nullptr;  // pattern table and row ids (pattern form only)
    uint8_t* d_pid = nullptr;
    int pat_major = 0;  // the pattern with the most rows, and its length
    int pat_major_len = 0;
    int pat_max_len = 0;
    double* d_V = nullptr;
    float* d_V32 = nullptr;
    double* d_w = nullptr;
    float* d_w32 = nullptr;
    double* d_y = nullptr;
    double* d_H = nullptr;
    double* d_h1 = nullptr;
    double* d_h2 = nullptr;
    double* d_coef = nullptr;
    double* d_cand = nullptr;
    double* d_expm_ws = nullptr;  // Pade workspace of the reference controller for m > EXPM_SMEM_K
    float* d_mlp = nullptr;
    float* d_mlp_win = nullptr;  // the network for solves with a window (may be null)
    double* d_partials = nullptr;
    GramState* d_gram = nullptr;
    double* d_gram_part = nullptr;
    unsigned int* d_counter = nullptr;
    unsigned int* d_bar = nullptr;  // the fused Lanczos cycle's grid-barrier words
    bool lanczos_fused = false;     // window-2 pattern-form bases in one cooperative launch
    DevState* d_state = nullptr;
    DevState* h_state = nullptr;
    mexk_step_t* d_log = nullptr;
    bool uploaded = false;
    bool use_graph = true;
    std::vector<GraphEntry> graphs;
};

namespace {

template <typename T>
int dalloc(T** p, size_t count) {
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), sizeof(T) * count);
    if (e != cudaSuccess) {
        set_cuda_error(e, "cudaMalloc", __FILE__, __LINE__);
        return MEXK_ERR_ALLOC;
    }
    return MEXK_OK;
}

template <typename T>
void dfree(T*& p) {
    if (p) cudaFree(p);
    p = nullptr;
}

// Whether A equals its transpose exactly (checked on the device once).
int matrix_symmetric(mexk_context_t ctx, int* sym) {
    if (ctx->symmetric < 0) {
        int* d_ok = nullptr;
        int rc = dalloc(&d_ok, 1);
        if (rc) return rc;
        rc = launch_symmetric_check(ctx->n, ctx->d_row_ptr, ctx->d_col, ctx->d_val, d_ok, ctx->stream);
        int ok = 0;
        if (!rc) {
            const cudaError_t e1 = cudaMemcpyAsync(&ok, d_ok, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
            const cudaError_t e2 = cudaStreamSynchronize(ctx->stream);
            if (e1 != cudaSuccess || e2 != cudaSuccess) {
                set_cuda_error(e1 != cudaSuccess ? e1 : e2, "symmetry check", __FILE__, __LINE__);
                rc = MEXK_ERR_CUDA;
            }
        }
        dfree(d_ok);
        if (rc) return rc;
        ctx->symmetric = ok ? 1 : 0;
    }
    *sym = ctx->symmetric;
    return MEXK_OK;
}

int check_params(mexk_context_t ctx, const mexk_params_t* p) {
    if (!ctx || !p) return MEXK_ERR_INVALID;
    if (!ctx->uploaded) return MEXK_ERR_NOT_READY;
    if (p->m < 1 || p->m > ctx->m_alloc || p->m > MEXK_M_MAX) {
        set_error_text("Krylov dimension m out of range (1..m_alloc_max)");
        return MEXK_ERR_INVALID;
    }
    if ((p->precision == MEXK_PREC_MIXED || p->controller != MEXK_CTRL_REFERENCE) && p->m > MEXK_M_MAX_MIXED) {
        set_error_text("mixed precision and the candidate-step controllers take m <= 64");
        return MEXK_ERR_UNSUPPORTED;
    }
    if (const mexk_stepping_t* ts = p->stepping) {
        // The reference reads these unchecked; values that would make its loop
        // misbehave (no progress, NaN steps) are refused here.
        if (!(ts->dt_min > 0.0) || !(ts->dt_max >= ts->dt_min) || !(ts->dt_init > 0.0) || !(ts->tol_step >= 0.0) ||
            !(ts->safety > 0.0) || !(ts->grow > 0.0) || !(ts->shrink > 0.0) || ts->max_steps < 0 ||
            ts->max_rejects < 1 || !std::isfinite(ts->dt_init) || !std::isfinite(ts->dt_max)) {
            set_error_text("time-stepping parameters out of range (dt_min > 0, dt_max >= dt_min, dt_init > 0, "
                           "safety, grow, shrink > 0, max_rejects >= 1)");
            return MEXK_ERR_INVALID;
        }
        if (ts->adapt_m && ts->m_step > 0 && ts->m_max > p->m) {
            // main.cu:1441-1444 refuses m beyond the allocation
            if (ts->m_max > ctx->m_alloc || ts->m_max >= ctx->n) {
                set_error_text("adapt_m: m_max exceeds the context's allocated Krylov dimension");
                return MEXK_ERR_INVALID;
            }
            if (p->precision == MEXK_PREC_MIXED || p->controller != MEXK_CTRL_REFERENCE) {
                set_error_text("adapt_m is implemented for the FP64 form with the reference controller");
                return MEXK_ERR_UNSUPPORTED;
            }
        }
    }
    // main.cu:1322-1326: m must be smaller than the number of rows.
    if (p->m >= ctx->n) {
        set_error_text("Requested Arnoldi m must be less than the number of rows");
        return MEXK_ERR_INVALID;
    }
    if (p->precision != MEXK_PREC_FP64 && p->precision != MEXK_PREC_MIXED) return MEXK_ERR_INVALID;
    if (p->controller < MEXK_CTRL_REFERENCE || p->controller > MEXK_CTRL_LEARNED) return MEXK_ERR_INVALID;
    if (p->controller == MEXK_CTRL_LEARNED && ctx->d_mlp == nullptr) {
        set_error_text("learned controller requested but no controller network is loaded");
        return MEXK_ERR_NOT_READY;
    }
    if (p->ortho_window != 0) {
        if (p->ortho_window < 2 || p->ortho_window > p->m) {
            set_error_text("ortho_window must be 0 or in 2..m");
            return MEXK_ERR_INVALID;
        }
        int sym = 0;
        const int rc = matrix_symmetric(ctx, &sym);
        if (rc) return rc;
        if (!sym) {
            set_error_text("a short-recurrence window needs a symmetric matrix");
            return MEXK_ERR_INVALID;
        }
    }
    return MEXK_OK;
}

// Gram state of a basis whose first columns are orthonormal: G = I, s = p = 1.
int reset_gram(mexk_context_t ctx, cudaStream_t s) {
    static GramState h0;
    static bool init = false;
    if (!init) {
        memset(&h0, 0, sizeof(h0));
        for (int i = 0; i < GRAM_LD; ++i) h0.G[i + i * GRAM_LD] = 1.0;
        for (int i = 0; i < GRAM_M + 2; ++i) h0.s[i] = h0.ip[i] = 1.0;
        h0.wsc = h0.psc = 1.0f;
        init = true;
    }
    MEXK_CK(cudaMemcpyAsync(ctx->d_gram, &h0, sizeof(GramState), cudaMemcpyHostToDevice, s));
    MEXK_CK(cudaStreamSynchronize(s));
    return MEXK_OK;
}

int ensure_mixed(mexk_context_t ctx) {
    if (ctx->d_V32) return MEXK_OK;
    int rc;
    if ((rc = dalloc(&ctx->d_V32, static_cast<size_t>(ctx->ldv) * (ctx->m_alloc + 1)))) return rc;
    if ((rc = dalloc(&ctx->d_w32, static_cast<size_t>(ctx->ldv)))) return rc;
    // Rows n..ldv-1 stay zero: the vectorised sweeps read and write them.
    MEXK_CK(cudaMemset(ctx->d_V32, 0, sizeof(float) * static_cast<size_t>(ctx->ldv) * (ctx->m_alloc + 1)));
    MEXK_CK(cudaMemset(ctx->d_w32, 0, sizeof(float) * static_cast<size_t>(ctx->ldv)));
    if ((rc = dalloc(&ctx->d_gram, 1))) return rc;
    if ((rc = dalloc(&ctx->d_gram_part, static_cast<size_t>(GRAM_MAX_ROW_BLOCKS) * GRAM_SLOTS))) return rc;
    if ((rc = reset_gram(ctx, ctx->stream))) return rc;
    if ((rc = dalloc(&ctx->d_val32, static_cast<size_t>(ctx->nnz) + 4))) return rc;
    if ((rc = launch_narrow_values(ctx->d_val, ctx->d_val32, static_cast<size_t>(ctx->nnz), ctx->stream))) return rc;
    ctx->spmv_form32 = ctx->d_pat ? MEXK_SPMV_PATTERN : ctx->spmv_narrow ? MEXK_SPMV_STAGED : MEXK_SPMV_DIRECT;
    MEXK_CK(cudaStreamSynchronize(ctx->stream));
    return MEXK_OK;
}

GsArgs gs_args(mexk_context_t ctx, int j, int reortho, bool fp32) {
    GsArgs g;
    g.n = ctx->n;
    g.k = j + 1;
    g.j = j;
    g.ldv = ctx->ldv;
    g.ldh = ctx->ldh;
    g.reortho = reortho ? 1 : 0;
    g.V = fp32 ? static_cast<const void*>(ctx->d_V32) : static_cast<const void*>(ctx->d_V);
    g.w = fp32 ? static_cast<void*>(ctx->d_w32) : static_cast<void*>(ctx->d_w);
    g.H = ctx->d_H;
    g.h1 = ctx->d_h1;
    g.h2 = ctx->d_h2;
    g.partials = ctx->d_partials;
    g.counter = ctx->d_counter;
    g.st = ctx->d_state;
    g.beta_out = nullptr;
    return g;
}

GramArgs gram_args(mexk_context_t ctx, int j, int reortho) {
    GramArgs g;
    g.n = ctx->n;
    g.j = j;
    g.ldv = ctx->ldv;
    g.ldh = ctx->ldh;
    g.reortho = reortho ? 1 : 0;
    g.V = ctx->d_V32;
    g.w = ctx->d_w32;
    g.H = ctx->d_H;
    g.gs = ctx->d_gram;
    g.part = ctx->d_gram_part;
    g.counter = ctx->d_counter;
    g.st = ctx->d_state;
    return g;
}

LiftArgs lift_args(mexk_context_t ctx, bool fp32) {
    LiftArgs l;
    l.n = ctx->n;
    l.ldv = ctx->ldv;
    l.V = fp32 ? static_cast<const void*>(ctx->d_V32) : static_cast<const void*>(ctx->d_V);
    l.coef = ctx->d_coef;
    l.y = ctx->d_y;
    l.partials = ctx->d_partials;
    l.counter = ctx->d_counter;
    l.st = ctx->d_state;
    l.scale = fp32 ? reinterpret_cast<const double*>(reinterpret_cast<const char*>(ctx->d_gram) +
                                                     offsetof(GramState, s))
                   : nullptr;
    return l;
}

// Arnoldi step j: w = A v_j, then orthogonalise into column j+1 and H(:, j).
// The FP64 form finishes the step (H(j+1, j), normalised column); the mixed
// form leaves H(j+1, j) to the next step's dot sweep or to finish_basis.
// A mixed-precision step j >= 1 over columns j-1 and j (every step of a
// window of 2, step 1 of full Arnoldi) takes its dot products from the SpMV's
// row sums and the previous update (no dot sweep of its own).
bool fused_step(int j, int window) {
    const int lo = window > 0 ? std::max(0, j + 1 - window) : 0;
    return j >= 1 && j + 1 - lo <= 2;
}

// Whether the last update of an m-column mixed basis (step m - 1) leaves
// |u_m|^2 as partials in column m's b slot: a two-column update sweep, and a
// slot below the |w|^2 one. The basis's last norm then needs no sweep.
bool norm_from_update(int m, int window) {
    if (m < 1 || m >= GRAM_M) return false;
    const int lo = window > 0 ? std::max(0, m - window) : 0;
    return m - lo <= 2;
}

// The context SpMV in its form for the precision: w = A u_j (dots: FP32, as
// for launch_spmv; not with the direct form).
int context_spmv(mexk_context_t ctx, int j, bool fp32, const int* skip, cudaStream_t s,
                 const GramArgs* dots = nullptr) {
    const size_t ldv = static_cast<size_t>(ctx->ldv);
    const int form = fp32 ? ctx->spmv_form32 : ctx->spmv_form64;
    if (form == MEXK_SPMV_PATTERN)
        return fp32 ? launch_spmv_pattern<float>(ctx->n, ctx->pat_major, ctx->pat_major_len, ctx->pat_max_len,
                                                 ctx->d_pid, ctx->d_pat, ctx->d_V32 + j * ldv, ctx->d_w32, skip, s,
                                                 dots)
                    : launch_spmv_pattern<double>(ctx->n, ctx->pat_major, ctx->pat_major_len, ctx->pat_max_len,
                                                  ctx->d_pid, ctx->d_pat, ctx->d_V + j * ldv, ctx->d_w, skip, s,
                                                  dots);
    const bool direct = form == MEXK_SPMV_DIRECT;
    if (direct && dots) return MEXK_ERR_UNSUPPORTED;
    return fp32 ? launch_spmv<float, float>(ctx->n, ctx->nblocks, ctx->d_tiles, ctx->d_col16, ctx->spmv_narrow,
                                            ctx->d_row_ptr, ctx->d_col, ctx->d_val32, ctx->d_V32 + j * ldv,
                                            ctx->d_w32, skip, &ctx->d_state->status, s, dots, direct)
                : launch_spmv<double, double>(ctx->n, ctx->nblocks, ctx->d_tiles, ctx->d_col16, ctx->spmv_narrow,
                                              ctx->d_row_ptr, ctx->d_col, ctx->d_val, ctx->d_V + j * ldv, ctx->d_w,
                                              skip, &ctx->d_state->status, s, dots, direct);
}

// m: size of the basis being built in order (0 for a step on its own: then
// the step does its own dot sweep, since the previous update may not have
// written its b partials).
int enqueue_step(mexk_context_t ctx, int j, int reortho, bool fp32, cudaStream_t s, int window = 0, int m = 0) {
    int rc;
    if (fp32) {
        GramArgs g = gram_args(ctx, j, reortho);
        g.lo = window > 0 ? std::max(0, j + 1 - window) : 0;
        // the step's dots ride on the staged and the pattern SpMV
        const bool fusable = m > 0 && ctx->spmv_form32 != MEXK_SPMV_DIRECT;
        const bool fuse = fusable && fused_step(j, window);
        g.b_blocks = fuse ? gram_update2_blocks(ctx->n) : 0;
        // window 2 (symmetric A) with the pattern SpMV: a_{j-1} from the update of step j-1
        g.sym = (window == 2 && ctx->spmv_form32 == MEXK_SPMV_PATTERN) ? 1 : 0;
        if ((rc = context_spmv(ctx, j, true, &ctx->d_state->breakdown, s, fuse ? &g : nullptr))) return rc;
        if (!fuse && (rc = launch_gram_dot(g, s))) return rc;
        g.write_b = (fusable && j + 1 < m && fused_step(j + 1, window)) ? 1 : 0;
        if (m > 0 && j + 1 == m && norm_from_update(m, window)) g.write_b = 1;  // for finish_basis
        return launch_gram_update(g, s);
    }
    if ((rc = context_spmv(ctx, j, false, &ctx->d_state->breakdown, s))) return rc;
    GsArgs g = gs_args(ctx, j, reortho, false);
    if (window > 0) {
        // CGS2 against the window's columns lo..j only (Lanczos for a symmetric A);
        // H(0:lo-1, j) stays at the zero the cycle starts from
        const int lo = std::max(0, j + 1 - window);
        g.V = ctx->d_V + static_cast<size_t>(lo) * ctx->ldv;
        g.k = j + 1 - lo;
        g.h_row0 = lo;
    }
    if ((rc = launch_gs_step(g, gs_grid_size(ctx->n, g.k), s))) return rc;
    return launch_normalize<double>(ctx->n, j, ctx->ldv, ctx->d_w, ctx->d_V, ctx->d_state, nullptr, s);
}

// After the last step j of a basis: H(j+1, j) of the mixed form. partials:
// the basis was built by enqueue_step with m = j + 1 and its window, whose
// last update left |u_{j+1}|^2 as partials (norm_from_update).
int finish_basis(mexk_context_t ctx, int j, bool fp32, cudaStream_t s, bool partials = false) {
    if (!fp32) return MEXK_OK;
    GramArgs g = gram_args(ctx, j, 1);
    if (partials) {
        g.b_blocks = gram_update2_blocks(ctx->n);
        return launch_gram_norm_partials(g, s);
    }
    return launch_gram_norm(g, s);
}

// The cycle's step controller over the k x k Hessenberg (k = m, or the
// breakdown size): the reference's (Pade exponential per attempt) or the
// candidate-step search (with the learned centre for MEXK_CTRL_LEARNED).
int enqueue_controller(mexk_context_t ctx, int m, int ctrl, mexk_step_t* log, cudaStream_t s, int window = 0) {
    if (ctrl == MEXK_CTRL_REFERENCE) {
        ControlArgs c;
        c.st = ctx->d_state;
        c.H = ctx->d_H;
        c.ldh = ctx->ldh;
        c.coef = ctx->d_coef;
        c.log = log;
        c.ws = ctx->d_expm_ws;
        return launch_controller(c, m, s);
    }
    SearchArgs c;
    c.st = ctx->d_state;
    c.H = ctx->d_H;
    c.ldh = ctx->ldh;
    c.coef = ctx->d_coef;
    c.log = log;
    c.cand = ctx->d_cand;
    c.counter = ctx->d_counter + 1;
    c.mlp = ctrl != MEXK_CTRL_LEARNED ? nullptr : (window > 0 && ctx->d_mlp_win) ? ctx->d_mlp_win : ctx->d_mlp;
    c.m_cap = ctx->m_alloc < ctx->n - 1 ? ctx->m_alloc : ctx->n - 1;
    return launch_controller_search(c, m, s);
}

// Whether a basis of m columns runs steps 1..m-1 as one cooperative launch
// (window 2 on a symmetric matrix in the row-pattern form, FP32 basis).
bool use_lanczos_cycle(mexk_context_t ctx, int m, bool fp32, int window) {
    return fp32 && window == 2 && m >= 2 && ctx->lanczos_fused && ctx->spmv_form32 == MEXK_SPMV_PATTERN &&
           lanczos_cycle_fits(ctx->n);
}

int enqueue_lanczos_cycle(mexk_context_t ctx, int m, int reortho, cudaStream_t s) {
    LanczosArgs a;
    a.n = ctx->n;
    a.j0 = 1;
    a.m = m;
    a.ldv = ctx->ldv;
    a.ldh = ctx->ldh;
    a.reortho = reortho ? 1 : 0;
    a.major = ctx->pat_major;
    a.major_len = ctx->pat_major_len;
    a.max_len = ctx->pat_max_len;
    a.npat = 0;
    a.pid = ctx->d_pid;
    a.T = ctx->d_pat;
    a.V = ctx->d_V32;
    a.H = ctx->d_H;
    a.gs = ctx->d_gram;
    a.st = ctx->d_state;
    a.part = ctx->d_gram_part;
    a.b_blocks = gram_update2_blocks(ctx->n);
    a.bar = ctx->d_bar;
    return launch_lanczos_cycle(a, s);
}

// One Krylov cycle: the unit that is captured into a graph.
template <typename TV>
int enqueue_cycle(mexk_context_t ctx, int m, int reortho, int ctrl, int window, cudaStream_t s) {
    const bool fp32 = sizeof(TV) == 4;
    TV* V = fp32 ? reinterpret_cast<TV*>(ctx->d_V32) : reinterpret_cast<TV*>(ctx->d_V);
    int rc;
    // a window's FP64 steps leave H(0:lo-1, j) alone: the cycle starts from zero
    if (!fp32 && window > 0)
        MEXK_CK(cudaMemsetAsync(ctx->d_H, 0, sizeof(double) * static_cast<size_t>(ctx->ldh) * m, s));
    const bool fused = use_lanczos_cycle(ctx, m, fp32, window);
    if (fused) {
        // step 0 as two kernels (its update writes step 1's b and a_0 partials), then the rest in one launch
        if ((rc = enqueue_step(ctx, 0, reortho, fp32, s, window, m))) return rc;
        if ((rc = enqueue_lanczos_cycle(ctx, m, reortho, s))) return rc;
    } else {
        for (int j = 0; j < m; ++j)
            if ((rc = enqueue_step(ctx, j, reortho, fp32, s, window, m))) return rc;
    }
    // the stepwise basis's last update left |u_m|^2 as partials where it could
    if ((rc = finish_basis(ctx, m - 1, fp32, s, !fused && fp32 && norm_from_update(m, window)))) return rc;
    if ((rc = enqueue_controller(ctx, m, ctrl, ctx->d_log, s, window))) return rc;
    const LiftArgs l = lift_args(ctx, fp32);
    if ((rc = launch_lift<TV>(l, gs_grid_size(ctx->n, 1), s))) return rc;
    return launch_restart<TV>(ctx->n, ctx->ldv, ctx->d_y, V, ctx->d_state, s);
}

int enqueue_cycle_any(mexk_context_t ctx, int m, int prec, int reortho, int ctrl, int window, cudaStream_t s) {
    return prec == MEXK_PREC_MIXED ? enqueue_cycle<float>(ctx, m, reortho, ctrl, window, s)
                                   : enqueue_cycle<double>(ctx, m, reortho, ctrl, window, s);
}

int get_graph(mexk_context_t ctx, int m, int prec, int reortho, int ctrl, int window, cudaGraphExec_t* out) {
    for (auto& g : ctx->graphs) {
        if (g.m == m && g.prec == prec && g.reortho == reortho && g.ctrl == ctrl && g.window == window) {
            *out = g.exec;
            return MEXK_OK;
        }
    }
    cudaGraph_t graph = nullptr;
    MEXK_CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    int rc = enqueue_cycle_any(ctx, m, prec, reortho, ctrl, window, ctx->stream);
    cudaError_t e = cudaStreamEndCapture(ctx->stream, &graph);
    if (rc != MEXK_OK) {
        if (graph) cudaGraphDestroy(graph);
        return rc;
    }
    if (e != cudaSuccess) {
        set_cuda_error(e, "cudaStreamEndCapture", __FILE__, __LINE__);
        return MEXK_ERR_CUDA;
    }
    cudaGraphExec_t exec = nullptr;
    e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
        set_cuda_error(e, "cudaGraphInstantiate", __FILE__, __LINE__);
        return MEXK_ERR_CUDA;
    }
    ctx->graphs.push_back({m, prec, reortho, ctrl, window, exec});
    *out = exec;
    return MEXK_OK;
}

void invalidate_graphs(mexk_context_t ctx) {
    cudaStreamSynchronize(ctx->stream);
    for (auto& g : ctx->graphs) cudaGraphExecDestroy(g.exec);
    ctx->graphs.clear();
}

// The reference's TimeSteppingParams defaults for ArnoldiParams
// (ArnoldiRunner constructor, main.cu:1292-1305).
mexk_stepping_t default_stepping(const mexk_params_t* p) {
    mexk_stepping_t ts;
    ts.dt_max = p->t;
    ts.dt_min = std::max(1e-12, p->t * 1e-6);
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
    return ts;
}

void init_state(DevState* st, const mexk_params_t* p, int log_cap) {
    memset(st, 0, sizeof(*st));
    const mexk_stepping_t ts = p->stepping ? *p->stepping : default_stepping(p);
    st->total_t = p->t;
    st->dt_max = ts.dt_max;
    st->dt_min = ts.dt_min;
    const double dt_init = ts.dt_init;
    st->tol = ts.tol_step;
    st->max_steps = ts.max_steps;
    st->max_rejects = ts.max_rejects;
    st->safety = ts.safety;
    st->grow = ts.grow;
    st->shrink = ts.shrink;
    st->adapt_m = (ts.adapt_m && ts.m_step > 0 && ts.m_max > p->m) ? 1 : 0;
    st->m_step = ts.m_step;
    st->m_max = ts.m_max;
    st->m_base = p->m;
    st->m = p->m;
    // compute_expmv (main.cu:1426-1434): clamp, then the first outer iteration's min.
    double dt = std::min(std::max(dt_init, st->dt_min), st->dt_max);
    st->t_done = 0.0;
    st->done = !(st->t_done < st->total_t && 0 < st->max_steps);
    dt = std::min(dt, st->total_t - st->t_done);
    st->dt = dt;
    st->k_used = p->m;
    st->m_next = p->m;
    st->ctrl = p->controller;
    const bool relax = p->controller != MEXK_CTRL_REFERENCE && p->precision == MEXK_PREC_MIXED;
    st->tol_floor_rel = relax ? 5.9604644775390625e-08 : 0.0;  // 2^-24, the FP32 unit roundoff
    st->err_budget_rel = relax ? 5e-7 : 0.0;
    st->log_cap = log_cap;
}

// y_host (optional): y is also copied there, ahead of the final
// synchronisation (one host round trip for the result and the state).
int solve(mexk_context_t ctx, const mexk_params_t* p, const double* v_dev, double* y_dev, cudaStream_t s,
          mexk_result_t* result, double* y_host = nullptr) {
    NvtxRange total_range("total_compute_expmv");
    int rc = check_params(ctx, p);
    if (rc) return rc;
    if (p->precision == MEXK_PREC_MIXED && (rc = ensure_mixed(ctx))) return rc;
    if (s == nullptr) s = ctx->stream;
    ctx->last_window = p->ortho_window;
    ctx->last_controller = p->controller;
    init_state(ctx->h_state, p, LOG_CAP);
    MEXK_CK(cudaMemcpyAsync(ctx->d_state, ctx->h_state, sizeof(DevState), cudaMemcpyHostToDevice, s));
    MEXK_CK(cudaMemsetAsync(ctx->d_bar, 0, sizeof(unsigned int) * 4, s));
    if (ctx->h_state->done) {
        // The reference never lifts when no step runs: y stays zero (main_cpu.cpp:467).
        MEXK_CK(cudaMemsetAsync(ctx->d_y, 0, sizeof(double) * ctx->n, s));
    } else {
        const int grid = gs_grid_size(ctx->n, 1);
        {
            NvtxRange init_range("init_q1");
            if (p->precision == MEXK_PREC_MIXED)
                rc = launch_init_start<float>(ctx->n, ctx->ldv, v_dev, ctx->d_V32, ctx->d_partials, ctx->d_counter,
                                              ctx->d_state, grid, s);
            else
                rc = launch_init_start<double>(ctx->n, ctx->ldv, v_dev, ctx->d_V, ctx->d_partials, ctx->d_counter,
                                               ctx->d_state, grid, s);
        }
        if (rc) return rc;
        if (ctx->use_graph && s != ctx->stream) MEXK_CK(cudaStreamSynchronize(s));
        // Every cycle ends with an accepted step or an abort, or (adapt_m)
        // with a larger basis requested after a reject, at most max_rejects
        // times per step; the extra margin only guards corrupt state.
        const long long per_step = 1 + (ctx->h_state->adapt_m ? ctx->h_state->max_rejects : 0);
        const long long max_cycles = (static_cast<long long>(ctx->h_state->max_steps) + 2) * per_step;
        const int reortho = p->reorthogonalize ? 1 : 0;
        int m_cycle = p->m;
        for (long long cyc = 0; cyc < max_cycles; ++cyc) {
            NvtxRange cycle_range("arnoldi_step_attempt");
            if (ctx->use_graph) {
                // Graphs are captured on the context stream and launched on `s`.
                cudaGraphExec_t exec = nullptr;
                if ((rc = get_graph(ctx, m_cycle, p->precision, reortho, p->controller, p->ortho_window, &exec)))
                    return rc;
                MEXK_CK(cudaGraphLaunch(exec, s));
            } else if ((rc = enqueue_cycle_any(ctx, m_cycle, p->precision, reortho, p->controller, p->ortho_window,
                                               s))) {
                return rc;
            }
            MEXK_CK(cudaMemcpyAsync(ctx->h_state, ctx->d_state, sizeof(DevState), cudaMemcpyDeviceToHost, s));
            MEXK_CK(cudaStreamSynchronize(s));
            if (ctx->h_state->done) break;
            if (ctx->h_state->status & ST_TIMEOUT) {
                set_error_text("a device wait gave up (bulk copy did not complete)");
                return MEXK_ERR_DEVICE;
            }
            const int mn = ctx->h_state->m_next;
            if (mn >= 1 && mn <= ctx->m_alloc && mn < ctx->n) m_cycle = mn;
        }
        if (!ctx->h_state->done) {
            set_error_text("solve did not finish within max_steps cycles");
            return MEXK_ERR_DEVICE;
        }
    }
    if (y_dev != ctx->d_y)
        MEXK_CK(cudaMemcpyAsync(y_dev, ctx->d_y, sizeof(double) * ctx->n, cudaMemcpyDeviceToDevice, s));
    if (y_host != nullptr)
        MEXK_CK(cudaMemcpyAsync(y_host, y_dev, sizeof(double) * ctx->n, cudaMemcpyDeviceToHost, s));
    MEXK_CK(cudaMemcpyAsync(ctx->h_state, ctx->d_state, sizeof(DevState), cudaMemcpyDeviceToHost, s));
    MEXK_CK(cudaStreamSynchronize(s));
    const DevState* st = ctx->h_state;
    if (st->status & ST_TIMEOUT) {
        set_error_text("a device wait gave up (bulk copy did not complete)");
        return MEXK_ERR_DEVICE;
    }
    if (result) {
        result->converged = st->converged;
        result->restarts_done = st->accepted;
        result->last_residual = st->last_residual;
        result->attempts = st->attempts;
        result->cycles = st->cycles;
        result->spmv_count = st->spmv_count;
        result->t_done = st->t_done;
        result->status = st->status;
    }
    return MEXK_OK;
}

}  // namespace

// ====================================================================== C ABI
namespace mexk {

int context_csr_begin(mexk_context_t ctx, int rows, long long nnz, int m_alloc_max, int** d_row_ptr, int** d_col,
                      double** d_val) {
    if (!ctx || rows < 1 || nnz < 0) return MEXK_ERR_INVALID;
    if (ctx->uploaded) return MEXK_ERR_NOT_READY;
    if (m_alloc_max < 1 || m_alloc_max > MEXK_M_MAX) return MEXK_ERR_INVALID;
    MEXK_CK(cudaSetDevice(ctx->device));
    dfree(ctx->d_row_ptr);  // left by an upload that failed
    dfree(ctx->d_col);
    dfree(ctx->d_val);
    ctx->n = rows;
    ctx->nnz = nnz;
    ctx->m_alloc = m_alloc_max;
    // Column stride: a multiple of 64 elements, so every column starts on a
    // 256-byte boundary and the vectorised sweeps cover whole 16-byte groups.
    ctx->ldv = (rows + 63) / 64 * 64;
    ctx->ldh = m_alloc_max + 1;
    int rc;
    // row_ptr, col_idx and values padded (zero tails): the SpMV copies whole
    // 16-byte groups
    if ((rc = dalloc(&ctx->d_row_ptr, static_cast<size_t>(rows) + 8))) return rc;
    MEXK_CK(cudaMemset(ctx->d_row_ptr, 0, sizeof(int) * (static_cast<size_t>(rows) + 8)));
    if ((rc = dalloc(&ctx->d_col, static_cast<size_t>(nnz) + 4))) return rc;
    MEXK_CK(cudaMemset(ctx->d_col + nnz, 0, sizeof(int) * 4));
    if ((rc = dalloc(&ctx->d_val, static_cast<size_t>(nnz) + 4))) return rc;
    MEXK_CK(cudaMemset(ctx->d_val + nnz, 0, sizeof(double) * 4));
    *d_row_ptr = ctx->d_row_ptr;
    *d_col = ctx->d_col;
    *d_val = ctx->d_val;
    return MEXK_OK;
}

int context_stream(mexk_context_t ctx, cudaStream_t* s) {
    MEXK_CK(cudaSetDevice(ctx->device));
    *s = ctx->stream;
    return MEXK_OK;
}

int context_csr_finish(mexk_context_t ctx, const int* row_ptr) {
    int rc;
    dfree(ctx->d_tiles);
    dfree(ctx->d_col16);
    SpmvSchedule sched;
    rc = build_spmv_schedule(ctx->n, row_ptr, ctx->d_col, &sched, ctx->stream);
    ctx->d_tiles = sched.d_tiles;
    ctx->d_col16 = sched.d_col16;
    if (rc) return rc;
    ctx->nblocks = sched.nblocks;
    ctx->spmv_narrow = sched.all_narrow;
    ctx->spmv_form64 = sched.all_narrow ? MEXK_SPMV_STAGED : MEXK_SPMV_DIRECT;
    const int m_alloc_max = ctx->m_alloc;
    const size_t vcount = static_cast<size_t>(ctx->ldv) * (m_alloc_max + 1);
    if ((rc = dalloc(&ctx->d_V, vcount))) return rc;
    MEXK_CK(cudaMemset(ctx->d_V, 0, sizeof(double) * vcount));
    if ((rc = dalloc(&ctx->d_w, ctx->ldv))) return rc;
    if ((rc = dalloc(&ctx->d_y, ctx->ldv))) return rc;
    MEXK_CK(cudaMemset(ctx->d_w, 0, sizeof(double) * ctx->ldv));
    MEXK_CK(cudaMemset(ctx->d_y, 0, sizeof(double) * ctx->ldv));
    const size_t hcount = static_cast<size_t>(ctx->ldh) * m_alloc_max;
    if ((rc = dalloc(&ctx->d_H, hcount))) return rc;
    MEXK_CK(cudaMemset(ctx->d_H, 0, sizeof(double) * hcount));
    if (m_alloc_max > EXPM_SMEM_K && (rc = dalloc(&ctx->d_expm_ws, expm_ws_doubles(m_alloc_max)))) return rc;
    if ((rc = dalloc(&ctx->d_h1, MEXK_M_MAX + 2))) return rc;
    if ((rc = dalloc(&ctx->d_h2, MEXK_M_MAX + 2))) return rc;
    if ((rc = dalloc(&ctx->d_coef, MEXK_M_MAX + 2))) return rc;
    if ((rc = dalloc(&ctx->d_cand, static_cast<size_t>(SEARCH_CAND) * CAND_STRIDE))) return rc;
    if ((rc = dalloc(&ctx->d_partials, static_cast<size_t>(PARTIAL_BLOCKS) * RED_STRIDE))) return rc;
    if ((rc = dalloc(&ctx->d_counter, 4))) return rc;
    MEXK_CK(cudaMemset(ctx->d_counter, 0, sizeof(unsigned int) * 4));
    if ((rc = dalloc(&ctx->d_bar, 4))) return rc;
    MEXK_CK(cudaMemset(ctx->d_bar, 0, sizeof(unsigned int) * 4));
    if ((rc = dalloc(&ctx->d_state, 1))) return rc;
    if ((rc = dalloc(&ctx->d_log, LOG_CAP))) return rc;
    cudaError_t e = cudaMallocHost(reinterpret_cast<void**>(&ctx->h_state), sizeof(DevState));
    if (e != cudaSuccess) {
        set_cuda_error(e, "cudaMallocHost", __FILE__, __LINE__);
        return MEXK_ERR_ALLOC;
    }
    memset(ctx->h_state, 0, sizeof(DevState));
    MEXK_CK(cudaMemcpy(ctx->d_state, ctx->h_state, sizeof(DevState), cudaMemcpyHostToDevice));
    // Row patterns: kept (and the pattern form chosen) when every row is one
    // of at most PAT_MAX patterns.
    dfree(ctx->d_pat);
    dfree(ctx->d_pid);
    const size_t npid = (static_cast<size_t>(ctx->n) + PAT_ROW_ALIGN - 1) / PAT_ROW_ALIGN * PAT_ROW_ALIGN;
    if ((rc = dalloc(&ctx->d_pat, 1))) return rc;
    if ((rc = dalloc(&ctx->d_pid, npid))) return rc;
    MEXK_CK(cudaMemsetAsync(ctx->d_pid, 0, npid, ctx->stream));
    bool pat_ok = false;
    if ((rc = build_row_patterns(ctx->n, ctx->d_row_ptr, ctx->d_col, ctx->d_val, ctx->d_pat, ctx->d_pid,
                                 &ctx->d_state->status, &pat_ok, &ctx->pat_major, &ctx->pat_major_len,
                                 &ctx->pat_max_len, ctx->stream)))
        return rc;
    MEXK_CK(cudaMemsetAsync(&ctx->d_state->status, 0, sizeof(int), ctx->stream));
    MEXK_CK(cudaStreamSynchronize(ctx->stream));
    if (pat_ok) {
        ctx->spmv_form64 = MEXK_SPMV_PATTERN;
    } else {
        dfree(ctx->d_pat);
        dfree(ctx->d_pid);
    }
    ctx->uploaded = true;
    return MEXK_OK;
}

}  // namespace mexk

extern "C" {

const char* mexk_error_string(int code) {
    switch (code) {
        case MEXK_OK: return "ok";
        case MEXK_ERR_INVALID: return "invalid argument";
        case MEXK_ERR_CUDA: return "CUDA runtime error";
        case MEXK_ERR_ALLOC: return "allocation failed";
        case MEXK_ERR_NOT_READY: return "context not ready (upload the matrix first)";
        case MEXK_ERR_DEVICE: return "device reported a failure";
        case MEXK_ERR_UNSUPPORTED: return "unsupported request";
    }
    return "unknown error";
}

const char* mexk_last_error_detail(void) { return g_err.c_str(); }

const char* mexk_version(void) { return "mexk 0.1 sm_103a"; }

int mexk_device_count(int* count) {
    if (!count) return MEXK_ERR_INVALID;
    *count = 0;
    MEXK_CK(cudaGetDeviceCount(count));
    return MEXK_OK;
}

int mexk_context_create(int device, mexk_context_t* out) {
    if (!out) return MEXK_ERR_INVALID;
    *out = nullptr;
    int count = 0;
    MEXK_CK(cudaGetDeviceCount(&count));
    if (device < 0 || device >= count) return MEXK_ERR_INVALID;
    MEXK_CK(cudaSetDevice(device));
    mexk_context_t c = new mexk_context_s();
    c->device = device;
    cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, device);
    const char* ng = getenv("MEXK_NO_GRAPH");
    c->use_graph = !(ng && ng[0] == '1');
    cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        set_cuda_error(e, "cudaStreamCreate", __FILE__, __LINE__);
        delete c;
        return MEXK_ERR_CUDA;
    }
    int rc = expm_init_attributes();
    // without its shared memory the fused Lanczos form stays off (lanczos_cycle_fits says no)
    if (rc == MEXK_OK && lanczos_cycle_prepare() != MEXK_OK) (void)cudaGetLastError();
    gs_prepare();
    if (rc) {
        cudaStreamDestroy(c->stream);
        delete c;
        return rc;
    }
    *out = c;
    return MEXK_OK;
}

int mexk_context_upload_csr(mexk_context_t ctx, int rows, long long nnz, const int* row_ptr, const int* col_idx,
                            const double* values, int m_alloc_max) {
    if (!ctx || rows < 1 || nnz < 0 || !row_ptr || (nnz > 0 && (!col_idx || !values))) return MEXK_ERR_INVALID;
    if (ctx->uploaded) return MEXK_ERR_NOT_READY;
    if (m_alloc_max < 1 || m_alloc_max > MEXK_M_MAX) return MEXK_ERR_INVALID;
    if (row_ptr[0] != 0 || row_ptr[rows] != nnz) {
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
    int *d_rp = nullptr, *d_ci = nullptr;
    double* d_va = nullptr;
    int rc = context_csr_begin(ctx, rows, nnz, m_alloc_max, &d_rp, &d_ci, &d_va);
    if (rc) return rc;
    MEXK_CK(cudaMemcpy(d_rp, row_ptr, sizeof(int) * (rows + 1), cudaMemcpyHostToDevice));
    if (nnz > 0) {
        MEXK_CK(cudaMemcpy(d_ci, col_idx, sizeof(int) * nnz, cudaMemcpyHostToDevice));
        MEXK_CK(cudaMemcpy(d_va, values, sizeof(double) * nnz, cudaMemcpyHostToDevice));
    }
    return context_csr_finish(ctx, row_ptr);
}

int mexk_context_destroy(mexk_context_t ctx) {
    if (!ctx) return MEXK_OK;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    for (auto& g : ctx->graphs) cudaGraphExecDestroy(g.exec);
    dfree(ctx->d_row_ptr);
    dfree(ctx->d_col);
    dfree(ctx->d_val);
    dfree(ctx->d_val32);
    dfree(ctx->d_tiles);
    dfree(ctx->d_col16);
    dfree(ctx->d_pat);
    dfree(ctx->d_pid);
    dfree(ctx->d_V);
    dfree(ctx->d_V32);
    dfree(ctx->d_w);
    dfree(ctx->d_w32);
    dfree(ctx->d_y);
    dfree(ctx->d_H);
    dfree(ctx->d_h1);
    dfree(ctx->d_h2);
    dfree(ctx->d_coef);
    dfree(ctx->d_cand);
    dfree(ctx->d_expm_ws);
    dfree(ctx->d_mlp);
    dfree(ctx->d_mlp_win);
    dfree(ctx->d_partials);
    dfree(ctx->d_gram);
    dfree(ctx->d_gram_part);
    dfree(ctx->d_counter);
    dfree(ctx->d_bar);
    dfree(ctx->d_state);
    dfree(ctx->d_log);
    if (ctx->h_state) cudaFreeHost(ctx->h_state);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return MEXK_OK;
}

void* mexk_context_stream(mexk_context_t ctx) { return ctx ? static_cast<void*>(ctx->stream) : nullptr; }

int mexk_expmv_device(mexk_context_t ctx, const mexk_params_t* p, const double* v_dev, double* y_dev,
                      void* stream, mexk_result_t* result) {
    if (!ctx || !v_dev || !y_dev) return MEXK_ERR_INVALID;
    MEXK_CK(cudaSetDevice(ctx->device));
    return solve(ctx, p, v_dev, y_dev, static_cast<cudaStream_t>(stream), result);
}

int mexk_expmv(mexk_context_t ctx, const mexk_params_t* p, const double* v_host, double* y_host,
               mexk_result_t* result) {
    if (!ctx || !v_host || !y_host) return MEXK_ERR_INVALID;
    int rc = check_params(ctx, p);
    if (rc) return rc;
    MEXK_CK(cudaSetDevice(ctx->device));
    const size_t bytes = sizeof(double) * ctx->n;
    // v goes through the work vector slot w (FP64, length >= n) as staging.
    MEXK_CK(cudaMemcpyAsync(ctx->d_w, v_host, bytes, cudaMemcpyHostToDevice, ctx->stream));
    // The start-vector kernels read v before any cycle overwrites w; y
    // comes back with the solve's final state.
    return solve(ctx, p, ctx->d_w, ctx->d_y, ctx->stream, result, y_host);
}

int mexk_get_steps(mexk_context_t ctx, mexk_step_t* steps, int cap, int* count) {
    if (!ctx || !ctx->uploaded || cap < 0 || (cap > 0 && !steps)) return MEXK_ERR_INVALID;
    MEXK_CK(cudaSetDevice(ctx->device));
    const int avail = std::min(ctx->h_state->nlog, LOG_CAP);
    if (count) *count = ctx->h_state->nlog;
    const int ncopy = std::min(avail, cap);
    if (ncopy > 0)
        MEXK_CK(cudaMemcpy(steps, ctx->d_log, sizeof(mexk_step_t) * ncopy, cudaMemcpyDeviceToHost));
    return MEXK_OK;
}

int mexk_context_set_basis(mexk_context_t ctx, int precision, const double* V_host, int ncols) {
    if (!ctx || !ctx->uploaded || !V_host || ncols < 1 || ncols > ctx->m_alloc + 1) return MEXK_ERR_INVALID;
    MEXK_CK(cudaSetDevice(ctx->device));
    const size_t n = static_cast<size_t>(ctx->n);
    if (precision == MEXK_PREC_FP64) {
        MEXK_CK(cudaMemcpy2D(ctx->d_V, sizeof(double) * ctx->ldv, V_host, sizeof(double) * n, sizeof(double) * n,
                             ncols, cudaMemcpyHostToDevice));
        return MEXK_OK;
    }
    int rc = ensure_mixed(ctx);
    if (rc) return rc;
    std::vector<float> f(n * ncols);
    for (size_t i = 0; i < f.size(); ++i) f[i] = static_cast<float>(V_host[i]);
    MEXK_CK(cudaMemcpy2D(ctx->d_V32, sizeof(float) * ctx->ldv, f.data(), sizeof(float) * n, sizeof(float) * n,
                         ncols, cudaMemcpyHostToDevice));
    // The given columns are taken as orthonormal: unit scales, G = I.
    return reset_gram(ctx, ctx->stream);
}

int mexk_context_get_basis(mexk_context_t ctx, int precision, double* V_host, int ncols) {
    if (!ctx || !ctx->uploaded || !V_host || ncols < 1 || ncols > ctx->m_alloc + 1) return MEXK_ERR_INVALID;
    MEXK_CK(cudaSetDevice(ctx->device));
    const size_t n = static_cast<size_t>(ctx->n);
    if (precision == MEXK_PREC_FP64) {
        MEXK_CK(cudaMemcpy2D(V_host, sizeof(double) * n, ctx->d_V, sizeof(double) * ctx->ldv, sizeof(double) * n,
                             ncols, cudaMemcpyDeviceToHost));
        return MEXK_OK;
    }
    if (!ctx->d_V32) return MEXK_ERR_NOT_READY;
    std::vector<float> f(n * ncols);
    MEXK_CK(cudaMemcpy2D(f.data(), sizeof(float) * n, ctx->d_V32, sizeof(float) * ctx->ldv, sizeof(float) * n,
                         ncols, cudaMemcpyDeviceToHost));
    // Stored columns are the basis vectors up to their scales.
    std::vector<double> sc(GRAM_M + 2);
    MEXK_CK(cudaMemcpy(sc.data(), reinterpret_cast<const char*>(ctx->d_gram) + offsetof(GramState, s),
                       sizeof(double) * sc.size(), cudaMemcpyDeviceToHost));
    for (int c = 0; c < ncols; ++c)
        for (size_t i = 0; i < n; ++i) V_host[c * n + i] = static_cast<double>(f[c * n + i]) * sc[c];
    return MEXK_OK;
}

int mexk_arnoldi_step(mexk_context_t ctx, int j, int reorthogonalize, int precision, double* h, double* beta,
                      int* ok) {
    if (!ctx || !ctx->uploaded || !h || !beta || !ok) return MEXK_ERR_INVALID;
    if (j < 0 || j >= ctx->m_alloc) return MEXK_ERR_INVALID;
    if (precision != MEXK_PREC_FP64 && precision != MEXK_PREC_MIXED) return MEXK_ERR_INVALID;
    MEXK_CK(cudaSetDevice(ctx->device));
    int rc;
    if (precision == MEXK_PREC_MIXED && (rc = ensure_mixed(ctx))) return rc;
    cudaStream_t s = ctx->stream;
    DevState* hs = ctx->h_state;
    memset(hs, 0, sizeof(DevState));
    hs->m = ctx->m_alloc;
    hs->k_used = ctx->m_alloc;
    MEXK_CK(cudaMemcpyAsync(ctx->d_state, hs, sizeof(DevState), cudaMemcpyHostToDevice, s));
    const bool fp32 = precision == MEXK_PREC_MIXED;
    if ((rc = enqueue_step(ctx, j, reorthogonalize, fp32, s))) return rc;
    if ((rc = finish_basis(ctx, j, fp32, s))) return rc;
    std::vector<double> col(static_cast<size_t>(ctx->ldh));
    MEXK_CK(cudaMemcpyAsync(col.data(), ctx->d_H + static_cast<size_t>(j) * ctx->ldh, sizeof(double) * ctx->ldh,
                            cudaMemcpyDeviceToHost, s));
    MEXK_CK(cudaMemcpyAsync(hs, ctx->d_state, sizeof(DevState), cudaMemcpyDeviceToHost, s));
    MEXK_CK(cudaStreamSynchronize(s));
    for (int i = 0; i <= j; ++i) h[i] = col[i];
    *beta = col[j + 1];
    *ok = hs->breakdown ? 0 : 1;
    return MEXK_OK;
}

// ---- stepping: the cycle's pieces driven from the host --------------------
int mexk_krylov_start(mexk_context_t ctx, int precision, const double* v_host, double* beta) {
    if (!ctx || !ctx->uploaded || !v_host || !beta) return MEXK_ERR_INVALID;
    if (precision != MEXK_PREC_FP64 && precision != MEXK_PREC_MIXED) return MEXK_ERR_INVALID;
    MEXK_CK(cudaSetDevice(ctx->device));
    int rc;
    if (precision == MEXK_PREC_MIXED && (rc = ensure_mixed(ctx))) return rc;
    cudaStream_t s = ctx->stream;
    memset(ctx->h_state, 0, sizeof(DevState));
    ctx->h_state->restart = 1;
    MEXK_CK(cudaMemcpyAsync(ctx->d_state, ctx->h_state, sizeof(DevState), cudaMemcpyHostToDevice, s));
    MEXK_CK(cudaMemcpyAsync(ctx->d_y, v_host, sizeof(double) * ctx->n, cudaMemcpyHostToDevice, s));
    const int grid = gs_grid_size(ctx->n, 1);
    rc = precision == MEXK_PREC_MIXED
             ? launch_init_start<float>(ctx->n, ctx->ldv, ctx->d_y, ctx->d_V32, ctx->d_partials, ctx->d_counter,
                                        ctx->d_state, grid, s)
             : launch_init_start<double>(ctx->n, ctx->ldv, ctx->d_y, ctx->d_V, ctx->d_partials, ctx->d_counter,
                                         ctx->d_state, grid, s);
    if (rc) return rc;
    MEXK_CK(cudaMemcpyAsync(ctx->h_state, ctx->d_state, sizeof(DevState), cudaMemcpyDeviceToHost, s));
    MEXK_CK(cudaStreamSynchronize(s));
    *beta = ctx->h_state->v_norm;
    return MEXK_OK;
}

int mexk_krylov_build(mexk_context_t ctx, int precision, int m, int reorthogonalize, double* H, int* k_used) {
    if (!ctx || !ctx->uploaded || !H || !k_used || m < 1 || m > ctx->m_alloc || m >= ctx->n)
        return MEXK_ERR_INVALID;
    if (precision != MEXK_PREC_FP64 && precision != MEXK_PREC_MIXED) return MEXK_ERR_INVALID;
    MEXK_CK(cudaSetDevice(ctx->device));
    int rc;
    if (precision == MEXK_PREC_MIXED && (rc = ensure_mixed(ctx))) return rc;
    cudaStream_t s = ctx->stream;
    DevState* hs = ctx->h_state;
    hs->done = 0;
    hs->breakdown = 0;
    hs->m = m;
    hs->k_used = m;
    MEXK_CK(cudaMemcpyAsync(ctx->d_state, hs, sizeof(DevState), cudaMemcpyHostToDevice, s));
    const bool fp32 = precision == MEXK_PREC_MIXED;
    for (int j = 0; j < m; ++j)
        if ((rc = enqueue_step(ctx, j, reorthogonalize, fp32, s))) return rc;
    if ((rc = finish_basis(ctx, m - 1, fp32, s))) return rc;
    MEXK_CK(cudaMemcpy2DAsync(H, sizeof(double) * (m + 1), ctx->d_H, sizeof(double) * ctx->ldh,
                              sizeof(double) * (m + 1), m, cudaMemcpyDeviceToHost, s));
    MEXK_CK(cudaMemcpyAsync(hs, ctx->d_state, sizeof(DevState), cudaMemcpyDeviceToHost, s));
    MEXK_CK(cudaStreamSynchronize(s));
    *k_used = hs->breakdown ? hs->k_used : m;
    // Entries below the subdiagonal and columns past a breakdown are zero.
    for (int j = 0; j < m; ++j)
        for (int i = 0; i <= m; ++i)
            if (i > j + 1 || j >= *k_used || (i == j + 1 && j == *k_used - 1 && hs->breakdown))
                H[i + static_cast<size_t>(j) * (m + 1)] = 0.0;
    return MEXK_OK;
}

int mexk_krylov_advance(mexk_context_t ctx, int precision, int k, const double* coef, double* beta) {
    if (!ctx || !ctx->uploaded || !coef || !beta || k < 1 || k > ctx->m_alloc + 1) return MEXK_ERR_INVALID;
    if (precision != MEXK_PREC_FP64 && precision != MEXK_PREC_MIXED) return MEXK_ERR_INVALID;
    MEXK_CK(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    DevState* hs = ctx->h_state;
    hs->done = 0;
    hs->lift = 1;
    hs->restart = 1;
    hs->k_lift = k;
    MEXK_CK(cudaMemcpyAsync(ctx->d_state, hs, sizeof(DevState), cudaMemcpyHostToDevice, s));
    MEXK_CK(cudaMemcpyAsync(ctx->d_coef, coef, sizeof(double) * k, cudaMemcpyHostToDevice, s));
    const bool fp32 = precision == MEXK_PREC_MIXED;
    if (fp32 && !ctx->d_V32) return MEXK_ERR_NOT_READY;
    const LiftArgs l = lift_args(ctx, fp32);
    int rc = fp32 ? launch_lift<float>(l, gs_grid_size(ctx->n, 1), s)
                  : launch_lift<double>(l, gs_grid_size(ctx->n, 1), s);
    if (rc) return rc;
    rc = fp32 ? launch_restart<float>(ctx->n, ctx->ldv, ctx->d_y, ctx->d_V32, ctx->d_state, s)
              : launch_restart<double>(ctx->n, ctx->ldv, ctx->d_y, ctx->d_V, ctx->d_state, s);
    if (rc) return rc;
    MEXK_CK(cudaMemcpyAsync(hs, ctx->d_state, sizeof(DevState), cudaMemcpyDeviceToHost, s));
    MEXK_CK(cudaStreamSynchronize(s));
    *beta = hs->v_norm;
    return MEXK_OK;
}

int mexk_krylov_result(mexk_context_t ctx, double* y_host) {
    if (!ctx || !ctx->uploaded || !y_host) return MEXK_ERR_INVALID;
    MEXK_CK(cudaSetDevice(ctx->device));
    MEXK_CK(cudaMemcpy(y_host, ctx->d_y, sizeof(double) * ctx->n, cudaMemcpyDeviceToHost));
    return MEXK_OK;
}

int mexk_context_set_controller(mexk_context_t ctx, const float* weights, int count) {
    if (!ctx || !weights || count != 4886) {
        set_error_text("controller network must have 4886 parameters");
        return MEXK_ERR_INVALID;
    }
    MEXK_CK(cudaSetDevice(ctx->device));
    int rc;
    if (!ctx->d_mlp && (rc = dalloc(&ctx->d_mlp, static_cast<size_t>(count)))) return rc;
    MEXK_CK(cudaMemcpy(ctx->d_mlp, weights, sizeof(float) * count, cudaMemcpyHostToDevice));
    return MEXK_OK;
}

int mexk_context_set_window_controller(mexk_context_t ctx, const float* weights, int count) {
    if (!ctx || !weights || count != 4886) {
        set_error_text("controller network must have 4886 parameters");
        return MEXK_ERR_INVALID;
    }
    MEXK_CK(cudaSetDevice(ctx->device));
    if (!ctx->d_mlp_win) {
        int rc;
        if ((rc = dalloc(&ctx->d_mlp_win, static_cast<size_t>(count)))) return rc;
        invalidate_graphs(ctx);  // captured window cycles hold the other network's address
    }
    MEXK_CK(cudaMemcpy(ctx->d_mlp_win, weights, sizeof(float) * count, cudaMemcpyHostToDevice));
    return MEXK_OK;
}

int mexk_context_get_spmv_form(mexk_context_t ctx, int precision, int* form) {
    if (!ctx || !ctx->uploaded || !form) return MEXK_ERR_INVALID;
    if (precision != MEXK_PREC_FP64 && precision != MEXK_PREC_MIXED) return MEXK_ERR_INVALID;
    int rc;
    if (precision == MEXK_PREC_MIXED) {
        MEXK_CK(cudaSetDevice(ctx->device));
        if ((rc = ensure_mixed(ctx))) return rc;
    }
    *form = precision == MEXK_PREC_MIXED ? ctx->spmv_form32 : ctx->spmv_form64;
    return MEXK_OK;
}

int mexk_context_set_spmv_form(mexk_context_t ctx, int precision, int form) {
    if (!ctx || !ctx->uploaded) return MEXK_ERR_INVALID;
    if (precision != MEXK_PREC_FP64 && precision != MEXK_PREC_MIXED) return MEXK_ERR_INVALID;
    if (form != MEXK_SPMV_STAGED && form != MEXK_SPMV_DIRECT && form != MEXK_SPMV_PATTERN) return MEXK_ERR_INVALID;
    if (form == MEXK_SPMV_PATTERN && !ctx->d_pat) {
        set_error_text("spmv form: the matrix has no row-pattern form (a row longer than 16 or > 256 patterns)");
        return MEXK_ERR_UNSUPPORTED;
    }
    int rc;
    if (precision == MEXK_PREC_MIXED) {
        MEXK_CK(cudaSetDevice(ctx->device));
        if ((rc = ensure_mixed(ctx))) return rc;  // its default must not undo the choice later
        ctx->spmv_form32 = form;
    } else {
        ctx->spmv_form64 = form;
    }
    // captured cycle graphs hold the other form's launches
    invalidate_graphs(ctx);
    return MEXK_OK;
}

int mexk_context_get_lanczos_form(mexk_context_t ctx, int* form) {
    if (!ctx || !ctx->uploaded || !form) return MEXK_ERR_INVALID;
    MEXK_CK(cudaSetDevice(ctx->device));
    int rc;
    if ((rc = ensure_mixed(ctx))) return rc;  // the mixed SpMV form is set there
    const bool applies = ctx->d_pat != nullptr && lanczos_cycle_fits(ctx->n) && ctx->spmv_form32 == MEXK_SPMV_PATTERN;
    *form = (ctx->lanczos_fused && applies) ? MEXK_LANCZOS_FUSED : MEXK_LANCZOS_STEPWISE;
    return MEXK_OK;
}

int mexk_context_set_lanczos_form(mexk_context_t ctx, int form) {
    if (!ctx || !ctx->uploaded) return MEXK_ERR_INVALID;
    if (form != MEXK_LANCZOS_STEPWISE && form != MEXK_LANCZOS_FUSED) return MEXK_ERR_INVALID;
    MEXK_CK(cudaSetDevice(ctx->device));
    ctx->lanczos_fused = form == MEXK_LANCZOS_FUSED;
    invalidate_graphs(ctx);  // captured cycles hold the other form's launches
    return MEXK_OK;
}

int mexk_profile_kernel(mexk_context_t ctx, int kind, int precision, int j, int iters, double* ms_per_launch) {
    if (!ctx || !ctx->uploaded || !ms_per_launch || iters < 1) return MEXK_ERR_INVALID;
    if (kind < 0 || kind >= MEXK_KERNEL_KINDS || j < 0 || j >= ctx->m_alloc) return MEXK_ERR_INVALID;
    if (precision != MEXK_PREC_FP64 && precision != MEXK_PREC_MIXED) return MEXK_ERR_INVALID;
    MEXK_CK(cudaSetDevice(ctx->device));
    int rc;
    if (precision == MEXK_PREC_MIXED && (rc = ensure_mixed(ctx))) return rc;
    const bool fp32 = precision == MEXK_PREC_MIXED;
    cudaStream_t s = ctx->stream;
    // A running state: k = j+1 basis columns, lift pending, nothing finished.
    DevState run;
    memset(&run, 0, sizeof(run));
    // The last solve's step size and norm (its H is still in place when the
    // controller is profiled before the Gram-Schmidt kernels).
    run.total_t = 1.0;
    run.dt = (ctx->h_state->dt > 0.0) ? ctx->h_state->dt : 1e-3;
    run.dt_max = 1.0;
    run.dt_min = 1e-12;
    run.tol = 1e300;  // every controller launch accepts its first attempt: one exponential
    run.v_norm = (ctx->h_state->v_norm > 0.0) ? ctx->h_state->v_norm : 1.0;
    run.m = j + 1;
    run.max_steps = 1 << 30;
    run.max_rejects = 20;
    run.safety = 0.8;
    run.grow = 1.5;
    run.shrink = 0.5;
    run.m_base = j + 1;
    run.k_used = j + 1;
    run.k_lift = j + 1;
    run.lift = 1;
    run.inv_beta = 1.0;
    run.log_cap = 0;
    DevState* h_run = nullptr;
    MEXK_CK(cudaMallocHost(reinterpret_cast<void**>(&h_run), sizeof(DevState)));
    *h_run = run;
    cudaEvent_t e0, e1;
    MEXK_CK(cudaEventCreate(&e0));
    MEXK_CK(cudaEventCreate(&e1));
    const GsArgs g = gs_args(ctx, j, 1, false);
    GramArgs ga = fp32 ? gram_args(ctx, j, 1) : GramArgs{};
    ga.lo = (fp32 && ctx->last_window > 0) ? std::max(0, j + 1 - ctx->last_window) : 0;
    const int grid = gs_grid_size(ctx->n, j + 1);
    double total = 0.0;
    rc = MEXK_OK;
    // One launch of the kind (rc: its status).
    auto launch_one = [&]() -> int {
        int r = MEXK_OK;
        switch (kind) {
            case MEXK_KERNEL_SPMV:
                r = context_spmv(ctx, j, fp32, nullptr, s);
                break;
            case MEXK_KERNEL_GS_DOT:
            case MEXK_KERNEL_GS_UPD_DOT:
            case MEXK_KERNEL_GS_UPD_NORM: {
                const GsMode mode = kind == MEXK_KERNEL_GS_DOT ? GS_DOT
                                    : kind == MEXK_KERNEL_GS_UPD_DOT ? GS_UPD_DOT
                                                                       : GS_UPD_NORM;
                r = fp32 ? MEXK_ERR_UNSUPPORTED : launch_gs<double>(mode, g, grid, s);
                break;
            }
            case MEXK_KERNEL_NORMALIZE:
                r = fp32 ? MEXK_ERR_UNSUPPORTED
                          : launch_normalize<double>(ctx->n, j, ctx->ldv, ctx->d_w, ctx->d_V, ctx->d_state, nullptr, s);
                break;
            case MEXK_KERNEL_GRAM_DOT:
                r = fp32 ? launch_gram_dot(ga, s) : MEXK_ERR_UNSUPPORTED;
                break;
            case MEXK_KERNEL_GRAM_UPDATE: {
                GramArgs gu = ga;  // as in a solve: b partials for a fused next step
                gu.write_b = (j + 1 < ctx->m_alloc && fused_step(j + 1, ctx->last_window)) ? 1 : 0;
                gu.sym = (ctx->last_window == 2 && ctx->spmv_form32 == MEXK_SPMV_PATTERN) ? 1 : 0;
                r = fp32 ? launch_gram_update(gu, s) : MEXK_ERR_UNSUPPORTED;
                break;
            }
            case MEXK_KERNEL_SPMV_DOTS: {
                if (!fp32 || !fused_step(j, ctx->last_window) || ctx->spmv_form32 == MEXK_SPMV_DIRECT) {
                    r = MEXK_ERR_UNSUPPORTED;
                    break;
                }
                GramArgs gd = ga;
                gd.b_blocks = gram_update2_blocks(ctx->n);
                gd.sym = (ctx->last_window == 2 && ctx->spmv_form32 == MEXK_SPMV_PATTERN) ? 1 : 0;
                r = context_spmv(ctx, j, true, nullptr, s, &gd);
                break;
            }
            case MEXK_KERNEL_GRAM_NORM:
                r = fp32 ? launch_gram_norm(ga, s) : MEXK_ERR_UNSUPPORTED;
                break;
            case MEXK_KERNEL_LANCZOS_CYCLE:
                // steps 1..j from the context's basis columns 0 and 1 (their
                // inputs stay untouched: launches repeat the same work)
                r = (fp32 && j >= 1 && use_lanczos_cycle(ctx, j + 1, true, ctx->last_window))
                        ? enqueue_lanczos_cycle(ctx, j + 1, 1, s)
                        : MEXK_ERR_UNSUPPORTED;
                break;
            case MEXK_KERNEL_LIFT: {
                const LiftArgs l = lift_args(ctx, fp32);
                r = fp32 ? launch_lift<float>(l, gs_grid_size(ctx->n, 1), s)
                          : launch_lift<double>(l, gs_grid_size(ctx->n, 1), s);
                break;
            }
            case MEXK_KERNEL_CONTROLLER:
                r = enqueue_controller(ctx, j + 1, ctx->last_controller, nullptr, s, ctx->last_window);
                break;
        }
        return r;
    };
    auto timed = [&](int count, double* ms_out) -> int {
        cudaError_t ce = cudaEventRecord(e0, s);
        int r = ce == cudaSuccess ? MEXK_OK : MEXK_ERR_CUDA;
        for (int k = 0; k < count && r == MEXK_OK; ++k) r = launch_one();
        if (r != MEXK_OK) return r;
        ce = cudaEventRecord(e1, s);
        if (ce == cudaSuccess) ce = cudaEventSynchronize(e1);
        float ms = 0.f;
        if (ce == cudaSuccess) ce = cudaEventElapsedTime(&ms, e0, e1);
        if (ce != cudaSuccess) {
            set_cuda_error(ce, "profile timing", __FILE__, __LINE__);
            return MEXK_ERR_CUDA;
        }
        *ms_out = ms;
        return MEXK_OK;
    };
    // Kinds that leave their inputs as they were (the SpMVs, the mixed
    // sweeps, the FP64 pass-1 dots) are timed as a back-to-back run of iters
    // launches (one event pair, as the launches follow one another in a
    // solve's graph) after one untimed launch. The others change the running
    // state or update w in place (controller, lift, the FP64 update passes,
    // normalise): each launch starts from a fresh copy of the state.
    const bool reset_each = !(kind == MEXK_KERNEL_SPMV || kind == MEXK_KERNEL_SPMV_DOTS ||
                              kind == MEXK_KERNEL_GRAM_DOT || kind == MEXK_KERNEL_GRAM_UPDATE ||
                              kind == MEXK_KERNEL_GRAM_NORM || kind == MEXK_KERNEL_GS_DOT ||
                              kind == MEXK_KERNEL_LANCZOS_CYCLE);
    if (reset_each) {
        for (int it = 0; it < iters && rc == MEXK_OK; ++it) {
            cudaError_t ce = cudaMemcpyAsync(ctx->d_state, h_run, sizeof(DevState), cudaMemcpyHostToDevice, s);
            if (ce != cudaSuccess) {
                set_cuda_error(ce, "profile setup", __FILE__, __LINE__);
                rc = MEXK_ERR_CUDA;
                break;
            }
            double ms = 0.0;
            rc = timed(1, &ms);
            total += ms;
        }
    } else {
        cudaError_t ce = cudaMemcpyAsync(ctx->d_state, h_run, sizeof(DevState), cudaMemcpyHostToDevice, s);
        if (ce != cudaSuccess) {
            set_cuda_error(ce, "profile setup", __FILE__, __LINE__);
            rc = MEXK_ERR_CUDA;
        }
        if (rc == MEXK_OK) rc = launch_one();
        if (rc == MEXK_OK) rc = timed(iters, &total);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFreeHost(h_run);
    if (rc == MEXK_OK) *ms_per_launch = total / iters;
    return rc;
}

}  // extern "C"
