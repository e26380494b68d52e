/*
 * mexk -- C ABI of the GB300 (sm_103a) restarted-Arnoldi exp(t*A)*v library.
 *
 * Plain pointers and sizes only. "Device" pointers are CUDA device addresses
 * on the context's device; "host" pointers are ordinary host memory.
 * Streams are passed as void* (a cudaStream_t; NULL = the context's own
 * stream for context calls, the legacy default stream for the free kernel
 * calls). Every function returns MEXK_OK or a MEXK_ERR_* code and never
 * exits the process; mexk_error_string() explains a code and
 * mexk_last_error_detail() gives the last failing CUDA call.
 *
 * The reference (kol-di/matrix-exp-krylov) has no library or FFI layer: its
 * solver is C++ classes compiled into main.cu. Each entry point below names
 * the reference code it replaces (file:line in that project).
 */
#ifndef MEXK_H
#define MEXK_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MEXK_OK 0
#define MEXK_ERR_INVALID 1     /* bad argument */
#define MEXK_ERR_CUDA 2        /* a CUDA runtime call failed */
#define MEXK_ERR_ALLOC 3       /* device or pinned allocation failed */
#define MEXK_ERR_NOT_READY 4   /* call order violated (e.g. expmv before upload) */
#define MEXK_ERR_DEVICE 5      /* the device reported a failure status */
#define MEXK_ERR_UNSUPPORTED 6 /* valid request this build does not handle */

/* Arithmetic of the Krylov basis and matrix values. */
#define MEXK_PREC_FP64 0  /* plain method: everything FP64 (the reference's path) */
#define MEXK_PREC_MIXED 1 /* A values, basis V_m and SpMV/Gram-Schmidt in FP32;
                             Hessenberg, norms, Pade and residual in FP64 */

/* Step-size control. */
#define MEXK_CTRL_REFERENCE 0 /* the reference's accept/reject heuristic (main.cu:1476-1516) */
#define MEXK_CTRL_SEARCH 1    /* per basis, the largest of 32 candidate steps whose
                                 residual estimate passes; reference heuristic if none.
                                 With MEXK_PREC_MIXED the FP32 basis cannot resolve a
                                 truncation error below its rounding of the current
                                 iterate y, so a step may also pass with
                                 err <= min(2^-24 |y|, 5e-7 |y| - E), E the sum of
                                 the errors already accepted: the accepted errors of
                                 a solve never add up to more than 5e-7 of the
                                 iterate's norm (beyond what tol itself allows) */
#define MEXK_CTRL_LEARNED 2   /* SEARCH centred on an MLP's step prediction, with the
                                 MLP also choosing the next cycle's Krylov dimension
                                 (at least half of the current one, rounded up to a
                                 multiple of 5, at most the allocation) */

/* Largest Krylov dimension m: MEXK_M_MAX for the plain method (FP64 and the
 * reference controller, the reference's ArnoldiParams default m = 100 among
 * them); MEXK_M_MAX_MIXED for mixed precision and the candidate-step
 * controllers, whose Gram matrix and candidate exponentials are held on chip. */
#define MEXK_M_MAX 128
#define MEXK_M_MAX_MIXED 64

/* Time-stepping parameters: the reference's TimeSteppingParams
 * (main.cu:1237-1250), read by compute_expmv on every solve (main.cu:1426,
 * 1476-1516). The step is accepted when err <= tol_step (or on breakdown);
 * an accepted step with err < 0.1 tol_step grows dt to
 * min(dt * grow * safety, dt_max); a rejected one either raises the Krylov
 * dimension by m_step (adapt_m, up to m_max) or shrinks dt to
 * max(dt * shrink * safety, dt_min); max_rejects rejects in a row abort the
 * solve and at most max_steps steps are accepted. */
typedef struct {
    double dt_init, dt_min, dt_max, tol_step;
    int max_steps, max_rejects;
    double safety, grow, shrink;
    int adapt_m, m_max, m_step;
} mexk_stepping_t;

/* Solver parameters. Mirrors ArnoldiParams (main.cu:1221-1230) plus the
 * precision choice. stepping = NULL derives the time-stepping parameters
 * from m, t, tol and max_restarts as the ArnoldiRunner constructor does
 * (main.cu:1292-1305). */
typedef struct {
    int m;               /* Krylov dimension, 1 <= m <= MEXK_M_MAX (MEXK_M_MAX_MIXED for
                            mixed precision or a candidate-step controller), m < n */
    double t;            /* total time */
    double tol;          /* per-step tolerance on the residual estimate */
    int max_restarts;    /* > 0: dt_init = t/max_restarts and at most that many
                            accepted steps; <= 0: dt_init = t, cap 1000 */
    int reorthogonalize; /* nonzero: second Gram-Schmidt pass (CLI always on) */
    int precision;       /* MEXK_PREC_* */
    int controller;      /* MEXK_CTRL_*: step-size control (0 = the reference's) */
    int ortho_window;    /* 0: orthogonalise against the whole basis (Arnoldi, the
                            reference's method). W >= 2 (symmetric A only, either
                            precision): against the last W basis vectors, the short
                            recurrence of Lanczos (FP64: CGS2 over the window); the
                            context verifies symmetry (MEXK_ERR_INVALID otherwise).
                            No reference counterpart. */
    const mexk_stepping_t* stepping; /* NULL: the defaults above. Otherwise used as
                            given with the reference controller; the candidate-step
                            controllers take dt_min, dt_max, tol_step, max_steps and
                            max_rejects from it and choose steps and m themselves.
                            adapt_m needs m_max <= the context's m_alloc_max. */
} mexk_params_t;

/* Outcome of one solve. converged / restarts_done / last_residual are the
 * reference's ArnoldiRunner public fields (main.cu:1258-1260). */
typedef struct {
    int converged;
    int restarts_done;    /* accepted time steps */
    double last_residual;
    int attempts;         /* accepted + rejected attempts ([STEP] lines) */
    int cycles;           /* Arnoldi basis builds (rejected attempts reuse the basis) */
    long long spmv_count; /* sparse products performed */
    double t_done;        /* time reached */
    int status;           /* device status bits, 0 = clean */
} mexk_result_t;

/* One accept/reject attempt: the fields of the reference's [STEP] line
 * (main.cu:1471-1474), and the Krylov dimension the attempt's basis was
 * built for (m_current of main.cu:1435; m_used is smaller after a breakdown),
 * which sizes the reference's "H_m column" lines (main.cu:1951). */
typedef struct {
    double t_done, dt, err;
    int m_used, accepts, rejects;
    int m_basis;
} mexk_step_t;

typedef struct mexk_context_s* mexk_context_t;

/* ---- library ---------------------------------------------------------- */
const char* mexk_error_string(int code);
/* Text of the last CUDA failure seen by this thread (empty if none). */
const char* mexk_last_error_detail(void);
/* Build identification, e.g. "mexk 0.1 sm_103a". */
const char* mexk_version(void);
/* Number of CUDA devices visible (cudaGetDeviceCount, main.cu:2146). */
int mexk_device_count(int* count);

/* ---- device context: replaces DeviceContext (main.cu:747-1125) -------- */
/* DeviceContext(dev_id) + init_handles() + create_streams()
 * (main.cu:806-868): selects the device and creates the context's stream. */
int mexk_context_create(int device, mexk_context_t* out);

/* DeviceContext::alloc_from + create_descriptors (main.cu:873-1067):
 * copies the CSR matrix (rows x rows, int32 indices, FP64 values, host
 * memory) to the device, allocates the basis for Krylov dimensions up to
 * m_alloc_max and builds the SpMV row-block schedule. The reference's
 * on/off-diagonal split and ghost buffers do not exist on one device.
 * Call once per context. */
int mexk_context_upload_csr(mexk_context_t ctx, int rows, long long nnz, const int* row_ptr,
                            const int* col_idx, const double* values, int m_alloc_max);

/* DeviceContext::destroy (main.cu:1069-1124). Safe on NULL. */
int mexk_context_destroy(mexk_context_t ctx);

/* The context's CUDA stream (a cudaStream_t). */
void* mexk_context_stream(mexk_context_t ctx);

/* ---- the hot path: ArnoldiRunner::compute_expmv (main.cu:1411-1571) ---- */
/* y = exp(t*A)*v with host vectors of length rows. Copies v in, runs the
 * whole restarted-Arnoldi solve on the device (basis build, fused
 * Gram-Schmidt, Pade exponential, accept/reject control, lift, restart)
 * and copies y out. result may be NULL. */
int mexk_expmv(mexk_context_t ctx, const mexk_params_t* p, const double* v_host, double* y_host,
               mexk_result_t* result);

/* Same with device vectors (FP64, length rows) on `stream` (NULL = the
 * context stream). Returns after the solve finished on the device. */
int mexk_expmv_device(mexk_context_t ctx, const mexk_params_t* p, const double* v_dev,
                      double* y_dev, void* stream, mexk_result_t* result);

/* Attempt log of the last solve ([STEP] lines). Writes up to cap entries,
 * *count = number available (may exceed cap). */
int mexk_get_steps(mexk_context_t ctx, mexk_step_t* steps, int cap, int* count);

/* ---- individual kernels (device pointers), for tests and composition -- */
/* w = A*x, CSR FP64 (replaces cusparseSpMV, main.cu:1722-1767). */
int mexk_spmv_f64(int rows, const int* row_ptr, const int* col_idx, const double* values,
                  const double* x, double* y, void* stream);
/* w = A*x with FP32 values and vectors, FP32 products and accumulation. */
int mexk_spmv_f32(int rows, const int* row_ptr, const int* col_idx, const float* values,
                  const float* x, float* y, void* stream);

/* One Arnoldi step j on the context's matrix: w = A*V[:,j], two
 * Gram-Schmidt passes (replaces orthogonalize_mgs, main.cu:1769-1876) and
 * normalisation with the breakdown test (normalize_new_vector,
 * main.cu:1878-1942). V is the context's FP64 basis, set with
 * mexk_context_set_basis. On return h[0..j] = H(0..j, j), *beta = H(j+1,j)
 * (0 on breakdown), *ok = 1 unless breakdown. Host outputs. */
int mexk_arnoldi_step(mexk_context_t ctx, int j, int reorthogonalize, int precision, double* h,
                      double* beta, int* ok);
/* Copy columns 0..ncols-1 of the context basis to/from host (column-major,
 * leading dimension rows) in the given precision's storage. */
int mexk_context_set_basis(mexk_context_t ctx, int precision, const double* V_host, int ncols);
int mexk_context_get_basis(mexk_context_t ctx, int precision, double* V_host, int ncols);

/* ---- Binary CSR v1 files ---------------------------------------------- */
typedef struct {
    long long rows, cols, nnz;
    int index_dtype;    /* 1 = u32, 2 = u64 */
    int value_dtype;    /* 1 = f32, 2 = f64 */
    unsigned int flags; /* bit 0 sorted, bit 1 no duplicates, bit 2 symmetric upper */
    int checks_passed;  /* load: 1 header, 2 indptr, 3 column range, 4 sorted / no-duplicate flags */
    double max_abs;     /* max |a_ij| over the entries (NaN skipped); set by the load */
    double seconds;     /* wall time of the load */
} mexk_bincsr_info_t;

/* Reads and checks the 64-byte header of a .bincsr file on the host (no
 * device work), with the checks and messages of CSRHost::from_binary_csr
 * (main.cu:265-330): MEXK_ERR_INVALID and mexk_last_error_detail() text on
 * failure. */
int mexk_bincsr_probe(const char* path, mexk_bincsr_info_t* info);

/* Loads a .bincsr file straight into the context (replaces
 * CSRHost::from_binary_csr + DeviceContext::alloc_from, main.cu:265-523 and
 * 873-1067, for a square matrix). The file is memory-mapped and streamed to
 * the device through pinned buffers; u64 indices are narrowed and f32 values
 * widened there, and the reference loader's checks (indptr, column range,
 * sorted / no-duplicate flags) run there too, reporting its first failure
 * with its message (MEXK_ERR_INVALID). Files with the symmetric_upper flag,
 * and non-square or empty matrices, return MEXK_ERR_UNSUPPORTED: CSRHost
 * loads them on the host (and the runner reports what it cannot solve). */
int mexk_context_load_bincsr(mexk_context_t ctx, const char* path, int m_alloc_max, mexk_bincsr_info_t* info);

/* E = exp(A) for a k-by-k FP64 matrix (device pointers, column-major,
 * leading dimensions lda/lde), single thread block Pade scaling-and-squaring
 * (replaces Eigen's MatrixXd::exp at main.cu:33-36). k <= MEXK_M_MAX. */
int mexk_expm_f64(int k, const double* A, int lda, double* E, int lde, void* stream);

/* ---- stepping: one cycle's pieces driven from the host ----------------- */
/* These expose the solve's steps for callers that choose steps themselves
 * (the learned controller's training sweeps). Host vectors/matrices.
 * start:   V[:,0] = v/|v| (init_q1, main.cu:1574); *beta = |v|.
 * build:   m Arnoldi steps from V[:,0] (the loop of main.cu:1451-1466);
 *          H receives the (m+1)-by-m Hessenberg matrix (column-major, ld m+1),
 *          *k_used the basis size (< m after a breakdown).
 * advance: y = sum_{i<k} coef[i] V[:,i] (the lift, main.cu:1980-2001, with
 *          coef = |v| exp(dt H_k) e1 computed by the caller), then V[:,0] =
 *          y/|y| (restart_from_y, main.cu:2023); *beta = |y|.
 * result:  copies the last y. */
int mexk_krylov_start(mexk_context_t ctx, int precision, const double* v_host, double* beta);
int mexk_krylov_build(mexk_context_t ctx, int precision, int m, int reorthogonalize, double* H, int* k_used);
int mexk_krylov_advance(mexk_context_t ctx, int precision, int k, const double* coef, double* beta);
int mexk_krylov_result(mexk_context_t ctx, double* y_host);

/* ---- learned step controller ----------------------------------------- */
/* Parameters of the controller network (8 -> 64 -> 64 -> 2, GELU, FP32):
 * W1[8][64], b1[64], W2[64][64], b2[64], W3[64][2], b3[2] (4866 trained
 * values) followed by feature mean[8], std[8], output mean[2], std[2]. */
#define MEXK_NET_PARAMS 4866
#define MEXK_NET_TOTAL 4886

/* Loads the network used by MEXK_CTRL_LEARNED (host array of
 * MEXK_NET_TOTAL floats). No reference counterpart (the reference's
 * controller is the fixed heuristic of main.cu:1476-1516). */
int mexk_context_set_controller(mexk_context_t ctx, const float* weights, int count);

/* Loads a second network, used by MEXK_CTRL_LEARNED for solves with a
 * short-recurrence window (ortho_window > 0, symmetric A), whose cycles cost
 * about linearly in m where full Gram-Schmidt cycles cost quadratically:
 * the two are trained on different cycle prices. Without it those solves use
 * the mexk_context_set_controller network. Same layout and count. */
int mexk_context_set_window_controller(mexk_context_t ctx, const float* weights, int count);

/* Network on N raw feature rows X[N][8] -> raw outputs Y[N][2] (device). */
int mexk_mlp_forward(const float* weights, const float* X, int N, float* Y, void* stream);
/* Gradient of the mean squared error of the normalised outputs over the
 * samples idx[0..count) of X[.][8] / T[.][2] into grad[MEXK_NET_PARAMS];
 * loss_parts receives 64 partial sums of squared errors; scratch holds
 * 64 * MEXK_NET_PARAMS floats. All device memory. */
int mexk_mlp_gradient(const float* weights, const float* X, const float* T, const int* idx, int count,
                      float* grad, float* loss_parts, float* scratch, void* stream);
/* One Adam step (beta 0.9/0.999, eps 1e-8, step >= 1) on the same loss;
 * adam_state holds 2 * MEXK_NET_PARAMS floats (zero before step 1). */
int mexk_mlp_adam_step(float* weights, float* adam_state, const float* X, const float* T, const int* idx,
                       int count, int step, float lr, float* loss_parts, float* scratch, void* stream);
/* The controller's view of a basis: out[0..7] = features of H (device,
 * leading dimension ldh >= k+1, 1 <= k <= MEXK_M_MAX_MIXED, the bases the
 * learned controller sees), out[8..9] = network outputs (0 if weights is
 * NULL), out[10] = log2 |H_k|_1. */
int mexk_controller_predict(const float* weights, const double* H, int ldh, int k, double rem, double tol,
                            double vnorm, double tau_prev, double err_prev, float* out, void* stream);

/* ---- allocation-free variant ------------------------------------------- */
/* Orthonormalises w against the k orthonormal FP64 columns of V (column-major,
 * leading dimension ldv) with the solver's Gram-Schmidt sweeps (two passes if
 * reorthogonalize, else one) and normalises it, without allocating anything:
 * for callers that cannot call cudaMalloc (a host that owns all device memory
 * through its own pool, an FFI runtime that only passes buffers, a request
 * path that must not allocate). All pointers are device memory of the current
 * device, and `stream` (NULL = the legacy default stream) must belong to that
 * device (MEXK_ERR_INVALID otherwise): on return (in stream order) h[0..k-1]
 * = V^T w summed over the passes, *beta = |w - V h| (0 on breakdown: norm <
 * 1e-14, NaN or Inf), q[0..n-1] = (w - V h) / beta (left untouched on
 * breakdown), and w holds the orthogonalised, unnormalised vector. Limits:
 * 1 <= k <= 64 (larger k: MEXK_ERR_INVALID); any n >= 1, the sweeps' grid
 * being capped at 1024 thread blocks (they stride over the rows). The
 * kernels' reduction scratch is a fixed 592 KB array in the library's device
 * memory, shared by all calls on a device; it keeps the last call's contents
 * (each call clears what must start at zero), so calls that overlap on the
 * GPU race and must be serialised. Every call looks up the array's device
 * address on the current device (cudaGetSymbolAddress); the first lookup on a
 * device loads the library's device code, so make the first call before any
 * stream capture. No counterpart in the reference: it orthogonalises only
 * inside orthogonalize_mgs with cuBLAS. */
int mexk_gram_schmidt_f64_noalloc(int n, int k, const double* V, int ldv, double* w,
                                  int reorthogonalize, double* h, double* beta, double* q,
                                  void* stream);

/* ---- batched solves ---------------------------------------------------- */
/* Many independent problems -- a CSR matrix, a time t and a block of up to
 * MEXK_BATCH_RHS right-hand sides each -- solved together in mixed
 * precision (FP32 matrix values and Krylov bases, FP64 Hessenberg, Gram
 * matrix, exponentials and results), every (problem, rhs) pair by the
 * reference method and step controller (ArnoldiRunner::compute_expmv,
 * main.cu:1411-1571) with its own step size. The reference solves one vector
 * per process; the batch has no reference counterpart beyond that method.
 * Problems are laid out in one row space and advanced in waves whose bases
 * fit the basis budget; one cycle of a wave is one CUDA graph launch. As for
 * MEXK_CTRL_SEARCH in mixed precision, a step of a right-hand side also
 * passes with err <= min(2^-24 |y|, 5e-7 |y| - E) (|y| its current iterate,
 * E its accepted errors so far): the FP32 bases do not resolve errors below
 * their rounding of y. */
#define MEXK_BATCH_RHS 16
#define MEXK_BATCH_M_MAX 32
typedef struct mexk_batch_s* mexk_batch_t;
typedef struct {
    int m;                 /* Krylov dimension, 1..MEXK_BATCH_M_MAX, < every problem's rows */
    double tol;            /* absolute a-posteriori error per accepted step, as ArnoldiParams::tol */
    int max_restarts;      /* as mexk_params_t.max_restarts */
    int reorthogonalize;
    long long basis_bytes; /* device memory for one wave's bases; 0 = 60% of the free memory at upload */
    int autotune;          /* 1 = choose the tile and sweep schedule by timing candidates on the first wave */
} mexk_batch_params_t;
typedef struct {
    int problems;
    int waves;
    int tile_rows;         /* rows per reduction tile */
    int dot_columns;       /* basis columns per block of the dot sweep */
    int spmm_unroll;       /* x gathers the SpMM issues together per row */
    int cycles;            /* graph launches over all waves in the last run */
    long long rows;        /* padded rows of the whole batch */
    long long nnz;
    double tune_ms;        /* time spent timing candidate schedules */
} mexk_batch_info_t;

/* Creates an empty batch for `device`; touches no device until upload. */
int mexk_batch_create(int device, const mexk_batch_params_t* p, mexk_batch_t* out);
/* Adds problem *index: CSR (int32, 0-based, rows x rows), time t and nrhs
 * (1..16) start vectors V, row-major rows x nrhs (V[i*nrhs + r]). The
 * arrays are read again by mexk_batch_upload and must stay valid until it
 * returns. Invalid input returns MEXK_ERR_INVALID (CSRHost checks,
 * main.cu:394-522). */
int mexk_batch_add(mexk_batch_t b, int rows, const int* row_ptr, const int* col_idx, const double* values,
                   double t, int nrhs, const double* V, int* index);
/* Copies every problem to the device, lays out the row space and plans the waves. */
int mexk_batch_upload(mexk_batch_t b);
/* Solves every (problem, rhs); may be called again (restarts from the start vectors). */
int mexk_batch_run(mexk_batch_t b);
/* Y: rows x nrhs row-major; results: nrhs entries (may be null). */
int mexk_batch_result(mexk_batch_t b, int problem, double* Y, mexk_result_t* results);
int mexk_batch_info(mexk_batch_t b, mexk_batch_info_t* info);
/* Times `iters` launches of one per-step kernel of the first wave at step j
 * with the schedule in use (after a run): kind 0 SpMM, 1 dot sweep (timing
 * only, states untouched), 2 update sweep. *ms_per_launch and the wave's
 * rows / nonzeros (for byte counts) are returned. */
int mexk_batch_profile(mexk_batch_t b, int kind, int j, int iters, double* ms_per_launch, long long* wave_rows,
                       long long* wave_nnz);
int mexk_batch_destroy(mexk_batch_t b);

/* ---- measurement ------------------------------------------------------ */
#define MEXK_KERNEL_SPMV 0
#define MEXK_KERNEL_GS_DOT 1      /* FP64: pass-1 dots */
#define MEXK_KERNEL_GS_UPD_DOT 2  /* FP64: pass-1 update fused with pass-2 dots */
#define MEXK_KERNEL_GS_UPD_NORM 3 /* FP64: pass-2 update + norm */
#define MEXK_KERNEL_NORMALIZE 4   /* FP64 */
#define MEXK_KERNEL_LIFT 5
#define MEXK_KERNEL_CONTROLLER 6   /* the step controller of the context's last solve */
#define MEXK_KERNEL_GRAM_DOT 7    /* mixed: dots with w and the newest column, Gram correction */
#define MEXK_KERNEL_GRAM_UPDATE 8 /* mixed: streaming update into the next column */
#define MEXK_KERNEL_GRAM_NORM 9   /* mixed: norm of the last column (once per basis) */
#define MEXK_KERNEL_SPMV_DOTS 10  /* mixed, steps j >= 1 over two columns: SpMV + the step's dots and finish */
#define MEXK_KERNEL_LANCZOS_CYCLE 11 /* mixed, window 2, fused form: steps 1..j of a basis in one launch */
#define MEXK_KERNEL_KINDS 12

/* Times `iters` launches of one solver kernel for Arnoldi step j (k = j+1
 * basis columns) on the context stream with CUDA events, on the context's
 * current basis and matrix (run a solve first), from a fresh running state:
 * the kinds whose launch leaves its inputs unchanged (SpMV, SpMV with dots,
 * the mixed sweeps, the FP64 pass-1 dots) run one untimed launch, then the
 * iters launches back to back between one event pair, as they follow one
 * another in a solve; the others (controller, lift, FP64 update passes,
 * normalise) get a fresh copy of the state and an event pair each.
 * *ms_per_launch = mean launch duration in milliseconds. No reference counterpart (the reference
 * times only the whole solve, METRIC total_compute_expmv_ms at main.cu:1570).
 * A kind marked FP64 or mixed returns MEXK_ERR_UNSUPPORTED for the other
 * precision. The mixed sweeps use the ortho_window, and the controller kind
 * the controller, of the context's last solve. */
int mexk_profile_kernel(mexk_context_t ctx, int kind, int precision, int j, int iters, double* ms_per_launch);

/* Which form of the context SpMV runs for a precision:
 * MEXK_SPMV_STAGED (persistent blocks, CSR row blocks staged into shared
 * memory by bulk copies), MEXK_SPMV_DIRECT (one block per CSR row block,
 * loads straight from HBM) or MEXK_SPMV_PATTERN (one byte per row naming one
 * of at most 256 distinct rows -- offsets col - row and values, at most 16
 * entries -- held in a table: stencil matrices). The staged and the pattern
 * form also accumulate the mixed two-column steps' dot products. At upload
 * the context picks the pattern form when every row is one of at most 256
 * such patterns (detected and verified on the device), else direct when
 * some row block's columns span 65,536 or more (gathers scattered over x,
 * where more blocks in flight keep more gathers outstanding), else staged;
 * the setter overrides that (MEXK_ERR_UNSUPPORTED: pattern form requested
 * for a matrix without one). All forms compute the same products and add
 * each row's in column order, so FP64 solves are bitwise equal under any;
 * mixed solves take the two-column steps' dots in a form-dependent order and
 * agree to rounding. No reference counterpart: the reference's SpMV is one
 * cuSPARSE call (main.cu:1743). */
#define MEXK_SPMV_STAGED 0
#define MEXK_SPMV_DIRECT 1
#define MEXK_SPMV_PATTERN 2
int mexk_context_get_spmv_form(mexk_context_t ctx, int precision, int* form);
int mexk_context_set_spmv_form(mexk_context_t ctx, int precision, int form);

/* How a short-recurrence basis (ortho_window = 2, mixed precision, a
 * symmetric matrix in the row-pattern SpMV form) runs its steps 1..m-1:
 * MEXK_LANCZOS_FUSED as one cooperative launch in which one thread block
 * per SM keeps its rows' ids and A u_j on chip and the blocks meet at two
 * bounded grid barriers per step; MEXK_LANCZOS_STEPWISE (the default) as two
 * launches per step (the SpMV with the step's dot products, the update).
 * The fused form applies when every block's rows fit its shared memory
 * (about 7 million rows on a 152-SM GB300); get reports the form a solve
 * would run. Both compute the same row sums and updates and sum the dot
 * products in different orders: solves agree to rounding. No reference
 * counterpart. */
#define MEXK_LANCZOS_STEPWISE 0
#define MEXK_LANCZOS_FUSED 1
int mexk_context_get_lanczos_form(mexk_context_t ctx, int* form);
int mexk_context_set_lanczos_form(mexk_context_t ctx, int form);

/* ---- testing hooks ------------------------------------------------------ */
/* enable != 0: from now on, thread block 0 of the staged CSR SpMV also waits
 * (1 ms limit) on a barrier that nothing arrives at, so its bounded wait runs
 * out: it drains its bulk copies in flight and sets the timeout status bit;
 * and thread block 0 of the fused Lanczos cycle leaves before its first grid
 * barrier, so the other blocks' bounded waits (1 s) run out. Either way the
 * solve returns MEXK_ERR_DEVICE and the context stays usable. enable = 0
 * restores normal operation. For failure-path tests only: it changes no
 * result of a solve that uses neither form. No reference counterpart (the
 * reference has no bounded device waits). */
int mexk_test_force_wait_timeout(int device, int enable);

#ifdef __cplusplus
}
#endif

#endif /* MEXK_H */
