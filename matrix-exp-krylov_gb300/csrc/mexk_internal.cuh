// Internal declarations shared by the mexk CUDA translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "mexk.h"

namespace mexk {

// ------------------------------------------------------------ errors
void set_cuda_error(cudaError_t e, const char* what, const char* file, int line);
void set_error_text(const std::string& s);

#define MEXK_CK(call)                                                   \
    do {                                                                \
        cudaError_t e_ = (call);                                        \
        if (e_ != cudaSuccess) {                                        \
            ::mexk::set_cuda_error(e_, #call, __FILE__, __LINE__);      \
            return MEXK_ERR_CUDA;                                       \
        }                                                               \
    } while (0)

#define MEXK_CK_LAUNCH(what)                                            \
    do {                                                                \
        cudaError_t e_ = cudaGetLastError();                            \
        if (e_ != cudaSuccess) {                                        \
            ::mexk::set_cuda_error(e_, what, __FILE__, __LINE__);       \
            return MEXK_ERR_CUDA;                                       \
        }                                                               \
    } while (0)

// ------------------------------------------------------------ device state
// Scalar state of one solve, resident in device memory. The controller
// fields follow ArnoldiRunner::compute_expmv (main.cu:1411-1571) and
// TimeSteppingParams (main.cu:1237-1250).
struct DevState {
    double total_t, t_done, dt, dt_min, dt_max, tol;
    double v_norm;        // |start vector| of the current segment
    double last_residual;
    double inv_beta;      // 1 / H(j+1, j) of the current Arnoldi step
    double restart_scale; // 1 / |y| (or 1) for the restart
    int m;
    int max_steps;
    int max_rejects;
    int accepted;
    int k_used;     // basis size of the cycle being built
    int k_lift;     // basis size used by the lift of the finished cycle
    int breakdown;  // set by the normalisation of the current cycle
    int done;       // solve finished (converged or not)
    int restart;    // the finished cycle was accepted and the solve goes on
    int converged;
    int status;     // error bits (0 = clean)
    int attempts;
    int cycles;
    int nlog;
    int log_cap;
    int lift;       // the finished cycle's lift is pending
    long long spmv_count;
    // step-size search / learned controller
    int ctrl;       // MEXK_CTRL_* of this solve
    int m_next;     // Krylov dimension of the next cycle
    double tau_prev;
    double err_prev;
    // Candidate-step control in FP32 storage does not resolve the truncation
    // error below the basis precision: a step also passes with
    // err <= min(tol_floor_rel*|v|, err_budget_rel*|v| - err_acc), |v| the
    // current iterate's norm and err_acc the errors accepted so far.
    double tol_floor_rel;
    double tol_base;  // the caller's tolerance (batch: tol is raised per segment from it)
    double err_budget_rel;
    double err_acc;
    // TimeSteppingParams (main.cu:1237-1250) as the caller set them.
    double safety, grow, shrink;
    int adapt_m, m_max, m_step;
    int m_base;     // ArnoldiParams::m: the Krylov dimension each step starts from
    int rejects;    // rejects of the current step carried across basis rebuilds (adapt_m)
};

// Status bits written by kernels.
enum : int {
    ST_LU_SINGULAR = 1,
    ST_SMEM = 2,
    ST_BAD_K = 4,
    ST_TIMEOUT = 8,  // a bounded wait gave up (the kernel skipped its work)
    ST_NONFINITE = 16,  // an exponential met Inf or NaN entries (non-finite input)
};

// ------------------------------------------------------------ constants
constexpr int SPMV_THREADS = 256;
constexpr int SPMV_TILE = 2048;     // nonzeros staged per row block
constexpr int SPMV_TILE_ROWS = 512; // rows per row block
constexpr int SEQ_ROW_MAX = 64;     // longest row summed by one thread (reference order)
constexpr int GS_THREADS = 256;
constexpr int RED_STRIDE = 72;      // doubles per block partial (>= GS_DOT_COLS + 2)
constexpr int GS_DOT_COLS = 64;     // basis columns one FP64 dot sweep reduces (larger k: column chunks)
constexpr int GS_MAX_GRID = 4096;   // largest grid of a Gram-Schmidt sweep (partials hold 4096 blocks)

// ------------------------------------------------------------ helpers
// Programmatic dependent launch: a kernel launched with launch_dependent()
// may start while the previous kernel of the stream finishes; it calls
// pdl_wait() before reading anything that kernel wrote, and the previous
// kernel calls pdl_trigger() once its blocks no longer need the launch held
// back. Both are no-ops for ordinary launches.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <typename... KArgs, typename... Args>
cudaError_t launch_dependent(void (*kernel)(KArgs...), int grid, int block, size_t smem, cudaStream_t s,
                             Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block-wide sum, result valid in thread 0. `scratch` holds >= 32 values.
template <typename T>
__device__ __forceinline__ T block_sum(T v, T* scratch) {
    v = warp_sum(v);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) scratch[warp] = v;
    __syncthreads();
    T s = 0;
    if (threadIdx.x == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        for (int i = 0; i < nw; ++i) s += scratch[i];
    }
    __syncthreads();
    return s;
}

// 16-byte row-group loads: RPT consecutive rows of one basis column.
template <int RPT, typename TV>
struct RowIO;
template <>
struct RowIO<1, double> {
    static __device__ __forceinline__ void ld(const double* p, double (&o)[1]) { o[0] = *p; }
    static __device__ __forceinline__ void ldg(const double* p, double (&o)[1]) { o[0] = __ldg(p); }
    static __device__ __forceinline__ void ldcs(const double* p, double (&o)[1]) { o[0] = __ldcs(p); }
    static __device__ __forceinline__ void st(double* p, const double (&o)[1]) { *p = o[0]; }
};
template <>
struct RowIO<2, double> {
    static __device__ __forceinline__ void put(const double2 t, double (&o)[2]) {
        o[0] = t.x;
        o[1] = t.y;
    }
    static __device__ __forceinline__ void ld(const double* p, double (&o)[2]) {
        put(*reinterpret_cast<const double2*>(p), o);
    }
    static __device__ __forceinline__ void ldg(const double* p, double (&o)[2]) {
        put(__ldg(reinterpret_cast<const double2*>(p)), o);
    }
    static __device__ __forceinline__ void ldcs(const double* p, double (&o)[2]) {
        put(__ldcs(reinterpret_cast<const double2*>(p)), o);
    }
    static __device__ __forceinline__ void st(double* p, const double (&o)[2]) {
        *reinterpret_cast<double2*>(p) = make_double2(o[0], o[1]);
    }
};
template <>
struct RowIO<1, float> {
    static __device__ __forceinline__ void ld(const float* p, float (&o)[1]) { o[0] = *p; }
    static __device__ __forceinline__ void ldg(const float* p, float (&o)[1]) { o[0] = __ldg(p); }
    static __device__ __forceinline__ void ldcs(const float* p, float (&o)[1]) { o[0] = __ldcs(p); }
    static __device__ __forceinline__ void st(float* p, const float (&o)[1]) { *p = o[0]; }
};
template <>
struct RowIO<4, float> {
    static __device__ __forceinline__ void put(const float4 t, float (&o)[4]) {
        o[0] = t.x;
        o[1] = t.y;
        o[2] = t.z;
        o[3] = t.w;
    }
    static __device__ __forceinline__ void ld(const float* p, float (&o)[4]) {
        put(*reinterpret_cast<const float4*>(p), o);
    }
    static __device__ __forceinline__ void ldg(const float* p, float (&o)[4]) {
        put(__ldg(reinterpret_cast<const float4*>(p)), o);
    }
    static __device__ __forceinline__ void ldcs(const float* p, float (&o)[4]) {
        put(__ldcs(reinterpret_cast<const float4*>(p)), o);
    }
    static __device__ __forceinline__ void st(float* p, const float (&o)[4]) {
        *reinterpret_cast<float4*>(p) = make_float4(o[0], o[1], o[2], o[3]);
    }
};

// Last-block-done handshake for grid reductions: every block has written its
// partials; returns true in exactly one block (the last to arrive), which
// then sees all partials. The counter is reset by that block. The block
// barrier orders every thread's writes before thread 0's release, and
// release and acquire are cumulative, so one thread per block synchronises
// (as a cooperative grid barrier does) rather than all of them.
__device__ __forceinline__ bool grid_last_block(unsigned int* counter, int* smem_flag) {
    __syncthreads();
    if (threadIdx.x == 0) {
        // one acquire-release atomic: releases this block's partials, and in the
        // last block acquires every other block's
        unsigned int ticket;
        asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], 1;" : "=r"(ticket) : "l"(counter) : "memory");
        const bool last = ticket == gridDim.x - 1;
        if (last) *counter = 0u;
        *smem_flag = last ? 1 : 0;
    }
    __syncthreads();
    return *smem_flag != 0;
}

// Deterministic reduction of partials[b * RED_STRIDE + c] over blocks
// b < nblocks for columns c < ncols by one block; out[c] in thread order.
// Uses up to blockDim.x threads; scratch holds blockDim.x doubles.
__device__ __forceinline__ void reduce_partials(const double* partials, int nblocks, int ncols,
                                                double* out_smem, double* scratch) {
    int groups = blockDim.x / (ncols > 0 ? ncols : 1);
    if (groups < 1) groups = 1;
    // power-of-two-free: thread t handles column c = t % ncols, group g = t / ncols
    const int t = threadIdx.x;
    const int c = t % ncols;
    const int g = t / ncols;
    double s = 0.0;
    if (g < groups) {
        // four independent running sums (their loads overlap), fixed combination order
        double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
        int b = g;
        for (; b + 3 * groups < nblocks; b += 4 * groups) {
            s0 += __ldcg(&partials[(size_t)b * RED_STRIDE + c]);
            s1 += __ldcg(&partials[(size_t)(b + groups) * RED_STRIDE + c]);
            s2 += __ldcg(&partials[(size_t)(b + 2 * groups) * RED_STRIDE + c]);
            s3 += __ldcg(&partials[(size_t)(b + 3 * groups) * RED_STRIDE + c]);
        }
        for (; b < nblocks; b += groups) s0 += __ldcg(&partials[(size_t)b * RED_STRIDE + c]);
        s = (s0 + s1) + (s2 + s3);
    }
    scratch[t] = s;
    __syncthreads();
    if (t < ncols) {
        double tot = 0.0;
        for (int q = 0; q < groups; ++q) tot += scratch[q * ncols + t];
        out_smem[t] = tot;
    }
    __syncthreads();
}

// ------------------------------------------------------------ SpMV
// Row-block schedule: rows [blocks[b], blocks[b+1]) form block b. A block
// holds <= tile nonzeros and <= tile_rows rows, or one longer row.
std::vector<int> build_row_blocks(int n, const int* row_ptr, int tile = SPMV_TILE, int tile_rows = SPMV_TILE_ROWS);
// The context SpMV's schedule, on the device: d_tiles[b] = {first row, first
// nonzero, offset of the block's 16-bit columns in d_col16 or -1, their base}
// (b <= nblocks), and the 16-bit column copy of the blocks whose columns span
// <= 65536 (made by a kernel from the device columns d_col; row_ptr is the
// host copy). The caller owns (cudaFree) d_tiles and d_col16.
struct SpmvSchedule {
    int nblocks = 0;
    int4* d_tiles = nullptr;
    uint16_t* d_col16 = nullptr;
    bool all_narrow = true;  // every staged row block has 16-bit columns
};
int build_spmv_schedule(int n, const int* row_ptr, const int* d_col, SpmvSchedule* out, cudaStream_t s);

// Row-pattern form of the context SpMV (spmv_pattern.cu): pattern p has
// len[p] <= PAT_LEN entries, column offsets off[p * PAT_LEN + q] (col - row,
// ascending) and values v64 / v32 (the FP32 copy rounded to nearest); row r
// is pattern pid[r]. keys / ids: the detection's hash table.
constexpr int PAT_MAX = 256;
constexpr int PAT_LEN = 16;
constexpr int PAT_SLOTS = 1024;
constexpr int PAT_ROW_ALIGN = 1024;  // pid is padded with zeros to a multiple of this
struct RowPatterns {
    unsigned long long keys[PAT_SLOTS];
    int ids[PAT_SLOTS];
    int count;
    int rows[PAT_MAX];  // rows of each pattern
    int len[PAT_MAX];
    int off[PAT_MAX * PAT_LEN];
    double v64[PAT_MAX * PAT_LEN];
    float v32[PAT_MAX * PAT_LEN];
};
// Detects the patterns of the device CSR (d_pid: n rounded up to
// PAT_ROW_ALIGN bytes, zero-filled by the caller); *ok when every row is one
// of at most PAT_MAX patterns of at most PAT_LEN entries; *major = the
// pattern with the most rows, *major_len its length, *max_len the longest
// pattern's. Synchronises s.
int build_row_patterns(int n, const int* d_row_ptr, const int* d_col, const double* d_val, RowPatterns* d_T,
                       uint8_t* d_pid, int* d_flags, bool* ok, int* major, int* major_len, int* max_len,
                       cudaStream_t s);

// Upload stages shared by mexk_context_upload_csr and the .bincsr loader:
// begin sets the sizes and allocates the context's CSR arrays (padded, zero
// tails); the caller fills row_ptr[0..rows], col_idx and values; finish
// builds the SpMV schedule from the device columns (row_ptr: the host copy)
// and allocates the solver's buffers.
int context_csr_begin(mexk_context_t ctx, int rows, long long nnz, int m_alloc_max, int** d_row_ptr, int** d_col,
                      double** d_val);
int context_csr_finish(mexk_context_t ctx, const int* row_ptr);
// Makes the context's device current; *s = its stream.
int context_stream(mexk_context_t ctx, cudaStream_t* s);

int launch_narrow_values(const double* src, float* dst, size_t count, cudaStream_t s);
// *ok = 1 when A equals its transpose exactly, else 0.
int launch_symmetric_check(int n, const int* row_ptr, const int* col_idx, const double* values, int* ok,
                           cudaStream_t s);

// Context SpMV over the schedule build_spmv_schedule made (tiles, col16 on
// the device). col16, col_idx, values and row_ptr are 16-byte aligned; col_idx and values have at least 3 readable
// entries past nnz, row_ptr at least n + 4 entries (row blocks are copied in
// whole 16-byte groups). A bulk copy that never completes sets ST_TIMEOUT in
// *status after a bounded wait; skip_flag (may be null) skips the product.
struct GramArgs;
// dots (FP32, a step j >= 1 over columns j-1 and j): the SpMV also
// accumulates that step's a = U^T w and |w|^2 and its last block finishes the
// step (the b partials come from the previous step's update, write_b).
// direct: the unstaged form, one thread block per row block (no dots).
template <typename TA, typename TX>
int launch_spmv(int n, int nblocks, const int4* tiles, const uint16_t* col16, bool all_narrow, const int* row_ptr,
                const int* col_idx, const TA* values, const TX* x, TX* y, const int* skip_flag, int* status,
                cudaStream_t s, const GramArgs* dots = nullptr, bool direct = false);
// w = A x in the pattern form; dots as for launch_spmv (FP32 only).
template <typename TX>
int launch_spmv_pattern(int n, int major, int major_len, int max_len, const uint8_t* pid, const RowPatterns* T,
                        const TX* x, TX* y, const int* skip_flag, cudaStream_t s, const GramArgs* dots = nullptr);

// ------------------------------------------------------------ Gram-Schmidt
enum GsMode : int { GS_DOT = 0, GS_UPD_DOT = 1, GS_UPD_NORM = 2 };

struct GsArgs {
    int n;
    int k;            // number of basis columns involved (j+1): the update sweeps use all
    int c0 = 0;       // the dot sweep reduces columns c0 .. c0+kd-1 (kd <= GS_DOT_COLS)
    int kd = 0;       //   (kd = 0: all k columns)
    int pass2 = 0;    // GS_DOT on a chunk of the second pass: results into h2 and H = h1 + h2
    int h_row0 = 0;   // V's first column is basis column h_row0 (a short-recurrence window):
                      //   the dots go to H rows h_row0.., the norm to H(j+1, j)
    int j;            // Arnoldi step (column of H)
    int ldv;          // basis leading dimension (elements)
    int ldh;          // H leading dimension
    int reortho;      // second pass enabled
    const void* V;    // basis, column-major, TV elements
    void* w;          // work vector, TV elements
    double* H;        // Hessenberg, column-major ldh x m
    double* h1;       // first-pass coefficients (k)
    double* h2;       // second-pass coefficients (k)
    double* partials; // grid partials
    unsigned int* counter;
    // Steps over <= 2 columns whose dot products the SpMV accumulates: the
    // update of step j also writes step j+1's b partials (write_b), over
    // b_blocks row blocks (the count step j+1's finish reads).
    int write_b = 0;
    int b_blocks = 0;
    DevState* st;     // may be null (standalone use): no flags read/written
    double* beta_out; // standalone use: |w| after the last pass
};

template <typename TV>
int launch_gs(GsMode mode, const GsArgs& a, int grid, cudaStream_t s);
// The FP64 CGS2 sweeps of one step (pass-1 dots, pass-1 update + pass-2
// dots, pass-2 update + norm); with more than GS_DOT_COLS columns the dots
// are reduced in column chunks, one launch each.
int launch_gs_step(const GsArgs& a, int grid, cudaStream_t s);
int gs_grid_size(int n, int k);
void gs_prepare();

template <typename TV>
int launch_normalize(int n, int j, int ldv, const TV* w, TV* V, const DevState* st,
                     const double* inv_beta, cudaStream_t s);

// ------------------------------------------------------------ Gram-corrected sweeps (FP32 basis)
// Column c of the FP32 basis stores u_c; the basis vector is v_c = s[c] * u_c.
constexpr int GRAM_M = MEXK_M_MAX_MIXED;    // largest Krylov dimension of the FP32 basis
constexpr int GRAM_LD = GRAM_M + 1;         // leading dimension of G
// partial slots: a [0,64), b [64,128), |w|^2 128; the fused Lanczos cycle's
// banks from 136 (lanczos_cycle.cu)
constexpr int GRAM_SLOTS = 2 * GRAM_M + 8 + 10;
constexpr int GRAM_BOFF = GRAM_M;
constexpr int GRAM_NWOFF = 2 * GRAM_M;
constexpr int GRAM_MAX_ROW_BLOCKS = 1024;
struct GramState {
    double G[GRAM_LD * GRAM_LD];  // Gram matrix V^T V (unit diagonal), column-major
    double s[GRAM_M + 2];     // column scales 1/|u_c|
    double ip[GRAM_M + 2];    // 1 / (pre-scale applied when column c was written)
    float coef[GRAM_M + 8];   // update coefficients s_c h_c of the current step
    float wsc, psc;               // update: u_{j+1} = psc * (wsc * w - sum coef_c u_c)
    // the part of a step's scalar chain from the previous update's partials
    // (step2_precompute): s_j, s_j^2, H(j, j-1), G(j-1, j), c_{j-1}, breakdown
    double pre[6];
};
struct GramArgs {
    int n, j, ldv, ldh, reortho;
    int lo = 0;        // first basis column of the step (0: all; j+1-W for a window of W)
    float* V;          // FP32 basis, column-major, ldv >= 4*ceil(n/4), rows n..ldv-1 zero
    const float* w;    // A u_j (unscaled), rows n..ldv-1 zero
    double* H;
    GramState* gs;
    double* part;      // GRAM_SLOTS x GRAM_MAX_ROW_BLOCKS: slot v of row block b at v * GRAM_MAX_ROW_BLOCKS + b
    unsigned int* counter;
    // Steps over <= 2 columns whose dot products the SpMV accumulates: the
    // update of step j also writes step j+1's b partials (write_b), over
    // b_blocks row blocks (the count step j+1's finish reads).
    int write_b = 0;
    int b_blocks = 0;
    // Symmetric A (a window of 2): u_{j-1}.(A u_j) = (A u_{j-1}).u_j, so the
    // update of step j-1, which holds w_{j-1} = A u_{j-1} and u_j, also writes
    // step j's a_{j-1} partials (into a slot j-1 over b_blocks row blocks) and
    // the SpMV of step j reads no u_{j-1}. sym on the update: write them; on
    // the SpMV with dots: read them.
    int sym = 0;
    DevState* st;
};
int device_sm_count();
int launch_gram_dot(const GramArgs& a, cudaStream_t s);
int launch_gram_update(const GramArgs& a, cudaStream_t s);
// Row blocks of the update sweep of a step over <= 2 columns (its b partials).
int gram_update2_blocks(int n);
// |u_{j+1}| -> H(j+1, j) and s[j+1] (the last step of a basis, or a single step).
int launch_gram_norm(const GramArgs& a, cudaStream_t s);
// The same from the |u_{j+1}|^2 partials of the last two-column update
// (write_b; a.b_blocks row blocks): one block, no sweep.
int launch_gram_norm_partials(const GramArgs& a, cudaStream_t s);

// Steps j0..m-1 of a Lanczos basis (window 2, symmetric A in the row-pattern
// form, FP32 basis) in one cooperative launch (lanczos_cycle.cu): per step
// the SpMV with its dot products, a grid barrier, the step's finish in every
// block, the update, a grid barrier. Step j0's b and a_{j0-1} partials come
// from the update of step j0-1 (over b_blocks row blocks). bar: three words
// (arrival count, abort flag, generation), zero before the first launch;
// the barriers leave them as they found them unless a wait gave up. Returns MEXK_ERR_UNSUPPORTED when the
// matrix's row blocks do not fit the kernel's shared memory.
struct LanczosArgs {
    int n, j0, m, ldv, ldh, reortho;
    int major, major_len, max_len, npat;
    const uint8_t* pid;
    const RowPatterns* T;
    float* V;
    double* H;
    GramState* gs;
    DevState* st;
    double* part;
    int b_blocks;
    unsigned* bar;
};
bool lanczos_cycle_fits(int n);
int lanczos_cycle_prepare();
int launch_lanczos_cycle(const LanczosArgs& a, cudaStream_t s);
// mexk_test_force_wait_timeout's part for the fused cycle (current device).
int lanczos_cycle_test_hook(int enable);

// ------------------------------------------------------------ expm / control
// Raises the dynamic shared-memory limits of the expm kernels; call once
// per device before any launch or stream capture.
int expm_init_attributes();
// Largest k whose Pade matrices fit in shared memory; larger k (up to
// MEXK_M_MAX) work in a global-memory workspace of expm_ws_doubles(k) doubles.
constexpr int EXPM_SMEM_K = 64;
size_t expm_ws_doubles(int k);
int launch_expm_standalone(int k, const double* A, int lda, double* E, int lde, int* status, double* ws,
                           cudaStream_t s);

struct ControlArgs {
    DevState* st;
    const double* H;
    int ldh;
    double* coef;       // lift coefficients (k+1)
    mexk_step_t* log;   // attempt log (log_cap entries)
    size_t h_stride = 0;     // batch: state b uses st + b, H + b*h_stride,
    size_t coef_stride = 0;  //        coef + b*coef_stride (no log)
    double* ws = nullptr;    // expm_ws_doubles(m) doubles of global memory for k > EXPM_SMEM_K
};
// One thread block per state (nstates > 1: a batch of independent solves).
int launch_controller(const ControlArgs& a, int m, cudaStream_t s, int nstates = 1);

// Candidate-step controller: one thread block per candidate step.
constexpr int SEARCH_CAND = 32;
constexpr int CAND_STRIDE = MEXK_M_MAX_MIXED + 2;  // err, tau, w_0..w_{k-1}
struct SearchArgs {
    DevState* st;
    const double* H;
    int ldh;
    double* coef;
    mexk_step_t* log;
    double* cand;           // SEARCH_CAND x CAND_STRIDE
    unsigned int* counter;
    const float* mlp;       // controller network weights, or null
    int m_cap;              // largest Krylov dimension the network may choose
};
int launch_controller_search(const SearchArgs& a, int m, cudaStream_t s);

// ------------------------------------------------------------ lift / restart
struct LiftArgs {
    int n, ldv;
    const void* V;
    const double* coef;
    double* y;
    double* partials;
    unsigned int* counter;
    // Steps over <= 2 columns whose dot products the SpMV accumulates: the
    // update of step j also writes step j+1's b partials (write_b), over
    // b_blocks row blocks (the count step j+1's finish reads).
    int write_b = 0;
    int b_blocks = 0;
    DevState* st;
    const double* scale = nullptr;  // per-column scale of the stored basis (FP32 basis)
};
template <typename TV>
int launch_lift(const LiftArgs& a, int grid, cudaStream_t s);
template <typename TV>
int launch_restart(int n, int ldv, const double* y, TV* V, const DevState* st, cudaStream_t s);

// Start vector: |v| by grid reduction, then V[:,0] = v * scale. The first
// kernel also initialises the controller fields.
template <typename TV>
int launch_init_start(int n, int ldv, const double* v, TV* V, double* partials,
                      unsigned int* counter, DevState* st, int grid, cudaStream_t s);

}  // namespace mexk
