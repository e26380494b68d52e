// K2: Gram-Schmidt sweeps over the Krylov basis, with the Hessenberg column
// and the normalisation written on the device.
//
// Replaces orthogonalize_mgs (reference main.cu:1769-1876: per basis vector
// a cublasDdot, an NCCL allreduce, a negate kernel, a cublasDaxpy and a D2H
// copy, twice) and normalize_new_vector (main.cu:1878-1942: cublasDnrm2,
// scalar kernels, two host syncs). Here step j runs three sweeps over the
// rows, each reading the basis columns 0..j once:
//   GS_DOT      h1 = V^T w                               (pass 1 dots)
//   GS_UPD_DOT  w -= V h1 ; h2 = V^T w ; H(:,j) = h1+h2  (pass 1 update fused
//                                                         with pass 2 dots)
//   GS_UPD_NORM w -= V h2 ; H(j+1,j) = |w|, breakdown test
// i.e. classical Gram-Schmidt with one re-orthogonalisation (CGS2), which
// equals the reference's two MGS passes in exact arithmetic. Each kernel
// reduces per-thread partials with warp butterflies, then across warps in
// shared memory, then across blocks with a last-block-done handshake
// (no spin waits), always in the same order, so results are deterministic.
// These are the FP64 form's sweeps (DFMA throughout); the mixed-precision
// form orthogonalises its FP32 basis in gram_mixed.cu.
#include "mexk_internal.cuh"

#include <limits.h>
#include <math.h>

namespace mexk {

namespace {

constexpr unsigned FULL = 0xffffffffu;

// Per-thread accumulator: FP64 FMA for FP64 data, compensated FP32 otherwise.
template <typename TV>
struct Acc;
template <>
struct Acc<double> {
    double s;
    __device__ __forceinline__ void zero() { s = 0.0; }
    __device__ __forceinline__ void fma_add(double a, double b) { s = fma(a, b, s); }
    __device__ __forceinline__ double value() const { return s; }
};
template <typename TV>
struct Compute;
template <>
struct Compute<double> {
    using type = double;
};

// Butterfly transpose-reduction of a[0..K) over the warp (K power of two,
// K <= 32): afterwards every lane l holds the warp total of index l % K.
template <int K>
__device__ __forceinline__ double transpose_reduce(double (&a)[K], int lane) {
#pragma unroll
    for (int s = K / 2; s >= 1; s >>= 1) {
        const bool upper = (lane & s) != 0;
#pragma unroll
        for (int i = 0; i < s; ++i) {
            const double send = upper ? a[i] : a[i + s];
            const double keep = upper ? a[i + s] : a[i];
            a[i] = keep + __shfl_xor_sync(FULL, send, s);
        }
    }
    double v = a[0];
#pragma unroll
    for (int s = K; s < 32; s <<= 1) v += __shfl_xor_sync(FULL, v, s);
    return v;
}

// Dot of RPT row values into an accumulator (DFMA chain).
template <int RPT>
__device__ __forceinline__ void acc_dot(Acc<double>& a, const double (&v)[RPT], const double (&w)[RPT]) {
#pragma unroll
    for (int i = 0; i < RPT; ++i) a.fma_add(v[i], w[i]);
}

// Grid stage shared by both sweep kernels: after every block wrote its
// partials, the last block to arrive sums them in block order and writes the
// Hessenberg entries, the next pass's coefficients, or the norm and the
// breakdown test (main.cu:1911). A dot sweep reduces columns c0..c0+ncols-1.
template <int MODE>
__device__ __forceinline__ void gs_finish(const GsArgs& a, int ncols, double* s_out, double* s_scratch, int* s_flag) {
    if (!grid_last_block(a.counter, s_flag)) return;
    reduce_partials(a.partials, gridDim.x, ncols, s_out, s_scratch);
    DevState* st = a.st;
    const int j = a.j;
    const int c = a.c0 + static_cast<int>(threadIdx.x);
    const size_t ldh = static_cast<size_t>(a.ldh);
    const size_t hr = static_cast<size_t>(a.h_row0) + c;  // the Hessenberg row of column c of V
    if (MODE == GS_DOT) {
        if (static_cast<int>(threadIdx.x) < ncols) {
            if (a.pass2) {
                a.h2[c] = s_out[threadIdx.x];
                if (a.H) a.H[hr + j * ldh] = a.h1[c] + s_out[threadIdx.x];
            } else {
                a.h1[c] = s_out[threadIdx.x];
                if (!a.reortho && a.H) a.H[hr + j * ldh] = s_out[threadIdx.x];
            }
        }
    } else if (MODE == GS_UPD_DOT) {
        if (static_cast<int>(threadIdx.x) < ncols) {
            a.h2[c] = s_out[threadIdx.x];
            if (a.H) a.H[hr + j * ldh] = a.h1[c] + s_out[threadIdx.x];
        }
    } else if (threadIdx.x == 0) {
        const double beta = sqrt(s_out[0]);
        const bool bad = beta < 1e-14 || isnan(beta) || isinf(beta);
        if (a.beta_out) *a.beta_out = bad ? 0.0 : beta;
        if (a.H && j + 1 < a.ldh) a.H[(j + 1) + j * ldh] = bad ? 0.0 : beta;
        if (st != nullptr) {
            if (bad) {
                st->breakdown = 1;
                st->k_used = j + 1;
            } else {
                st->inv_beta = 1.0 / beta;
            }
        }
    }
}

// Update part of a row group: s += sum_c h_c V[r0.., c] for columns
// cb0 .. k-1 in order (CH at a time).
template <int CH, typename TV, int RPT, typename TC>
__device__ __forceinline__ void gs_upd_cols(const TV* __restrict__ V, size_t ldv, size_t r0, int cb, int k,
                                           const TC* s_h, TC (&s)[RPT]) {
    using IO = RowIO<RPT, TV>;
    TV vv[CH][RPT];
#pragma unroll
    for (int cc = 0; cc < CH; ++cc)
        if (cb + cc < k) IO::ld(V + (cb + cc) * ldv + r0, vv[cc]);
#pragma unroll
    for (int cc = 0; cc < CH; ++cc)
        if (cb + cc < k) {
            const TC h = s_h[cb + cc];
#pragma unroll
            for (int i = 0; i < RPT; ++i) s[i] = fma(static_cast<TC>(vv[cc][i]), h, s[i]);
        }
}

// One row group (RPT rows starting at r0) of a sweep: the update subtracts
// sum_c h_c V[:, c] over all k columns, the dots reduce columns c0..c0+kd-1
// (kd <= KMAX). Columns are read in chunks of CH so that only the
// accumulators stay live across the loop; in the KEEP form (every column's
// rows fit in registers; the launch guarantees c0 = 0 and kd = k <= KMAX)
// each column is loaded once.
template <int KMAX, int MODE, typename TV, int RPT>
__device__ __forceinline__ void gs_rows(const TV* __restrict__ V, size_t ldv, TV* __restrict__ w, size_t r0,
                                       int k, int c0, int kd, const typename Compute<TV>::type* s_h,
                                       Acc<TV> (&acc)[KMAX], Acc<TV>& nacc) {
    using TC = typename Compute<TV>::type;
    using IO = RowIO<RPT, TV>;
    constexpr int CH = 8;
    constexpr bool KEEP = KMAX * RPT * sizeof(TV) <= 128;
    TV wv[RPT];
    IO::ld(w + r0, wv);
    TC wr[RPT];
#pragma unroll
    for (int i = 0; i < RPT; ++i) wr[i] = static_cast<TC>(wv[i]);
    if constexpr (KEEP) {
        TV vv[KMAX][RPT];
#pragma unroll
        for (int c = 0; c < KMAX; ++c)
            if (c < k) IO::ldcs(V + c * ldv + r0, vv[c]);
        if (MODE != GS_DOT) {
            TC s[RPT];
#pragma unroll
            for (int i = 0; i < RPT; ++i) s[i] = TC(0);
#pragma unroll
            for (int c = 0; c < KMAX; ++c)
                if (c < k) {
                    const TC h = s_h[c];
#pragma unroll
                    for (int i = 0; i < RPT; ++i) s[i] = fma(static_cast<TC>(vv[c][i]), h, s[i]);
                }
#pragma unroll
            for (int i = 0; i < RPT; ++i) {
                wr[i] = wr[i] - s[i];
                wv[i] = static_cast<TV>(wr[i]);
            }
            IO::st(w + r0, wv);
        }
        if (MODE != GS_UPD_NORM) {
#pragma unroll
            for (int c = 0; c < KMAX; ++c)
                if (c < k) {
                    TC vc[RPT];
#pragma unroll
                    for (int i = 0; i < RPT; ++i) vc[i] = static_cast<TC>(vv[c][i]);
                    acc_dot<RPT>(acc[c], vc, wr);
                }
        } else {
            acc_dot<RPT>(nacc, wr, wr);
        }
    } else {
        if (MODE != GS_DOT) {
            TC s[RPT];
#pragma unroll
            for (int i = 0; i < RPT; ++i) s[i] = TC(0);
#pragma unroll
            for (int cb = 0; cb < KMAX; cb += CH)
                if (cb < k) gs_upd_cols<CH, TV, RPT, TC>(V, ldv, r0, cb, k, s_h, s);
            // bases wider than the sweep's width (FP64, more than GS_DOT_COLS
            // columns; the launch picks the full width for those)
            if constexpr (KMAX == GS_DOT_COLS)
                for (int cb = KMAX; cb < k; cb += CH) gs_upd_cols<CH, TV, RPT, TC>(V, ldv, r0, cb, k, s_h, s);
#pragma unroll
            for (int i = 0; i < RPT; ++i) {
                wr[i] = wr[i] - s[i];
                wv[i] = static_cast<TV>(wr[i]);
            }
            IO::st(w + r0, wv);
        }
        if (MODE != GS_UPD_NORM) {
            const TV* Vd = V + static_cast<size_t>(c0) * ldv;
#pragma unroll
            for (int cb = 0; cb < KMAX; cb += CH) {
                if (cb < kd) {
                    TV vv[CH][RPT];
#pragma unroll
                    for (int cc = 0; cc < CH; ++cc)
                        if (cb + cc < kd) {
                            if (MODE == GS_UPD_DOT) IO::ldg(Vd + (cb + cc) * ldv + r0, vv[cc]);
                            else IO::ldcs(Vd + (cb + cc) * ldv + r0, vv[cc]);
                        }
#pragma unroll
                    for (int cc = 0; cc < CH; ++cc)
                        if (cb + cc < kd) {
                            TC vc[RPT];
#pragma unroll
                            for (int i = 0; i < RPT; ++i) vc[i] = static_cast<TC>(vv[cc][i]);
                            acc_dot<RPT>(acc[cb + cc], vc, wr);
                        }
                }
            }
        } else {
            acc_dot<RPT>(nacc, wr, wr);
        }
    }
}

// Register cap per width so that 3 / 2 / 1 blocks of 256 threads stay resident.
// The fused update+dot sweep keeps more values live: one block fewer.
template <int KMAX, int MODE>
constexpr int gs_min_blocks() {
    return KMAX <= 16 ? (MODE == GS_UPD_DOT ? 2 : 3) : (KMAX <= 32 ? 2 : 1);
}

template <int KMAX, int MODE, typename TV, int RPT>
__global__ void __launch_bounds__(GS_THREADS, (gs_min_blocks<KMAX, MODE>())) gs_kernel(GsArgs a) {
    using TC = typename Compute<TV>::type;
    constexpr int NW = GS_THREADS / 32;
    constexpr int KR = KMAX < 32 ? KMAX : 32;  // width of one butterfly
    constexpr int NB = KMAX / KR;               // butterflies per thread
    __shared__ double s_red[NW][KMAX + 1];
    __shared__ double s_out[KMAX + 1];
    __shared__ double s_scratch[GS_THREADS];
    __shared__ TC s_h[MEXK_M_MAX];
    __shared__ int s_flag;

    DevState* st = a.st;
    if (st != nullptr && (st->breakdown || st->done)) return;
    const int k = a.k;
    const int c0 = a.c0;
    const int kd = a.kd > 0 ? a.kd : k;
    const int n = a.n;
    const size_t ldv = static_cast<size_t>(a.ldv);
    const TV* __restrict__ V = static_cast<const TV*>(a.V);
    TV* __restrict__ w = static_cast<TV*>(a.w);
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;

    if (MODE != GS_DOT) {
        const double* hin = (MODE == GS_UPD_DOT || !a.reortho) ? a.h1 : a.h2;
        for (int c = threadIdx.x; c < k; c += GS_THREADS) s_h[c] = static_cast<TC>(hin[c]);
        __syncthreads();
    }

    Acc<TV> acc[KMAX];
    Acc<TV> nacc;
#pragma unroll
    for (int c = 0; c < KMAX; ++c) acc[c].zero();
    nacc.zero();

    // launch_gs refuses n > INT_MAX - GS_MAX_GRID * GS_THREADS: no counter overflows
    const int stride = gridDim.x * GS_THREADS;
    const int ngroups = n / RPT;
    for (int g = blockIdx.x * GS_THREADS + threadIdx.x; g < ngroups; g += stride)
        gs_rows<KMAX, MODE, TV, RPT>(V, ldv, w, static_cast<size_t>(g) * RPT, k, c0, kd, s_h, acc, nacc);
    if (RPT > 1) {
        for (int r = ngroups * RPT + blockIdx.x * GS_THREADS + threadIdx.x; r < n; r += stride)
            gs_rows<KMAX, MODE, TV, 1>(V, ldv, w, static_cast<size_t>(r), k, c0, kd, s_h, acc, nacc);
    }

    // ---- block reduction
    int ncols;
    if (MODE != GS_UPD_NORM) {
        ncols = kd;
#pragma unroll
        for (int b = 0; b < NB; ++b) {
            double part[KR];
#pragma unroll
            for (int i = 0; i < KR; ++i) part[i] = acc[b * KR + i].value();
            const double v = transpose_reduce<KR>(part, lane);
            if (lane < KR) s_red[warp][b * KR + lane] = v;
        }
    } else {
        ncols = 1;
        double v = nacc.value();
        v = warp_sum(v);
        if (lane == 0) s_red[warp][0] = v;
    }
    __syncthreads();
    if (static_cast<int>(threadIdx.x) < ncols) {
        double s = 0.0;
#pragma unroll
        for (int q = 0; q < NW; ++q) s += s_red[q][threadIdx.x];
        a.partials[static_cast<size_t>(blockIdx.x) * RED_STRIDE + threadIdx.x] = s;
    }

    gs_finish<MODE>(a, ncols, s_out, s_scratch, &s_flag);
}

// V[:,j+1] = w * (1/beta), the reference's multiply by the reciprocal.
template <typename TV>
__global__ void __launch_bounds__(256) normalize_kernel(int n, int j, int ldv, const TV* __restrict__ w,
                                                        TV* __restrict__ V, const DevState* st,
                                                        const double* inv_beta_ptr) {
    if (st != nullptr && (st->breakdown || st->done)) return;
    const TV inv = static_cast<TV>(st != nullptr ? st->inv_beta : *inv_beta_ptr);
    TV* q = V + static_cast<size_t>(j + 1) * ldv;
    constexpr int RPT = 16 / sizeof(TV);
    const bool vec = (reinterpret_cast<uintptr_t>(q) % 16 == 0) && (reinterpret_cast<uintptr_t>(w) % 16 == 0);
    const int stride = gridDim.x * blockDim.x;
    int r0 = 0;
    if (vec) {
        const int ng = n / RPT;
        for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < ng; g += stride) {
            TV t[RPT];
            RowIO<RPT, TV>::ldcs(w + static_cast<size_t>(g) * RPT, t);
#pragma unroll
            for (int i = 0; i < RPT; ++i) t[i] = t[i] * inv;
            RowIO<RPT, TV>::st(q + static_cast<size_t>(g) * RPT, t);
        }
        r0 = ng * RPT;
    }
    for (int r = r0 + blockIdx.x * blockDim.x + threadIdx.x; r < n; r += stride) q[r] = w[r] * inv;
}

template <int KMAX, int MODE, typename TV, int RPT>
int launch_one(const GsArgs& a, int grid, cudaStream_t s) {
    gs_kernel<KMAX, MODE, TV, RPT><<<grid, GS_THREADS, 0, s>>>(a);
    MEXK_CK_LAUNCH("gs_kernel");
    return MEXK_OK;
}

// 16-byte row groups need 16-byte aligned columns: every column start
// (V + c*ldv) and w. Otherwise one row per thread.
template <typename TV>
bool vector_ok(const GsArgs& a) {
    constexpr int RPT = 16 / sizeof(TV);
    return (reinterpret_cast<uintptr_t>(a.V) % 16 == 0) && (reinterpret_cast<uintptr_t>(a.w) % 16 == 0) &&
           (a.ldv % RPT == 0);
}

template <int KMAX, int MODE, typename TV>
int launch_k(const GsArgs& a, int grid, cudaStream_t s) {
    constexpr int RPT = 16 / sizeof(TV);
    if (vector_ok<TV>(a)) return launch_one<KMAX, MODE, TV, RPT>(a, grid, s);
    return launch_one<KMAX, MODE, TV, 1>(a, grid, s);
}

// The width is set by the columns the sweep reduces (the update-and-norm
// sweep reduces none: its width only decides whether columns stay in registers).
template <int MODE, typename TV>
int launch_mode(const GsArgs& a, int grid, cudaStream_t s) {
    const int kd = MODE == GS_UPD_NORM ? (a.k < GS_DOT_COLS ? a.k : GS_DOT_COLS) : (a.kd > 0 ? a.kd : a.k);
    // A chunk of a wider basis (dot columns other than all k) takes a width
    // whose row groups do not stay in registers (those assume the dot
    // columns are the update's).
    const bool chunk = a.c0 != 0 || kd != a.k;
    if (chunk) return kd <= 32 ? launch_k<32, MODE, TV>(a, grid, s) : launch_k<GS_DOT_COLS, MODE, TV>(a, grid, s);
    if (kd <= 8) return launch_k<8, MODE, TV>(a, grid, s);
    if (kd <= 16) return launch_k<16, MODE, TV>(a, grid, s);
    if (kd <= 32) return launch_k<32, MODE, TV>(a, grid, s);
    if (kd <= GS_DOT_COLS) return launch_k<GS_DOT_COLS, MODE, TV>(a, grid, s);
    return MEXK_ERR_UNSUPPORTED;
}

}  // namespace

namespace {

template <int KMAX, int MODE, typename TV, int RPT>
int occupancy_of() {
    static int occ = -1;
    if (occ < 0) {
        int b = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, gs_kernel<KMAX, MODE, TV, RPT>, GS_THREADS, 0) !=
            cudaSuccess)
            b = 1;
        occ = b > 0 ? b : 1;
    }
    return occ;
}

// Resident blocks per SM shared by the three sweeps of one width.
template <int KMAX, typename TV>
int occupancy_k() {
    constexpr int RPT = 16 / sizeof(TV);
    int o = occupancy_of<KMAX, GS_DOT, TV, RPT>();
    o = min(o, occupancy_of<KMAX, GS_UPD_DOT, TV, RPT>());
    o = min(o, occupancy_of<KMAX, GS_UPD_NORM, TV, RPT>());
    return o;
}

template <typename TV>
int occupancy_for(int k) {
    if (k <= 8) return occupancy_k<8, TV>();
    if (k <= 16) return occupancy_k<16, TV>();
    if (k <= 32) return occupancy_k<32, TV>();
    return occupancy_k<64, TV>();
}

}  // namespace

// One wave of resident blocks (at most 4 per SM), fewer for short vectors.
int gs_grid_size(int n, int k) {
    int per_sm = occupancy_for<double>(k);
    if (per_sm > 4) per_sm = 4;
    constexpr int rpt = 2;
    const long long need = (static_cast<long long>(n) + rpt * GS_THREADS - 1) / (rpt * GS_THREADS);
    long long g = static_cast<long long>(device_sm_count()) * per_sm;
    if (need < g) g = need;
    if (g < 1) g = 1;
    return static_cast<int>(g);
}

// Resolves every occupancy query once, outside any stream capture.
void gs_prepare() {
    for (int k : {8, 16, 32, 64}) (void)gs_grid_size(1 << 20, k);
}

template <typename TV>
int launch_gs(GsMode mode, const GsArgs& a, int grid, cudaStream_t s) {
    const int kd = a.kd > 0 ? a.kd : a.k;
    if (a.k < 1 || a.k > MEXK_M_MAX || a.c0 < 0 || a.c0 + kd > a.k) return MEXK_ERR_INVALID;
    if (a.n < 1 || a.n > INT_MAX - GS_MAX_GRID * GS_THREADS || grid < 1 || grid > GS_MAX_GRID) {
        set_error_text("Gram-Schmidt sweep: n or grid out of range");
        return MEXK_ERR_INVALID;
    }
    if (mode != GS_UPD_NORM && kd > GS_DOT_COLS) return MEXK_ERR_UNSUPPORTED;
    switch (mode) {
        case GS_DOT: return launch_mode<GS_DOT, TV>(a, grid, s);
        case GS_UPD_DOT: return launch_mode<GS_UPD_DOT, TV>(a, grid, s);
        case GS_UPD_NORM: return launch_mode<GS_UPD_NORM, TV>(a, grid, s);
    }
    return MEXK_ERR_INVALID;
}

int launch_gs_step(const GsArgs& g0, int grid, cudaStream_t s) {
    int rc;
    if (g0.k <= GS_DOT_COLS) {
        GsArgs g = g0;
        g.c0 = 0;
        g.kd = 0;
        g.pass2 = 0;
        if ((rc = launch_gs<double>(GS_DOT, g, grid, s))) return rc;
        if (g.reortho && (rc = launch_gs<double>(GS_UPD_DOT, g, grid, s))) return rc;
        return launch_gs<double>(GS_UPD_NORM, g, grid, s);
    }
    GsArgs g = g0;
    g.pass2 = 0;
    for (int c0 = 0; c0 < g0.k; c0 += GS_DOT_COLS) {  // pass-1 dots, one launch per column chunk
        g.c0 = c0;
        g.kd = g0.k - c0 < GS_DOT_COLS ? g0.k - c0 : GS_DOT_COLS;
        if ((rc = launch_gs<double>(GS_DOT, g, grid, s))) return rc;
    }
    if (g0.reortho) {
        // pass-1 update of every column fused with the first chunk's pass-2
        // dots, then the other chunks' pass-2 dots on the updated vector
        g.c0 = 0;
        g.kd = GS_DOT_COLS;
        if ((rc = launch_gs<double>(GS_UPD_DOT, g, grid, s))) return rc;
        g.pass2 = 1;
        for (int c0 = GS_DOT_COLS; c0 < g0.k; c0 += GS_DOT_COLS) {
            g.c0 = c0;
            g.kd = g0.k - c0 < GS_DOT_COLS ? g0.k - c0 : GS_DOT_COLS;
            if ((rc = launch_gs<double>(GS_DOT, g, grid, s))) return rc;
        }
    }
    g.c0 = 0;
    g.kd = 0;
    g.pass2 = 0;
    return launch_gs<double>(GS_UPD_NORM, g, grid, s);
}

template <typename TV>
int launch_normalize(int n, int j, int ldv, const TV* w, TV* V, const DevState* st,
                     const double* inv_beta, cudaStream_t s) {
    int grid = (n / (16 / static_cast<int>(sizeof(TV))) + 255) / 256;
    if (grid > 2048) grid = 2048;
    if (grid < 1) grid = 1;
    normalize_kernel<TV><<<grid, 256, 0, s>>>(n, j, ldv, w, V, st, inv_beta);
    MEXK_CK_LAUNCH("normalize_kernel");
    return MEXK_OK;
}

template int launch_gs<double>(GsMode, const GsArgs&, int, cudaStream_t);
template int launch_normalize<double>(int, int, int, const double*, double*, const DevState*,
                                      const double*, cudaStream_t);

}  // namespace mexk
