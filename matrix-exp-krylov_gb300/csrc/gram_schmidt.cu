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
// FP64 storage accumulates with DFMA; FP32 storage (mixed precision)
// multiplies in FP32 and accumulates each thread's terms with Kahan
// compensation before the FP64 block and grid stages.
#include "mexk_internal.cuh"

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
template <>
struct Acc<float> {
    float s, c;
    __device__ __forceinline__ void zero() {
        s = 0.f;
        c = 0.f;
    }
    __device__ __forceinline__ void fma_add(float a, float b) {
        const float y = __fmaf_rn(a, b, -c);
        const float t = __fadd_rn(s, y);
        c = __fsub_rn(__fsub_rn(t, s), y);
        s = t;
    }
    __device__ __forceinline__ double value() const { return static_cast<double>(s) - static_cast<double>(c); }
};

template <typename TV>
struct Compute;
template <>
struct Compute<double> {
    using type = double;
};
template <>
struct Compute<float> {
    using type = float;
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

template <int KMAX, int MODE, typename TV>
__global__ void __launch_bounds__(GS_THREADS) gs_kernel(GsArgs a) {
    using TC = typename Compute<TV>::type;
    constexpr int NW = GS_THREADS / 32;
    constexpr int KR = KMAX < 32 ? KMAX : 32;  // width of one butterfly
    constexpr int NB = KMAX / KR;               // butterflies per thread
    __shared__ double s_red[NW][KMAX + 1];
    __shared__ double s_out[KMAX + 1];
    __shared__ double s_scratch[GS_THREADS];
    __shared__ int s_flag;

    DevState* st = a.st;
    if (st != nullptr && (st->breakdown || st->done)) return;
    const int k = a.k;
    const int n = a.n;
    const size_t ldv = static_cast<size_t>(a.ldv);
    const TV* __restrict__ V = static_cast<const TV*>(a.V);
    TV* __restrict__ w = static_cast<TV*>(a.w);
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;

    TC hreg[KMAX];
    if (MODE != GS_DOT) {
        const double* hin = (MODE == GS_UPD_DOT || !a.reortho) ? a.h1 : a.h2;
#pragma unroll
        for (int c = 0; c < KMAX; ++c) hreg[c] = (c < k) ? static_cast<TC>(hin[c]) : TC(0);
    }

    Acc<TV> acc[KMAX];
    Acc<TV> nacc;
#pragma unroll
    for (int c = 0; c < KMAX; ++c) acc[c].zero();
    nacc.zero();

    const int stride = gridDim.x * GS_THREADS;
    for (int r = blockIdx.x * GS_THREADS + threadIdx.x; r < n; r += stride) {
        TC wr = static_cast<TC>(w[r]);
        if (MODE != GS_DOT) {
            TC s = TC(0);
#pragma unroll
            for (int c = 0; c < KMAX; ++c)
                if (c < k) s = fma(static_cast<TC>(V[c * ldv + r]), hreg[c], s);
            wr = wr - s;
            w[r] = static_cast<TV>(wr);
        }
        if (MODE != GS_UPD_NORM) {
#pragma unroll
            for (int c = 0; c < KMAX; ++c)
                if (c < k) acc[c].fma_add(static_cast<TC>(__ldg(&V[c * ldv + r])), wr);
        } else {
            nacc.fma_add(wr, wr);
        }
    }

    // ---- block reduction
    int ncols;
    if (MODE != GS_UPD_NORM) {
        ncols = k;
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
    if (threadIdx.x < ncols) {
        double s = 0.0;
#pragma unroll
        for (int q = 0; q < NW; ++q) s += s_red[q][threadIdx.x];
        a.partials[static_cast<size_t>(blockIdx.x) * RED_STRIDE + threadIdx.x] = s;
    }

    // ---- grid reduction by the last block
    if (!grid_last_block(a.counter, &s_flag)) return;
    reduce_partials(a.partials, gridDim.x, ncols, s_out, s_scratch);
    const int j = a.j;
    const size_t ldh = static_cast<size_t>(a.ldh);
    if (MODE == GS_DOT) {
        if (threadIdx.x < k) {
            a.h1[threadIdx.x] = s_out[threadIdx.x];
            if (!a.reortho && a.H) a.H[threadIdx.x + j * ldh] = s_out[threadIdx.x];
        }
    } else if (MODE == GS_UPD_DOT) {
        if (threadIdx.x < k) {
            a.h2[threadIdx.x] = s_out[threadIdx.x];
            if (a.H) a.H[threadIdx.x + j * ldh] = a.h1[threadIdx.x] + s_out[threadIdx.x];
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

template <typename TV>
__global__ void __launch_bounds__(256) normalize_kernel(int n, int j, int ldv, const TV* __restrict__ w,
                                                        TV* __restrict__ V, const DevState* st,
                                                        const double* inv_beta_ptr) {
    if (st != nullptr && (st->breakdown || st->done)) return;
    const double inv = st != nullptr ? st->inv_beta : *inv_beta_ptr;
    TV* q = V + static_cast<size_t>(j + 1) * ldv;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x)
        q[r] = static_cast<TV>(static_cast<double>(w[r]) * inv);
}

template <int KMAX, int MODE, typename TV>
int launch_one(const GsArgs& a, int grid, cudaStream_t s) {
    gs_kernel<KMAX, MODE, TV><<<grid, GS_THREADS, 0, s>>>(a);
    MEXK_CK_LAUNCH("gs_kernel");
    return MEXK_OK;
}

template <int MODE, typename TV>
int launch_mode(const GsArgs& a, int grid, cudaStream_t s) {
    if (a.k <= 8) return launch_one<8, MODE, TV>(a, grid, s);
    if (a.k <= 16) return launch_one<16, MODE, TV>(a, grid, s);
    if (a.k <= 32) return launch_one<32, MODE, TV>(a, grid, s);
    if (a.k <= 64) return launch_one<64, MODE, TV>(a, grid, s);
    return MEXK_ERR_UNSUPPORTED;
}

}  // namespace

int gs_grid_size(int n, int k, bool fp32) {
    static int sms = 0;
    if (sms == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    }
    // Wide accumulator sets cost registers: fewer resident blocks per SM.
    int per_sm = 4;
    if (!fp32 && k > 32) per_sm = 1;
    else if (!fp32 && k > 16) per_sm = 2;
    else if (fp32 && k > 32) per_sm = 2;
    const long long need = (static_cast<long long>(n) + GS_THREADS - 1) / GS_THREADS;
    long long g = static_cast<long long>(sms) * per_sm;
    if (need < g) g = need;
    if (g < 1) g = 1;
    return static_cast<int>(g);
}

template <typename TV>
int launch_gs(GsMode mode, const GsArgs& a, int grid, cudaStream_t s) {
    if (a.k < 1 || a.k > MEXK_M_MAX) return MEXK_ERR_INVALID;
    switch (mode) {
        case GS_DOT: return launch_mode<GS_DOT, TV>(a, grid, s);
        case GS_UPD_DOT: return launch_mode<GS_UPD_DOT, TV>(a, grid, s);
        case GS_UPD_NORM: return launch_mode<GS_UPD_NORM, TV>(a, grid, s);
    }
    return MEXK_ERR_INVALID;
}

template <typename TV>
int launch_normalize(int n, int j, int ldv, const TV* w, TV* V, const DevState* st,
                     const double* inv_beta, cudaStream_t s) {
    int grid = (n + 255) / 256;
    if (grid > 4096) grid = 4096;
    if (grid < 1) grid = 1;
    normalize_kernel<TV><<<grid, 256, 0, s>>>(n, j, ldv, w, V, st, inv_beta);
    MEXK_CK_LAUNCH("normalize_kernel");
    return MEXK_OK;
}

template int launch_gs<double>(GsMode, const GsArgs&, int, cudaStream_t);
template int launch_gs<float>(GsMode, const GsArgs&, int, cudaStream_t);
template int launch_normalize<double>(int, int, int, const double*, double*, const DevState*,
                                      const double*, cudaStream_t);
template int launch_normalize<float>(int, int, int, const float*, float*, const DevState*,
                                     const double*, cudaStream_t);

}  // namespace mexk
