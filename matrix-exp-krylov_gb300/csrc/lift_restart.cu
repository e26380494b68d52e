// K4: lift y = |v| V_k w_H with the norm of y for the restart, the restart
// q1 = y/|y| and the start vector q1 = v/|v|.
//
// The reference lifts with one pageable H2D copy of the coefficient and one
// cublasDaxpy per basis column (small_expm_and_lift, main.cu:1980-2001),
// rereading and rewriting y k times, then restart_from_y
// (main.cu:2023-2073) runs Dnrm2, an allreduce, a host sync, Dscal and two
// D2D copies; init_q1 (main.cu:1574-1633) does the same for v. Here the
// lift reads each basis column once, accumulates every row in one FMA chain
// in column order (the axpy order), writes y once and reduces |y|^2 in the
// same pass; the restart is a single scale into V[:,0]. The norm guard
// |x| > 1e-14 follows the CPU twin (main_cpu.cpp:480, 596).
#include "mexk_internal.cuh"

#include <math.h>

namespace mexk {

namespace {

constexpr int LIFT_THREADS = 256;
constexpr int LIFT_BLOCKS_PER_SM = 6;  // a strided multi-column read wants many warps in flight

// The double of a float, exactly (the value F2F produces), by integer
// operations for normal numbers and zero: the conversion otherwise runs on
// this GPU's FP64 units, which execute about two lanes per clock per SM.
// Subnormal, infinite and NaN inputs take the hardware conversion.
__device__ __forceinline__ double widen(float f) {
    const unsigned u = __float_as_uint(f);
    const unsigned e = (u >> 23) & 0xffu;
    if (e == 0u || e == 0xffu) {
        if ((u & 0x7fffffffu) == 0u) return __hiloint2double(static_cast<int>(u & 0x80000000u), 0);
        return static_cast<double>(f);
    }
    const unsigned hi = (u & 0x80000000u) | ((e + 896u) << 20) | ((u >> 3) & 0xfffffu);
    const unsigned lo = u << 29;
    return __hiloint2double(static_cast<int>(hi), static_cast<int>(lo));
}

// RPT rows of y = sum_c coef_c V_c over the columns with nonzero
// coefficients, loaded 4 at a time (16-byte
// row groups; 40 registers, so 6 blocks of 256 threads fit an SM). FP64 basis: one DFMA chain per row in column order (the axpy
// order). FP32 basis: FP32 products summed with compensation and widened
// once per row, so the FP64 pipe does O(1) work per row, not O(k).
template <typename TV, int RPT>
__device__ __forceinline__ void lift_rows(const TV* __restrict__ V, size_t ldv, size_t r0, int k, const double* c64,
                                          const float* c32, double (&y)[RPT]) {
    constexpr int CH = 4;
    using IO = RowIO<RPT, TV>;
    if constexpr (sizeof(TV) == 8) {
        double s[RPT];
#pragma unroll
        for (int i = 0; i < RPT; ++i) s[i] = 0.0;
        for (int cb = 0; cb < k; cb += CH) {
            TV vv[CH][RPT];
#pragma unroll
            for (int cc = 0; cc < CH; ++cc)
                if (cb + cc < k && c64[cb + cc] != 0.0) IO::ldcs(V + (cb + cc) * ldv + r0, vv[cc]);
#pragma unroll
            for (int cc = 0; cc < CH; ++cc)
                if (cb + cc < k && c64[cb + cc] != 0.0) {
#pragma unroll
                    for (int i = 0; i < RPT; ++i) s[i] = fma(c64[cb + cc], static_cast<double>(vv[cc][i]), s[i]);
                }
        }
#pragma unroll
        for (int i = 0; i < RPT; ++i) y[i] = s[i];
    } else {
        float s[RPT], comp[RPT];
#pragma unroll
        for (int i = 0; i < RPT; ++i) s[i] = comp[i] = 0.f;
        for (int cb = 0; cb < k; cb += CH) {
            TV vv[CH][RPT];
#pragma unroll
            for (int cc = 0; cc < CH; ++cc)
                if (cb + cc < k && c32[cb + cc] != 0.0f) IO::ldcs(V + (cb + cc) * ldv + r0, vv[cc]);
#pragma unroll
            for (int cc = 0; cc < CH; ++cc)
                if (cb + cc < k && c32[cb + cc] != 0.0f) {
#pragma unroll
                    for (int i = 0; i < RPT; ++i) {
                        const float yv = __fmaf_rn(c32[cb + cc], static_cast<float>(vv[cc][i]), -comp[i]);
                        const float t = __fadd_rn(s[i], yv);
                        comp[i] = __fsub_rn(__fsub_rn(t, s[i]), yv);
                        s[i] = t;
                    }
                }
        }
#pragma unroll
        for (int i = 0; i < RPT; ++i) y[i] = widen(s[i]) - widen(comp[i]);
    }
}

template <typename TV>
__global__ void __launch_bounds__(LIFT_THREADS, LIFT_BLOCKS_PER_SM) lift_kernel(LiftArgs a) {
    constexpr int RPT = 16 / sizeof(TV);
    __shared__ double s_coef[MEXK_M_MAX + 1];
    __shared__ float s_coef32[MEXK_M_MAX + 1];
    __shared__ double s_red[32];
    __shared__ double s_out[1];
    __shared__ double s_scratch[LIFT_THREADS];
    __shared__ int s_flag;
    // launched as a dependent of the controller: its state and coefficients
    // are read after the wait; the restart may launch meanwhile
    pdl_wait();
    pdl_trigger();
    DevState* st = a.st;
    if (!st->lift) return;
    const int k = st->k_lift;
    for (int i = threadIdx.x; i < k; i += blockDim.x) {
        // a zero coefficient drops its column, as the reference's lift skips
        // it (main.cu:1993): 0 * Inf or NaN entries must not reach y
        const double c = (a.coef[i] == 0.0) ? 0.0 : (a.scale ? a.coef[i] * a.scale[i] : a.coef[i]);
        s_coef[i] = c;
        s_coef32[i] = static_cast<float>(c);
    }
    __syncthreads();
    const TV* __restrict__ V = static_cast<const TV*>(a.V);
    const size_t ldv = static_cast<size_t>(a.ldv);
    const bool vec = (reinterpret_cast<uintptr_t>(V) % 16 == 0) && (a.ldv % RPT == 0) &&
                     (reinterpret_cast<uintptr_t>(a.y) % 16 == 0);
    const int stride = gridDim.x * LIFT_THREADS;
    double nacc = 0.0;
    int r_tail = 0;
    if (vec) {
        const int ng = a.n / RPT;
        for (int g = blockIdx.x * LIFT_THREADS + threadIdx.x; g < ng; g += stride) {
            double y[RPT];
            lift_rows<TV, RPT>(V, ldv, static_cast<size_t>(g) * RPT, k, s_coef, s_coef32, y);
#pragma unroll
            for (int i = 0; i < RPT; i += 2) {
                *reinterpret_cast<double2*>(a.y + static_cast<size_t>(g) * RPT + i) = make_double2(y[i], y[i + 1]);
                nacc = fma(y[i], y[i], nacc);
                nacc = fma(y[i + 1], y[i + 1], nacc);
            }
        }
        r_tail = ng * RPT;
    }
    for (int r = r_tail + blockIdx.x * LIFT_THREADS + threadIdx.x; r < a.n; r += stride) {
        double y[1];
        lift_rows<TV, 1>(V, ldv, static_cast<size_t>(r), k, s_coef, s_coef32, y);
        a.y[r] = y[0];
        nacc = fma(y[0], y[0], nacc);
    }
    nacc = warp_sum(nacc);
    if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = nacc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int q = 0; q < LIFT_THREADS / 32; ++q) t += s_red[q];
        a.partials[static_cast<size_t>(blockIdx.x) * RED_STRIDE] = t;
    }
    if (!grid_last_block(a.counter, &s_flag)) return;
    reduce_partials(a.partials, gridDim.x, 1, s_out, s_scratch);
    if (threadIdx.x == 0) {
        const double nrm = sqrt(s_out[0]);
        st->restart_scale = nrm > 1e-14 ? 1.0 / nrm : 1.0;
        if (st->restart) st->v_norm = nrm;
        st->lift = 0;
    }
}

// |x|^2 of the start vector -> v_norm and restart_scale (init_q1).
__global__ void __launch_bounds__(LIFT_THREADS)
    start_norm_kernel(int n, const double* __restrict__ x, double* partials, unsigned int* counter,
                      DevState* st) {
    __shared__ double s_red[32];
    __shared__ double s_out[1];
    __shared__ double s_scratch[LIFT_THREADS];
    __shared__ int s_flag;
    double nacc = 0.0;
    for (int r = blockIdx.x * LIFT_THREADS + threadIdx.x; r < n; r += gridDim.x * LIFT_THREADS)
        nacc = fma(x[r], x[r], nacc);
    nacc = warp_sum(nacc);
    if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = nacc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int q = 0; q < LIFT_THREADS / 32; ++q) t += s_red[q];
        partials[static_cast<size_t>(blockIdx.x) * RED_STRIDE] = t;
    }
    if (!grid_last_block(counter, &s_flag)) return;
    reduce_partials(partials, gridDim.x, 1, s_out, s_scratch);
    if (threadIdx.x == 0) {
        const double nrm = sqrt(s_out[0]);
        st->v_norm = nrm;
        st->restart_scale = nrm > 1e-14 ? 1.0 / nrm : 1.0;
    }
}

// V[:,0] = x * scale. FP64: the reference's x * (1/|x|). FP32 basis: one
// narrowing conversion per element, then an FP32 multiply.
template <typename TV>
__global__ void __launch_bounds__(256) restart_kernel(int n, const double* __restrict__ x, TV* __restrict__ V0,
                                                      const DevState* st, int force) {
    pdl_wait();  // a dependent of the lift (no-op after a plain launch)
    pdl_trigger();
    if (!force && !st->restart) return;
    const TV sc = static_cast<TV>(st->restart_scale);
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x)
        V0[r] = static_cast<TV>(__ldcs(&x[r])) * sc;
}

int elementwise_grid(int n) {
    int g = (n + 255) / 256;
    if (g > 8192) g = 8192;
    return g < 1 ? 1 : g;
}

}  // namespace

template <typename TV>
int launch_lift(const LiftArgs& a, int /*grid*/, cudaStream_t s) {
    constexpr int RPT = 16 / static_cast<int>(sizeof(TV));
    const long long need = (static_cast<long long>(a.n) + RPT * LIFT_THREADS - 1) / (RPT * LIFT_THREADS);
    const long long cap = static_cast<long long>(device_sm_count()) * LIFT_BLOCKS_PER_SM;
    const int grid = static_cast<int>(need < cap ? (need < 1 ? 1 : need) : cap);
    const cudaError_t e = launch_dependent(lift_kernel<TV>, grid, LIFT_THREADS, 0, s, a);
    if (e != cudaSuccess) {
        set_cuda_error(e, "lift_kernel", __FILE__, __LINE__);
        return MEXK_ERR_CUDA;
    }
    return MEXK_OK;
}

template <typename TV>
int launch_restart(int n, int ldv, const double* y, TV* V, const DevState* st, cudaStream_t s) {
    (void)ldv;
    const cudaError_t e = launch_dependent(restart_kernel<TV>, elementwise_grid(n), 256, 0, s, n, y, V, st, 0);
    if (e != cudaSuccess) {
        set_cuda_error(e, "restart_kernel", __FILE__, __LINE__);
        return MEXK_ERR_CUDA;
    }
    return MEXK_OK;
}

template <typename TV>
int launch_init_start(int n, int ldv, const double* v, TV* V, double* partials, unsigned int* counter,
                      DevState* st, int grid, cudaStream_t s) {
    (void)ldv;
    start_norm_kernel<<<grid, LIFT_THREADS, 0, s>>>(n, v, partials, counter, st);
    MEXK_CK_LAUNCH("start_norm_kernel");
    restart_kernel<TV><<<elementwise_grid(n), 256, 0, s>>>(n, v, V, st, 1);
    MEXK_CK_LAUNCH("restart_kernel");
    return MEXK_OK;
}

template int launch_lift<double>(const LiftArgs&, int, cudaStream_t);
template int launch_lift<float>(const LiftArgs&, int, cudaStream_t);
template int launch_restart<double>(int, int, const double*, double*, const DevState*, cudaStream_t);
template int launch_restart<float>(int, int, const double*, float*, const DevState*, cudaStream_t);
template int launch_init_start<double>(int, int, const double*, double*, double*, unsigned int*, DevState*,
                                       int, cudaStream_t);
template int launch_init_start<float>(int, int, const double*, float*, double*, unsigned int*, DevState*, int,
                                      cudaStream_t);

}  // namespace mexk
