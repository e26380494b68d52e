// K1: CSR sparse matrix-vector product w = A*x on sm_103a.
//
// Replaces cusparseSpMV (reference main.cu:1722-1767, called with a fresh
// dense-vector descriptor per call). Design: the rows are cut into row
// blocks of at most SPMV_TILE nonzeros and SPMV_TILE_ROWS rows (one row
// per block when a row is longer), so every thread block streams a
// contiguous range of values and column indices with coalesced loads,
// whatever the row-length distribution (Laplacian stencils, Zipf rows).
// Phase 1 multiplies value * x[col] into shared memory; phase 2 sums each
// row's products. Rows of at most SEQ_ROW_MAX nonzeros are summed in column
// order by one thread, so their FP64 result equals the reference's serial
// loop (main_cpu.cpp:388-397) bit for bit: one rounded product per nonzero,
// added left to right. Longer rows (the power-law tails) are summed by one
// warp each, and rows longer than a tile by the whole block, in fixed
// orders (deterministic, within rounding of the serial sum). The gathers of x are
// served from L2 (x is one basis column, read right after it was written).
#include "mexk_internal.cuh"

namespace mexk {

std::vector<int> build_row_blocks(int n, const int* row_ptr) {
    std::vector<int> blocks;
    blocks.reserve(static_cast<size_t>(n) / 64 + 2);
    blocks.push_back(0);
    int r = 0;
    while (r < n) {
        const int start = r;
        const long long len0 = static_cast<long long>(row_ptr[r + 1]) - row_ptr[r];
        if (len0 > SPMV_TILE) {
            ++r;
        } else {
            long long acc = 0;
            while (r < n && r - start < SPMV_TILE_ROWS) {
                const long long len = static_cast<long long>(row_ptr[r + 1]) - row_ptr[r];
                if (acc + len > SPMV_TILE) break;
                acc += len;
                ++r;
            }
        }
        blocks.push_back(r);
    }
    return blocks;
}

template <typename T>
struct AccType;
template <>
struct AccType<double> {
    using type = double;
};
template <>
struct AccType<float> {
    using type = float;
};

// Four consecutive values starting at a 16-byte boundary.
template <typename TA>
struct Quad;
template <>
struct Quad<float> {
    static __device__ __forceinline__ void ld(const float* p, float (&o)[4]) {
        const float4 t = __ldcs(reinterpret_cast<const float4*>(p));
        o[0] = t.x;
        o[1] = t.y;
        o[2] = t.z;
        o[3] = t.w;
    }
};
template <>
struct Quad<double> {
    static __device__ __forceinline__ void ld(const double* p, double (&o)[4]) {
        const double2 t0 = __ldcs(reinterpret_cast<const double2*>(p));
        const double2 t1 = __ldcs(reinterpret_cast<const double2*>(p) + 1);
        o[0] = t0.x;
        o[1] = t0.y;
        o[2] = t1.x;
        o[3] = t1.y;
    }
};

// Groups of 4 nonzeros one thread covers in a tile (the tile's span, widened
// down to a multiple of 4, has at most SPMV_TILE + 3 entries).
constexpr int SPMV_QUADS = ((SPMV_TILE + 3 + 3) / 4 + SPMV_THREADS - 1) / SPMV_THREADS;

// VEC: values and column indices are 16-byte aligned arrays padded by at
// least 3 entries past nnz, so whole aligned groups of 4 may be loaded; every
// thread issues all its column/value loads, then all its x gathers.
template <typename TA, typename TX, bool VEC>
__global__ void __launch_bounds__(SPMV_THREADS)
    spmv_rowblock_kernel(int nblocks, const int* __restrict__ blocks, const int* __restrict__ row_ptr,
                         const int* __restrict__ col_idx, const TA* __restrict__ values,
                         const TX* __restrict__ x, TX* __restrict__ y, const int* __restrict__ skip) {
    using TP = typename AccType<TX>::type;
    __shared__ TP prod[SPMV_TILE];
    __shared__ TP red[32];
    __shared__ int s_long[SPMV_TILE / (SEQ_ROW_MAX + 1) + 1];
    __shared__ int s_nlong;
    pdl_wait();
    if (skip != nullptr && *skip) return;
    const int tid = threadIdx.x;
    const int lane = tid & 31;
    for (int b = blockIdx.x; b < nblocks; b += gridDim.x) {
        if (tid == 0) s_nlong = 0;
        const int r0 = blocks[b];
        const int r1 = blocks[b + 1];
        const int e0 = row_ptr[r0];
        const int e1 = row_ptr[r1];
        const int cnt = e1 - e0;
        if (cnt > SPMV_TILE) {
            // One long row: the block splits its nonzeros, then a tree sum.
            TP s = 0;
            for (int e = e0 + tid; e < e1; e += SPMV_THREADS) {
                const TP p = static_cast<TP>(__ldcs(&values[e])) * static_cast<TP>(__ldg(&x[__ldcs(&col_idx[e])]));
                s += p;
            }
            s = block_sum(s, red);
            if (tid == 0) y[r0] = static_cast<TX>(s);
            continue;
        }
        // Row extents for phase 2, fetched alongside phase 1.
        constexpr int RPT = SPMV_TILE_ROWS / SPMV_THREADS;
        int ra[RPT], rz[RPT];
#pragma unroll
        for (int q = 0; q < RPT; ++q) {
            const int r = r0 + tid + q * SPMV_THREADS;
            ra[q] = r < r1 ? row_ptr[r] : 0;
            rz[q] = r < r1 ? row_ptr[r + 1] : 0;
        }
        // Phase 1: coalesced stream of (value, column) pairs.
        if constexpr (VEC) {
            const int base = e0 & ~3;
            const int nq = (e1 - base + 3) >> 2;
            int4 cq[SPMV_QUADS];
            TA aq[SPMV_QUADS][4];
#pragma unroll
            for (int q = 0; q < SPMV_QUADS; ++q) {
                const int g = tid + q * SPMV_THREADS;
                if (g < nq) {
                    cq[q] = __ldcs(reinterpret_cast<const int4*>(col_idx + base) + g);
                    Quad<TA>::ld(values + base + 4 * g, aq[q]);
                }
            }
            TP xq[SPMV_QUADS][4];
#pragma unroll
            for (int q = 0; q < SPMV_QUADS; ++q) {
                const int g = tid + q * SPMV_THREADS;
                const int e = base + 4 * g;
                const int c4[4] = {cq[q].x, cq[q].y, cq[q].z, cq[q].w};
#pragma unroll
                for (int i = 0; i < 4; ++i)
                    xq[q][i] = (g < nq && e + i >= e0 && e + i < e1) ? static_cast<TP>(__ldg(&x[c4[i]])) : TP(0);
            }
#pragma unroll
            for (int q = 0; q < SPMV_QUADS; ++q) {
                const int g = tid + q * SPMV_THREADS;
                const int e = base + 4 * g;
#pragma unroll
                for (int i = 0; i < 4; ++i)
                    if (g < nq && e + i >= e0 && e + i < e1) prod[e + i - e0] = static_cast<TP>(aq[q][i]) * xq[q][i];
            }
        } else {
#pragma unroll 4
            for (int e = tid; e < cnt; e += SPMV_THREADS) {
                const int c = __ldcs(&col_idx[e0 + e]);
                const TA a = __ldcs(&values[e0 + e]);
                prod[e] = static_cast<TP>(a) * static_cast<TP>(__ldg(&x[c]));
            }
        }
        __syncthreads();
        // Phase 2: rows of at most SEQ_ROW_MAX nonzeros are summed left to
        // right by one thread (the reference's order); longer rows go to a
        // list and are summed by one warp each.
#pragma unroll
        for (int q = 0; q < RPT; ++q) {
            const int r = r0 + tid + q * SPMV_THREADS;
            if (r < r1) {
                if (rz[q] - ra[q] > SEQ_ROW_MAX) {
                    s_long[atomicAdd(&s_nlong, 1)] = r;
                } else {
                    TP s = 0;
                    for (int p = ra[q] - e0; p < rz[q] - e0; ++p) s += prod[p];
                    y[r] = static_cast<TX>(s);
                }
            }
        }
        __syncthreads();
        if (b + static_cast<int>(gridDim.x) >= nblocks) pdl_trigger();  // this block's last row block
        // Each lane sums its strided share in order, then a fixed butterfly:
        // the result does not depend on which warp takes the row.
        for (int i = tid >> 5; i < s_nlong; i += SPMV_THREADS / 32) {
            const int r = s_long[i];
            const int a = row_ptr[r] - e0;
            const int z = row_ptr[r + 1] - e0;
            TP s = 0;
            for (int p = a + lane; p < z; p += 32) s += prod[p];
            s = warp_sum(s);
            if (lane == 0) y[r] = static_cast<TX>(s);
        }
        __syncthreads();
    }
}

template <typename TA, typename TX>
int launch_spmv(int n, int nblocks, const int* blocks, const int* row_ptr, const int* col_idx,
                const TA* values, const TX* x, TX* y, const int* skip_flag, cudaStream_t s, bool padded) {
    if (n <= 0 || nblocks <= 0) return MEXK_OK;
    const int grid = nblocks < 1048576 ? nblocks : 1048576;
    const bool vec = padded && reinterpret_cast<uintptr_t>(col_idx) % 16 == 0 &&
                     reinterpret_cast<uintptr_t>(values) % 16 == 0;
    if (vec)
    {
        const cudaError_t e = launch_dependent(spmv_rowblock_kernel<TA, TX, true>, grid, SPMV_THREADS, 0, s,
                                               nblocks, blocks, row_ptr, col_idx, values, x, y, skip_flag);
        if (e != cudaSuccess) {
            set_cuda_error(e, "spmv_rowblock_kernel", __FILE__, __LINE__);
            return MEXK_ERR_CUDA;
        }
        return MEXK_OK;
    }
    else
        spmv_rowblock_kernel<TA, TX, false><<<grid, SPMV_THREADS, 0, s>>>(nblocks, blocks, row_ptr, col_idx,
                                                                          values, x, y, skip_flag);
    MEXK_CK_LAUNCH("spmv_rowblock_kernel");
    return MEXK_OK;
}

template int launch_spmv<double, double>(int, int, const int*, const int*, const int*, const double*,
                                         const double*, double*, const int*, cudaStream_t, bool);
template int launch_spmv<float, float>(int, int, const int*, const int*, const int*, const float*,
                                       const float*, float*, const int*, cudaStream_t, bool);

// FP32 copy of the FP64 matrix values for the mixed-precision form
// (round to nearest).
__global__ void narrow_kernel(const double* __restrict__ src, float* __restrict__ dst, size_t count) {
    for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < count;
         i += static_cast<size_t>(gridDim.x) * blockDim.x)
        dst[i] = __double2float_rn(src[i]);
}

int launch_narrow_values(const double* src, float* dst, size_t count, cudaStream_t s) {
    if (count == 0) return MEXK_OK;
    const size_t want = (count + 255) / 256;
    const int grid = static_cast<int>(want < 4096 ? want : 4096);
    narrow_kernel<<<grid, 256, 0, s>>>(src, dst, count);
    MEXK_CK_LAUNCH("narrow_kernel");
    return MEXK_OK;
}

// A == A^T exactly: every entry (r, c, v) has an entry (c, r, v). One thread
// per row scans, for each of its entries, row c for column r.
__global__ void symmetric_check_kernel(int n, const int* __restrict__ row_ptr, const int* __restrict__ col_idx,
                                       const double* __restrict__ values, int* __restrict__ ok) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        for (int e = row_ptr[r]; e < row_ptr[r + 1]; ++e) {
            const int c = col_idx[e];
            const double v = values[e];
            bool found = false;
            for (int f = row_ptr[c]; f < row_ptr[c + 1]; ++f)
                if (col_idx[f] == r && values[f] == v) {
                    found = true;
                    break;
                }
            if (!found) {
                atomicAnd(ok, 0);
                return;
            }
        }
    }
}

__global__ void set_one_kernel(int* p) { *p = 1; }

int launch_symmetric_check(int n, const int* row_ptr, const int* col_idx, const double* values, int* ok,
                           cudaStream_t s) {
    set_one_kernel<<<1, 1, 0, s>>>(ok);
    MEXK_CK_LAUNCH("set_one_kernel");
    if (n <= 0) return MEXK_OK;
    const int grid = (n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096;
    symmetric_check_kernel<<<grid, 256, 0, s>>>(n, row_ptr, col_idx, values, ok);
    MEXK_CK_LAUNCH("symmetric_check_kernel");
    return MEXK_OK;
}

// Free-standing C entry points: build the schedule on the host from a device
// row_ptr copy. Meant for tests and one-off products; the solver keeps the
// schedule resident.
template <typename TA, typename TX>
static int spmv_standalone(int rows, const int* row_ptr, const int* col_idx, const TA* values,
                           const TX* x, TX* y, void* stream) {
    if (rows < 0 || (rows > 0 && (!row_ptr || !x || !y))) return MEXK_ERR_INVALID;
    if (rows == 0) return MEXK_OK;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    std::vector<int> rp(static_cast<size_t>(rows) + 1);
    MEXK_CK(cudaMemcpyAsync(rp.data(), row_ptr, sizeof(int) * rp.size(), cudaMemcpyDeviceToHost, s));
    MEXK_CK(cudaStreamSynchronize(s));
    std::vector<int> blocks = build_row_blocks(rows, rp.data());
    int* d_blocks = nullptr;
    MEXK_CK(cudaMallocAsync(reinterpret_cast<void**>(&d_blocks), sizeof(int) * blocks.size(), s));
    MEXK_CK(cudaMemcpyAsync(d_blocks, blocks.data(), sizeof(int) * blocks.size(), cudaMemcpyHostToDevice, s));
    int rc = launch_spmv<TA, TX>(rows, static_cast<int>(blocks.size()) - 1, d_blocks, row_ptr, col_idx,
                                 values, x, y, nullptr, s, false);
    cudaError_t e = cudaFreeAsync(d_blocks, s);
    if (rc == MEXK_OK && e != cudaSuccess) {
        set_cuda_error(e, "cudaFreeAsync", __FILE__, __LINE__);
        rc = MEXK_ERR_CUDA;
    }
    if (rc == MEXK_OK) MEXK_CK(cudaStreamSynchronize(s));
    return rc;
}

}  // namespace mexk

extern "C" int mexk_spmv_f64(int rows, const int* row_ptr, const int* col_idx, const double* values,
                             const double* x, double* y, void* stream) {
    return mexk::spmv_standalone<double, double>(rows, row_ptr, col_idx, values, x, y, stream);
}

extern "C" int mexk_spmv_f32(int rows, const int* row_ptr, const int* col_idx, const float* values,
                             const float* x, float* y, void* stream) {
    return mexk::spmv_standalone<float, float>(rows, row_ptr, col_idx, values, x, y, stream);
}
