// K1: CSR sparse matrix-vector product w = A*x on sm_103a.
//
// Replaces cusparseSpMV (reference main.cu:1722-1767, called with a fresh
// dense-vector descriptor per call). Design: the rows are cut into row
// blocks of at most SPMV_TILE nonzeros and SPMV_TILE_ROWS rows (one row
// per block when a row is longer), so every thread block streams a
// contiguous range of values and column indices with coalesced loads,
// whatever the row-length distribution (Laplacian stencils, Zipf rows).
// Phase 1 multiplies value * x[col] into shared memory; phase 2 sums each
// row's products. In a context (padded, aligned arrays) each thread block is
// persistent over a contiguous range of row blocks and double-buffers them:
// while it multiplies and sums one row block, the bulk-copy engine (TMA,
// cp.async.bulk) brings the next one's column indices, values and row
// pointers into shared memory, so the matrix stream never waits on the
// gather -> sum chain of a row block. Rows of at most SEQ_ROW_MAX nonzeros are summed in column
// order by one thread, so their FP64 result equals the reference's serial
// loop (main_cpu.cpp:388-397) bit for bit: one rounded product per nonzero,
// added left to right. Longer rows (the power-law tails) are summed by one
// warp each, and rows longer than a tile by the whole block, in fixed
// orders (deterministic, within rounding of the serial sum). The gathers of x are
// served from L2 (x is one basis column, read right after it was written).
#include "gram_step.cuh"

#include <algorithm>
#include <climits>

namespace mexk {

std::vector<int> build_row_blocks(int n, const int* row_ptr, int tile, int tile_rows) {
    std::vector<int> blocks;
    blocks.reserve(static_cast<size_t>(n) / 64 + 2);
    blocks.push_back(0);
    int r = 0;
    while (r < n) {
        const int start = r;
        const long long len0 = static_cast<long long>(row_ptr[r + 1]) - row_ptr[r];
        if (len0 > tile) {
            ++r;
        } else {
            long long acc = 0;
            while (r < n && r - start < tile_rows) {
                const long long len = static_cast<long long>(row_ptr[r + 1]) - row_ptr[r];
                if (acc + len > tile) break;
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

// Free-standing form (any alignment): one row block per thread block.
template <typename TA, typename TX>
__global__ void __launch_bounds__(SPMV_THREADS)
    spmv_rowblock_kernel(int nblocks, const int* __restrict__ blocks, const int* __restrict__ row_ptr,
                         const int* __restrict__ col_idx, const TA* __restrict__ values,
                         const TX* __restrict__ x, TX* __restrict__ y) {
    using TP = typename AccType<TX>::type;
    __shared__ TP prod[SPMV_TILE];
    __shared__ TP red[32];
    __shared__ int s_long[SPMV_TILE / (SEQ_ROW_MAX + 1) + 1];
    __shared__ int s_nlong;
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
#pragma unroll 4
        for (int e = tid; e < cnt; e += SPMV_THREADS) {
            const int c = __ldcs(&col_idx[e0 + e]);
            const TA a = __ldcs(&values[e0 + e]);
            prod[e] = static_cast<TP>(a) * static_cast<TP>(__ldg(&x[c]));
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

// ------------------------------------------------------------ bulk-copy staging
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_init_fence() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
// One arrival (the issuing thread's) plus `bytes` of transaction count.
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(
                     smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}
// L2 policy for data read once: evicted first, so that streaming the matrix
// does not push the basis vectors the next kernels read out of L2.
__device__ __forceinline__ uint64_t l2_evict_first_policy() {
    uint64_t pol;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}
// Global -> shared bulk copy (16-byte aligned addresses, size a multiple of 16)
// completing on `bar`.
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar,
                                              uint64_t pol) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], "
        "%4;" ::"r"(smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar)), "l"(pol)
        : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Orders this thread's earlier shared-memory accesses before later bulk copies.
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// Bounded wait for the phase of `bar` with the given parity: false after
// limit_ns (default about a second: the copies did not complete).
__device__ __noinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, unsigned long long limit_ns = 1000000000ull) {
    if (mbar_try_wait(bar, parity)) return true;
    const unsigned long long t0 = global_ns();
    while (!mbar_try_wait(bar, parity))
        if (global_ns() - t0 > limit_ns) return false;
    return true;
}

// Testing hook (mexk_test_force_wait_timeout): when set, block 0 of the
// staged SpMV also waits, with a 1 ms limit, on an mbarrier that nothing
// arrives at, so its bounded wait runs out and the timeout path (drain the
// copies in flight, ST_TIMEOUT, MEXK_ERR_DEVICE) runs without any fault.
__device__ int g_test_dead_wait = 0;
constexpr unsigned long long TEST_DEAD_WAIT_NS = 1000000ull;

// Shape of the context SpMV: threads per block, most nonzeros and rows per
// row block, shared-memory buffers per block, resident blocks per SM the
// register budget is set for.
constexpr int ST_THREADS = 256;
constexpr int ST_TILE = 2048;
constexpr int ST_ROWS = 512;
constexpr int ST_STAGES = 2;  // buffers (measured: 3 and 4 slower, 39.6 / 45.3 us against 38.0 on heat2048 FP32)
constexpr int ST_MINB = 5;

// Shared-memory image of one row block: the 16-byte groups of column indices
// (32-bit, or 16-bit offsets when NARROW: every staged row block of the
// matrix has them) and values its nonzeros span, then row_ptr from its first
// row rounded down to a multiple of 4 through its end row. The compact NARROW
// image leaves more of the SM's shared storage to L1, which serves the x
// gathers (heat2048 FP32: 38.0 against 38.8 us).
template <typename TA, bool NARROW>
struct TileStage {
    static constexpr int QMAX = (ST_TILE + 6) / 4;  // groups of 4 a row block spans
    static constexpr int COL = NARROW ? (QMAX * 8 + 15) / 16 * 16 : QMAX * 16;
    static constexpr int VAL = QMAX * 4 * static_cast<int>(sizeof(TA));
    static constexpr int RP = (ST_ROWS + 4 + 3) / 4 * 16;
    static constexpr int BYTES = COL + VAL + RP;
    static constexpr int STAGES = ST_STAGES;
    static_assert(COL % 16 == 0 && VAL % 16 == 0 && RP % 16 == 0, "bulk copies need 16-byte pieces");
};
constexpr int ST_QUADS = (TileStage<float, false>::QMAX + ST_THREADS - 1) / ST_THREADS;
constexpr int ST_RPT = (ST_ROWS + ST_THREADS - 1) / ST_THREADS;

template <typename TA, typename TP>
__device__ __forceinline__ void smem_quad(const TA* p, TP (&o)[4]);
template <>
__device__ __forceinline__ void smem_quad<float, float>(const float* p, float (&o)[4]) {
    const float4 t = *reinterpret_cast<const float4*>(p);
    o[0] = t.x;
    o[1] = t.y;
    o[2] = t.z;
    o[3] = t.w;
}
template <>
__device__ __forceinline__ void smem_quad<double, double>(const double* p, double (&o)[4]) {
    const double2 t0 = reinterpret_cast<const double2*>(p)[0];
    const double2 t1 = reinterpret_cast<const double2*>(p)[1];
    o[0] = t0.x;
    o[1] = t0.y;
    o[2] = t1.x;
    o[3] = t1.y;
}

// One warp per staged row block: the span of its columns; when it is at most
// 65536, the columns minus their minimum go to the block's slot of col16 (at
// the positions e - (first nonzero rounded down to 4) of its 16-byte groups;
// the slot was zeroed), else the block keeps 32-bit columns (z = -1).
__global__ void narrow_columns_kernel(int nblocks, int4* __restrict__ tiles, const int* __restrict__ col_idx,
                                      uint16_t* __restrict__ col16, int* __restrict__ all_narrow) {
    const int lane = threadIdx.x & 31;
    const int b = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (b >= nblocks) return;
    const int4 t = tiles[b];
    if (t.z < 0) return;  // one long row: streamed directly
    const int e0 = t.y, e1 = tiles[b + 1].y;
    int lo = INT_MAX, hi = INT_MIN;
    for (int e = e0 + lane; e < e1; e += 32) {
        const int c = col_idx[e];
        lo = min(lo, c);
        hi = max(hi, c);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    if (e1 == e0) lo = hi = 0;
    if (static_cast<long long>(hi) - lo > 65535) {
        if (lane == 0) {
            tiles[b].z = -1;
            atomicAnd(all_narrow, 0);
        }
        return;
    }
    const int base = e0 & ~3;
    for (int e = e0 + lane; e < e1; e += 32) col16[t.z + (e - base)] = static_cast<uint16_t>(col_idx[e] - lo);
    if (lane == 0) tiles[b].w = lo;
}

int build_spmv_schedule(int n, const int* row_ptr, const int* d_col, SpmvSchedule* out, cudaStream_t s) {
    const std::vector<int> blocks = build_row_blocks(n, row_ptr, ST_TILE, ST_ROWS);
    const int nb = static_cast<int>(blocks.size()) - 1;
    std::vector<int4> tiles(blocks.size());
    size_t slots = 0;
    for (int b = 0; b < nb; ++b) {
        const int r0 = blocks[b], e0 = row_ptr[r0], e1 = row_ptr[blocks[b + 1]];
        int off = -1;
        if (e1 - e0 <= ST_TILE) {
            const int base = e0 & ~3;
            const size_t nq = static_cast<size_t>(e1 - base + 3) >> 2;
            if (slots + 4 * nq + 8 > static_cast<size_t>(INT_MAX)) return MEXK_ERR_UNSUPPORTED;
            off = static_cast<int>(slots);
            slots += (4 * nq + 7) & ~static_cast<size_t>(7);
        }
        tiles[b] = make_int4(r0, e0, off, 0);
    }
    tiles[nb] = make_int4(n, row_ptr[n], -1, 0);
    out->nblocks = nb;
    out->all_narrow = true;
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&out->d_tiles), sizeof(int4) * tiles.size());
    if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&out->d_col16), sizeof(uint16_t) * (slots + 8));
    int* d_flag = nullptr;
    if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&d_flag), sizeof(int));
    if (e != cudaSuccess) {
        cudaFree(d_flag);
        set_cuda_error(e, "cudaMalloc", __FILE__, __LINE__);
        return MEXK_ERR_ALLOC;
    }
    const int one = 1;
    int flag = 1;
    e = cudaMemcpyAsync(out->d_tiles, tiles.data(), sizeof(int4) * tiles.size(), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(out->d_col16, 0, sizeof(uint16_t) * (slots + 8), s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_flag, &one, sizeof(int), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && nb > 0) {
        narrow_columns_kernel<<<(nb + 7) / 8, 256, 0, s>>>(nb, out->d_tiles, d_col, out->d_col16, d_flag);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(&flag, d_flag, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(d_flag);
    if (e != cudaSuccess) {
        set_cuda_error(e, "SpMV schedule", __FILE__, __LINE__);
        return MEXK_ERR_CUDA;
    }
    out->all_narrow = flag != 0;
    return MEXK_OK;
}

// Context form. tiles[b] = {first row, first nonzero, offset of its 16-bit
// columns in col16 or -1, their base} of row block b (b <= nblocks);
// col_idx/values 16-byte aligned with >= 3 entries past nnz, the column
// indices there zero; row_ptr with >= n + 4 entries. A row block whose
// columns span at most 65536 is staged from col16 (2 bytes per nonzero
// instead of 4). Thread block g
// takes row blocks [t0, t1) through SL::STAGES buffers: thread 0 issues the
// bulk copies of row block i + STAGES - 1 once every thread has finished
// row block i - 1 (whose buffer it reuses). Every staged 16-byte group is
// multiplied whole (its column indices are all valid, those outside the row
// block included), the products overwrite the staged values, and the row
// sums read only the row block's own. Row blocks of one long row are not
// staged: the block streams them directly.
//
// DOTS (FP32 mixed form, a step j >= 1 over columns lo = j-1 and j): every
// thread that writes a row sum w_r also accumulates u_{j-1,r} w_r, u_{j,r} w_r
// and w_r^2 (FP32 per thread); each block then writes its partials (FP64
// over the warps), and the last block to finish runs the step's finish
// (step2_finish: b partials from the previous update). This replaces the
// step's separate dot sweep.
template <typename TA, typename TX, bool NARROW, bool DOTS>
__global__ void __launch_bounds__(ST_THREADS, ST_MINB)
    spmv_stream_kernel(int nblocks, const int4* __restrict__ tiles, const uint16_t* __restrict__ col16,
                       const int* __restrict__ row_ptr, const int* __restrict__ col_idx,
                       const TA* __restrict__ values, const TX* __restrict__ x,
                       TX* __restrict__ y, const int* __restrict__ skip, int* __restrict__ status, GramArgs ga) {
    using TP = typename AccType<TX>::type;
    using SL = TileStage<TA, NARROW>;
    constexpr int S = SL::STAGES;
    static_assert(sizeof(TA) == sizeof(TP), "products overwrite the staged values");
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) uint64_t bar[S];
    __shared__ __align__(8) uint64_t dead_bar;  // the testing hook's barrier: never arrived at
    __shared__ TP red[32];
    __shared__ int s_long[ST_TILE / (SEQ_ROW_MAX + 1) + 1];
    __shared__ int s_nlong;
    const int tid = threadIdx.x;
    const int lane = tid & 31;
    const int g = blockIdx.x, G = gridDim.x;
    const int per = nblocks / G, extra = nblocks % G;
    const int t0 = g * per + (g < extra ? g : extra);
    const int t1 = t0 + per + (g < extra ? 1 : 0);
    auto staged = [&](int i) { return tiles[i + 1].y - tiles[i].y <= ST_TILE; };
    float da0 = 0.f, da1 = 0.f, dw = 0.f;  // DOTS: u_{j-1}.w, u_j.w, |w|^2
    auto dots_with = [&](float up, float uj, TP s) {
        if constexpr (DOTS) {
            const float sf = static_cast<float>(s);
            da0 = fmaf(up, sf, da0);
            da1 = fmaf(uj, sf, da1);
            dw = fmaf(sf, sf, dw);
        }
    };
    auto dots = [&](int r, TP s) {  // rows summed outside the thread's own (long rows)
        if constexpr (DOTS) {
            const size_t ldv = static_cast<size_t>(ga.ldv);
            dots_with(ga.V[static_cast<size_t>(ga.lo) * ldv + r], ga.V[static_cast<size_t>(ga.j) * ldv + r], s);
        }
    };
    auto issue = [&](int i, uint64_t pol) {  // thread 0
        const int4 a = tiles[i], b = tiles[i + 1];
        if (b.y - a.y > ST_TILE) return;
        const int s = (i - t0) % S;
        unsigned char* st = smem + s * SL::BYTES;
        const int base = a.y & ~3;
        const uint32_t nq = static_cast<uint32_t>((b.y - base + 3) >> 2);
        const int rbase = a.x & ~3;
        const uint32_t nrp = static_cast<uint32_t>((b.x + 1 - rbase + 3) & ~3);
        const bool nar = NARROW || a.z >= 0;
        const uint32_t bc = nar ? (nq + 1u) / 2u * 16u : nq * 16u;
        const uint32_t bv = nq * 4u * static_cast<uint32_t>(sizeof(TA)), br = nrp * 4u;
        mbar_arrive_expect_tx(&bar[s], bc + bv + br);
        if (nq > 0) {
            if (nar)
                bulk_copy_g2s(st, col16 + a.z, bc, &bar[s], pol);
            else
                bulk_copy_g2s(st, col_idx + base, bc, &bar[s], pol);
            bulk_copy_g2s(st + SL::COL, values + base, bv, &bar[s], pol);
        }
        bulk_copy_g2s(st + SL::COL + SL::VAL, row_ptr + rbase, br, &bar[s], pol);
    };
    uint64_t pol = 0;
    if (tid == 0) {
        pol = l2_evict_first_policy();
        for (int s = 0; s < S; ++s) mbar_init(&bar[s], 1);
        mbar_init(&dead_bar, 1);
        mbar_init_fence();
        // The matrix is never written by a kernel: its first row blocks are
        // requested before waiting for the previous kernel of the stream.
        for (int i = t0; i < t1 && i < t0 + S - 1; ++i) issue(i, pol);
    }
    __syncthreads();
    pdl_wait();
    const bool skipped = __syncthreads_or(skip != nullptr && *skip) != 0;
    unsigned phase = 0;  // bit s: parity of the next completion of buffer s
    int i = t0;
    bool fail = false;
    for (; i < t1 && !skipped; ++i) {
        const bool st_i = staged(i);
        const int sb = (i - t0) % S;
        bool ok = true;
        if (st_i) ok = mbar_wait(&bar[sb], (phase >> sb) & 1u);
        if (i == t0 && g == 0 && tid == 0 && g_test_dead_wait != 0)
            ok = mbar_wait(&dead_bar, 0u, TEST_DEAD_WAIT_NS) && ok;
        // also: every thread has finished row block i - 1
        if (__syncthreads_or(!ok)) {
            fail = true;
            break;
        }
        if (st_i) phase ^= 1u << sb;
        if (tid == 0 && i + S - 1 < t1) issue(i + S - 1, pol);
        if (i == t1 - 1) pdl_trigger();  // this block's last row block
        const int4 ta = tiles[i], tb = tiles[i + 1];
        const int r0 = ta.x, r1 = tb.x, e0 = ta.y, e1 = tb.y;
        if (!st_i) {
            // One long row: the block splits its nonzeros, then a tree sum.
            TP s = 0;
            for (int e = e0 + tid; e < e1; e += ST_THREADS)
                s += static_cast<TP>(__ldcs(&values[e])) * static_cast<TP>(__ldg(&x[__ldcs(&col_idx[e])]));
            s = block_sum(s, red);
            if (tid == 0) {
                y[r0] = static_cast<TX>(s);
                dots(r0, s);
            }
            continue;
        }
        unsigned char* st = smem + sb * SL::BYTES;
        const bool narrow = NARROW || ta.z >= 0;
        TP* sv = reinterpret_cast<TP*>(st + SL::COL);  // values, then products (entry e at e - base)
        const int* srp = reinterpret_cast<const int*>(st + SL::COL + SL::VAL);
        const int base = e0 & ~3;
        const int nq = (e1 - base + 3) >> 2;
        const int rbase = r0 & ~3;
        if (tid == 0) s_nlong = 0;
        // DOTS: the basis entries of the thread's own rows, requested now so
        // that they arrive during phase 1.
        float pre_p[ST_RPT], pre_j[ST_RPT];
        if constexpr (DOTS) {
            const size_t ldv = static_cast<size_t>(ga.ldv);
#pragma unroll
            for (int q = 0; q < ST_RPT; ++q) {
                const int r = r0 + tid + q * ST_THREADS;
                pre_p[q] = r < r1 ? __ldg(ga.V + static_cast<size_t>(ga.lo) * ldv + r) : 0.f;
                pre_j[q] = r < r1 ? __ldg(ga.V + static_cast<size_t>(ga.j) * ldv + r) : 0.f;
            }
        }
        // Phase 1: every gather of the thread issued together.
        int4 cq[ST_QUADS];
        if (narrow) {
            const uint2* sc = reinterpret_cast<const uint2*>(st);
            const int cb = ta.w;
#pragma unroll
            for (int q = 0; q < ST_QUADS; ++q) {
                const int gq = tid + q * ST_THREADS;
                const uint2 w = gq < nq ? sc[gq] : make_uint2(0u, 0u);
                cq[q] = make_int4(cb + static_cast<int>(w.x & 0xffffu), cb + static_cast<int>(w.x >> 16),
                                  cb + static_cast<int>(w.y & 0xffffu), cb + static_cast<int>(w.y >> 16));
            }
        } else {
            const int4* sc = reinterpret_cast<const int4*>(st);
#pragma unroll
            for (int q = 0; q < ST_QUADS; ++q) {
                const int gq = tid + q * ST_THREADS;
                cq[q] = gq < nq ? sc[gq] : make_int4(0, 0, 0, 0);
            }
        }
        TP xq[ST_QUADS][4];
#pragma unroll
        for (int q = 0; q < ST_QUADS; ++q) {
            xq[q][0] = static_cast<TP>(__ldg(&x[cq[q].x]));
            xq[q][1] = static_cast<TP>(__ldg(&x[cq[q].y]));
            xq[q][2] = static_cast<TP>(__ldg(&x[cq[q].z]));
            xq[q][3] = static_cast<TP>(__ldg(&x[cq[q].w]));
        }
#pragma unroll
        for (int q = 0; q < ST_QUADS; ++q) {
            const int gq = tid + q * ST_THREADS;
            if (gq < nq) {
                TP aq[4];
                smem_quad<TA, TP>(sv + 4 * gq, aq);
#pragma unroll
                for (int k = 0; k < 4; ++k) sv[4 * gq + k] = aq[k] * xq[q][k];
            }
        }
        __syncthreads();
        // Phase 2: rows of at most SEQ_ROW_MAX nonzeros left to right by one
        // thread; longer rows to a list, one warp each.
#pragma unroll
        for (int q = 0; q < ST_RPT; ++q) {
            const int r = r0 + tid + q * ST_THREADS;
            if (r < r1) {
                const int ra = srp[r - rbase], rz = srp[r + 1 - rbase];
                if (rz - ra > SEQ_ROW_MAX) {
                    s_long[atomicAdd(&s_nlong, 1)] = r;
                } else {
                    TP s = 0;
                    for (int p = ra - base; p < rz - base; ++p) s += sv[p];
                    y[r] = static_cast<TX>(s);
                    if constexpr (DOTS) dots_with(pre_p[q], pre_j[q], s);
                }
            }
        }
        __syncthreads();
        for (int li = tid >> 5; li < s_nlong; li += ST_THREADS / 32) {
            const int r = s_long[li];
            const int a = srp[r - rbase] - base;
            const int z = srp[r + 1 - rbase] - base;
            TP s = 0;
            for (int p = a + lane; p < z; p += 32) s += sv[p];
            s = warp_sum(s);
            if (lane == 0) {
                y[r] = static_cast<TX>(s);
                dots(r, s);
            }
        }
        // this thread's writes to the buffer before the next bulk copy into it
        fence_proxy_async_smem();
    }
    if (skipped || fail) {
        if (fail && tid == 0) atomicOr(status, ST_TIMEOUT);
        // No copy may still be writing this block's shared memory when it
        // exits: wait (bounded) for those issued and not consumed.
        for (int k = i; k < t1 && k < i + S - 1; ++k) {
            if (!staged(k)) continue;
            const int sb = (k - t0) % S;
            mbar_wait(&bar[sb], (phase >> sb) & 1u);
            phase ^= 1u << sb;
        }
    }
    if constexpr (DOTS) {
        // Every block that ran (a timed-out one too, so that the arrival count
        // stays whole) writes its partials; the last one finishes the step.
        if (skipped) return;
        if (blockIdx.x == 0) step2_precompute<16>(ga, ga.b_blocks);  // the chain's first part, as above
        __shared__ double s_red[8][3];
        const float r0 = warp_sum(da0), r1 = warp_sum(da1), r2 = warp_sum(dw);
        if (lane == 0) {
            s_red[tid >> 5][0] = r0;
            s_red[tid >> 5][1] = r1;
            s_red[tid >> 5][2] = r2;
        }
        const int jj = ga.j;
        step_write_partials(s_red, ga.part, blockIdx.x, [&](int q) { return q < 2 ? jj - 1 + q : GRAM_NWOFF; });
        __shared__ int s_flag;
        if (!grid_last_block(ga.counter, &s_flag)) return;
        step2_finish_pre<16>(ga, gridDim.x);
    }
}

// Global 16-byte group of 4 values, streamed (read once).
template <typename TA>
__device__ __forceinline__ void gquad(const TA* p, TA (&o)[4]);
template <>
__device__ __forceinline__ void gquad<float>(const float* p, float (&o)[4]) {
    const float4 t = __ldcs(reinterpret_cast<const float4*>(p));
    o[0] = t.x;
    o[1] = t.y;
    o[2] = t.z;
    o[3] = t.w;
}
template <>
__device__ __forceinline__ void gquad<double>(const double* p, double (&o)[4]) {
    const double2 t0 = __ldcs(reinterpret_cast<const double2*>(p));
    const double2 t1 = __ldcs(reinterpret_cast<const double2*>(p) + 1);
    o[0] = t0.x;
    o[1] = t0.y;
    o[2] = t1.x;
    o[3] = t1.y;
}

// Context form without staging, one thread block per row block (the same
// schedule): the block loads its 16-byte groups of columns and values
// directly, gathers x for every entry of those groups (the padding columns
// are zero, so no range tests), keeps the products in shared memory and sums
// the rows as spmv_stream_kernel does (same products, same order). Many
// short-lived blocks let the scheduler keep more gathers in flight than the
// persistent staged form: for matrices whose columns scatter over all of x
// (every product a separate gather, e.g. the power-law rows) this form is
// faster, for banded ones the staged form is. A context runs this form when
// some row block's columns span 65,536 or more (the staged form's 16-bit
// column layout does not apply).
template <typename TA, typename TX>
__global__ void __launch_bounds__(ST_THREADS)
    spmv_direct_kernel(int nblocks, const int4* __restrict__ tiles, const int* __restrict__ row_ptr,
                       const int* __restrict__ col_idx, const TA* __restrict__ values, const TX* __restrict__ x,
                       TX* __restrict__ y, const int* __restrict__ skip) {
    using TP = typename AccType<TX>::type;
    constexpr int QMAX = TileStage<TA, false>::QMAX;
    __shared__ TP prod[QMAX * 4];
    __shared__ TP red[32];
    __shared__ int s_long[ST_TILE / (SEQ_ROW_MAX + 1) + 1];
    __shared__ int s_nlong;
    const int tid = threadIdx.x;
    const int lane = tid & 31;
    const int b = blockIdx.x;
    const int4 ta = tiles[b], tb = tiles[b + 1];
    const int r0 = ta.x, r1 = tb.x, e0 = ta.y, e1 = tb.y;
    // the matrix is never written by a kernel: its loads may start before the
    // previous kernel of the stream has finished
    int ra[ST_RPT], rz[ST_RPT];
#pragma unroll
    for (int q = 0; q < ST_RPT; ++q) {
        const int r = r0 + tid + q * ST_THREADS;
        ra[q] = r < r1 ? row_ptr[r] : 0;
        rz[q] = r < r1 ? row_ptr[r + 1] : 0;
    }
    if (e1 - e0 > ST_TILE) {
        pdl_wait();
        if (skip != nullptr && *skip) return;
        if (b == static_cast<int>(gridDim.x) - 1) pdl_trigger();
        // One long row: the block splits its nonzeros, then a tree sum.
        TP s = 0;
        for (int e = e0 + tid; e < e1; e += ST_THREADS)
            s += static_cast<TP>(__ldcs(&values[e])) * static_cast<TP>(__ldg(&x[__ldcs(&col_idx[e])]));
        s = block_sum(s, red);
        if (tid == 0) y[r0] = static_cast<TX>(s);
        return;
    }
    const int base = e0 & ~3;
    const int nq = (e1 - base + 3) >> 2;
    int4 cq[ST_QUADS];
    TA aq[ST_QUADS][4];
#pragma unroll
    for (int q = 0; q < ST_QUADS; ++q) {
        const int gq = tid + q * ST_THREADS;
        if (gq < nq) {
            cq[q] = __ldcs(reinterpret_cast<const int4*>(col_idx + base) + gq);
            gquad<TA>(values + base + 4 * gq, aq[q]);
        } else {
            cq[q] = make_int4(0, 0, 0, 0);
        }
    }
    pdl_wait();
    if (skip != nullptr && *skip) return;
    if (b == static_cast<int>(gridDim.x) - 1) pdl_trigger();
    if (tid == 0) s_nlong = 0;
    TP xq[ST_QUADS][4];
#pragma unroll
    for (int q = 0; q < ST_QUADS; ++q) {
        xq[q][0] = static_cast<TP>(__ldg(&x[cq[q].x]));
        xq[q][1] = static_cast<TP>(__ldg(&x[cq[q].y]));
        xq[q][2] = static_cast<TP>(__ldg(&x[cq[q].z]));
        xq[q][3] = static_cast<TP>(__ldg(&x[cq[q].w]));
    }
#pragma unroll
    for (int q = 0; q < ST_QUADS; ++q) {
        const int gq = tid + q * ST_THREADS;
        if (gq < nq) {
#pragma unroll
            for (int k = 0; k < 4; ++k) prod[4 * gq + k] = static_cast<TP>(aq[q][k]) * xq[q][k];
        }
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < ST_RPT; ++q) {
        const int r = r0 + tid + q * ST_THREADS;
        if (r < r1) {
            if (rz[q] - ra[q] > SEQ_ROW_MAX) {
                s_long[atomicAdd(&s_nlong, 1)] = r;
            } else {
                TP s = 0;
                for (int p = ra[q] - base; p < rz[q] - base; ++p) s += prod[p];
                y[r] = static_cast<TX>(s);
            }
        }
    }
    __syncthreads();
    for (int li = tid >> 5; li < s_nlong; li += ST_THREADS / 32) {
        const int r = s_long[li];
        const int a = row_ptr[r] - base;
        const int z = row_ptr[r + 1] - base;
        TP s = 0;
        for (int p = a + lane; p < z; p += 32) s += prod[p];
        s = warp_sum(s);
        if (lane == 0) y[r] = static_cast<TX>(s);
    }
}

template <typename TA, typename TX, bool NARROW, bool DOTS>
int launch_spmv_as(int nblocks, const int4* tiles, const uint16_t* col16, const int* row_ptr, const int* col_idx,
                   const TA* values, const TX* x, TX* y, const int* skip_flag, int* status, const GramArgs& ga,
                   cudaStream_t s) {
    using SL = TileStage<TA, NARROW>;
    constexpr size_t smem = SL::STAGES * SL::BYTES;
    auto kern = spmv_stream_kernel<TA, TX, NARROW, DOTS>;
    static int resident = 0;  // thread blocks per SM (one device type per process)
    if (resident == 0) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
        if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, kern, ST_THREADS, smem);
        if (e != cudaSuccess || resident < 1) {
            resident = 0;
            set_cuda_error(e == cudaSuccess ? cudaErrorInvalidConfiguration : e, "spmv_stream_kernel setup", __FILE__,
                           __LINE__);
            return MEXK_ERR_CUDA;
        }
    }
    long long cap = static_cast<long long>(device_sm_count()) * resident;
    if (DOTS && cap > GRAM_MAX_ROW_BLOCKS) cap = GRAM_MAX_ROW_BLOCKS;  // one partial slot per block
    const int grid = static_cast<int>(nblocks < cap ? nblocks : cap);
    const cudaError_t e = launch_dependent(kern, grid, ST_THREADS, smem, s, nblocks, tiles, col16, row_ptr, col_idx,
                                           values, x, y, skip_flag, status, ga);
    if (e != cudaSuccess) {
        set_cuda_error(e, "spmv_stream_kernel", __FILE__, __LINE__);
        return MEXK_ERR_CUDA;
    }
    return MEXK_OK;
}

template <typename TA, typename TX>
int launch_spmv_direct(int nblocks, const int4* tiles, const int* row_ptr, const int* col_idx, const TA* values,
                       const TX* x, TX* y, const int* skip_flag, cudaStream_t s) {
    const cudaError_t e = launch_dependent(spmv_direct_kernel<TA, TX>, nblocks, ST_THREADS, 0, s, nblocks, tiles,
                                           row_ptr, col_idx, values, x, y, skip_flag);
    if (e != cudaSuccess) {
        set_cuda_error(e, "spmv_direct_kernel", __FILE__, __LINE__);
        return MEXK_ERR_CUDA;
    }
    return MEXK_OK;
}

template <typename TA, typename TX>
int launch_spmv(int n, int nblocks, const int4* tiles, const uint16_t* col16, bool all_narrow, const int* row_ptr,
                const int* col_idx, const TA* values, const TX* x, TX* y, const int* skip_flag, int* status,
                cudaStream_t s, const GramArgs* dots, bool direct) {
    if (n <= 0 || nblocks <= 0) return MEXK_OK;
    if (reinterpret_cast<uintptr_t>(col_idx) % 16 != 0 || reinterpret_cast<uintptr_t>(values) % 16 != 0 ||
        reinterpret_cast<uintptr_t>(row_ptr) % 16 != 0 || reinterpret_cast<uintptr_t>(col16) % 16 != 0) {
        set_error_text("spmv: context arrays must be 16-byte aligned");
        return MEXK_ERR_INVALID;
    }
    const GramArgs none{};
    if (direct && !dots) return launch_spmv_direct<TA, TX>(nblocks, tiles, row_ptr, col_idx, values, x, y, skip_flag, s);
    if constexpr (sizeof(TX) == 4) {
        if (dots) {
            // the staged form takes u_{j-1}.w itself (sym is the pattern form's)
            if (dots->j < 1 || dots->lo != dots->j - 1 || dots->b_blocks < 1 || dots->sym) return MEXK_ERR_INVALID;
            return all_narrow ? launch_spmv_as<TA, TX, true, true>(nblocks, tiles, col16, row_ptr, col_idx, values,
                                                                    x, y, skip_flag, status, *dots, s)
                              : launch_spmv_as<TA, TX, false, true>(nblocks, tiles, col16, row_ptr, col_idx, values,
                                                                     x, y, skip_flag, status, *dots, s);
        }
    } else if (dots) {
        return MEXK_ERR_UNSUPPORTED;
    }
    return all_narrow ? launch_spmv_as<TA, TX, true, false>(nblocks, tiles, col16, row_ptr, col_idx, values, x, y,
                                                             skip_flag, status, none, s)
                      : launch_spmv_as<TA, TX, false, false>(nblocks, tiles, col16, row_ptr, col_idx, values, x, y,
                                                              skip_flag, status, none, s);
}

template int launch_spmv<double, double>(int, int, const int4*, const uint16_t*, bool, const int*, const int*,
                                         const double*, const double*, double*, const int*, int*, cudaStream_t,
                                         const GramArgs*, bool);
template int launch_spmv<float, float>(int, int, const int4*, const uint16_t*, bool, const int*, const int*,
                                       const float*, const float*, float*, const int*, int*, cudaStream_t,
                                       const GramArgs*, bool);

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
// A == A^T exactly: every entry (r, c, v) has an entry (c, r, v). Row c is
// searched by bisection (its columns ascending, as the loaders and stencil
// generators give them); a row that bisection misses is scanned only when it
// is short (<= 64 entries) -- a long unsorted row makes the check answer
// "not symmetric" rather than cost a serial scan per entry. Threads stop once
// any of them found an asymmetry.
__global__ void symmetric_check_kernel(int n, const int* __restrict__ row_ptr, const int* __restrict__ col_idx,
                                       const double* __restrict__ values, int* __restrict__ ok) {
    for (long long rr = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; rr < n;
         rr += static_cast<long long>(gridDim.x) * blockDim.x) {
        if (*reinterpret_cast<volatile int*>(ok) == 0) return;
        const int r = static_cast<int>(rr);
        for (int e = row_ptr[r]; e < row_ptr[r + 1]; ++e) {
            const int c = col_idx[e];
            const double v = values[e];
            const int f0 = row_ptr[c], f1 = row_ptr[c + 1];
            int lo = f0, hi = f1;  // first position with col_idx >= r
            while (lo < hi) {
                const int mid = lo + (hi - lo) / 2;
                if (col_idx[mid] < r) lo = mid + 1;
                else hi = mid;
            }
            bool found = false;
            for (int f = lo; f < f1 && col_idx[f] == r; ++f)
                if (values[f] == v) {
                    found = true;
                    break;
                }
            if (!found && f1 - f0 <= 64) {
                for (int f = f0; f < f1; ++f)
                    if (col_idx[f] == r && values[f] == v) {
                        found = true;
                        break;
                    }
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
    const int nb = static_cast<int>(blocks.size()) - 1;
    int rc = MEXK_OK;
    spmv_rowblock_kernel<TA, TX><<<nb < 1048576 ? nb : 1048576, SPMV_THREADS, 0, s>>>(nb, d_blocks, row_ptr, col_idx,
                                                                                     values, x, y);
    const cudaError_t le = cudaGetLastError();
    if (le != cudaSuccess) {
        set_cuda_error(le, "spmv_rowblock_kernel", __FILE__, __LINE__);
        rc = MEXK_ERR_CUDA;
    }
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

extern "C" int mexk_test_force_wait_timeout(int device, int enable) {
    int count = 0;
    MEXK_CK(cudaGetDeviceCount(&count));
    if (device < 0 || device >= count) return MEXK_ERR_INVALID;
    MEXK_CK(cudaSetDevice(device));
    const int v = enable ? 1 : 0;
    MEXK_CK(cudaMemcpyToSymbol(mexk::g_test_dead_wait, &v, sizeof(int)));
    const int rc = mexk::lanczos_cycle_test_hook(enable);
    if (rc != MEXK_OK) return rc;
    MEXK_CK(cudaDeviceSynchronize());
    return MEXK_OK;
}
