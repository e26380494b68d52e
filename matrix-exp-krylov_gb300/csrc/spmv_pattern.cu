// Row-pattern form of the context SpMV w = A x (replaces the cusparseSpMV of
// the reference's spmv_on_off, main.cu:1722-1767, like the other forms).
//
// Stencil matrices repeat a handful of rows: the 5-point heat operator has
// nine kinds (interior, four edges, four corners), each the same column
// offsets (col - row) and the same values. The pattern form stores one byte
// per row -- which of at most 256 distinct patterns (length <= 16, offsets
// ascending, values) the row is -- and reads offsets and values from the
// pattern table, which stays in L1. The matrix stream of the CSR forms
// (6-12 bytes per nonzero) becomes 1 byte per row: an SpMV moves n bytes,
// x once and w once.
//
// The form is exact: a row's products value * x[row + offset] are formed in
// column order and added left to right from zero, which is the order of the
// CSR forms' one-thread rows (<= 64 nonzeros), so FP64 results are bitwise
// those of the CSR forms. Detection runs on the device at upload: every row
// hashes (length, offsets, value bits) into an open-addressing table whose
// first inserter of a key takes the next pattern id and writes the pattern;
// a second pass looks each row's id up and compares the row with its
// pattern entry by entry (a hash collision, a row longer than 16 or more
// than 256 patterns leaves the context on the CSR forms).
#include <algorithm>
#include <vector>

#include "gram_step.cuh"

namespace mexk {

namespace {

constexpr int PAT_THREADS = 256;

// Probes of the hash table per key: a detection that succeeds holds at most
// PAT_MAX keys in PAT_SLOTS slots (a quarter full), so a longer probe
// sequence means too many patterns.
constexpr int PAT_PROBES = 64;

// Flags of the detection passes.
constexpr int PAT_LONG_ROW = 1;
constexpr int PAT_TOO_MANY = 2;
constexpr int PAT_MISMATCH = 4;

// splitmix64's output function (Steele, Lea, Flood 2014) as the mixing step.
__device__ __forceinline__ uint64_t pat_mix(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

// Key of row r (never 0), or 0 when the row is longer than PAT_LEN.
__device__ __forceinline__ uint64_t pat_row_key(int r, const int* __restrict__ row_ptr,
                                                const int* __restrict__ col_idx, const double* __restrict__ values) {
    const int e0 = row_ptr[r], e1 = row_ptr[r + 1];
    if (e1 - e0 > PAT_LEN) return 0;
    uint64_t h = pat_mix(0x9e3779b97f4a7c15ULL + static_cast<uint64_t>(e1 - e0));
    for (int e = e0; e < e1; ++e) {
        h = pat_mix(h ^ static_cast<uint32_t>(col_idx[e] - r));
        h = pat_mix(h ^ static_cast<uint64_t>(__double_as_longlong(values[e])));
    }
    return h | 1ull;
}

__global__ void pattern_insert_kernel(int n, const int* __restrict__ row_ptr, const int* __restrict__ col_idx,
                                      const double* __restrict__ values, RowPatterns* T, int* flags) {
    const int lane = threadIdx.x & 31;
    const int stride = gridDim.x * blockDim.x;
    // whole warps run every iteration (the match below takes the full mask)
    const int nw = (n + 31) & ~31;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < nw; r += stride) {
        // a failed detection stops at once (the warp decides together)
        if (__any_sync(0xffffffffu, *reinterpret_cast<volatile int*>(flags) != 0)) return;
        const uint64_t key = r < n ? pat_row_key(r, row_ptr, col_idx, values) : 0;
        if (r < n && key == 0) atomicOr(flags, PAT_LONG_ROW);
        const unsigned peers = __match_any_sync(0xffffffffu, key);
        if (key == 0 || lane != __ffs(peers) - 1) continue;
        // one lane per distinct key of the warp inserts it
        unsigned slot = static_cast<unsigned>(key) & (PAT_SLOTS - 1);
        bool done = false;
        for (int probe = 0; probe < PAT_PROBES && !done; ++probe, slot = (slot + 1) & (PAT_SLOTS - 1)) {
            unsigned long long k = *reinterpret_cast<volatile unsigned long long*>(&T->keys[slot]);
            if (k == 0) k = atomicCAS(&T->keys[slot], 0ull, static_cast<unsigned long long>(key));
            if (k == 0) {  // this lane inserted the key: take an id, write the pattern
                const int id = atomicAdd(&T->count, 1);
                if (id >= PAT_MAX) {
                    atomicOr(flags, PAT_TOO_MANY);
                } else {
                    T->ids[slot] = id;
                    const int e0 = row_ptr[r], len = row_ptr[r + 1] - e0;
                    T->len[id] = len;
                    for (int q = 0; q < len; ++q) {
                        T->off[id * PAT_LEN + q] = col_idx[e0 + q] - r;
                        T->v64[id * PAT_LEN + q] = values[e0 + q];
                        T->v32[id * PAT_LEN + q] = __double2float_rn(values[e0 + q]);
                    }
                }
                done = true;
            } else if (k == key) {
                done = true;
            }
        }
        if (!done) atomicOr(flags, PAT_TOO_MANY);
    }
}

__global__ void pattern_assign_kernel(int n, const int* __restrict__ row_ptr, const int* __restrict__ col_idx,
                                      const double* __restrict__ values, RowPatterns* __restrict__ T,
                                      uint8_t* __restrict__ pid, int* flags) {
    const int lane = threadIdx.x & 31;
    const int stride = gridDim.x * blockDim.x;
    const int nw = (n + 31) & ~31;  // whole warps run every iteration (the row count match)
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < nw; r += stride) {
        if (__any_sync(0xffffffffu, *reinterpret_cast<volatile int*>(flags) != 0)) return;  // failed: stop
        const uint64_t key = r < n ? pat_row_key(r, row_ptr, col_idx, values) : 0;
        int id = -1;
        if (key != 0) {  // rows without a key are flagged by the insert pass
            unsigned slot = static_cast<unsigned>(key) & (PAT_SLOTS - 1);
            for (int probe = 0; probe < PAT_PROBES; ++probe, slot = (slot + 1) & (PAT_SLOTS - 1)) {
                const unsigned long long k = T->keys[slot];
                if (k == key) {
                    id = T->ids[slot];
                    break;
                }
                if (k == 0) break;
            }
            if (id < 0 || id >= PAT_MAX) {
                atomicOr(flags, PAT_MISMATCH);
                id = -1;
            } else {
                const int e0 = row_ptr[r], len = row_ptr[r + 1] - e0;
                bool same = T->len[id] == len;
                for (int q = 0; q < len && same; ++q)
                    same = T->off[id * PAT_LEN + q] == col_idx[e0 + q] - r &&
                           __double_as_longlong(T->v64[id * PAT_LEN + q]) == __double_as_longlong(values[e0 + q]);
                if (!same) atomicOr(flags, PAT_MISMATCH);
                pid[r] = static_cast<uint8_t>(id);
            }
        }
        // rows per pattern, one atomic per distinct id of the warp
        const unsigned peers = __match_any_sync(0xffffffffu, id);
        if (id >= 0 && lane == __ffs(peers) - 1) atomicAdd(&T->rows[id], __popc(peers));
    }
}

template <typename TX>
__device__ __forceinline__ const TX* pat_values(const RowPatterns* T);
template <>
__device__ __forceinline__ const double* pat_values<double>(const RowPatterns* T) {
    return T->v64;
}
template <>
__device__ __forceinline__ const float* pat_values<float>(const RowPatterns* T) {
    return T->v32;
}

__device__ __forceinline__ double pat_mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float pat_mul(float a, float b) { return __fmul_rn(a, b); }

constexpr int PAT_RPT = 4;  // rows per thread and chunk
constexpr int PAT_CHUNK = PAT_THREADS * PAT_RPT;
static_assert(PAT_ROW_ALIGN % PAT_CHUNK == 0, "a chunk's ids lie inside the padded id array");
static_assert(PAT_RPT % 2 == 0, "the generic rows go in pairs");
constexpr unsigned PAT_FULL = 0xffffffffu;

// In its k-th chunk c (blocks stride over the chunks), warp w of a block
// takes the 128 consecutive rows of slice (w + k) mod 8: row i of lane l is
// c * PAT_CHUNK + 128 slice + 32 i + l (its ids, w and the gathers of one
// entry are whole 128-byte lines). Rotating the slices spreads the rows
// that meet a boundary -- at fixed places of every chunk on a grid whose
// lines are a multiple of the chunk -- over all warps. LMAX
// bounds every pattern's length; the major pattern (the one with the most
// rows) has major_len entries, whose offsets and values are held in
// registers from the start. A warp whose 128 rows are all major goes
// straight to its gathers; any other warp takes each non-major row's
// offsets and values from the table -- all entries of a row (two rows
// without DOTS, whose registers allow it) requested together, so a boundary
// costs a round trip per row, not one per entry -- unless all its rows share
// one pattern (a boundary line of a stencil: that pattern's entries are
// loaded once for the warp and the rows take the major pattern's loop). Either way a row's products are formed and added in
// entry order from zero. With DOTS (FP32 mixed form, a step j >= 1 over
// columns j-1 and j; DOTS 2: symmetric A, u_{j-1} w taken from the previous
// update as w_{j-1} u_j) each row sum also accumulates u_{j-1} w, u_j w, |w|^2
// and the last block finishes the step, as the staged CSR form does.
template <typename TX, int DOTS, int LMAX>
__global__ void __launch_bounds__(PAT_THREADS, 4)
    spmv_pattern_kernel(int n, int major, int major_len, const uint8_t* __restrict__ pid,
                        const RowPatterns* __restrict__ T, const TX* __restrict__ x, TX* __restrict__ y,
                        const int* __restrict__ skip, GramArgs ga) {
    const int tid = threadIdx.x;
    const int lane = tid & 31;
    const int nchunk = (n + PAT_CHUNK - 1) / PAT_CHUNK;
    constexpr int NW = PAT_THREADS / 32;
    const int warp = tid >> 5;
    // the thread's first row within its k-th chunk
    auto wrow = [&](int k) { return ((warp + k) % NW) * (32 * PAT_RPT) + lane; };
    const TX* __restrict__ tv = pat_values<TX>(T);
    const int* __restrict__ toff = T->off;
    const int* __restrict__ tlen = T->len;
    int ids[PAT_RPT];
    // Addresses: one base pointer per row group or pattern entry, the rows
    // 32 i apart at constant offsets from it (no 64-bit index arithmetic
    // per row and entry).
    auto load_ids = [&](int cc, int k) {  // pid is zero-padded to whole chunks
        const uint8_t* __restrict__ pb = pid + (static_cast<size_t>(cc) * PAT_CHUNK + wrow(k));
#pragma unroll
        for (int i = 0; i < PAT_RPT; ++i) ids[i] = cc < nchunk ? __ldg(pb + i * 32) : 0;
    };
    // the matrix is never written by a kernel: the major pattern and the
    // first ids load before the wait
    int mo[LMAX];
    TX ma[LMAX];
#pragma unroll
    for (int q = 0; q < LMAX; ++q) {
        const bool on = q < major_len;
        mo[q] = on ? __ldg(toff + major * PAT_LEN + q) : 0;
        ma[q] = on ? __ldg(tv + major * PAT_LEN + q) : TX(0);
    }
    int c = blockIdx.x;
    load_ids(c, 0);
    pdl_wait();
    if (skip != nullptr && *skip) return;
    pdl_trigger();
    float da0 = 0.f, da1 = 0.f, dw = 0.f;
    // DOTS: columns j-1 and j of the basis
    const float* __restrict__ vlo =
        DOTS == 1 ? ga.V + static_cast<size_t>(ga.lo) * static_cast<size_t>(ga.ldv) : nullptr;
    const float* __restrict__ vj = DOTS ? ga.V + static_cast<size_t>(ga.j) * static_cast<size_t>(ga.ldv) : nullptr;
    for (int k = 0; c < nchunk; c += gridDim.x, ++k) {
        const int r0 = c * PAT_CHUNK + wrow(k);
        int cur[PAT_RPT];
#pragma unroll
        for (int i = 0; i < PAT_RPT; ++i) cur[i] = ids[i];
        load_ids(c + gridDim.x, k + 1);
        float up[PAT_RPT], uj[PAT_RPT];
        if constexpr (DOTS == 1) {
            const float* __restrict__ vb = vlo + r0;
#pragma unroll
            for (int i = 0; i < PAT_RPT; ++i) up[i] = r0 + i * 32 < n ? __ldg(vb + i * 32) : 0.f;
        }
        auto load_uj = [&]() {  // u_j = x at the thread's rows
            if constexpr (DOTS) {
                const float* __restrict__ vb = vj + r0;
#pragma unroll
                for (int i = 0; i < PAT_RPT; ++i) uj[i] = r0 + i * 32 < n ? __ldg(vb + i * 32) : 0.f;
            }
        };
        // rows [r0, r0 + 32 i] in range and their sums in s: store, accumulate the dots
        auto emit = [&](const TX (&s)[PAT_RPT], bool all_in) {
            TX* __restrict__ yb = y + r0;
#pragma unroll
            for (int i = 0; i < PAT_RPT; ++i) {
                const int r = r0 + i * 32;
                if (all_in || r < n) {
                    yb[i * 32] = s[i];
                    if constexpr (DOTS) {
                        const float sf = static_cast<float>(s[i]);
                        if constexpr (DOTS == 1) da0 = fmaf(up[i], sf, da0);
                        da1 = fmaf(uj[i], sf, da1);
                        dw = fmaf(sf, sf, dw);
                    }
                }
            }
        };
        const bool all_in = r0 + (PAT_RPT - 1) * 32 < n;
        bool all_major = all_in;
#pragma unroll
        for (int i = 0; i < PAT_RPT; ++i) all_major = all_major && cur[i] == major;
        // one pattern over all of the warp's rows (a boundary line of a stencil)
        const int p0 = __shfl_sync(PAT_FULL, cur[0], 0);
        bool uniform = all_in;
#pragma unroll
        for (int i = 0; i < PAT_RPT; ++i) uniform = uniform && cur[i] == p0;
        TX s[PAT_RPT];
        if (!__all_sync(PAT_FULL, all_major) && __all_sync(PAT_FULL, uniform)) {
            // that pattern's entries once for the warp (broadcast loads), then
            // the gathers as for the major pattern, summed in the same order
            const int plen = __ldg(tlen + p0);
            int po[LMAX];
            TX pa[LMAX];
#pragma unroll
            for (int q = 0; q < LMAX; ++q) {
                const bool on = q < plen;
                po[q] = on ? __ldg(toff + p0 * PAT_LEN + q) : 0;
                pa[q] = on ? __ldg(tv + p0 * PAT_LEN + q) : TX(0);
            }
            const TX* xe[LMAX];
#pragma unroll
            for (int q = 0; q < LMAX; ++q) xe[q] = x + (r0 + po[q]);
            load_uj();
#pragma unroll
            for (int i = 0; i < PAT_RPT; ++i) {
                TX acc = TX(0);
#pragma unroll
                for (int q = 0; q < LMAX; ++q) {
                    if (q < plen) {
                        const TX xq = __ldg(xe[q] + i * 32);
                        acc += pat_mul(pa[q], xq);
                    }
                }
                s[i] = acc;
            }
            emit(s, true);
        } else if (__all_sync(PAT_FULL, all_major)) {
            const TX* xe[LMAX];
#pragma unroll
            for (int q = 0; q < LMAX; ++q) xe[q] = x + (r0 + mo[q]);
            load_uj();  // the rows' own lines, just gathered: L1 hits
#pragma unroll
            for (int i = 0; i < PAT_RPT; ++i) {
                TX acc = TX(0);
#pragma unroll
                for (int q = 0; q < LMAX; ++q) {
                    if (q < major_len) {
                        const TX xq = __ldg(xe[q] + i * 32);
                        acc += pat_mul(ma[q], xq);
                    }
                }
                s[i] = acc;
            }
            emit(s, true);
        } else {
            load_uj();
            constexpr int GP = DOTS == 1 ? 1 : 2;  // rows whose entries are in flight together (DOTS 1: registers)
            int len[PAT_RPT];
#pragma unroll
            for (int i = 0; i < PAT_RPT; ++i)
                len[i] = r0 + i * 32 < n ? (cur[i] == major ? major_len : __ldg(tlen + cur[i])) : 0;
#pragma unroll
            for (int i0 = 0; i0 < PAT_RPT; i0 += GP) {
                TX av[GP][LMAX], xv[GP][LMAX];
#pragma unroll
                for (int h = 0; h < GP; ++h) {
                    const int i = i0 + h;
                    const bool maj = cur[i] == major;
                    const int* to = toff + cur[i] * PAT_LEN;
                    const TX* ta = tv + cur[i] * PAT_LEN;
#pragma unroll
                    for (int q = 0; q < LMAX; ++q) {
                        const bool on = q < len[i];
                        const int o = maj ? mo[q] : (on ? __ldg(to + q) : 0);
                        av[h][q] = maj ? ma[q] : (on ? __ldg(ta + q) : TX(0));
                        xv[h][q] = on ? __ldg(x + (r0 + i * 32 + o)) : TX(0);
                    }
                }
#pragma unroll
                for (int h = 0; h < GP; ++h) {
                    TX acc = TX(0);
#pragma unroll
                    for (int q = 0; q < LMAX; ++q)
                        if (q < len[i0 + h]) acc += pat_mul(av[h][q], xv[h][q]);
                    s[i0 + h] = acc;
                }
            }
            emit(s, false);
        }
    }
    if constexpr (DOTS) {
        // block 0: the chain's first part from the previous update's partials,
        // done while the other blocks finish their rows
        if (blockIdx.x == 0) step2_precompute<20>(ga, ga.b_blocks);
        __shared__ double s_red[8][3];
        const float r0 = warp_sum(da0), r1 = warp_sum(da1), r2 = warp_sum(dw);
        if (lane == 0) {
            s_red[tid >> 5][0] = r0;
            s_red[tid >> 5][1] = r1;
            s_red[tid >> 5][2] = r2;
        }
        const int jj = ga.j;
        // DOTS 2 (symmetric A): a_{j-1} comes from the previous update, not from this sweep
        step_write_partials(s_red, ga.part, blockIdx.x, [&](int q) {
            return q == 0 ? (DOTS == 1 ? jj - 1 : -1) : q == 1 ? jj : GRAM_NWOFF;
        });
        __shared__ int s_flag;
        if (!grid_last_block(ga.counter, &s_flag)) return;
        step2_finish_pre<20>(ga, gridDim.x);  // <= 640 blocks: one round of partial loads
    }
}

template <typename TX, int DOTS, int LMAX>
int launch_pattern_as(int n, int major, int major_len, const uint8_t* pid, const RowPatterns* T, const TX* x,
                      TX* y, const int* skip, const GramArgs& ga, cudaStream_t s) {
    auto kern = spmv_pattern_kernel<TX, DOTS, LMAX>;
    static int resident = 0;  // thread blocks per SM (one device type per process)
    if (resident == 0) {
        const cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, kern, PAT_THREADS, 0);
        if (e != cudaSuccess || resident < 1) {
            resident = 0;
            set_cuda_error(e == cudaSuccess ? cudaErrorInvalidConfiguration : e, "spmv_pattern_kernel setup",
                           __FILE__, __LINE__);
            return MEXK_ERR_CUDA;
        }
    }
    const long long nchunk = (static_cast<long long>(n) + PAT_CHUNK - 1) / PAT_CHUNK;
    long long cap = static_cast<long long>(device_sm_count()) * resident;
    if (DOTS && cap > GRAM_MAX_ROW_BLOCKS) cap = GRAM_MAX_ROW_BLOCKS;  // one partial slot per block
    const int grid = static_cast<int>(nchunk < cap ? nchunk : cap);
    const cudaError_t e =
        launch_dependent(kern, grid, PAT_THREADS, 0, s, n, major, major_len, pid, T, x, y, skip, ga);
    if (e != cudaSuccess) {
        set_cuda_error(e, "spmv_pattern_kernel", __FILE__, __LINE__);
        return MEXK_ERR_CUDA;
    }
    return MEXK_OK;
}

// The longest pattern picks the kernel: the stencils' 3, 5, 7 and 9 entries
// (1-D, 2-D, 3-D, 2-D nine-point) unroll exactly.
template <typename TX, int DOTS>
int launch_pattern_len(int n, int major, int major_len, int max_len, const uint8_t* pid, const RowPatterns* T,
                       const TX* x, TX* y, const int* skip, const GramArgs& ga, cudaStream_t s) {
    if (max_len <= 3) return launch_pattern_as<TX, DOTS, 3>(n, major, major_len, pid, T, x, y, skip, ga, s);
    if (max_len <= 5) return launch_pattern_as<TX, DOTS, 5>(n, major, major_len, pid, T, x, y, skip, ga, s);
    if (max_len <= 7) return launch_pattern_as<TX, DOTS, 7>(n, major, major_len, pid, T, x, y, skip, ga, s);
    if (max_len <= 9) return launch_pattern_as<TX, DOTS, 9>(n, major, major_len, pid, T, x, y, skip, ga, s);
    return launch_pattern_as<TX, DOTS, PAT_LEN>(n, major, major_len, pid, T, x, y, skip, ga, s);
}

}  // namespace

int build_row_patterns(int n, const int* d_row_ptr, const int* d_col, const double* d_val, RowPatterns* d_T,
                       uint8_t* d_pid, int* d_flags, bool* ok, int* major, int* major_len, int* max_len,
                       cudaStream_t s) {
    *ok = false;
    *major = 0;
    *major_len = 0;
    *max_len = 0;
    if (n <= 0) return MEXK_OK;
    MEXK_CK(cudaMemsetAsync(d_T, 0, sizeof(RowPatterns), s));
    MEXK_CK(cudaMemsetAsync(d_flags, 0, sizeof(int), s));
    const long long want = (static_cast<long long>(n) + 255) / 256;
    const int grid = static_cast<int>(want < 8192 ? want : 8192);
    pattern_insert_kernel<<<grid, 256, 0, s>>>(n, d_row_ptr, d_col, d_val, d_T, d_flags);
    MEXK_CK_LAUNCH("pattern_insert_kernel");
    int flags = -1;
    MEXK_CK(cudaMemcpyAsync(&flags, d_flags, sizeof(int), cudaMemcpyDeviceToHost, s));
    MEXK_CK(cudaStreamSynchronize(s));
    if (flags != 0) return MEXK_OK;  // a row longer than PAT_LEN or too many patterns
    pattern_assign_kernel<<<grid, 256, 0, s>>>(n, d_row_ptr, d_col, d_val, d_T, d_pid, d_flags);
    MEXK_CK_LAUNCH("pattern_assign_kernel");
    MEXK_CK(cudaMemcpyAsync(&flags, d_flags, sizeof(int), cudaMemcpyDeviceToHost, s));
    MEXK_CK(cudaStreamSynchronize(s));
    *ok = flags == 0;
    if (*ok) {
        int count = 0;
        std::vector<int> len(PAT_MAX), rows(PAT_MAX);
        MEXK_CK(cudaMemcpy(&count, &d_T->count, sizeof(int), cudaMemcpyDeviceToHost));
        MEXK_CK(cudaMemcpy(len.data(), d_T->len, sizeof(int) * PAT_MAX, cudaMemcpyDeviceToHost));
        MEXK_CK(cudaMemcpy(rows.data(), d_T->rows, sizeof(int) * PAT_MAX, cudaMemcpyDeviceToHost));
        for (int q = 1; q < count && q < PAT_MAX; ++q)
            if (rows[q] > rows[*major]) *major = q;
        *major_len = len[*major];
        for (int q = 0; q < count && q < PAT_MAX; ++q) *max_len = std::max(*max_len, len[q]);
    }
    return MEXK_OK;
}

template <typename TX>
int launch_spmv_pattern(int n, int major, int major_len, int max_len, const uint8_t* pid, const RowPatterns* T,
                        const TX* x, TX* y, const int* skip_flag, cudaStream_t s, const GramArgs* dots) {
    if (n <= 0) return MEXK_OK;
    if (reinterpret_cast<uintptr_t>(pid) % 16 != 0 || reinterpret_cast<uintptr_t>(y) % (4 * sizeof(TX)) != 0) {
        set_error_text("spmv: pattern ids and w must be 16-byte aligned");
        return MEXK_ERR_INVALID;
    }
    const GramArgs none{};
    if constexpr (sizeof(TX) == 4) {
        if (dots) {
            if (dots->j < 1 || dots->lo != dots->j - 1 || dots->b_blocks < 1) return MEXK_ERR_INVALID;
            return dots->sym
                       ? launch_pattern_len<TX, 2>(n, major, major_len, max_len, pid, T, x, y, skip_flag, *dots, s)
                       : launch_pattern_len<TX, 1>(n, major, major_len, max_len, pid, T, x, y, skip_flag, *dots, s);
        }
    } else if (dots) {
        return MEXK_ERR_UNSUPPORTED;
    }
    return launch_pattern_len<TX, 0>(n, major, major_len, max_len, pid, T, x, y, skip_flag, none, s);
}

template int launch_spmv_pattern<double>(int, int, int, int, const uint8_t*, const RowPatterns*, const double*,
                                         double*, const int*, cudaStream_t, const GramArgs*);
template int launch_spmv_pattern<float>(int, int, int, int, const uint8_t*, const RowPatterns*, const float*, float*,
                                        const int*, cudaStream_t, const GramArgs*);

}  // namespace mexk
