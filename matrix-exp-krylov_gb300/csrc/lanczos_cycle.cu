// The steps of a short-recurrence (Lanczos, window 2) basis in one
// cooperative launch: the mixed-precision form's hot loop for symmetric
// stencil matrices (the row-pattern SpMV form).
//
// Per step the two-kernel form runs the pattern SpMV with the step's dot
// products (its last block finishes the step) and then the update sweep:
// w = A u_j travels to HBM and back, the row ids are read again every step,
// and two launches per step put the dependency chain SpMV -> reduction ->
// finish -> update -> next SpMV through kernel boundaries. Here one thread
// block per SM owns a fixed range of rows for the whole basis:
//   phase A  w = A u_j on its rows (ids and w in shared memory), u_j.w, |w|^2
//   barrier
//   phase B  every block sums the partials and runs the step's finish
//            (step2_chain, the same arithmetic as the two-kernel form;
//            block 0 stores H, the Gram entries and scales)
//   phase C  u_{j+1} = p (s_j w - (c_{j-1} u_{j-1} + c_j u_j)) on its rows,
//            and the next step's u_j.u_{j+1}, |u_{j+1}|^2, w_j.u_{j+1}
//   barrier
// so a step reads the gathered u_j (L2-resident: written by the previous
// phase C) and writes u_{j+1}, nothing else. The barriers are an arrival
// counter and a generation word with a bounded wait (about a second of
// %globaltimer): on expiry a block raises the abort word and ST_TIMEOUT and
// every block leaves; a cooperative launch guarantees that all blocks are
// resident, so the wait normally takes microseconds. Partials of phases A and C go to separate
// banks by step parity, so a block still summing step j's partials never
// sees them overwritten. Row sums and update arithmetic are those of the
// two-kernel form (products in entry order from zero; the update's FMA
// order); the dot products are summed in another order, so the two forms
// agree to rounding.
#include "gram_step.cuh"

namespace mexk {

namespace {

constexpr int LC_THREADS = 1024;
constexpr int LC_NW = LC_THREADS / 32;
constexpr int LC_GROUP = 128;        // rows of a warp's group (4 per lane)
constexpr int LC_SLOT_A = 2 * GRAM_M + 8;  // bank A(p) = {a_j, |w|^2} at LC_SLOT_A + 2 p
constexpr int LC_SLOT_C = LC_SLOT_A + 4;   // bank C(p) = {u_j.u_{j+1}, |u_{j+1}|^2, w_j.u_{j+1}} at LC_SLOT_C + 3 p
static_assert(LC_SLOT_C + 6 <= GRAM_SLOTS, "partial banks inside the slot array");
constexpr unsigned long long LC_WAIT_NS = 1000000000ull;

// Testing hook (mexk_test_force_wait_timeout): when set, block 0 leaves
// before its first grid barrier, so every other block's bounded wait runs
// out and the timeout path runs without any fault.
__device__ int g_test_lc_lost_block = 0;
size_t g_lc_smem_max = 0;  // dynamic shared memory a block may take (set by lanczos_cycle_prepare)

__device__ __forceinline__ unsigned long long lc_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Grid barrier: bar[0] counts the arrivals of the current barrier, bar[2]
// is its generation (the last block to arrive resets the count, then moves
// the generation on: the words return to their state after every barrier,
// so consecutive launches need no reset), bar[1] is the abort word. Returns
// true when every block arrived, false (after raising the abort word and,
// on expiry of the bounded wait, ST_TIMEOUT) when the wait gave up or
// another block gave up.
__device__ bool lc_barrier(unsigned* bar, int* status) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned* vbar = bar;
        const unsigned gen = vbar[2];
        __threadfence();
        int ok = 1;
        if (atomicAdd(&bar[0], 1u) == gridDim.x - 1) {
            atomicExch(&bar[0], 0u);
            __threadfence();
            atomicAdd(&bar[2], 1u);
        } else {
            const unsigned long long t0 = lc_ns();
            while (vbar[2] == gen) {
                if (vbar[1] != 0u) {
                    ok = 0;
                    break;
                }
                if (lc_ns() - t0 > LC_WAIT_NS) {
                    atomicExch(&bar[1], 1u);
                    atomicOr(status, ST_TIMEOUT);
                    ok = 0;
                    break;
                }
            }
        }
        __threadfence();
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// Block sums of NV FP32 per-thread values (FP64 over the warps, fixed order)
// into the row block's slots slot0 + v of the partial array.
template <int NV>
__device__ __forceinline__ void lc_write_partials(const float (&v)[NV], double* part, int slot0) {
    __shared__ double s_red[LC_NW][NV];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < NV; ++q) {
        const float r = warp_sum(v[q]);
        if (lane == 0) s_red[warp][q] = r;
    }
    __syncthreads();
    // warp q < NV sums value q over the 32 warps as an FP64 butterfly (five
    // dependent adds, not a chain of 32: FP64 adds take ~64 cycles here)
    static_assert(LC_NW == 32, "one lane per warp");
    if (warp < NV) {
        double t = s_red[lane][warp];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (lane == 0) part[static_cast<size_t>(slot0 + warp) * GRAM_MAX_ROW_BLOCKS + blockIdx.x] = t;
    }
}

__device__ __forceinline__ float lc_dot4(const float4& a, const float4& b) {
    return fmaf(a.x, b.x, fmaf(a.y, b.y, fmaf(a.z, b.z, a.w * b.w)));
}

template <int LMAX>
__global__ void __launch_bounds__(LC_THREADS, 1) lanczos_cycle_kernel(LanczosArgs a, int rows) {
    extern __shared__ __align__(16) unsigned char lc_smem[];
    const int tid = threadIdx.x;
    const int lane = tid & 31, warp = tid >> 5;
    const int r0 = blockIdx.x * rows;
    const int nr = min(a.n - r0, rows);  // > 0: the grid covers the rows exactly
    const int nr4 = (nr + 3) & ~3;
    float* s_w = reinterpret_cast<float*>(lc_smem);
    uint8_t* s_id = reinterpret_cast<uint8_t*>(s_w + rows);
    // constant during the solve: the block's row ids (16-byte loads; the id
    // array is zero-padded to whole 1024-row chunks), the major pattern
    const uint4* pid4 = reinterpret_cast<const uint4*>(a.pid + r0);
    for (int i = tid; i < (nr + 15) / 16; i += LC_THREADS) reinterpret_cast<uint4*>(s_id)[i] = __ldg(pid4 + i);
    for (int i = nr + tid; i < nr4; i += LC_THREADS) s_w[i] = 0.f;  // the update's float4 tail
    const float* __restrict__ tv = a.T->v32;
    const int* __restrict__ toff = a.T->off;
    const int* __restrict__ tlen = a.T->len;
    const int major = a.major, major_len = a.major_len;
    int mo[LMAX];
    float ma[LMAX];
#pragma unroll
    for (int q = 0; q < LMAX; ++q) {
        const bool on = q < major_len;
        mo[q] = on ? __ldg(toff + major * PAT_LEN + q) : 0;
        ma[q] = on ? __ldg(tv + major * PAT_LEN + q) : 0.f;
    }
    int q0 = -1;  // the major pattern's entry at offset 0, if any
#pragma unroll
    for (int q = 0; q < LMAX; ++q)
        if (q < major_len && mo[q] == 0) q0 = q;
    pdl_wait();
    DevState* st = a.st;
    if (st->breakdown || st->done) return;
    GramState* gs = a.gs;
    __shared__ double s_tot[5];
    __shared__ double s_carry[2];  // s_j and the next column's 1 / pre-scale
    __shared__ float s_sc[4];      // c_{j-1}, c_j, s_j, p
    __shared__ int s_bad;
    double s0 = gs->s[a.j0 - 1];
    double ip_j = gs->ip[a.j0];
    const size_t ldv = static_cast<size_t>(a.ldv);
    __syncthreads();
    for (int j = a.j0; j < a.m; ++j) {
        // ---- phase A: w = A u_j on the block's rows; u_j.w and |w|^2
        const float* uj = a.V + static_cast<size_t>(j) * ldv;
        float dsum[2] = {0.f, 0.f};
        for (int base = warp * LC_GROUP; base < nr; base += LC_NW * LC_GROUP) {
            int id[4];
            bool all_major = base + LC_GROUP <= nr;
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int rel = base + i * 32 + lane;
                id[i] = rel < nr ? s_id[rel] : major;
                all_major = all_major && id[i] == major;
            }
            float sum[4], ur[4];
            if (__all_sync(0xffffffffu, all_major)) {
                const float* xb = uj + r0 + base + lane;
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    float acc = 0.f;
#pragma unroll
                    for (int q = 0; q < LMAX; ++q) {
                        if (q < major_len) {
                            const float xq = xb[i * 32 + mo[q]];
                            if (q == q0) ur[i] = xq;
                            acc += __fmul_rn(ma[q], xq);
                        }
                    }
                    sum[i] = acc;
                    if (q0 < 0) ur[i] = xb[i * 32];
                }
            } else {
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    const int rel = base + i * 32 + lane;
                    float acc = 0.f, u = 0.f;
                    if (rel < nr) {
                        const int r = r0 + rel;
                        const int len = id[i] == major ? major_len : __ldg(tlen + id[i]);
                        const int* to = toff + id[i] * PAT_LEN;
                        const float* ta = tv + id[i] * PAT_LEN;
#pragma unroll
                        for (int q = 0; q < LMAX; ++q) {
                            if (q < len) {
                                const int o = id[i] == major ? mo[q] : __ldg(to + q);
                                const float av = id[i] == major ? ma[q] : __ldg(ta + q);
                                acc += __fmul_rn(av, uj[r + o]);
                            }
                        }
                        u = uj[r];
                    }
                    sum[i] = acc;
                    ur[i] = u;
                }
            }
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int rel = base + i * 32 + lane;
                if (rel < nr) {
                    s_w[rel] = sum[i];
                    dsum[0] = fmaf(ur[i], sum[i], dsum[0]);
                    dsum[1] = fmaf(sum[i], sum[i], dsum[1]);
                }
            }
        }
        lc_write_partials<2>(dsum, a.part, LC_SLOT_A + 2 * (j & 1));
        if (j == a.j0 && blockIdx.x == 0 && g_test_lc_lost_block != 0) return;
        if (!lc_barrier(a.bar, &st->status)) return;

        const float4* u4 = reinterpret_cast<const float4*>(uj + r0);
        const float4* p4 = reinterpret_cast<const float4*>(a.V + static_cast<size_t>(j - 1) * ldv + r0);
        const int nq = nr4 / 4;

        // ---- phase B: the step's finish in every block (the same sums and
        // arithmetic everywhere: every block reaches the same values)
        const int pa = LC_SLOT_A + 2 * (j & 1), pc = LC_SLOT_C + 3 * ((j - 1) & 1);
        const bool first = j == a.j0;
        const int G = static_cast<int>(gridDim.x);
        // tot = {a_{j-1}, a_j, b_{j-1}, b_j, |w|^2}
        step_sum_partials<8>(
            a.part, 5,
            [&](int v) {
                switch (v) {
                    case 0: return first ? j - 1 : pc + 2;
                    case 1: return pa;
                    case 2: return first ? GRAM_BOFF + j - 1 : pc;
                    case 3: return first ? GRAM_BOFF + j : pc + 1;
                    default: return pa + 1;
                }
            },
            [&](int v) { return (first && v != 1 && v != 4) ? a.b_blocks : G; }, s_tot);
        __syncthreads();
        if (tid == 0) {
            const Step2Out o = step2_chain(s_tot, 2, j, a.reortho, s0, ip_j);
            if (blockIdx.x == 0) {
                GramArgs g;
                g.n = a.n;
                g.j = j;
                g.lo = j - 1;
                g.ldv = a.ldv;
                g.ldh = a.ldh;
                g.reortho = a.reortho;
                g.V = a.V;
                g.H = a.H;
                g.gs = gs;
                g.st = st;
                step2_store(g, 2, o, s0);
            }
            s_bad = o.bad ? 1 : 0;
            s_carry[0] = o.sj;
            s_carry[1] = o.ip;
            s_sc[0] = static_cast<float>(s0 * o.hp);
            s_sc[1] = static_cast<float>(o.sj * o.hj);
            s_sc[2] = static_cast<float>(o.sj);
            s_sc[3] = static_cast<float>(o.p);
        }
        if (blockIdx.x == 0)  // H(0:j-2, j) = 0: outside the window
            for (int r = tid; r < j - 1; r += LC_THREADS) a.H[r + static_cast<size_t>(j) * a.ldh] = 0.0;
        __syncthreads();
        if (s_bad) return;  // breakdown at step j (the same decision in every block)
        s0 = s_carry[0];
        ip_j = s_carry[1];

        // ---- phase C: u_{j+1} on the block's rows, the next step's sums
        const float cp = s_sc[0], cj = s_sc[1], wsc = s_sc[2], psc = s_sc[3];
        float4* o4 = reinterpret_cast<float4*>(a.V + static_cast<size_t>(j + 1) * ldv + r0);
        const float4* w4 = reinterpret_cast<const float4*>(s_w);
        float nx[3] = {0.f, 0.f, 0.f};  // u_j.u_{j+1}, |u_{j+1}|^2, w_j.u_{j+1}
        auto upd = [&](const float4& x, const float4& u, const float4& v, int i) {
            float4 sv;
            sv.x = fmaf(u.x, cj, fmaf(v.x, cp, 0.f));
            sv.y = fmaf(u.y, cj, fmaf(v.y, cp, 0.f));
            sv.z = fmaf(u.z, cj, fmaf(v.z, cp, 0.f));
            sv.w = fmaf(u.w, cj, fmaf(v.w, cp, 0.f));
            float4 r;
            r.x = fmaf(x.x, wsc, -sv.x) * psc;
            r.y = fmaf(x.y, wsc, -sv.y) * psc;
            r.z = fmaf(x.z, wsc, -sv.z) * psc;
            r.w = fmaf(x.w, wsc, -sv.w) * psc;
            o4[i] = r;
            nx[0] += lc_dot4(u, r);
            nx[1] += lc_dot4(r, r);
            nx[2] += lc_dot4(x, r);
        };
        // four row groups per thread and round: their loads in flight together
        int i = tid;
        for (; i + 3 * LC_THREADS < nq; i += 4 * LC_THREADS) {
            float4 x[4], u[4], v[4];
#pragma unroll
            for (int h = 0; h < 4; ++h) {
                u[h] = u4[i + h * LC_THREADS];
                v[h] = p4[i + h * LC_THREADS];
                x[h] = w4[i + h * LC_THREADS];
            }
#pragma unroll
            for (int h = 0; h < 4; ++h) upd(x[h], u[h], v[h], i + h * LC_THREADS);
        }
        for (; i < nq; i += LC_THREADS) upd(w4[i], u4[i], p4[i], i);
        if (j + 1 < a.m) lc_write_partials<3>(nx, a.part, LC_SLOT_C + 3 * (j & 1));
        if (!lc_barrier(a.bar, &st->status)) return;
    }
}

// Rows per block: the rows split over one block per SM, rounded up to whole
// warp groups (their ids start 128-byte aligned).
int lc_rows(int n) {
    const int G = device_sm_count();
    long long r = (static_cast<long long>(n) + G - 1) / G;
    r = (r + LC_GROUP - 1) / LC_GROUP * LC_GROUP;
    return static_cast<int>(r);
}

size_t lc_smem_bytes(int rows) { return static_cast<size_t>(rows) * (sizeof(float) + 1); }

template <int LMAX>
int lc_launch_as(const LanczosArgs& a, cudaStream_t s) {
    const int rows = lc_rows(a.n);
    const int grid = (a.n + rows - 1) / rows;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(LC_THREADS);
    cfg.dynamicSmemBytes = lc_smem_bytes(rows);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const cudaError_t e = cudaLaunchKernelEx(&cfg, lanczos_cycle_kernel<LMAX>, a, rows);
    if (e != cudaSuccess) {
        set_cuda_error(e, "lanczos_cycle_kernel", __FILE__, __LINE__);
        return MEXK_ERR_CUDA;
    }
    return MEXK_OK;
}

}  // namespace

bool lanczos_cycle_fits(int n) {
    if (n < 1) return false;
    const int rows = lc_rows(n);
    return lc_smem_bytes(rows) <= g_lc_smem_max && (n + rows - 1) / rows <= GRAM_MAX_ROW_BLOCKS;
}

// Raises every instantiation's dynamic shared-memory limit to what the
// device allows a block beside the kernel's static shared memory; call per
// device before any launch or stream capture.
template <int LMAX>
int lc_prepare_as(int optin, size_t* common) {
    cudaFuncAttributes fa;
    MEXK_CK(cudaFuncGetAttributes(&fa, lanczos_cycle_kernel<LMAX>));
    const int bytes = optin - static_cast<int>(fa.sharedSizeBytes);
    if (bytes <= 0) return MEXK_ERR_UNSUPPORTED;
    MEXK_CK(cudaFuncSetAttribute(lanczos_cycle_kernel<LMAX>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    if (*common == 0 || static_cast<size_t>(bytes) < *common) *common = static_cast<size_t>(bytes);
    return MEXK_OK;
}

int lanczos_cycle_prepare() {
    int dev = 0, optin = 0;
    MEXK_CK(cudaGetDevice(&dev));
    MEXK_CK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    size_t common = 0;
    int rc;
    if ((rc = lc_prepare_as<3>(optin, &common)) || (rc = lc_prepare_as<5>(optin, &common)) ||
        (rc = lc_prepare_as<7>(optin, &common)) || (rc = lc_prepare_as<9>(optin, &common)) ||
        (rc = lc_prepare_as<PAT_LEN>(optin, &common)))
        return rc;
    g_lc_smem_max = common;
    return MEXK_OK;
}

int lanczos_cycle_test_hook(int enable) {
    const int v = enable ? 1 : 0;
    MEXK_CK(cudaMemcpyToSymbol(g_test_lc_lost_block, &v, sizeof(int)));
    return MEXK_OK;
}

int launch_lanczos_cycle(const LanczosArgs& a, cudaStream_t s) {
    if (a.j0 < 1 || a.m > GRAM_M || a.j0 >= a.m || !lanczos_cycle_fits(a.n) || a.ldv % 4 != 0 || a.b_blocks < 1 ||
        reinterpret_cast<uintptr_t>(a.V) % 16 != 0 || reinterpret_cast<uintptr_t>(a.pid) % 16 != 0)
        return MEXK_ERR_UNSUPPORTED;
    if (a.max_len <= 3) return lc_launch_as<3>(a, s);
    if (a.max_len <= 5) return lc_launch_as<5>(a, s);
    if (a.max_len <= 7) return lc_launch_as<7>(a, s);
    if (a.max_len <= 9) return lc_launch_as<9>(a, s);
    return lc_launch_as<PAT_LEN>(a, s);
}

}  // namespace mexk
