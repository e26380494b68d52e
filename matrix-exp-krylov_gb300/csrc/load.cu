// Binary CSR v1 (.bincsr) straight into a context.
//
// The reference reads a .bincsr file into host vectors with std::ifstream,
// checks every entry on the host (indptr order and range, column range, the
// sorted / no-duplicate flags), narrows u64 indices and widens f32 values
// element by element (CSRHost::from_binary_csr, main.cu:265-523), then
// copies the arrays to the device (DeviceContext::alloc_from, main.cu:873).
// For large files those host loops dominate the wall time. Here the file is
// memory-mapped, copied by a few host threads into two pinned chunks that
// alternate with the host-to-device copies, and everything else runs on the
// device: u64 -> int32 narrowing, f32 -> f64 widening, the checks (in the
// reference's order, reporting its first failure with its message), max|a_ij|
// for the command line's t clamp, and the SpMV schedule.
//
// Format (the reference's docs/binary_csr_v1.md): a 64-byte little-endian
// header -- magic "CSR\0\0\0\0\1", u32 version, u32 flags (bit 0 sorted, 1 no
// duplicates, 2 symmetric upper), u64 nrows, ncols, nnz, u32 index dtype
// (1 u32, 2 u64), u32 value dtype (1 f32, 2 f64), two reserved zero u64 --
// then indptr[nrows+1], indices[nnz], data[nnz], unpadded.
#include "mexk_internal.cuh"

#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <chrono>
#include <climits>
#include <cstring>
#include <limits>
#include <string>
#include <thread>
#include <vector>

namespace mexk {
namespace {

struct BinHeader {
    uint32_t version, flags;
    uint64_t nr, nc, nz;
    uint32_t idt, vdt;
};

uint32_t le32(const unsigned char* p) {
    return static_cast<uint32_t>(p[0]) | (static_cast<uint32_t>(p[1]) << 8) | (static_cast<uint32_t>(p[2]) << 16) |
           (static_cast<uint32_t>(p[3]) << 24);
}
uint64_t le64(const unsigned char* p) { return static_cast<uint64_t>(le32(p)) | (static_cast<uint64_t>(le32(p + 4)) << 32); }

int fail(const std::string& msg) {
    set_error_text(msg);
    return MEXK_ERR_INVALID;
}

// The header checks of CSRHost::from_binary_csr, in its order and with its
// messages (main.cu:265-330).
int parse_header(const unsigned char* h, uint64_t file_size, const std::string& fn, BinHeader* out) {
    if (file_size < 64) return fail("Error: Binary CSR file too small (expected at least 64 bytes): " + fn);
    static const unsigned char magic[8] = {'C', 'S', 'R', 0, 0, 0, 0, 1};
    if (std::memcmp(h, magic, 8) != 0) return fail("Error: Invalid Binary CSR magic in " + fn);
    BinHeader b;
    b.version = le32(h + 8);
    b.flags = le32(h + 12);
    b.nr = le64(h + 16);
    b.nc = le64(h + 24);
    b.nz = le64(h + 32);
    b.idt = le32(h + 40);
    b.vdt = le32(h + 44);
    const uint64_t res0 = le64(h + 48), res1 = le64(h + 56);
    if (b.version != 1)
        return fail("Error: Unsupported Binary CSR version " + std::to_string(b.version) + " in " + fn);
    if (b.idt != 1 && b.idt != 2) return fail("Error: Unsupported index_dtype=" + std::to_string(b.idt) + " in " + fn);
    if (b.vdt != 1 && b.vdt != 2) return fail("Error: Unsupported value_dtype=" + std::to_string(b.vdt) + " in " + fn);
    if (res0 != 0 || res1 != 0) return fail("Error: Reserved header fields must be zero in " + fn);
    const uint64_t imax = static_cast<uint64_t>(std::numeric_limits<int>::max());
    if (b.nr > imax || b.nc > imax || b.nz > imax)
        return fail("Error: Matrix dimensions/nnz exceed int32 limits used by solver in " + fn);
    const uint64_t ib = b.idt == 1 ? 4 : 8, vb = b.vdt == 1 ? 4 : 8;
    const uint64_t expected = 64 + (b.nr + 1) * ib + b.nz * ib + b.nz * vb;
    if (expected != file_size)
        return fail("Error: Binary CSR size mismatch in " + fn + " (expected " + std::to_string(expected) +
                    " bytes, got " + std::to_string(file_size) + ")");
    *out = b;
    return MEXK_OK;
}

void fill_info(const BinHeader& b, mexk_bincsr_info_t* info) {
    if (!info) return;
    info->rows = static_cast<long long>(b.nr);
    info->cols = static_cast<long long>(b.nc);
    info->nnz = static_cast<long long>(b.nz);
    info->index_dtype = static_cast<int>(b.idt);
    info->value_dtype = static_cast<int>(b.vdt);
    info->flags = b.flags;
    info->checks_passed = 1;
}

// ------------------------------------------------------------ device checks
// First failures, each the smallest index found (atomicMin), ULLONG_MAX = none.
struct LoadChecks {
    unsigned long long first_decrease;  // row r with indptr[r] > indptr[r+1]
    unsigned long long first_bad_col;   // k with indices[k] >= ncols
    unsigned long long first_bad_row;   // 2 r + (0 unsorted, 1 duplicate)
    unsigned long long ptr0, ptrn;      // indptr[0], indptr[nrows]
    unsigned long long max_abs_bits;    // max |a_ij| as ordered bits (non-negative doubles)
};

template <typename TI>
__global__ void check_indptr_kernel(const TI* __restrict__ p, long long nr, LoadChecks* c) {
    for (long long r = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; r < nr;
         r += static_cast<long long>(gridDim.x) * blockDim.x)
        if (static_cast<unsigned long long>(p[r]) > static_cast<unsigned long long>(p[r + 1]))
            atomicMin(&c->first_decrease, static_cast<unsigned long long>(r));
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        c->ptr0 = static_cast<unsigned long long>(p[0]);
        c->ptrn = static_cast<unsigned long long>(p[nr]);
    }
}

// indptr as int32 (after the checks: every entry <= nnz <= INT_MAX).
__global__ void narrow_indptr_kernel(const unsigned long long* __restrict__ p, int* __restrict__ out, long long n1) {
    for (long long r = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; r < n1;
         r += static_cast<long long>(gridDim.x) * blockDim.x)
        out[r] = static_cast<int>(p[r]);
}

// One chunk of indices [k0, k0 + count): the range check and, for u64 files,
// the narrowing into the context's int32 columns.
template <typename TI>
__global__ void indices_kernel(const TI* __restrict__ src, int* __restrict__ dst, long long k0, long long count,
                               unsigned long long ncols, LoadChecks* c) {
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < count;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const unsigned long long v = static_cast<unsigned long long>(src[i]);
        if (v >= ncols) atomicMin(&c->first_bad_col, static_cast<unsigned long long>(k0 + i));
        if (sizeof(TI) == 8) dst[i] = static_cast<int>(v);
    }
}

// One chunk of values: f32 widened into the context's f64 values (f64 files
// are copied as they are), and max |a_ij| (NaN skipped, as std::max skips it).
template <typename TV>
__global__ void values_kernel(const TV* __restrict__ src, double* __restrict__ dst, long long count, LoadChecks* c) {
    double m = 0.0;
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < count;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const double v = static_cast<double>(src[i]);
        if (sizeof(TV) == 4) dst[i] = v;
        const double a = fabs(v);
        if (a > m) m = a;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0 && m > 0.0) atomicMax(&c->max_abs_bits, static_cast<unsigned long long>(__double_as_longlong(m)));
}

// The sorted / no-duplicate flags, one thread per row: the first violation of
// the row decides its kind; the smallest row wins.
__global__ void check_rows_kernel(const int* __restrict__ rp, const int* __restrict__ ci, long long nr, int sorted,
                                  int nodup, LoadChecks* c) {
    for (long long r = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; r < nr;
         r += static_cast<long long>(gridDim.x) * blockDim.x) {
        for (int p = rp[r] + 1; p < rp[r + 1]; ++p) {
            const int a = ci[p - 1], b = ci[p];
            if (sorted && a > b) {
                atomicMin(&c->first_bad_row, 2ull * static_cast<unsigned long long>(r));
                break;
            }
            if (nodup && a == b) {
                atomicMin(&c->first_bad_row, 2ull * static_cast<unsigned long long>(r) + 1ull);
                break;
            }
        }
    }
}

int grid_for(long long n) { return static_cast<int>(std::max(1LL, std::min<long long>((n + 255) / 256, 8192))); }

// Host -> device streaming through two pinned chunks: while chunk c is copied
// to the device, the host threads fill chunk c + 1 from the mapped file.
class Streamer {
  public:
    static constexpr size_t CHUNK = 64ull << 20;
    Streamer(cudaStream_t s) : s_(s) {}
    ~Streamer() {
        for (int b = 0; b < 2; ++b) {
            if (ev_[b]) {
                cudaEventSynchronize(ev_[b]);
                cudaEventDestroy(ev_[b]);
            }
            if (pin_[b]) cudaFreeHost(pin_[b]);
        }
    }
    int init() {
        for (int b = 0; b < 2; ++b) {
            cudaError_t e = cudaHostAlloc(reinterpret_cast<void**>(&pin_[b]), CHUNK, cudaHostAllocWriteCombined);
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev_[b], cudaEventDisableTiming);
            if (e != cudaSuccess) {
                set_cuda_error(e, "pinned staging", __FILE__, __LINE__);
                return MEXK_ERR_ALLOC;
            }
        }
        threads_ = static_cast<int>(std::max(1u, std::min(8u, std::thread::hardware_concurrency())));
        return MEXK_OK;
    }
    // Copies bytes [src, src + bytes) to dst in chunks; after each chunk's
    // copy, per_chunk(offset, length) may enqueue work on the stream that
    // reads the chunk at dst + offset.
    template <typename ChunkFn>
    int copy(const unsigned char* src, size_t bytes, unsigned char* dst, ChunkFn per_chunk) {
        for (size_t off = 0; off < bytes; off += CHUNK) {
            const size_t len = std::min(CHUNK, bytes - off);
            const int b = cur_;
            cur_ ^= 1;
            cudaError_t e = cudaEventSynchronize(ev_[b]);  // this buffer's previous copy is done
            if (e != cudaSuccess) return cuda_fail(e);
            fill(pin_[b], src + off, len);
            e = cudaMemcpyAsync(dst + off, pin_[b], len, cudaMemcpyHostToDevice, s_);
            if (e != cudaSuccess) return cuda_fail(e);
            const int rc = per_chunk(off, len);
            if (rc) return rc;
            e = cudaEventRecord(ev_[b], s_);
            if (e != cudaSuccess) return cuda_fail(e);
        }
        return MEXK_OK;
    }

  private:
    void fill(unsigned char* dst, const unsigned char* src, size_t len) {
        const size_t per = (len + threads_ - 1) / threads_;
        if (threads_ == 1 || len < (4u << 20)) {
            std::memcpy(dst, src, len);
            return;
        }
        std::vector<std::thread> th;
        th.reserve(threads_);
        for (int t = 0; t < threads_; ++t) {
            const size_t a = t * per, z = std::min(len, a + per);
            if (a >= z) break;
            th.emplace_back([=] { std::memcpy(dst + a, src + a, z - a); });
        }
        for (auto& x : th) x.join();
    }
    static int cuda_fail(cudaError_t e) {
        set_cuda_error(e, "bincsr streaming", __FILE__, __LINE__);
        return MEXK_ERR_CUDA;
    }
    cudaStream_t s_;
    unsigned char* pin_[2] = {nullptr, nullptr};
    cudaEvent_t ev_[2] = {nullptr, nullptr};
    int cur_ = 0;
    int threads_ = 1;
};

struct Mapped {
    int fd = -1;
    void* p = MAP_FAILED;
    size_t size = 0;
    ~Mapped() {
        if (p != MAP_FAILED) munmap(p, size);
        if (fd >= 0) close(fd);
    }
};

int map_file(const char* path, Mapped* m) {
    const std::string fn(path);
    m->fd = open(path, O_RDONLY);
    if (m->fd < 0) return fail("Error: Could not open binary CSR file " + fn);
    struct stat st;
    if (fstat(m->fd, &st) != 0) return fail("Error: Could not open binary CSR file " + fn);
    m->size = static_cast<size_t>(st.st_size);
    if (m->size < 64) return fail("Error: Binary CSR file too small (expected at least 64 bytes): " + fn);
    m->p = mmap(nullptr, m->size, PROT_READ, MAP_PRIVATE, m->fd, 0);
    if (m->p == MAP_FAILED) return fail("Error: Failed to read 64-byte header from " + fn);
    madvise(m->p, m->size, MADV_SEQUENTIAL);
    return MEXK_OK;
}

template <typename T>
struct DevBuf {
    T* p = nullptr;
    ~DevBuf() {
        if (p) cudaFree(p);
    }
    int alloc(size_t count) {
        const cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&p), sizeof(T) * std::max<size_t>(count, 1));
        if (e != cudaSuccess) {
            set_cuda_error(e, "cudaMalloc", __FILE__, __LINE__);
            return MEXK_ERR_ALLOC;
        }
        return MEXK_OK;
    }
};

#define LOAD_CK(call)                                             \
    do {                                                          \
        const cudaError_t e_ = (call);                            \
        if (e_ != cudaSuccess) {                                  \
            set_cuda_error(e_, #call, __FILE__, __LINE__);        \
            return MEXK_ERR_CUDA;                                 \
        }                                                         \
    } while (0)

int load(mexk_context_t ctx, const char* path, int m_alloc_max, mexk_bincsr_info_t* info, cudaStream_t s) {
    const auto t_start = std::chrono::steady_clock::now();
    const std::string fn(path);
    Mapped map;
    int rc = map_file(path, &map);
    if (rc) return rc;
    const unsigned char* base = static_cast<const unsigned char*>(map.p);
    BinHeader h;
    if (info) info->checks_passed = 0;
    if ((rc = parse_header(base, map.size, fn, &h))) return rc;
    fill_info(h, info);
    if (h.flags & 4u) {
        set_error_text("symmetric_upper files are expanded on the host: load them with CSRHost::from_binary_csr");
        return MEXK_ERR_UNSUPPORTED;
    }
    if (h.nr < 1) {
        set_error_text("the solver needs a matrix with at least one row");
        return MEXK_ERR_UNSUPPORTED;
    }
    const long long nr = static_cast<long long>(h.nr), nz = static_cast<long long>(h.nz);
    const size_t ib = h.idt == 1 ? 4 : 8;
    const unsigned char* f_ptr = base + 64;
    const unsigned char* f_idx = f_ptr + (h.nr + 1) * ib;
    const unsigned char* f_val = f_idx + h.nz * ib;

    int *d_rp = nullptr, *d_ci = nullptr;
    double* d_va = nullptr;
    if ((rc = context_csr_begin(ctx, static_cast<int>(nr), nz, m_alloc_max, &d_rp, &d_ci, &d_va))) return rc;
    DevBuf<LoadChecks> chk;
    if ((rc = chk.alloc(1))) return rc;
    LoadChecks c0;
    std::memset(&c0, 0, sizeof(c0));
    c0.first_decrease = c0.first_bad_col = c0.first_bad_row = ULLONG_MAX;
    LOAD_CK(cudaMemcpyAsync(chk.p, &c0, sizeof(c0), cudaMemcpyHostToDevice, s));
    // Wide staging for u64 indptr (checked before narrowing) and for chunks
    // that need converting (u64 indices, f32 values).
    DevBuf<unsigned char> wide;
    const size_t wide_bytes = std::max<size_t>(h.idt == 2 ? (h.nr + 1) * 8 : 0, Streamer::CHUNK);
    if ((rc = wide.alloc(wide_bytes))) return rc;
    Streamer st(s);
    if ((rc = st.init())) return rc;
    auto none = [](size_t, size_t) { return MEXK_OK; };

    // indptr
    if (h.idt == 1) {
        if ((rc = st.copy(f_ptr, (h.nr + 1) * 4, reinterpret_cast<unsigned char*>(d_rp), none))) return rc;
        check_indptr_kernel<uint32_t><<<grid_for(nr), 256, 0, s>>>(reinterpret_cast<const uint32_t*>(d_rp), nr,
                                                                   chk.p);
    } else {
        if ((rc = st.copy(f_ptr, (h.nr + 1) * 8, wide.p, none))) return rc;
        check_indptr_kernel<unsigned long long>
            <<<grid_for(nr), 256, 0, s>>>(reinterpret_cast<const unsigned long long*>(wide.p), nr, chk.p);
    }
    LOAD_CK(cudaGetLastError());
    LoadChecks c;
    LOAD_CK(cudaMemcpyAsync(&c, chk.p, sizeof(c), cudaMemcpyDeviceToHost, s));
    LOAD_CK(cudaStreamSynchronize(s));
    if (c.ptr0 != 0) return fail("Error: indptr[0] must be 0 in " + fn);
    if (c.first_decrease != ULLONG_MAX)
        return fail("Error: indptr is not non-decreasing at row " + std::to_string(c.first_decrease) + " in " + fn);
    if (c.ptrn != h.nz) return fail("Error: indptr[nrows] != nnz in " + fn);
    if (info) info->checks_passed = 2;
    if (h.idt == 2) {
        narrow_indptr_kernel<<<grid_for(nr + 1), 256, 0, s>>>(reinterpret_cast<const unsigned long long*>(wide.p),
                                                              d_rp, nr + 1);
        LOAD_CK(cudaGetLastError());
    }

    // indices: range check (and narrowing) chunk by chunk
    const unsigned long long ncols = h.nc;
    if (h.idt == 1) {
        rc = st.copy(f_idx, h.nz * 4, reinterpret_cast<unsigned char*>(d_ci), [&](size_t off, size_t len) {
            const long long k0 = static_cast<long long>(off / 4), cnt = static_cast<long long>(len / 4);
            indices_kernel<uint32_t><<<grid_for(cnt), 256, 0, s>>>(reinterpret_cast<const uint32_t*>(d_ci) + k0,
                                                                   nullptr, k0, cnt, ncols, chk.p);
            return cudaGetLastError() == cudaSuccess ? MEXK_OK : MEXK_ERR_CUDA;
        });
    } else {
        // chunks land in the staging buffer (offset taken modulo the chunk)
        for (size_t off = 0; off < h.nz * 8 && rc == MEXK_OK; off += Streamer::CHUNK) {
            const size_t len = std::min(Streamer::CHUNK, h.nz * 8 - off);
            rc = st.copy(f_idx + off, len, wide.p, [&](size_t, size_t l) {
                const long long k0 = static_cast<long long>(off / 8), cnt = static_cast<long long>(l / 8);
                indices_kernel<unsigned long long><<<grid_for(cnt), 256, 0, s>>>(
                    reinterpret_cast<const unsigned long long*>(wide.p), d_ci + k0, k0, cnt, ncols, chk.p);
                return cudaGetLastError() == cudaSuccess ? MEXK_OK : MEXK_ERR_CUDA;
            });
        }
    }
    if (rc) return rc;
    // values: widening and max |a_ij|
    if (h.vdt == 2) {
        rc = st.copy(f_val, h.nz * 8, reinterpret_cast<unsigned char*>(d_va), [&](size_t off, size_t len) {
            const long long k0 = static_cast<long long>(off / 8), cnt = static_cast<long long>(len / 8);
            values_kernel<double><<<grid_for(cnt), 256, 0, s>>>(d_va + k0, nullptr, cnt, chk.p);
            return cudaGetLastError() == cudaSuccess ? MEXK_OK : MEXK_ERR_CUDA;
        });
    } else {
        for (size_t off = 0; off < h.nz * 4 && rc == MEXK_OK; off += Streamer::CHUNK) {
            const size_t len = std::min(Streamer::CHUNK, h.nz * 4 - off);
            rc = st.copy(f_val + off, len, wide.p, [&](size_t, size_t l) {
                const long long k0 = static_cast<long long>(off / 4), cnt = static_cast<long long>(l / 4);
                values_kernel<float><<<grid_for(cnt), 256, 0, s>>>(reinterpret_cast<const float*>(wide.p),
                                                                   d_va + k0, cnt, chk.p);
                return cudaGetLastError() == cudaSuccess ? MEXK_OK : MEXK_ERR_CUDA;
            });
        }
    }
    if (rc) return rc;
    LOAD_CK(cudaMemcpyAsync(&c, chk.p, sizeof(c), cudaMemcpyDeviceToHost, s));
    LOAD_CK(cudaStreamSynchronize(s));
    if (c.first_bad_col != ULLONG_MAX)
        return fail("Error: Column index out of range at k=" + std::to_string(c.first_bad_col) + " in " + fn);
    if (info) info->checks_passed = 3;
    const int sorted = (h.flags & 1u) != 0, nodup = (h.flags & 2u) != 0;
    if (sorted || nodup) {
        check_rows_kernel<<<grid_for(nr), 256, 0, s>>>(d_rp, d_ci, nr, sorted, nodup, chk.p);
        LOAD_CK(cudaGetLastError());
        LOAD_CK(cudaMemcpyAsync(&c, chk.p, sizeof(c), cudaMemcpyDeviceToHost, s));
        LOAD_CK(cudaStreamSynchronize(s));
        if (c.first_bad_row != ULLONG_MAX) {
            const std::string r = std::to_string(c.first_bad_row / 2);
            if (c.first_bad_row % 2 == 0)
                return fail("Error: Row " + r + " is not sorted but sorted flag is set in " + fn);
            return fail("Error: Row " + r + " has duplicates but no_duplicates flag is set in " + fn);
        }
    }
    if (info) info->checks_passed = 4;
    if (h.nr != h.nc) {  // a valid file the solver cannot use (the runner reports it)
        set_error_text("the solver needs a square matrix");
        return MEXK_ERR_UNSUPPORTED;
    }
    // The schedule needs indptr on the host: the validated int32 copy.
    std::vector<int> rp(static_cast<size_t>(nr) + 1);
    LOAD_CK(cudaMemcpyAsync(rp.data(), d_rp, sizeof(int) * rp.size(), cudaMemcpyDeviceToHost, s));
    LOAD_CK(cudaStreamSynchronize(s));
    if ((rc = context_csr_finish(ctx, rp.data()))) return rc;
    if (info) {
        double m;
        std::memcpy(&m, &c.max_abs_bits, sizeof(m));
        info->max_abs = m;
        info->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
    }
    return MEXK_OK;
}

}  // namespace
}  // namespace mexk

extern "C" int mexk_bincsr_probe(const char* path, mexk_bincsr_info_t* info) {
    using namespace mexk;
    if (!path) return MEXK_ERR_INVALID;
    const std::string fn(path);
    const int fd = open(path, O_RDONLY);
    if (fd < 0) return fail("Error: Could not open binary CSR file " + fn);
    struct stat st;
    unsigned char h[64];
    int rc = MEXK_OK;
    if (fstat(fd, &st) != 0) {
        rc = fail("Error: Could not open binary CSR file " + fn);
    } else if (st.st_size < 64) {
        rc = fail("Error: Binary CSR file too small (expected at least 64 bytes): " + fn);
    } else if (pread(fd, h, 64, 0) != 64) {
        rc = fail("Error: Failed to read 64-byte header from " + fn);
    } else {
        BinHeader b;
        rc = parse_header(h, static_cast<uint64_t>(st.st_size), fn, &b);
        if (rc == MEXK_OK) {
            fill_info(b, info);
            if (info) info->max_abs = info->seconds = 0.0;
        } else if (info) {
            info->checks_passed = 0;
        }
    }
    close(fd);
    return rc;
}

extern "C" int mexk_context_load_bincsr(mexk_context_t ctx, const char* path, int m_alloc_max,
                                        mexk_bincsr_info_t* info) {
    using namespace mexk;
    if (!ctx || !path) return MEXK_ERR_INVALID;
    cudaStream_t s = nullptr;
    const int rc = context_stream(ctx, &s);
    if (rc) return rc;
    return load(ctx, path, m_alloc_max, info, s);
}
