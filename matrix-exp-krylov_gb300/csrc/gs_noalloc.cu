// Allocation-free Gram-Schmidt orthonormalisation of one vector.
//
// Some callers cannot allocate device memory at the moment they need this
// step: a host program that owns every device buffer through its own pool
// or arena, a language runtime that binds the C ABI over FFI and only hands
// over pre-allocated buffers, or a service whose request path is forbidden
// from calling cudaMalloc after start-up (allocation can block or fail under
// fragmentation). mexk_gram_schmidt_f64_noalloc runs the same three sweeps as
// the solver's Arnoldi step (pass-1 dots, pass-1 update + pass-2 dots,
// pass-2 update + norm) and the normalisation, but keeps its grid-reduction
// scratch in one fixed array in this file's device memory instead of memory
// a context allocated.
//
// The scratch array is shared by every call in the process on a given
// device and keeps the previous call's contents; each call clears the parts
// that must start at zero. Calls that overlap on the GPU (different streams
// or threads without ordering between them) race on it and give wrong
// results; serialise them.
#include "mexk_internal.cuh"


namespace mexk {
namespace {

// Largest grid the kernels may use with this scratch (gs_grid_size gives at
// most 4 blocks per SM: 608 on a 152-SM GB300); larger grids are capped, the
// sweeps stride over the rows.
constexpr int NOALLOC_MAX_BLOCKS = 1024;
// Largest basis this entry point orthogonalises against (one dot sweep).
constexpr int NOALLOC_K_MAX = 64;
static_assert(NOALLOC_K_MAX <= GS_DOT_COLS, "one dot sweep per pass");

// Byte layout of the scratch array.
constexpr size_t OFF_PARTIALS = 0;
constexpr size_t SZ_PARTIALS = sizeof(double) * NOALLOC_MAX_BLOCKS * RED_STRIDE;
constexpr size_t OFF_H1 = OFF_PARTIALS + SZ_PARTIALS;
constexpr size_t OFF_H2 = OFF_H1 + sizeof(double) * (NOALLOC_K_MAX + 2);
constexpr size_t OFF_STATE = (OFF_H2 + sizeof(double) * (NOALLOC_K_MAX + 2) + 255) / 256 * 256;
constexpr size_t OFF_COUNTER = (OFF_STATE + sizeof(DevState) + 255) / 256 * 256;
constexpr size_t SCRATCH_BYTES = OFF_COUNTER + 256;

// Every device that loads the library holds this array (about 600 KB) until
// the process exits.
static __device__ __align__(256) unsigned char g_gs_scratch[SCRATCH_BYTES];

// Device address of g_gs_scratch on the current device. Host code cannot
// use the symbol itself: on the host it names a stand-in, not device memory.
// Looked up on every call (no cache): after a device reset the module, and
// with it the array, may sit at another address.
int scratch_address(unsigned char** out) {
    void* p = nullptr;
    MEXK_CK(cudaGetSymbolAddress(&p, g_gs_scratch));
    *out = static_cast<unsigned char*>(p);
    return MEXK_OK;
}

}  // namespace
}  // namespace mexk

extern "C" int mexk_gram_schmidt_f64_noalloc(int n, int k, const double* V, int ldv, double* w,
                                              int reorthogonalize, double* h, double* beta, double* q,
                                              void* stream) {
    using namespace mexk;
    if (n < 1 || ldv < n || !V || !w || !h || !beta || !q) {
        set_error_text("mexk_gram_schmidt_f64_noalloc: bad pointer or size");
        return MEXK_ERR_INVALID;
    }
    if (k < 1 || k > NOALLOC_K_MAX) {
        set_error_text("mexk_gram_schmidt_f64_noalloc: k must be in 1..64 (scratch holds 64 coefficients)");
        return MEXK_ERR_INVALID;
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (s != nullptr) {
        // The scratch address belongs to the current device: so must the stream.
        int dev = 0, sdev = 0;
        MEXK_CK(cudaGetDevice(&dev));
        MEXK_CK(cudaStreamGetDevice(s, &sdev));
        if (sdev != dev) {
            set_error_text("mexk_gram_schmidt_f64_noalloc: the stream belongs to another device than the current one");
            return MEXK_ERR_INVALID;
        }
    }
    unsigned char* base = nullptr;
    int rc = scratch_address(&base);
    if (rc != MEXK_OK) return rc;
    int grid = gs_grid_size(n, k);
    if (grid > NOALLOC_MAX_BLOCKS) grid = NOALLOC_MAX_BLOCKS;
    DevState* st = reinterpret_cast<DevState*>(base + OFF_STATE);
    // A fresh running state (no breakdown, not done) and a zero block counter.
    MEXK_CK(cudaMemsetAsync(base + OFF_STATE, 0, SCRATCH_BYTES - OFF_STATE, s));
    GsArgs g;
    g.n = n;
    g.k = k;
    g.j = 0;      // with ldh = 1 the kernels write h[0..k-1] and leave beta to beta_out
    g.ldv = ldv;
    g.ldh = 1;
    g.reortho = reorthogonalize ? 1 : 0;
    g.V = V;
    g.w = w;
    g.H = h;
    g.h1 = reinterpret_cast<double*>(base + OFF_H1);
    g.h2 = reinterpret_cast<double*>(base + OFF_H2);
    g.partials = reinterpret_cast<double*>(base + OFF_PARTIALS);
    g.counter = reinterpret_cast<unsigned int*>(base + OFF_COUNTER);
    g.st = st;
    g.beta_out = beta;
    if ((rc = launch_gs_step(g, grid, s))) return rc;
    // q = w / beta (column j+1 = 0 of q); skipped on breakdown.
    return launch_normalize<double>(n, -1, ldv, w, q, st, nullptr, s);
}
