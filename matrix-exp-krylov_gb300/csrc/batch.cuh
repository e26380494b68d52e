// Batched solves: many independent matrices, each with a block of up to 16
// right-hand sides, advanced together (mixed precision: FP32 matrix values
// and bases, FP64 Hessenberg, Gram matrix, exponentials and results).
//
// Row space: the problems' rows are concatenated, each problem padded to a
// multiple of 64 rows (padding rows are empty and their vectors zero), so
// every 64-row chunk and every tile belongs to one problem. Vectors are
// RHS-interleaved: row r of a vector holds the 16 right-hand sides of that
// row (64 bytes), so a thread owns one row quarter (a float4 of 4 RHS).
// State b = problem * 16 + rhs is an independent solve with its own
// DevState, Hessenberg, Gram matrix and scales (one column of the block is
// never mixed with another: these are 16 separate Krylov bases that share
// the matrix reads).
//
// A wave is a contiguous range of problems whose bases fit the memory
// budget; one cycle of a wave (m Arnoldi steps over every active state, the
// controllers, lifts and restarts) is one captured CUDA graph.
#pragma once

#include "mexk_internal.cuh"

namespace mexk {
namespace batch {

constexpr int BR = 16;                     // right-hand sides per row
constexpr int BT = 256;                    // threads per block
constexpr int BROWS = BT / 4;              // rows per block pass (64)
constexpr int BM_MAX = 32;                 // largest Krylov dimension
constexpr int BLD = BM_MAX + 1;            // leading dimension of H and G per state
constexpr int A_OFF = 0;                   // tile partial slots: a[c][r]
constexpr int B_OFF = BR * BM_MAX;         //                     b[c][r]
constexpr int W_OFF = 2 * BR * BM_MAX;     //                     |w|^2[r] (or |y|^2[r])
constexpr int BPS = 2 * BR * BM_MAX + BR;  // doubles per tile partial (1040)

struct Layout {
    int P;                 // problems in the wave
    int T;                 // tiles of the wave
    int C0, C1;            // 64-row chunks [C0, C1) of the wave (global chunk index)
    long long R0;          // first global row of the wave (vectors U, W index row - R0)
    const int* tile_prob;  // [T] problem (global index)
    const long long* tile_row0;  // [T] first global row
    const int* tile_nrows;       // [T] rows (multiple of 64)
    const int* ptile0;     // [global problem] first tile of the problem in this wave
    const int* ptiles;     // [global problem] tiles of the problem in this wave
    const int* chunk_prob; // [global chunk] problem
    const long long* prow0;     // [global problem] first global row
    const long long* row_ptr;   // [global rows + 1] CSR over all problems, local columns
    const int* col;
    const float* val;
    float* U;              // basis: column c at U + c * ldu, rows R0.. of the wave
    size_t ldu;            // floats per basis column (wave rows * 16)
    float* W;              // A u_j of the wave
    const double* V0;      // FP64 start vectors, all global rows [row][16]
    double* Y;             // FP64 results, all global rows [row][16]
    DevState* st;          // [global problem * 16 + rhs]
    double* H;             // per state BLD x BM_MAX, column-major
    double* G;             // per state BLD x BLD
    double* s;             // per state BLD+1 column scales
    double* pre;           // per state BLD+1 pre-scales
    float* coef;           // per state BLD update coefficients
    float* wsc;            // per state
    float* psc;            // per state
    double* coefl;         // per state BLD lift coefficients (from the controller)
    double* part;          // [T][BPS]
    unsigned int* pcount;  // [global problem] arrival counters
    int* pdone;            // [global problem] every state of the problem finished
    int* active;           // states still running after the cycle (one int)
};

// Per-step kernels; gg = columns per block of the dot sweep (2 or 4),
// unroll = x gathers issued together per row by the SpMM (4 or 8).
int launch_spmm(const Layout& L, int j, int unroll, cudaStream_t s);
int launch_dot(const Layout& L, int j, int reortho, int gg, int tune, cudaStream_t s);
int launch_update(const Layout& L, int j, cudaStream_t s);
int launch_norm_last(const Layout& L, int j, cudaStream_t s);
// Cycle kernels.
int launch_lift(const Layout& L, int k_max, int start, cudaStream_t s);
// from_start: u_0 from the start vectors V0, else from the lifted Y.
int launch_restart(const Layout& L, int from_start, cudaStream_t s);
int launch_status(const Layout& L, int p0, int p1, cudaStream_t s);

}  // namespace batch
}  // namespace mexk
