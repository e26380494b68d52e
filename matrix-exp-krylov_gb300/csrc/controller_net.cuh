// Step-size / Krylov-dimension network of the learned controller: features
// of a built Arnoldi basis and the forward pass of an 8 -> 64 -> 64 -> 2 MLP
// with GELU activations (FP32). Shared by the controller kernel and the
// standalone prediction / training entry points.
#pragma once

#include <math.h>

#include "mexk_internal.cuh"

namespace mexk {
namespace net {

constexpr int IN = 8;
constexpr int HID = 64;
constexpr int OUT = 2;
// Parameter layout (floats): W1[IN][HID], b1[HID], W2[HID][HID], b2[HID],
// W3[HID][OUT], b3[OUT], then the fixed input/output normalisation.
constexpr int W1 = 0;
constexpr int B1 = W1 + IN * HID;
constexpr int W2 = B1 + HID;
constexpr int B2 = W2 + HID * HID;
constexpr int W3 = B2 + HID;
constexpr int B3 = W3 + HID * OUT;
constexpr int TRAINABLE = B3 + OUT;  // 4866
constexpr int FMEAN = TRAINABLE;
constexpr int FSTD = FMEAN + IN;
constexpr int OMEAN = FSTD + IN;
constexpr int OSTD = OMEAN + OUT;
constexpr int TOTAL = OSTD + OUT;  // 4886

// Krylov dimensions the network may choose (one captured graph each).
constexpr int M_MIN = 10;
constexpr int M_MAX = 60;
constexpr int M_STEP = 5;

__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float x) {
    const float cdf = 0.5f * (1.0f + erff(x * 0.70710678118654752f));
    const float pdf = 0.39894228040143268f * expf(-0.5f * x * x);
    return cdf + x * pdf;
}

// Features of the basis H_k (column-major, leading dimension ldh; the
// subdiagonal entry H(k, k-1) included):
//   f0 log2(|H_k|_1 * remaining time)       f4 k / 64
//   f1 log2(H(k,k-1) / |H_k|_1)              f5 |H above the superdiagonal|_F / |H_k|_F
//   f2 subdiagonal log2-decay per column     f6 log2(previous step * |H_k|_1)
//      over the last half of the basis       f7 log2(previous estimate / tolerance)
//   f3 log2(tolerance / |v|)
// Every thread of the block calls it (k <= 64): thread j sums column j of
// H_k in row order (|H_k|_1 is the largest such sum), warp 0 combines the
// columns (the two squared-norm sums as a fixed xor butterfly: every lane
// ends with the same bits), lane 0 writes f. FP64 adds take about 64 clocks
// here, so a single thread's O(k^2) chain cost tens of microseconds. col:
// 192 doubles of shared scratch; n1: one shared double. Returns |H_k|_1 to
// every thread; deterministic.
__device__ inline double basis_features(const double* H, int ldh, int k, double rem, double tol, double vnorm,
                                        double tau_prev, double err_prev, float* f, double* col, double* n1_out) {
    const int t = threadIdx.x;
    for (int j = t; j < 64; j += blockDim.x) {
        double cs = 0.0, fr = 0.0, up = 0.0;
        if (j < k) {
            for (int i = 0; i <= j + 1 && i < k; ++i) {
                const double h = H[i + static_cast<size_t>(j) * ldh];
                cs += fabs(h);
                fr += h * h;
                if (i < j - 1) up += h * h;
            }
        }
        col[j] = cs;
        col[64 + j] = fr;
        col[128 + j] = up;
    }
    __syncthreads();
    if (t < 32) {
        double n1 = fmax(col[t], col[t + 32]);
        double fro = col[64 + t] + col[96 + t];
        double upper = col[128 + t] + col[160 + t];
        for (int o = 16; o >= 1; o >>= 1) {
            n1 = fmax(n1, __shfl_xor_sync(0xffffffffu, n1, o));
            fro += __shfl_xor_sync(0xffffffffu, fro, o);
            upper += __shfl_xor_sync(0xffffffffu, upper, o);
        }
        if (t == 0) {
            const double tiny = 1e-300;
            n1 = n1 > tiny ? n1 : tiny;
            const double hk = fabs(H[k + static_cast<size_t>(k - 1) * ldh]);
            const int jm = k / 2;  // column of the mid-basis subdiagonal
            const double hm = fabs(H[(jm + 1) + static_cast<size_t>(jm) * ldh]);
            const double span = (k - 1 - jm) > 0 ? static_cast<double>(k - 1 - jm) : 1.0;
            f[0] = static_cast<float>(log2(n1 * (rem > tiny ? rem : tiny)));
            f[1] = static_cast<float>(log2(hk / n1 + 1e-30));
            f[2] = static_cast<float>((log2(hk + tiny) - log2(hm + tiny)) / span);
            f[3] = static_cast<float>(log2(tol / (vnorm > tiny ? vnorm : tiny)));
            f[4] = static_cast<float>(k) / 64.0f;
            f[5] = static_cast<float>(fro > 0.0 ? sqrt(upper / fro) : 0.0);
            f[6] = tau_prev > 0.0 ? static_cast<float>(log2(tau_prev * n1)) : f[0];
            f[7] = err_prev > 0.0 ? static_cast<float>(log2(err_prev / tol)) : 0.0f;
            for (int i = 0; i < IN; ++i) {
                if (!isfinite(f[i])) f[i] = 0.0f;
                f[i] = fminf(fmaxf(f[i], -200.0f), 200.0f);
            }
            *n1_out = n1;
        }
    }
    __syncthreads();
    return *n1_out;
}

// Forward pass by the first HID threads of a block (all threads must call:
// it synchronises). in: raw features (shared); out[0..1] raw outputs
// (shared). a1/a2: HID-float shared scratch.
__device__ inline void mlp_forward_block(const float* __restrict__ w, const float* in, float* a1, float* a2,
                                         float* out) {
    const int t = threadIdx.x;
    if (t < HID) {
        float z = w[B1 + t];
        for (int i = 0; i < IN; ++i) z = fmaf((in[i] - w[FMEAN + i]) / w[FSTD + i], w[W1 + i * HID + t], z);
        a1[t] = gelu(z);
    }
    __syncthreads();
    if (t < HID) {
        float z = w[B2 + t];
        for (int i = 0; i < HID; ++i) z = fmaf(a1[i], w[W2 + i * HID + t], z);
        a2[t] = gelu(z);
    }
    __syncthreads();
    if (t < OUT) {
        float z = w[B3 + t];
        for (int i = 0; i < HID; ++i) z = fmaf(a2[i], w[W3 + i * OUT + t], z);
        out[t] = z * w[OSTD + t] + w[OMEAN + t];
    }
    __syncthreads();
}

// Network outputs -> (log2 of the step centre times |H_k|_1, next m).
__device__ __forceinline__ int next_m_from(float o1, int m_cap) {
    o1 = fminf(fmaxf(o1, 0.0f), 1.0f);  // also maps NaN (a broken network) to M_MIN
    const float mf = static_cast<float>(M_MIN) + o1 * static_cast<float>(M_MAX - M_MIN);
    int mq = static_cast<int>(rintf(mf / M_STEP)) * M_STEP;
    mq = mq < M_MIN ? M_MIN : (mq > M_MAX ? M_MAX : mq);
    return mq < m_cap ? mq : m_cap;
}

}  // namespace net
}  // namespace mexk
