// Training and inference kernels of the learned step controller's network
// (8 -> 64 -> 64 -> 2, GELU, FP32), plus the standalone feature/prediction
// entry used to check the controller kernel's view of a basis.
//
// Training minimises the mean squared error of the normalised outputs with
// Adam. One thread block of 64 threads (one per hidden unit) runs forward
// and backward for chunks of 16 samples, keeps its share of the gradient in
// registers and writes one partial gradient; a second kernel sums the
// partials in block order (deterministic) and applies the Adam update.
#include "controller_net.cuh"

#include <vector>

namespace mexk {
namespace {

using namespace net;

constexpr int SB = 16;           // samples per chunk
constexpr int GRAD_BLOCKS = 64;  // partial gradients per minibatch

struct Stage {
    float xn[SB][IN];
    float z1[SB][HID], a1[SB][HID];
    float z2[SB][HID], a2[SB][HID];
    float d2[SB][HID];
    float dz3[SB][OUT];
    float loss[SB * OUT];
};

// Gradient of the batch loss over samples idx[0..count) (a minibatch) into
// partial[blockIdx.x][TRAINABLE] and the summed squared error into
// loss_part[blockIdx.x].
__global__ void __launch_bounds__(HID) mlp_grad_kernel(const float* __restrict__ w, const float* __restrict__ X,
                                                       const float* __restrict__ T, const int* __restrict__ idx,
                                                       int count, float* __restrict__ partial,
                                                       float* __restrict__ loss_part) {
    __shared__ Stage S;
    const int t = threadIdx.x;
    float gW1[IN], gW2[HID], gW3[OUT], gb1 = 0.f, gb2 = 0.f, gb3 = 0.f, lsum = 0.f;
#pragma unroll
    for (int i = 0; i < IN; ++i) gW1[i] = 0.f;
#pragma unroll
    for (int i = 0; i < HID; ++i) gW2[i] = 0.f;
#pragma unroll
    for (int c = 0; c < OUT; ++c) gW3[c] = 0.f;
    const float inv_count = 1.0f / (static_cast<float>(count) * OUT);
    for (int base = blockIdx.x * SB; base < count; base += gridDim.x * SB) {
        const int ns = min(SB, count - base);
        for (int e = t; e < SB * IN; e += HID) {
            const int s = e / IN, i = e % IN;
            S.xn[s][i] = (s < ns) ? (X[static_cast<size_t>(idx[base + s]) * IN + i] - w[FMEAN + i]) / w[FSTD + i] : 0.f;
        }
        __syncthreads();
        for (int s = 0; s < SB; ++s) {
            float z = w[B1 + t];
            for (int i = 0; i < IN; ++i) z = fmaf(S.xn[s][i], w[W1 + i * HID + t], z);
            S.z1[s][t] = z;
            S.a1[s][t] = gelu(z);
        }
        __syncthreads();
        for (int s = 0; s < SB; ++s) {
            float z = w[B2 + t];
            for (int i = 0; i < HID; ++i) z = fmaf(S.a1[s][i], w[W2 + i * HID + t], z);
            S.z2[s][t] = z;
            S.a2[s][t] = gelu(z);
        }
        __syncthreads();
        if (t < SB * OUT) {
            const int s = t / OUT, c = t % OUT;
            float z = w[B3 + c];
            for (int i = 0; i < HID; ++i) z = fmaf(S.a2[s][i], w[W3 + i * OUT + c], z);
            float d = 0.f, l = 0.f;
            if (s < ns) {
                const float tn = (T[static_cast<size_t>(idx[base + s]) * OUT + c] - w[OMEAN + c]) / w[OSTD + c];
                const float r = z - tn;
                d = 2.0f * r * inv_count;
                l = r * r;
            }
            S.dz3[s][c] = d;
            S.loss[t] = l;
        }
        __syncthreads();
        if (t == 0)
            for (int q = 0; q < SB * OUT; ++q) lsum += S.loss[q];
        // layer 3 and the hidden-2 error
        for (int s = 0; s < SB; ++s) {
            float da = 0.f;
#pragma unroll
            for (int c = 0; c < OUT; ++c) {
                gW3[c] = fmaf(S.a2[s][t], S.dz3[s][c], gW3[c]);
                da = fmaf(S.dz3[s][c], w[W3 + t * OUT + c], da);
            }
            S.d2[s][t] = da * gelu_grad(S.z2[s][t]);
        }
        if (t < OUT)
            for (int s = 0; s < SB; ++s) gb3 += S.dz3[s][t];
        __syncthreads();
        // layer 2 and the hidden-1 error
        for (int s = 0; s < SB; ++s) {
            const float dz = S.d2[s][t];
            gb2 += dz;
#pragma unroll
            for (int i = 0; i < HID; ++i) gW2[i] = fmaf(S.a1[s][i], dz, gW2[i]);
        }
        float d1[SB];
        for (int s = 0; s < SB; ++s) {
            float da = 0.f;
            for (int o = 0; o < HID; ++o) da = fmaf(S.d2[s][o], w[W2 + t * HID + o], da);
            d1[s] = da * gelu_grad(S.z1[s][t]);
        }
        // layer 1
        for (int s = 0; s < SB; ++s) {
            gb1 += d1[s];
#pragma unroll
            for (int i = 0; i < IN; ++i) gW1[i] = fmaf(S.xn[s][i], d1[s], gW1[i]);
        }
        __syncthreads();
    }
    float* P = partial + static_cast<size_t>(blockIdx.x) * TRAINABLE;
#pragma unroll
    for (int i = 0; i < IN; ++i) P[W1 + i * HID + t] = gW1[i];
    P[B1 + t] = gb1;
#pragma unroll
    for (int i = 0; i < HID; ++i) P[W2 + i * HID + t] = gW2[i];
    P[B2 + t] = gb2;
#pragma unroll
    for (int c = 0; c < OUT; ++c) P[W3 + t * OUT + c] = gW3[c];
    if (t < OUT) P[B3 + t] = gb3;
    if (t == 0) loss_part[blockIdx.x] = lsum;
}

// grad = sum of the partials in block order; optionally an Adam step.
__global__ void mlp_reduce_adam_kernel(const float* __restrict__ partial, int nparts, float* __restrict__ grad,
                                       float* __restrict__ w, float* __restrict__ mom, float* __restrict__ vel,
                                       float lr, float b1t, float b2t, int apply) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= TRAINABLE) return;
    float g = 0.f;
    for (int b = 0; b < nparts; ++b) g += partial[static_cast<size_t>(b) * TRAINABLE + p];
    if (grad) grad[p] = g;
    if (!apply) return;
    const float beta1 = 0.9f, beta2 = 0.999f, eps = 1e-8f;
    const float m = beta1 * mom[p] + (1.f - beta1) * g;
    const float v = beta2 * vel[p] + (1.f - beta2) * g * g;
    mom[p] = m;
    vel[p] = v;
    w[p] -= lr * (m / (1.f - b1t)) / (sqrtf(v / (1.f - b2t)) + eps);
}

__global__ void mlp_forward_kernel(const float* __restrict__ w, const float* __restrict__ X, int N,
                                   float* __restrict__ Y) {
    __shared__ float in[IN], a1[HID], a2[HID], out[OUT];
    for (int s = blockIdx.x; s < N; s += gridDim.x) {
        if (threadIdx.x < IN) in[threadIdx.x] = X[static_cast<size_t>(s) * IN + threadIdx.x];
        __syncthreads();
        mlp_forward_block(w, in, a1, a2, out);
        if (threadIdx.x < OUT) Y[static_cast<size_t>(s) * OUT + threadIdx.x] = out[threadIdx.x];
        __syncthreads();
    }
}

__global__ void predict_kernel(const float* __restrict__ w, const double* __restrict__ H, int ldh, int k,
                               double rem, double tol, double vnorm, double tau_prev, double err_prev,
                               float* __restrict__ out) {
    __shared__ float f[IN], a1[HID], a2[HID], o[OUT];
    __shared__ double col[192], n1s;
    const double n1 = basis_features(H, ldh, k, rem, tol, vnorm, tau_prev, err_prev, f, col, &n1s);
    if (w != nullptr) mlp_forward_block(w, f, a1, a2, o);
    if (threadIdx.x < IN) out[threadIdx.x] = f[threadIdx.x];
    if (threadIdx.x < OUT) out[IN + threadIdx.x] = (w != nullptr) ? o[threadIdx.x] : 0.f;
    if (threadIdx.x == 0) out[IN + OUT] = static_cast<float>(log2(n1));
}

}  // namespace
}  // namespace mexk

using namespace mexk;

extern "C" int mexk_mlp_forward(const float* weights, const float* X, int N, float* Y, void* stream) {
    if (!weights || !X || !Y || N < 0) return MEXK_ERR_INVALID;
    if (N == 0) return MEXK_OK;
    const int grid = N < 4096 ? N : 4096;
    mlp_forward_kernel<<<grid, net::HID, 0, static_cast<cudaStream_t>(stream)>>>(weights, X, N, Y);
    MEXK_CK_LAUNCH("mlp_forward_kernel");
    return MEXK_OK;
}

extern "C" int mexk_mlp_gradient(const float* weights, const float* X, const float* T, const int* idx, int count,
                                 float* grad, float* loss_parts, float* scratch, void* stream) {
    if (!weights || !X || !T || !idx || !grad || !loss_parts || !scratch || count < 1) return MEXK_ERR_INVALID;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    mlp_grad_kernel<<<GRAD_BLOCKS, net::HID, 0, s>>>(weights, X, T, idx, count, scratch, loss_parts);
    MEXK_CK_LAUNCH("mlp_grad_kernel");
    mlp_reduce_adam_kernel<<<(net::TRAINABLE + 255) / 256, 256, 0, s>>>(scratch, GRAD_BLOCKS, grad, nullptr,
                                                                          nullptr, nullptr, 0.f, 0.f, 0.f, 0);
    MEXK_CK_LAUNCH("mlp_reduce_adam_kernel");
    return MEXK_OK;
}

extern "C" int mexk_mlp_adam_step(float* weights, float* adam_state, const float* X, const float* T,
                                  const int* idx, int count, int step, float lr, float* loss_parts, float* scratch,
                                  void* stream) {
    if (!weights || !adam_state || !X || !T || !idx || !loss_parts || !scratch || count < 1 || step < 1)
        return MEXK_ERR_INVALID;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    mlp_grad_kernel<<<GRAD_BLOCKS, net::HID, 0, s>>>(weights, X, T, idx, count, scratch, loss_parts);
    MEXK_CK_LAUNCH("mlp_grad_kernel");
    const float b1t = powf(0.9f, static_cast<float>(step));
    const float b2t = powf(0.999f, static_cast<float>(step));
    mlp_reduce_adam_kernel<<<(net::TRAINABLE + 255) / 256, 256, 0, s>>>(
        scratch, GRAD_BLOCKS, nullptr, weights, adam_state, adam_state + net::TRAINABLE, lr, b1t, b2t, 1);
    MEXK_CK_LAUNCH("mlp_reduce_adam_kernel");
    return MEXK_OK;
}

extern "C" int mexk_controller_predict(const float* weights, const double* H, int ldh, int k, double rem, double tol,
                                       double vnorm, double tau_prev, double err_prev, float* out, void* stream) {
    if (!H || !out || k < 1 || k > MEXK_M_MAX_MIXED || ldh < k + 1) return MEXK_ERR_INVALID;
    predict_kernel<<<1, net::HID, 0, static_cast<cudaStream_t>(stream)>>>(weights, H, ldh, k, rem, tol, vnorm,
                                                                          tau_prev, err_prev, out);
    MEXK_CK_LAUNCH("predict_kernel");
    return MEXK_OK;
}
