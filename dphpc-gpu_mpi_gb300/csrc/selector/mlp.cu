// mlp.cu — the learned algorithm selector's network, trained on the GPU by these kernels.
//
// No counterpart in the reference (one algorithm per collective there).  A 12 -> 64 -> 64 -> 4 fp32 MLP
// (ReLU hidden layers) maps call features (message size, rank count, datatype, operator, occupancy, kind)
// to predicted log-time of each reduction variant (DIRECT, TREE, RING, STAGED).  Loss: per sample, the
// squared error of the outputs whose variant was measured (mask), summed, averaged over the batch.
// Parameter layout (shared with the CPU oracle's fp64 restatement and the in-kernel inference):
//   W1[64][12], b1[64], W2[64][64], b2[64], W3[4][64], b3[4].
#include <cuda_runtime.h>

#include "gpumpi.h"

namespace {

constexpr int IN = 12, H = 64, OUT = 4;
constexpr int W1 = 0, B1 = W1 + H * IN, W2 = B1 + H, B2 = W2 + H * H, W3 = B2 + H, B3 = W3 + OUT * H;
constexpr int NP = B3 + OUT;
static_assert(NP == GPUMPI_MLP_NPARAMS, "parameter layout");
constexpr int SPB = 32;  // samples per block

// One block of 64 threads: thread j owns hidden unit j of both layers (and output j < 4).
// Gradients of the block's samples accumulate in shared memory, then go to `grads` with atomics.
__global__ void __launch_bounds__(64) mlp_grad_kernel(const float* __restrict__ p, const float* __restrict__ x,
                                                      const float* __restrict__ t, const float* __restrict__ mask,
                                                      int batch, float* __restrict__ grads, float* __restrict__ loss) {
    __shared__ float sx[IN], h1[H], h2[H], dz2[H], dy[OUT], sloss;
    __shared__ float gW2[H * H];
    const int j = (int)threadIdx.x;
    float gW1[IN], gb1 = 0.f, gb2 = 0.f, gW3[OUT], gb3 = 0.f;
    for (int i = 0; i < IN; i++) gW1[i] = 0.f;
    for (int o = 0; o < OUT; o++) gW3[o] = 0.f;
    for (int i = 0; i < H; i++) gW2[j * H + i] = 0.f;
    if (j == 0) sloss = 0.f;
    const int s0 = (int)blockIdx.x * SPB;
    for (int s = s0; s < s0 + SPB && s < batch; s++) {
        __syncthreads();
        if (j < IN) sx[j] = x[(long long)s * IN + j];
        __syncthreads();
        float z1 = p[B1 + j];
        for (int i = 0; i < IN; i++) z1 = fmaf(p[W1 + j * IN + i], sx[i], z1);
        h1[j] = z1 > 0.f ? z1 : 0.f;
        __syncthreads();
        float z2 = p[B2 + j];
        for (int i = 0; i < H; i++) z2 = fmaf(p[W2 + j * H + i], h1[i], z2);
        h2[j] = z2 > 0.f ? z2 : 0.f;
        __syncthreads();
        if (j < OUT) {
            float y = p[B3 + j];
            for (int i = 0; i < H; i++) y = fmaf(p[W3 + j * H + i], h2[i], y);
            const float m = mask[(long long)s * OUT + j];
            const float d = y - t[(long long)s * OUT + j];
            dy[j] = 2.f * m * d / (float)batch;
            atomicAdd(&sloss, m * d * d);
        }
        __syncthreads();
        // output layer: thread j accumulates column j of W3 for every output
        float dh2 = 0.f;
        for (int o = 0; o < OUT; o++) {
            gW3[o] = fmaf(dy[o], h2[j], gW3[o]);
            dh2 = fmaf(p[W3 + o * H + j], dy[o], dh2);
        }
        if (j < OUT) gb3 += dy[j];
        const float d2 = z2 > 0.f ? dh2 : 0.f;
        dz2[j] = d2;
        gb2 += d2;
        for (int i = 0; i < H; i++) gW2[j * H + i] = fmaf(d2, h1[i], gW2[j * H + i]);
        __syncthreads();
        float dh1 = 0.f;
        for (int k = 0; k < H; k++) dh1 = fmaf(p[W2 + k * H + j], dz2[k], dh1);
        const float d1 = z1 > 0.f ? dh1 : 0.f;
        gb1 += d1;
        for (int i = 0; i < IN; i++) gW1[i] = fmaf(d1, sx[i], gW1[i]);
    }
    __syncthreads();
    for (int i = 0; i < IN; i++) atomicAdd(&grads[W1 + j * IN + i], gW1[i]);
    atomicAdd(&grads[B1 + j], gb1);
    for (int i = 0; i < H; i++) atomicAdd(&grads[W2 + j * H + i], gW2[j * H + i]);
    atomicAdd(&grads[B2 + j], gb2);
    for (int o = 0; o < OUT; o++) atomicAdd(&grads[W3 + o * H + j], gW3[o]);
    if (j < OUT) atomicAdd(&grads[B3 + j], gb3);
    if (j == 0 && loss) atomicAdd(loss, sloss / (float)batch);
}

__global__ void __launch_bounds__(64) mlp_forward_kernel(const float* __restrict__ p, const float* __restrict__ x,
                                                         int batch, float* __restrict__ y) {
    __shared__ float sx[IN], h1[H], h2[H];
    const int j = (int)threadIdx.x;
    const int s0 = (int)blockIdx.x * SPB;
    for (int s = s0; s < s0 + SPB && s < batch; s++) {
        __syncthreads();
        if (j < IN) sx[j] = x[(long long)s * IN + j];
        __syncthreads();
        float z1 = p[B1 + j];
        for (int i = 0; i < IN; i++) z1 = fmaf(p[W1 + j * IN + i], sx[i], z1);
        h1[j] = z1 > 0.f ? z1 : 0.f;
        __syncthreads();
        float z2 = p[B2 + j];
        for (int i = 0; i < H; i++) z2 = fmaf(p[W2 + j * H + i], h1[i], z2);
        h2[j] = z2 > 0.f ? z2 : 0.f;
        __syncthreads();
        if (j < OUT) {
            float o = p[B3 + j];
            for (int i = 0; i < H; i++) o = fmaf(p[W3 + j * H + i], h2[i], o);
            y[(long long)s * OUT + j] = o;
        }
    }
}

__global__ void mlp_adam_kernel(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                                float* __restrict__ v, int step, float lr, float b1, float b2, float eps, float wd) {
    const int i = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (i >= NP) return;
    const float gi = g[i] + wd * p[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float mh = mi / (1.f - powf(b1, (float)step));
    const float vh = vi / (1.f - powf(b2, (float)step));
    p[i] -= lr * mh / (sqrtf(vh) + eps);
}

}  // namespace

extern "C" {

// Gradient of the masked loss over a batch (device buffers); grads (NP floats) and *loss are overwritten.
int gpumpi_mlp_loss_grad(const float* params, const float* x, const float* t, const float* mask, int batch,
                         float* grads, float* loss, void* stream) {
    if (!params || !x || !t || !mask || !grads || batch <= 0) return GPUMPI_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    if (cudaMemsetAsync(grads, 0, sizeof(float) * NP, s) != cudaSuccess) return GPUMPI_ERR_CUDA;
    if (loss && cudaMemsetAsync(loss, 0, sizeof(float), s) != cudaSuccess) return GPUMPI_ERR_CUDA;
    mlp_grad_kernel<<<(batch + SPB - 1) / SPB, 64, 0, s>>>(params, x, t, mask, batch, grads, loss);
    return cudaGetLastError() == cudaSuccess ? GPUMPI_SUCCESS : GPUMPI_ERR_LAUNCH;
}

int gpumpi_mlp_forward(const float* params, const float* x, int batch, float* y, void* stream) {
    if (!params || !x || !y || batch <= 0) return GPUMPI_ERR_ARG;
    mlp_forward_kernel<<<(batch + SPB - 1) / SPB, 64, 0, (cudaStream_t)stream>>>(params, x, batch, y);
    return cudaGetLastError() == cudaSuccess ? GPUMPI_SUCCESS : GPUMPI_ERR_LAUNCH;
}

// One Adam step (step counts from 1) with decoupled weight decay wd.
int gpumpi_mlp_adam_step(float* params, const float* grads, float* m, float* v, int step, float lr, float wd,
                         void* stream) {
    if (!params || !grads || !m || !v || step < 1) return GPUMPI_ERR_ARG;
    mlp_adam_kernel<<<(NP + 255) / 256, 256, 0, (cudaStream_t)stream>>>(params, grads, m, v, step, lr, 0.9f, 0.999f,
                                                                        1e-8f, wd);
    return cudaGetLastError() == cudaSuccess ? GPUMPI_SUCCESS : GPUMPI_ERR_LAUNCH;
}

}  // extern "C"
