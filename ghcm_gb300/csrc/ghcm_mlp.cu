// Training and inference kernels of the schedule MLP (12 -> 64 -> 64 -> 1,
// ReLU hidden layers, sigmoid output, FP32), written out by hand:
//
//   k_mlp_forward  one thread per sample, the parameters staged in shared
//                  memory (every thread of a warp reads the same weight: a
//                  broadcast), the first hidden layer in registers;
//   k_mlp_grad     64 samples per CTA: forward and backward pass per thread
//                  (activations and their gradients kept in padded shared
//                  rows), then the CTA sums each parameter's gradient over its
//                  samples - thread t owns parameters t, t + 64, ... so every
//                  reduction reads one broadcast row and one contiguous row -
//                  and adds it to the global gradient with one atomic;
//   k_adam         one thread per parameter: Adam with bias correction, then
//                  clears the gradient.
//
// Loss: binary cross-entropy on the logit, positives weighted by pos_weight.
// The parameter layout (ghcm_internal.h) is the one the in-kernel scorer
// (ghcm_learn.cuh) reads. No counterpart in the reference.
#include "ghcm_host.h"

#include <algorithm>
#include <cmath>
#include <vector>

namespace ghcm {
namespace {

constexpr int kTrainCta = 64;        // samples (threads) per gradient CTA
constexpr int kRow = kHidden + 1;    // padded shared row: thread s at bank (s + k) % 32

struct GradSmem {
    float p[kParams];
    float x[kTrainCta][kFeatures];
    float h1[kTrainCta][kRow];
    float h2[kTrainCta][kRow];
    float dh1[kTrainCta][kRow];
    float dh2[kTrainCta][kRow];
    float dz[kTrainCta];
    float loss[kTrainCta / 32];
};

__device__ __forceinline__ float sigmoidf(float z) { return 1.f / (1.f + expf(-z)); }

// log(1 + exp(-|z|)) + max(z, 0) - y z, the BCE of a logit, weighted
__device__ __forceinline__ float bce_logit(float z, float y, float pos_weight) {
    float const sp = log1pf(expf(-fabsf(z)));
    float const lp1 = -(sp + fmaxf(-z, 0.f));  // log sigmoid(z)
    float const lp0 = -(sp + fmaxf(z, 0.f));   // log (1 - sigmoid(z))
    return -(pos_weight * y * lp1 + (1.f - y) * lp0);
}

__global__ void k_mlp_forward(const float* __restrict__ P, const float* __restrict__ X, uint32_t n,
                              float* __restrict__ out) {
    extern __shared__ float sp[];
    for (int i = threadIdx.x; i < kParams; i += blockDim.x) sp[i] = P[i];
    __syncthreads();
    uint32_t const s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    float x[kFeatures];
#pragma unroll
    for (int i = 0; i < kFeatures; ++i) x[i] = X[static_cast<size_t>(s) * kFeatures + i];
    float h1[kHidden];
#pragma unroll
    for (int k = 0; k < kHidden; ++k) {
        float a = sp[kOffB1 + k];
#pragma unroll
        for (int i = 0; i < kFeatures; ++i) a = fmaf(sp[kOffW1 + i * kHidden + k], x[i], a);
        h1[k] = fmaxf(a, 0.f);
    }
    float z = sp[kOffB3];
    for (int j = 0; j < kHidden; ++j) {
        float a = sp[kOffB2 + j];
#pragma unroll
        for (int k = 0; k < kHidden; ++k) a = fmaf(sp[kOffW2 + k * kHidden + j], h1[k], a);
        z = fmaf(sp[kOffW3 + j], fmaxf(a, 0.f), z);
    }
    out[s] = sigmoidf(z);
}

// Gradient of the summed loss over samples [first, first + count), added to G;
// the summed loss is added to *loss_sum.
__global__ void __launch_bounds__(kTrainCta) k_mlp_grad(const float* __restrict__ P, const float* __restrict__ X,
                                                        const float* __restrict__ Y, uint32_t first, uint32_t count,
                                                        float pos_weight, float* __restrict__ G,
                                                        float* __restrict__ loss_sum) {
    extern __shared__ __align__(16) unsigned char raw[];
    GradSmem& sm = *reinterpret_cast<GradSmem*>(raw);
    int const t = threadIdx.x;
    for (int i = t; i < kParams; i += kTrainCta) sm.p[i] = P[i];
    uint32_t const local = blockIdx.x * kTrainCta + static_cast<uint32_t>(t);
    bool const valid = local < count;
    size_t const s = static_cast<size_t>(first) + local;
#pragma unroll
    for (int i = 0; i < kFeatures; ++i) sm.x[t][i] = valid ? X[s * kFeatures + i] : 0.f;
    __syncthreads();
    const float* p = sm.p;

    // forward
    float h1[kHidden];
#pragma unroll
    for (int k = 0; k < kHidden; ++k) {
        float a = p[kOffB1 + k];
#pragma unroll
        for (int i = 0; i < kFeatures; ++i) a = fmaf(p[kOffW1 + i * kHidden + k], sm.x[t][i], a);
        h1[k] = fmaxf(a, 0.f);
        sm.h1[t][k] = h1[k];
    }
    float z = p[kOffB3];
    for (int j = 0; j < kHidden; ++j) {
        float a = p[kOffB2 + j];
#pragma unroll
        for (int k = 0; k < kHidden; ++k) a = fmaf(p[kOffW2 + k * kHidden + j], h1[k], a);
        a = fmaxf(a, 0.f);
        sm.h2[t][j] = a;
        z = fmaf(p[kOffW3 + j], a, z);
    }
    float const y = valid ? Y[s] : 0.f;
    float const pr = sigmoidf(z);
    float const dz = valid ? (y > 0.5f ? pos_weight * (pr - 1.f) : pr) : 0.f;
    float loss = valid ? bce_logit(z, y, pos_weight) : 0.f;
    sm.dz[t] = dz;

    // backward through the hidden layers
    for (int j = 0; j < kHidden; ++j) sm.dh2[t][j] = (sm.h2[t][j] > 0.f) ? dz * p[kOffW3 + j] : 0.f;
#pragma unroll
    for (int k = 0; k < kHidden; ++k) {
        float a = 0.f;
        if (h1[k] > 0.f)
            for (int j = 0; j < kHidden; ++j) a = fmaf(p[kOffW2 + k * kHidden + j], sm.dh2[t][j], a);
        sm.dh1[t][k] = a;
    }
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) loss += __shfl_xor_sync(0xffffffffu, loss, o);
    if ((t & 31) == 0) sm.loss[t >> 5] = loss;
    __syncthreads();
    if (t == 0) {
        float l = 0.f;
        for (int w = 0; w < kTrainCta / 32; ++w) l += sm.loss[w];
        atomicAdd(loss_sum, l);
    }

    // parameter gradients summed over the CTA's samples
    for (int q = t; q < kParams; q += kTrainCta) {
        float g = 0.f;
        if (q < kOffB1) {
            int const i = (q - kOffW1) / kHidden, k = (q - kOffW1) % kHidden;
            for (int r = 0; r < kTrainCta; ++r) g = fmaf(sm.x[r][i], sm.dh1[r][k], g);
        } else if (q < kOffW2) {
            int const k = q - kOffB1;
            for (int r = 0; r < kTrainCta; ++r) g += sm.dh1[r][k];
        } else if (q < kOffB2) {
            int const k = (q - kOffW2) / kHidden, j = (q - kOffW2) % kHidden;
            for (int r = 0; r < kTrainCta; ++r) g = fmaf(sm.h1[r][k], sm.dh2[r][j], g);
        } else if (q < kOffW3) {
            int const j = q - kOffB2;
            for (int r = 0; r < kTrainCta; ++r) g += sm.dh2[r][j];
        } else if (q < kOffB3) {
            int const j = q - kOffW3;
            for (int r = 0; r < kTrainCta; ++r) g = fmaf(sm.dz[r], sm.h2[r][j], g);
        } else {
            for (int r = 0; r < kTrainCta; ++r) g += sm.dz[r];
        }
        atomicAdd(&G[q], g);
    }
}

__global__ void k_adam(float* __restrict__ P, float* __restrict__ G, float* __restrict__ M, float* __restrict__ V,
                       float lr, float b1, float b2, float eps, float bc1, float bc2, float scale) {
    int const i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kParams) return;
    float const g = G[i] * scale;
    G[i] = 0.f;
    float const m = b1 * M[i] + (1.f - b1) * g;
    float const v = b2 * V[i] + (1.f - b2) * g * g;
    M[i] = m;
    V[i] = v;
    P[i] -= lr * (m / bc1) / (sqrtf(v / bc2) + eps);
}

size_t grad_smem() { return sizeof(GradSmem); }

cudaError_t launch_grad(const float* P, const float* X, const float* Y, uint32_t first, uint32_t count,
                        float pos_weight, float* G, float* loss_sum, cudaStream_t st) {
    static bool attr = false;
    if (!attr) {
        cudaError_t const e =
            cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(grad_smem()));
        if (e != cudaSuccess) return e;
        attr = true;
    }
    unsigned const grid = (count + kTrainCta - 1) / kTrainCta;
    if (grid == 0) return cudaSuccess;
    k_mlp_grad<<<grid, kTrainCta, grad_smem(), st>>>(P, X, Y, first, count, pos_weight, G, loss_sum);
    return cudaGetLastError();
}

}  // namespace
}  // namespace ghcm

using namespace ghcm;

extern "C" {

int ghcm_train_config_default(ghcm_train_config* cfg) {
    if (!cfg) return GHCM_ERR_BAD_ARG;
    *cfg = ghcm_train_config{};
    cfg->epochs = 20;
    cfg->batch = 4096;
    cfg->lr = 1e-3f;
    cfg->beta1 = 0.9f;
    cfg->beta2 = 0.999f;
    cfg->adam_eps = 1e-8f;
    cfg->pos_weight = 1.f;
    return GHCM_OK;
}

int ghcm_mlp_forward(const float* d_params, const float* d_x, uint32_t n, float* d_prob, void* stream) {
    if (!d_params || (n && (!d_x || !d_prob))) return GHCM_ERR_BAD_ARG;
    if (n == 0) return GHCM_OK;
    unsigned const tb = 128;
    k_mlp_forward<<<(n + tb - 1) / tb, tb, kParams * sizeof(float), static_cast<cudaStream_t>(stream)>>>(d_params, d_x,
                                                                                                       n, d_prob);
    return map_cuda(cudaGetLastError());
}

int ghcm_mlp_grad(const float* d_params, const float* d_x, const float* d_y, uint32_t n, float pos_weight,
                  float* d_grad, float* d_loss_sum, void* stream) {
    if (!d_params || !d_grad || !d_loss_sum || (n && (!d_x || !d_y))) return GHCM_ERR_BAD_ARG;
    if (!(pos_weight > 0.f) || !std::isfinite(pos_weight)) return GHCM_ERR_BAD_ARG;
    return map_cuda(launch_grad(d_params, d_x, d_y, 0u, n, pos_weight, d_grad, d_loss_sum,
                                static_cast<cudaStream_t>(stream)));
}

int ghcm_mlp_train(const float* d_x, const float* d_y, uint32_t n, float* d_params, const ghcm_train_config* cfg,
                   void* stream, float* epoch_losses) {
    if (!d_x || !d_y || !d_params || !cfg || n == 0) return GHCM_ERR_BAD_ARG;
    if (cfg->epochs == 0 || cfg->batch == 0 || !(cfg->lr > 0.f) || !(cfg->beta1 >= 0.f && cfg->beta1 < 1.f) ||
        !(cfg->beta2 >= 0.f && cfg->beta2 < 1.f) || !(cfg->adam_eps > 0.f) || !(cfg->pos_weight > 0.f))
        return GHCM_ERR_BAD_ARG;
    for (uint32_t r : cfg->reserved)
        if (r != 0u) return GHCM_ERR_BAD_ARG;
    cudaStream_t const st = static_cast<cudaStream_t>(stream);
    DevBuf buf;  // grad | m | v | per-epoch loss sums
    size_t const pbytes = align_up(kParams * sizeof(float), 256);
    if (!buf.reserve(3 * pbytes + cfg->epochs * sizeof(float))) return GHCM_ERR_OOM;
    float* G = reinterpret_cast<float*>(buf.as<char>());
    float* M = reinterpret_cast<float*>(buf.as<char>() + pbytes);
    float* V = reinterpret_cast<float*>(buf.as<char>() + 2 * pbytes);
    float* L = reinterpret_cast<float*>(buf.as<char>() + 3 * pbytes);
    cudaError_t e = cudaMemsetAsync(buf.p, 0, buf.bytes, st);
    double b1t = 1.0, b2t = 1.0;
    for (uint32_t ep = 0; ep < cfg->epochs && e == cudaSuccess; ++ep) {
        for (uint32_t first = 0; first < n && e == cudaSuccess; first += cfg->batch) {
            uint32_t const count = std::min(cfg->batch, n - first);
            e = launch_grad(d_params, d_x, d_y, first, count, cfg->pos_weight, G, L + ep, st);
            b1t *= cfg->beta1;
            b2t *= cfg->beta2;
            if (e == cudaSuccess) {
                k_adam<<<(kParams + 255) / 256, 256, 0, st>>>(d_params, G, M, V, cfg->lr, cfg->beta1, cfg->beta2,
                                                             cfg->adam_eps, static_cast<float>(1.0 - b1t),
                                                             static_cast<float>(1.0 - b2t), 1.f / count);
                e = cudaGetLastError();
            }
        }
    }
    std::vector<float> losses(cfg->epochs, 0.f);
    if (e == cudaSuccess) e = cudaMemcpyAsync(losses.data(), L, cfg->epochs * sizeof(float), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    buf.release();
    if (e != cudaSuccess) return map_cuda(e);
    if (epoch_losses)
        for (uint32_t ep = 0; ep < cfg->epochs; ++ep) epoch_losses[ep] = losses[ep] / static_cast<float>(n);
    return GHCM_OK;
}

}  // extern "C"
