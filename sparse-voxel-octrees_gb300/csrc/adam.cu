// adam.cu — one-pass Adam update of the per-leaf shading parameters.
//
// The optimisation loop of the differentiable path updates two parameter
// arrays of 3 floats per octree word (hundreds of millions of values) every
// step.  svo_adam_step: one kernel reads p, g, m, v and writes p, m, v (and
// zeroes g for the next accumulation): 28-32 bytes per value, one pass,
// HBM-bound.  svo_adam_step_leaves: the same update over only the leaves the
// adjoint has ever touched (a list kept by svo_diff_backward_l2), with
// results identical to the dense pass.
//
// Update (Kingma & Ba, "Adam", 2015; no weight decay, no amsgrad), with the
// bias corrections folded into two scalars computed on the host in double:
//   m = b1 m + (1 - b1) g,   v = b2 v + (1 - b2) g^2,
//   p -= (lr / (1 - b1^t)) m / (sqrt(v) / sqrt(1 - b2^t) + eps).
#include <cmath>

#include "svo_internal.h"

namespace svo {
namespace {

struct AdamArgs {
    float b1, b2, one_minus_b1, one_minus_b2, step_size, inv_bc2_sqrt, eps;
    int zero_grad;
};

__device__ __forceinline__ void adam_one(float &p, float &g, float &m, float &v, const AdamArgs &a) {
    m = a.b1 * m + a.one_minus_b1 * g;
    v = a.b2 * v + a.one_minus_b2 * g * g;
    float denom = sqrtf(v) * a.inv_bc2_sqrt + a.eps;
    p -= a.step_size * m / denom;
    if (a.zero_grad) g = 0.0f;
}

__global__ void k_adam_vec4(float4 *__restrict__ p, float4 *__restrict__ g, float4 *__restrict__ m,
                            float4 *__restrict__ v, uint64_t n4, AdamArgs a) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += (uint64_t)gridDim.x * blockDim.x) {
        float4 P = p[i], G = g[i], M = m[i], V = v[i];
        adam_one(P.x, G.x, M.x, V.x, a);
        adam_one(P.y, G.y, M.y, V.y, a);
        adam_one(P.z, G.z, M.z, V.z, a);
        adam_one(P.w, G.w, M.w, V.w, a);
        p[i] = P;
        m[i] = M;
        v[i] = V;
        if (a.zero_grad) g[i] = G;
    }
}

__global__ void k_adam_scalar(float *__restrict__ p, float *__restrict__ g, float *__restrict__ m, float *__restrict__ v,
                              uint64_t begin, uint64_t n, AdamArgs a) {
    for (uint64_t i = begin + (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        float P = p[i], G = g[i], M = m[i], V = v[i];
        adam_one(P, G, M, V, a);
        p[i] = P;
        m[i] = M;
        v[i] = V;
        if (a.zero_grad) g[i] = G;
    }
}

// The leaves of leaf_list only: a leaf outside the list has had no gradient
// since its moments were zero (the list holds every leaf the adjoint touched),
// so the dense update would leave its parameters, moments and gradient
// exactly as they are (m = v = 0 gives p -= step_size * 0 / eps).
__global__ void k_adam_leaves(float *__restrict__ p, float *__restrict__ g, float *__restrict__ m,
                              float *__restrict__ v, uint32_t width, const uint32_t *__restrict__ list,
                              const uint32_t *__restrict__ count, uint64_t cap, uint64_t n_values, AdamArgs a) {
    const uint64_t n = min((uint64_t)__ldg(count), cap) * width;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t leaf = __ldg(list + i / width);
        const uint64_t k = leaf * width + i % width;
        if (k >= n_values) continue;
        float P = p[k], G = g[k], M = m[k], V = v[k];
        adam_one(P, G, M, V, a);
        p[k] = P;
        m[k] = M;
        v[k] = V;
        if (a.zero_grad) g[k] = G;
    }
}

int adam_args(float lr, float beta1, float beta2, float eps, int step, int zero_grad, AdamArgs &a) {
    if (step < 1) return set_error(SVO_ERR_INVALID, "step must be >= 1");
    if (!(beta1 >= 0.0f && beta1 < 1.0f && beta2 >= 0.0f && beta2 < 1.0f))
        return set_error(SVO_ERR_INVALID, "betas must lie in [0, 1)");
    a.b1 = beta1;
    a.b2 = beta2;
    a.one_minus_b1 = 1.0f - beta1;
    a.one_minus_b2 = 1.0f - beta2;
    const double bc1 = 1.0 - std::pow((double)beta1, (double)step);
    const double bc2 = 1.0 - std::pow((double)beta2, (double)step);
    a.step_size = (float)((double)lr / bc1);
    a.inv_bc2_sqrt = (float)(1.0 / std::sqrt(bc2));
    a.eps = eps;
    a.zero_grad = zero_grad ? 1 : 0;
    return SVO_OK;
}

}  // namespace
}  // namespace svo

using namespace svo;

extern "C" int svo_adam_step_leaves(float *params, float *grads, float *exp_avg, float *exp_avg_sq, uint64_t n_values,
                                    uint32_t width, const uint32_t *leaf_list, const uint32_t *leaf_count,
                                    uint64_t leaf_capacity, float lr, float beta1, float beta2, float eps, int step,
                                    int zero_grad, svo_stream stream) {
    clear_error();
    if (!params || !grads || !exp_avg || !exp_avg_sq || !leaf_list || !leaf_count || width == 0)
        return set_error(SVO_ERR_INVALID, "bad arguments");
    AdamArgs a;
    int rc = adam_args(lr, beta1, beta2, eps, step, zero_grad, a);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    int dev = 0, sms = 0;
    SVO_CUDA_TRY(cudaGetDevice(&dev));
    SVO_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    // the listed count is read on the device (no host round trip); the grid
    // strides over whatever it holds
    k_adam_leaves<<<(unsigned)sms * 8, 256, 0, st>>>(params, grads, exp_avg, exp_avg_sq, width, leaf_list, leaf_count,
                                                     leaf_capacity, n_values, a);
    SVO_CUDA_TRY(cudaGetLastError());
    return SVO_OK;
}

extern "C" int svo_adam_step(float *params, float *grads, float *exp_avg, float *exp_avg_sq, uint64_t n, float lr,
                             float beta1, float beta2, float eps, int step, int zero_grad, svo_stream stream) {
    clear_error();
    if (n == 0) return SVO_OK;
    if (!params || !grads || !exp_avg || !exp_avg_sq) return set_error(SVO_ERR_INVALID, "null argument");
    AdamArgs a;
    int rc = adam_args(lr, beta1, beta2, eps, step, zero_grad, a);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    int dev = 0, sms = 0;
    SVO_CUDA_TRY(cudaGetDevice(&dev));
    SVO_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const unsigned grid = (unsigned)sms * 8;
    const bool aligned = ((uintptr_t)params | (uintptr_t)grads | (uintptr_t)exp_avg | (uintptr_t)exp_avg_sq) % 16 == 0;
    uint64_t done = 0;
    if (aligned && n >= 4) {
        uint64_t n4 = n / 4;
        k_adam_vec4<<<grid, 256, 0, st>>>((float4 *)params, (float4 *)grads, (float4 *)exp_avg, (float4 *)exp_avg_sq,
                                          n4, a);
        SVO_CUDA_TRY(cudaGetLastError());
        done = n4 * 4;
    }
    if (done < n) {
        k_adam_scalar<<<grid, 256, 0, st>>>(params, grads, exp_avg, exp_avg_sq, done, n, a);
        SVO_CUDA_TRY(cudaGetLastError());
    }
    return SVO_OK;
}
