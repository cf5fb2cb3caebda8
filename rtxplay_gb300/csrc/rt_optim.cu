// rt_optim.cu -- the device-side pieces of an inverse-rendering loop: an L2
// image loss with its gradient, and an Adam step on a parameter vector.
//
// No counterpart in the reference (it renders only).  With rt_batch_launch,
// rt_batch_adjoint and rt_batch_set_albedos they make an optimisation
// iteration that never copies parameters or images through the host:
//   launch -> rt_l2_loss_grad -> adjoint -> rt_adam_step -> set_albedos.
#include <cmath>

#include "rt_internal.h"

namespace rt {
namespace {

constexpr int kThreads = 256;

// L = sum over pixels and channels of (clamp(I, 0, 1) - T)^2; writes
// dL/d(clamp(I)) = 2 (clamp(I) - T) and adds L to *loss (block sums, one
// double atomic per block).
__global__ void k_l2(const rt_float3* __restrict__ image, const rt_float3* __restrict__ target,
                     rt_float3* __restrict__ grad, uint32_t n, double* loss) {
    __shared__ double part[kThreads / 32];
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    double l = 0.0;
    if (p < n) {
        const rt_float3 I = image[p], T = target[p];
        const float c[3] = {fminf(fmaxf(I.x, 0.f), 1.f), fminf(fmaxf(I.y, 0.f), 1.f), fminf(fmaxf(I.z, 0.f), 1.f)};
        const float t[3] = {T.x, T.y, T.z};
        float g[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float e = c[k] - t[k];
            g[k] = 2.f * e;
            l += double(e) * double(e);
        }
        grad[p] = rt_float3{g[0], g[1], g[2]};
    }
    if (!loss) return;
    for (int o = 16; o > 0; o >>= 1) l += __shfl_down_sync(0xFFFFFFFFu, l, o);
    if ((threadIdx.x & 31u) == 0) part[threadIdx.x >> 5] = l;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < kThreads / 32; ++w) s += part[w];
        atomicAdd(loss, s);
    }
}

// Adam (Kingma and Ba 2015), in place on float parameters with a double
// gradient; bc1 = 1 - beta1^t and bc2 = 1 - beta2^t come from the host.  The
// parameter is clamped to [lo, hi] after the step (albedos stay in [0, 1]).
__global__ void k_adam(float* __restrict__ theta, const double* __restrict__ grad, float* __restrict__ m,
                       float* __restrict__ v, uint32_t n, float lr, float b1, float b2, float eps, float bc1,
                       float bc2, float lo, float hi) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float g = float(grad[i]);
    const float mi = b1 * m[i] + (1.f - b1) * g;
    const float vi = b2 * v[i] + (1.f - b2) * (g * g);
    m[i] = mi;
    v[i] = vi;
    const float mh = mi / bc1;
    const float vh = vi / bc2;
    const float th = theta[i] - lr * mh / (sqrtf(vh) + eps);
    theta[i] = fminf(fmaxf(th, lo), hi);
}

// The same step with the step number on the device (an iteration captured
// into a CUDA graph replays the same kernel arguments): t = *step + 1, the
// bias corrections from it; k_step_advance then stores t.
__global__ void k_adam_dev(float* __restrict__ theta, const double* __restrict__ grad, float* __restrict__ m,
                           float* __restrict__ v, uint32_t n, float lr, float b1, float b2, float eps,
                           const uint32_t* __restrict__ step, float lo, float hi) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double t = double(*step) + 1.0;
    const float bc1 = float(1.0 - pow(double(b1), t));
    const float bc2 = float(1.0 - pow(double(b2), t));
    const float g = float(grad[i]);
    const float mi = b1 * m[i] + (1.f - b1) * g;
    const float vi = b2 * v[i] + (1.f - b2) * (g * g);
    m[i] = mi;
    v[i] = vi;
    const float mh = mi / bc1;
    const float vh = vi / bc2;
    const float th = theta[i] - lr * mh / (sqrtf(vh) + eps);
    theta[i] = fminf(fmaxf(th, lo), hi);
}

__global__ void k_step_advance(uint32_t* step) { *step += 1u; }

}  // namespace
}  // namespace rt

using namespace rt;

extern "C" {

rt_status rt_l2_loss_grad(const rt_float3* image, const rt_float3* target, rt_float3* grad_image, unsigned int n,
                          double* loss, void* stream) {
    return guarded([&] {
        RT_REQUIRE(image && target && grad_image, "image/target/grad_image is NULL");
        if (n == 0) return;
        k_l2<<<(n + kThreads - 1) / kThreads, kThreads, 0, as_stream(stream)>>>(image, target, grad_image, n, loss);
        RT_CHECK_LAUNCH();
    });
}

rt_status rt_adam_step(float* theta, const double* grad, float* m, float* v, unsigned int n, float lr, float beta1,
                       float beta2, float eps, unsigned int step, float lo, float hi, void* stream) {
    return guarded([&] {
        RT_REQUIRE(theta && grad && m && v, "theta/grad/m/v is NULL");
        RT_REQUIRE(step >= 1, "step counts from 1");
        RT_REQUIRE(beta1 >= 0.f && beta1 < 1.f && beta2 >= 0.f && beta2 < 1.f, "betas must be in [0, 1)");
        if (n == 0) return;
        const float bc1 = float(1.0 - std::pow(double(beta1), double(step)));
        const float bc2 = float(1.0 - std::pow(double(beta2), double(step)));
        k_adam<<<(n + kThreads - 1) / kThreads, kThreads, 0, as_stream(stream)>>>(theta, grad, m, v, n, lr, beta1,
                                                                                   beta2, eps, bc1, bc2, lo, hi);
        RT_CHECK_LAUNCH();
    });
}

rt_status rt_adam_step_device(float* theta, const double* grad, float* m, float* v, unsigned int n, float lr,
                              float beta1, float beta2, float eps, unsigned int* step, float lo, float hi,
                              void* stream) {
    return guarded([&] {
        RT_REQUIRE(theta && grad && m && v && step, "theta/grad/m/v/step is NULL");
        RT_REQUIRE(beta1 >= 0.f && beta1 < 1.f && beta2 >= 0.f && beta2 < 1.f, "betas must be in [0, 1)");
        cudaStream_t s = as_stream(stream);
        if (n) {
            k_adam_dev<<<(n + kThreads - 1) / kThreads, kThreads, 0, s>>>(theta, grad, m, v, n, lr, beta1, beta2, eps,
                                                                          step, lo, hi);
            RT_CHECK_LAUNCH();
        }
        k_step_advance<<<1, 1, 0, s>>>(step);
        RT_CHECK_LAUNCH();
    });
}

}  // extern "C"
