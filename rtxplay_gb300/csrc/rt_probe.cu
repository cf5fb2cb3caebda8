// rt_probe.cu -- a bandwidth probe for the roofline figures.
//
// No counterpart in the reference.  The traversal kernel's bytes are served
// mostly by L1 and L2 (its node and primitive working set is the upper part
// of the hierarchy), so its L2 byte rate is reported against an L2 copy
// bandwidth measured on the same device: a plain copy of a buffer pair that
// fits in L2, repeated inside one launch so that launch gaps do not count,
// with loads and stores that bypass L1 (.cg), timed with CUDA events.
#include <algorithm>

#include "rt_internal.h"

namespace rt {
namespace {

constexpr int kProbeThreads = 256;

__global__ void __launch_bounds__(kProbeThreads) k_copy_cg(const float4* __restrict__ src, float4* __restrict__ dst,
                                                           size_t n, unsigned reps) {
    const size_t stride = size_t(gridDim.x) * blockDim.x;
    for (unsigned r = 0; r < reps; ++r) {
        for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
            __stcg(dst + i, __ldcg(src + i));
        }
    }
}

}  // namespace
}  // namespace rt

using namespace rt;

extern "C" rt_status rt_measure_copy_bandwidth(size_t bytes, unsigned int reps, double* gbs, void* stream) {
    return guarded([&] {
        RT_REQUIRE(gbs != nullptr, "gbs is NULL");
        RT_REQUIRE(bytes >= 4096 && bytes % 16 == 0, "bytes must be a multiple of 16, at least 4096");
        RT_REQUIRE(reps >= 1, "reps must be >= 1");
        cudaStream_t s = as_stream(stream);
        DevBuf a, b;
        a.reserve(bytes);
        b.reserve(bytes);
        RT_CUDA(cudaMemsetAsync(a.p, 0, bytes, s));
        const size_t n = bytes / 16;
        int per_sm = 0;
        RT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, reinterpret_cast<const void*>(k_copy_cg),
                                                              kProbeThreads, 0));
        const unsigned grid = unsigned(std::max(1, per_sm) * sm_count());
        k_copy_cg<<<grid, kProbeThreads, 0, s>>>(a.as<float4>(), b.as<float4>(), n, 2u);   // warm-up, loads L2
        RT_CHECK_LAUNCH();
        cudaEvent_t e0, e1;
        RT_CUDA(cudaEventCreate(&e0));
        RT_CUDA(cudaEventCreate(&e1));
        float ms = 0.f;
        try {
            RT_CUDA(cudaEventRecord(e0, s));
            k_copy_cg<<<grid, kProbeThreads, 0, s>>>(a.as<float4>(), b.as<float4>(), n, reps);
            RT_CHECK_LAUNCH();
            RT_CUDA(cudaEventRecord(e1, s));
            RT_CUDA(cudaEventSynchronize(e1));
            RT_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        } catch (...) {
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            throw;
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        *gbs = 2.0 * double(bytes) * reps / (double(ms) * 1e-3) / 1e9;   // bytes read + written
    });
}
