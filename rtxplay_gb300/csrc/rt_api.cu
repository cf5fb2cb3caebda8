// rt_api.cu -- C ABI glue: error reporting, version, camera set-up.
#include <atomic>
#include <cmath>
#include <cstdio>
#include <string>

#include "rt_device.cuh"
#include "rt_internal.h"

namespace rt {
namespace {
thread_local std::string g_last_error;
std::atomic<long long> g_fail_alloc{0};   // allocations until the injected failure (0: none)
}

bool injected_alloc_failure() {
    long long n = g_fail_alloc.load();
    while (n > 0) {
        if (g_fail_alloc.compare_exchange_weak(n, n - 1)) return n == 1;
    }
    return false;
}

bool stream_capturing(cudaStream_t s) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    RT_CUDA(cudaStreamIsCapturing(s, &cs));
    RT_REQUIRE(cs != cudaStreamCaptureStatusInvalidated, "the stream's capture has been invalidated");
    return cs == cudaStreamCaptureStatusActive;
}

int& capture_no_alloc() {
    static thread_local int depth = 0;
    return depth;
}

void set_last_error(const std::string& msg) { g_last_error = msg; }
void clear_last_error() { g_last_error.clear(); }

void throw_cuda(cudaError_t e, const char* what, const char* file, int line) {
    char buf[512];
    std::snprintf(buf, sizeof(buf), "CUDA error %d (%s) in %s at %s:%d", int(e), cudaGetErrorString(e), what, file,
                  line);
    throw Error(e == cudaErrorMemoryAllocation ? RT_ERR_OUT_OF_MEMORY : RT_ERR_CUDA, buf);
}

// SM count of the current device, cached per device ordinal (atomics: host
// threads may ask concurrently; a race only repeats the query).
int sm_count() {
    constexpr int kMaxDevices = 64;
    static std::atomic<int> cache[kMaxDevices];
    int dev = 0;
    RT_CUDA(cudaGetDevice(&dev));
    if (dev >= 0 && dev < kMaxDevices) {
        const int c = cache[dev].load(std::memory_order_relaxed);
        if (c > 0) return c;
    }
    int n = 0;
    RT_CUDA(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev));
    if (dev >= 0 && dev < kMaxDevices) cache[dev].store(n, std::memory_order_relaxed);
    return n;
}

}  // namespace rt

using namespace rt;

extern "C" {

const char* rt_last_error_string(void) { return g_last_error.c_str(); }

rt_status rt_debug_fail_alloc(unsigned int n) {
    g_fail_alloc.store((long long)n);
    return RT_OK;
}

#ifdef RT_CHECKS
const char* rt_version(void) { return "rtxplay_gb300 0.1 sm_103a bounds-checked"; }
#else
const char* rt_version(void) { return "rtxplay_gb300 0.1 sm_103a"; }
#endif

// Camera::set (optx/camera.h:30-48) in binary32 on the host; the compiler
// contracts nothing here (-ffp-contract=off), matching the CPU oracle.
rt_status rt_camera_set(rt_camera* cam, rt_float3 eye, rt_float3 pat, rt_float3 vup, float fov, float aspratio,
                        float aperture, float fostance) {
    return guarded([&] {
        RT_REQUIRE(cam != nullptr, "cam is NULL");
        const float3 E = make_float3(eye.x, eye.y, eye.z), P = make_float3(pat.x, pat.y, pat.z),
                     U = make_float3(vup.x, vup.y, vup.z);
        const float3 w = unitV(sub(E, P));
        const float3 u = unitV(cross(U, w));
        const float3 v = cross(w, u);
        const float kPi = 3.14159265358979323846f;
        const float h = 2.f * tanf(.5f * (fov * kPi / 180.f));
        const float wd = h * aspratio;
        const float3 hvec = mul(fostance * h / 2.f, v);
        const float3 wvec = mul(fostance * wd / 2.f, u);
        const float3 dvec = mul(fostance, w);
        cam->eye = eye;
        cam->pat = pat;
        cam->vup = vup;
        cam->fov = fov;
        cam->aspratio = aspratio;
        cam->aperture = aperture;
        cam->fostance = fostance;
        cam->u = rt_float3{u.x, u.y, u.z};
        cam->v = rt_float3{v.x, v.y, v.z};
        cam->w = rt_float3{w.x, w.y, w.z};
        cam->hvec = rt_float3{hvec.x, hvec.y, hvec.z};
        cam->wvec = rt_float3{wvec.x, wvec.y, wvec.z};
        cam->dvec = rt_float3{dvec.x, dvec.y, dvec.z};
    });
}

}  // extern "C"
