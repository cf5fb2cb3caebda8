// rt_internal.h -- host-side helpers shared by the library's translation units.
#pragma once

#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include "../../include/rt_api.h"

namespace rt {

// Exception carried to the C ABI boundary, where it becomes an rt_status and
// the thread's last-error string (never thrown across the ABI).
struct Error : std::runtime_error {
    rt_status status;
    Error(rt_status s, const std::string& m) : std::runtime_error(m), status(s) {}
};

void set_last_error(const std::string& msg);
void clear_last_error();

[[noreturn]] void throw_cuda(cudaError_t e, const char* what, const char* file, int line);

// NVTX range for the scope (header-only NVTX v3: a no-op unless a profiler
// such as ncu or nsys is attached; `ncu --nvtx --nvtx-include` filters by it).
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

// Fault injection (rt_debug_fail_alloc): true when this device allocation is
// the one chosen to fail.
bool injected_alloc_failure();

// Stream capture: true while `s` is being captured into a CUDA graph.  Calls
// that support capture enqueue only stream-ordered work then (no host reads,
// no synchronisation) and may not grow a device buffer: inside a
// CaptureNoAlloc scope a DevBuf that would have to allocate throws instead.
bool stream_capturing(cudaStream_t s);
int& capture_no_alloc();
struct CaptureNoAlloc {
    bool on;
    explicit CaptureNoAlloc(bool enable) : on(enable) { if (on) ++capture_no_alloc(); }
    ~CaptureNoAlloc() { if (on) --capture_no_alloc(); }
    CaptureNoAlloc(const CaptureNoAlloc&) = delete;
    CaptureNoAlloc& operator=(const CaptureNoAlloc&) = delete;
};

#define RT_CUDA(call)                                                        \
    do {                                                                     \
        cudaError_t rt_e_ = (call);                                          \
        if (rt_e_ != cudaSuccess) ::rt::throw_cuda(rt_e_, #call, __FILE__, __LINE__); \
    } while (0)

#define RT_CHECK_LAUNCH() RT_CUDA(cudaGetLastError())

#define RT_REQUIRE(cond, msg)                                                \
    do {                                                                     \
        if (!(cond)) throw ::rt::Error(RT_ERR_INVALID_ARG, (msg));           \
    } while (0)

// Runs `body`, mapping exceptions to an rt_status.
template <class F>
rt_status guarded(F&& body) {
    try {
        clear_last_error();
        body();
        return RT_OK;
    } catch (const Error& e) {
        set_last_error(e.what());
        return e.status;
    } catch (const std::bad_alloc&) {
        set_last_error("host allocation failed");
        return RT_ERR_OUT_OF_MEMORY;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return RT_ERR_INTERNAL;
    }
}

// Owning device buffer (cudaMalloc/cudaFree), grow-only.
struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    DevBuf(DevBuf&& o) noexcept : p(o.p), bytes(o.bytes) { o.p = nullptr; o.bytes = 0; }
    DevBuf& operator=(DevBuf&& o) noexcept {
        if (this != &o) { release(); p = o.p; bytes = o.bytes; o.p = nullptr; o.bytes = 0; }
        return *this;
    }
    ~DevBuf() { release(); }
    void release() noexcept {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    void reserve(size_t n) {
        if (n <= bytes) return;
        if (capture_no_alloc())
            throw Error(RT_ERR_INVALID_ARG, "a device buffer would have to grow inside a stream capture: make the "
                                            "same call once before capturing");
        release();
        if (n == 0) return;
        if (injected_alloc_failure())
            throw Error(RT_ERR_OUT_OF_MEMORY, "cudaMalloc of " + std::to_string(n) + " bytes failed (injected)");
        cudaError_t e = cudaMalloc(&p, n);
        if (e == cudaErrorMemoryAllocation) {
            cudaGetLastError();
            throw Error(RT_ERR_OUT_OF_MEMORY, "cudaMalloc of " + std::to_string(n) + " bytes failed");
        }
        if (e != cudaSuccess) throw_cuda(e, "cudaMalloc", __FILE__, __LINE__);
        bytes = n;
    }
    template <class T>
    T* as() const { return static_cast<T*>(p); }
};

inline cudaStream_t as_stream(void* s) { return static_cast<cudaStream_t>(s); }

// Number of SMs of the current device (cached per process).
int sm_count();

// ---- scan / sort (rt_sort.cu) ----
// Exclusive prefix sum of n uint32 on the device; `tmp` is grown as needed.
void scan_exclusive_u32(const uint32_t* in, uint32_t* out, uint32_t n, DevBuf& tmp, cudaStream_t s);
// Stable LSD radix sort of (key, value) pairs, 8-bit digits, `bits` low key
// bits significant; keys/vals are sorted in place using `tmp` as scratch.
void radix_sort_pairs_u32(uint32_t* keys, uint32_t* vals, uint32_t n, int bits, DevBuf& tmp, cudaStream_t s);
void radix_sort_pairs_u64(unsigned long long* keys, uint32_t* vals, uint32_t n, int bits, DevBuf& tmp,
                          cudaStream_t s);

}  // namespace rt
