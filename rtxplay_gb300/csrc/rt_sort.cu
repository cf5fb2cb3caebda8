// rt_sort.cu -- device prefix sum and stable LSD radix sort.
//
// The LBVH builder sorts (Morton code, primitive id) pairs and the
// tessellator sorts vertex keys with these kernels.  The sort is a classic
// three-step LSD pass per 8-bit digit: per-tile digit histograms, one
// exclusive scan over the digit-major histogram table, then a stable scatter
// that ranks equal digits inside a tile with warp match/ballot and per-warp
// counts in shared memory.  No kernel waits on another block, so nothing here
// can spin.  Stability makes the result bit-exact against std::stable_sort.
#include <algorithm>
#include <cstdint>
#include <mutex>
#include <string>
#include <vector>

#include "rt_internal.h"

namespace rt {
namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;   // 1024 elements per block

// Words of scratch that scan_rec needs for n elements: the partial sums of
// every level of its recursion, plus one.  Both the allocating sort and the
// fixed-scratch sort size their scan tree with this one function.
constexpr size_t scan_tmp_words(uint32_t n) {
    size_t words = 0;
    while (n > uint32_t(kScanTile)) {
        n = (n + kScanTile - 1) / kScanTile;
        words += n;
    }
    return words + 1;
}

// Block-wide exclusive scan of one value per thread; returns the block total.
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t x, uint32_t& total) {
    __shared__ uint32_t warp_sums[kScanThreads / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t inc = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, inc, o);
        if (lane >= o) inc += y;
    }
    if (lane == 31) warp_sums[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < kScanThreads / 32 ? warp_sums[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < kScanThreads / 32) warp_sums[lane] = w;   // inclusive warp prefix
    }
    __syncthreads();
    const uint32_t warp_off = warp == 0 ? 0u : warp_sums[warp - 1];
    total = warp_sums[kScanThreads / 32 - 1];
    __syncthreads();
    return warp_off + inc - x;
}

__global__ void k_scan_partials(const uint32_t* __restrict__ in, uint32_t n, uint32_t* __restrict__ partials) {
    const uint32_t base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    uint32_t s = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i)
        if (base + i < n) s += in[base + i];
    uint32_t total;
    block_exclusive_scan(s, total);
    if (threadIdx.x == 0) partials[blockIdx.x] = total;
}

__global__ void k_scan_apply(const uint32_t* in, uint32_t* out, uint32_t n, const uint32_t* __restrict__ offsets) {
    const uint32_t base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    uint32_t v[kScanItems];
    uint32_t s = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        v[i] = base + i < n ? in[base + i] : 0u;
        s += v[i];
    }
    uint32_t total;
    uint32_t run = block_exclusive_scan(s, total) + (offsets ? offsets[blockIdx.x] : 0u);
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        if (base + i < n) out[base + i] = run;
        run += v[i];
    }
}

void scan_rec(const uint32_t* in, uint32_t* out, uint32_t n, uint32_t* tmp, cudaStream_t s) {
    const uint32_t nb = (n + kScanTile - 1) / kScanTile;
    if (nb <= 1) {
        k_scan_apply<<<1, kScanThreads, 0, s>>>(in, out, n, nullptr);
        RT_CHECK_LAUNCH();
        return;
    }
    uint32_t* partials = tmp;
    k_scan_partials<<<nb, kScanThreads, 0, s>>>(in, n, partials);
    RT_CHECK_LAUNCH();
    scan_rec(partials, partials, nb, tmp + nb, s);
    k_scan_apply<<<nb, kScanThreads, 0, s>>>(in, out, n, partials);
    RT_CHECK_LAUNCH();
}


// ------------------------------------------------------------- radix sort
constexpr int kSortThreads = 256;
constexpr int kSortWarps = kSortThreads / 32;
constexpr int kSortItems = 16;
constexpr int kSortTile = kSortThreads * kSortItems;   // 4096 keys per block
constexpr int kRadix = 256;

template <class K>
__device__ __forceinline__ uint32_t digit_of(K k, int shift) {
    return uint32_t(k >> shift) & (kRadix - 1);
}

template <class K>
__global__ void __launch_bounds__(kSortThreads) k_radix_hist(const K* __restrict__ keys, uint32_t n, int shift,
                                                             uint32_t* __restrict__ hist, uint32_t nblocks) {
    __shared__ uint32_t cnt[kRadix];
    cnt[threadIdx.x] = 0;
    __syncthreads();
    const uint32_t tile = blockIdx.x * kSortTile;
#pragma unroll 4
    for (int r = 0; r < kSortItems; ++r) {
        const uint32_t pos = tile + r * kSortThreads + threadIdx.x;
        if (pos < n) atomicAdd(&cnt[digit_of(keys[pos], shift)], 1u);
    }
    __syncthreads();
    hist[threadIdx.x * nblocks + blockIdx.x] = cnt[threadIdx.x];
}

template <class K>
__global__ void __launch_bounds__(kSortThreads) k_radix_scatter(const K* __restrict__ keys, const uint32_t* __restrict__ vals,
                                                                uint32_t n, int shift, const uint32_t* __restrict__ offsets,
                                                                uint32_t nblocks, K* __restrict__ keys_out,
                                                                uint32_t* __restrict__ vals_out) {
    __shared__ uint32_t base[kRadix];
    __shared__ uint32_t wcnt[kSortWarps][kRadix];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t lanemask_lt = (1u << lane) - 1u;
    base[threadIdx.x] = offsets[threadIdx.x * nblocks + blockIdx.x];
    const uint32_t tile = blockIdx.x * kSortTile;
    for (int r = 0; r < kSortItems; ++r) {
#pragma unroll
        for (int w = 0; w < kSortWarps; ++w) wcnt[w][threadIdx.x] = 0;
        __syncthreads();
        const uint32_t pos = tile + r * kSortThreads + threadIdx.x;
        const bool valid = pos < n;
        K k = 0;
        uint32_t v = 0, d = 0, rank = 0;
        const uint32_t vmask = __ballot_sync(0xFFFFFFFFu, valid);
        if (valid) {
            k = keys[pos];
            v = vals[pos];
            d = digit_of(k, shift);
            const uint32_t peers = __match_any_sync(vmask, d);
            rank = __popc(peers & lanemask_lt);
            if (rank == 0) wcnt[warp][d] = __popc(peers);
        }
        __syncthreads();
        if (valid) {
            uint32_t prefix = 0;
            for (int w = 0; w < warp; ++w) prefix += wcnt[w][d];
            const uint32_t dst = base[d] + prefix + rank;
            keys_out[dst] = k;
            vals_out[dst] = v;
        }
        __syncthreads();
        uint32_t add = 0;
#pragma unroll
        for (int w = 0; w < kSortWarps; ++w) add += wcnt[w][threadIdx.x];
        base[threadIdx.x] += add;
        __syncthreads();
    }
}

template <class K>
void radix_sort_pairs(K* keys, uint32_t* vals, uint32_t n, int bits, DevBuf& tmp, cudaStream_t s) {
    if (n <= 1 || bits <= 0) return;
    const uint32_t nblocks = (n + kSortTile - 1) / kSortTile;
    const uint32_t nhist = kRadix * nblocks;
    auto align = [](size_t b) { return (b + 255) & ~size_t(255); };
    const size_t off_keys = 0;
    const size_t off_vals = off_keys + align(size_t(n) * sizeof(K));
    const size_t off_hist = off_vals + align(size_t(n) * sizeof(uint32_t));
    const size_t off_scan = off_hist + align(size_t(nhist) * sizeof(uint32_t));
    const size_t total = off_scan + align(scan_tmp_words(nhist) * sizeof(uint32_t));
    tmp.reserve(total);
    char* b = tmp.as<char>();
    K* alt_keys = reinterpret_cast<K*>(b + off_keys);
    uint32_t* alt_vals = reinterpret_cast<uint32_t*>(b + off_vals);
    uint32_t* hist = reinterpret_cast<uint32_t*>(b + off_hist);
    uint32_t* scan_tmp = reinterpret_cast<uint32_t*>(b + off_scan);

    K* src_k = keys;
    uint32_t* src_v = vals;
    K* dst_k = alt_keys;
    uint32_t* dst_v = alt_vals;
    const int passes = (bits + 7) / 8;
    for (int p = 0; p < passes; ++p) {
        const int shift = 8 * p;
        k_radix_hist<K><<<nblocks, kSortThreads, 0, s>>>(src_k, n, shift, hist, nblocks);
        RT_CHECK_LAUNCH();
        scan_rec(hist, hist, nhist, scan_tmp, s);
        k_radix_scatter<K><<<nblocks, kSortThreads, 0, s>>>(src_k, src_v, n, shift, hist, nblocks, dst_k, dst_v);
        RT_CHECK_LAUNCH();
        std::swap(src_k, dst_k);
        std::swap(src_v, dst_v);
    }
    if (src_k != keys) {
        RT_CUDA(cudaMemcpyAsync(keys, src_k, size_t(n) * sizeof(K), cudaMemcpyDeviceToDevice, s));
        RT_CUDA(cudaMemcpyAsync(vals, src_v, size_t(n) * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s));
    }
}

}  // namespace

void scan_exclusive_u32(const uint32_t* in, uint32_t* out, uint32_t n, DevBuf& tmp, cudaStream_t s) {
    if (n == 0) return;
    tmp.reserve(scan_tmp_words(n) * sizeof(uint32_t));
    scan_rec(in, out, n, tmp.as<uint32_t>(), s);
}

void radix_sort_pairs_u32(uint32_t* keys, uint32_t* vals, uint32_t n, int bits, DevBuf& tmp, cudaStream_t s) {
    radix_sort_pairs<uint32_t>(keys, vals, n, std::min(bits, 32), tmp, s);
}

void radix_sort_pairs_u64(unsigned long long* keys, uint32_t* vals, uint32_t n, int bits, DevBuf& tmp,
                          cudaStream_t s) {
    radix_sort_pairs<unsigned long long>(keys, vals, n, std::min(bits, 64), tmp, s);
}

}  // namespace rt

// ---------------------------------------------------------------------------
// Allocation-free variant of the pair sort.
//
// Some callers cannot allocate device memory while they run: a host engine
// that reserves all device memory for its own pool up front, or a per-frame
// loop where a cudaMalloc/cudaFree would synchronise the whole device and
// stall the frame.  For them rt_radix_sort_pairs_noalloc sorts out of a fixed
// scratch array that lives in this library's device image instead of a
// cudaMalloc'd buffer.  The array is reserved on every GPU that loads the
// library and stays reserved until the process exits.
namespace rt {
namespace {

constexpr uint32_t kNoAllocMaxPairs = 1u << 18;   // 262,144 (key, value) pairs

struct NoAllocLayout {
    size_t keys, vals, hist, scan, total;
};

// Offsets of the sort's scratch inside the fixed array, for n pairs of
// key_bytes-wide keys (alternate keys and values, digit histograms, scan tree).
constexpr size_t noalloc_align(size_t b) { return (b + 255) & ~size_t(255); }
constexpr NoAllocLayout noalloc_layout(uint32_t n, size_t key_bytes) {
    const uint32_t nblocks = (n + kSortTile - 1) / kSortTile;
    const uint32_t nhist = kRadix * nblocks;
    const size_t keys = 0;
    const size_t vals = keys + noalloc_align(size_t(n) * key_bytes);
    const size_t hist = vals + noalloc_align(size_t(n) * sizeof(uint32_t));
    const size_t scan = hist + noalloc_align(size_t(nhist) * sizeof(uint32_t));
    const size_t total = scan + noalloc_align(scan_tmp_words(nhist) * sizeof(uint32_t));
    return NoAllocLayout{keys, vals, hist, scan, total};
}

constexpr size_t kNoAllocScratchBytes = noalloc_layout(kNoAllocMaxPairs, 8).total;   // about 3.1 MiB

// The fixed scratch.  Host code must not take its address directly (on the
// host the name is only a stand-in); the device address comes from
// cudaGetSymbolAddress, once per device.
static __device__ __align__(256) unsigned char g_noalloc_sort_scratch[kNoAllocScratchBytes];

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
void* g_noalloc_ptr[kNoAllocMaxDevices] = {};

// Device address of the scratch on the current device.  The first call on a
// device sets it up.  Later calls made outside a stream capture look it up
// again (a cheap query), so a cudaDeviceReset between calls, which reloads
// the module at a possibly different address, leaves no stale pointer behind;
// calls made during a capture use the address cached by the last lookup.
unsigned char* noalloc_scratch(cudaStream_t s) {
    int dev = 0;
    RT_CUDA(cudaGetDevice(&dev));
    RT_REQUIRE(dev >= 0 && dev < kNoAllocMaxDevices, "device ordinal out of range for the fixed scratch");
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cap) != cudaSuccess) {   // e.g. the legacy stream while another captures
        (void)cudaGetLastError();
        cap = cudaStreamCaptureStatusActive;
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[dev] || cap == cudaStreamCaptureStatusNone) {
        void* p = nullptr;
        RT_CUDA(cudaGetSymbolAddress(&p, g_noalloc_sort_scratch));
        g_noalloc_ptr[dev] = p;
    }
    return static_cast<unsigned char*>(g_noalloc_ptr[dev]);
}

template <class K>
void radix_sort_pairs_fixed(K* keys, uint32_t* vals, uint32_t n, int bits, unsigned char* scratch, cudaStream_t s) {
    if (n <= 1 || bits <= 0) return;
    const NoAllocLayout L = noalloc_layout(n, sizeof(K));
    RT_REQUIRE(L.total <= kNoAllocScratchBytes, "no-allocation sort scratch too small");
    const uint32_t nblocks = (n + kSortTile - 1) / kSortTile;
    const uint32_t nhist = kRadix * nblocks;
    K* alt_keys = reinterpret_cast<K*>(scratch + L.keys);
    uint32_t* alt_vals = reinterpret_cast<uint32_t*>(scratch + L.vals);
    uint32_t* hist = reinterpret_cast<uint32_t*>(scratch + L.hist);
    uint32_t* scan_tmp = reinterpret_cast<uint32_t*>(scratch + L.scan);
    // Every pass writes all of hist and the scan tree before reading them, so
    // nothing in the shared scratch has to be cleared between calls.
    K* src_k = keys;
    uint32_t* src_v = vals;
    K* dst_k = alt_keys;
    uint32_t* dst_v = alt_vals;
    const int passes = (bits + 7) / 8;
    for (int p = 0; p < passes; ++p) {
        const int shift = 8 * p;
        k_radix_hist<K><<<nblocks, kSortThreads, 0, s>>>(src_k, n, shift, hist, nblocks);
        RT_CHECK_LAUNCH();
        scan_rec(hist, hist, nhist, scan_tmp, s);
        k_radix_scatter<K><<<nblocks, kSortThreads, 0, s>>>(src_k, src_v, n, shift, hist, nblocks, dst_k, dst_v);
        RT_CHECK_LAUNCH();
        std::swap(src_k, dst_k);
        std::swap(src_v, dst_v);
    }
    if (src_k != keys) {
        RT_CUDA(cudaMemcpyAsync(keys, src_k, size_t(n) * sizeof(K), cudaMemcpyDeviceToDevice, s));
        RT_CUDA(cudaMemcpyAsync(vals, src_v, size_t(n) * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s));
    }
}

}  // namespace
}  // namespace rt

// Same result as rt_radix_sort_pairs, but no device allocation: the scratch is
// the fixed array above, so n is limited to 262,144 pairs.  Stream-ordered,
// returns without synchronising.  The first call on a device looks up the
// array's device address; make that first call before any stream capture.
// All calls share the one array: calls whose work can overlap on the GPU (on
// different streams, or from several host threads) race on it.
extern "C" rt_status rt_radix_sort_pairs_noalloc(void* keys, unsigned int* vals, unsigned int n,
                                                 unsigned int key_bits, void* stream) {
    using namespace rt;
    return guarded([&] {
        RT_REQUIRE(keys != nullptr && vals != nullptr, "keys/vals are NULL");
        RT_REQUIRE(key_bits >= 1 && key_bits <= 64, "key_bits must be 1..64");
        if (n > kNoAllocMaxPairs)
            throw Error(RT_ERR_INVALID_ARG, "rt_radix_sort_pairs_noalloc: n = " + std::to_string(n) +
                                                " exceeds the fixed scratch limit of " +
                                                std::to_string(kNoAllocMaxPairs) + " pairs");
        cudaStream_t s = as_stream(stream);
        unsigned char* scratch = noalloc_scratch(s);
        if (key_bits <= 32)
            radix_sort_pairs_fixed<uint32_t>(static_cast<uint32_t*>(keys), vals, n, int(key_bits), scratch, s);
        else
            radix_sort_pairs_fixed<unsigned long long>(static_cast<unsigned long long*>(keys), vals, n,
                                                       int(key_bits), scratch, s);
    });
}
