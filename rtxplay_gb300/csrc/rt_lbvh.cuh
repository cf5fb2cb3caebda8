// rt_lbvh.cuh -- device helpers shared by the hierarchy builders: record
// boxes, orderable float keys, Morton expansion, segment lookup and the
// Karras 2012 hierarchy over sorted codes.
#pragma once

#include "rt_scene.h"

namespace rt {
namespace {

struct Box3 {
    float3 lo, hi;
};

__device__ __forceinline__ Box3 prim_box(const float4* __restrict__ rec) {
    const float4 a = rec[0], b = rec[1], c = rec[2];
    if (__float_as_uint(c.w) == kPrimInstance) return Box3{xyz(a), xyz(b)};
    if (__float_as_uint(c.w) == kPrimTriangle) {
        return Box3{mk(fminf(fminf(a.x, b.x), c.x), fminf(fminf(a.y, b.y), c.y), fminf(fminf(a.z, b.z), c.z)),
                    mk(fmaxf(fmaxf(a.x, b.x), c.x), fmaxf(fmaxf(a.y, b.y), c.y), fmaxf(fmaxf(a.z, b.z), c.z))};
    }
    const float r = b.x;
    return Box3{mk(a.x - r, a.y - r, a.z - r), mk(a.x + r, a.y + r, a.z + r)};
}

__device__ __forceinline__ float3 centroid(const Box3& b) { return mul(0.5f, add(b.lo, b.hi)); }

__device__ __forceinline__ uint32_t ford(float f) {   // float -> order-preserving u32
    const uint32_t b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float fdeord(uint32_t o) {
    return __uint_as_float((o & 0x80000000u) ? (o & 0x7FFFFFFFu) : ~o);
}

__device__ __forceinline__ uint32_t expand10(uint32_t x) {
    x = (x * 0x00010001u) & 0xFF0000FFu;
    x = (x * 0x00000101u) & 0x0F00F00Fu;
    x = (x * 0x00000011u) & 0xC30C30C3u;
    x = (x * 0x00000005u) & 0x49249249u;
    return x;
}
__device__ __forceinline__ unsigned long long expand20(unsigned long long x) {
    x &= 0xFFFFFull;
    x = (x | x << 32) & 0x001F00000000FFFFull;
    x = (x | x << 16) & 0x001F0000FF0000FFull;
    x = (x | x << 8) & 0x100F00F00F00F00Full;
    x = (x | x << 4) & 0x10C30C30C30C30C3ull;
    x = (x | x << 2) & 0x1249249249249249ull;
    return x;
}
__device__ __forceinline__ float quantf(float c, float lo, float ext, float cells) {
    const float f = ext > 0.f ? (c - lo) / ext : 0.f;
    const float q = f * cells;
    const float top = cells - 1.f;
    return q < 0.f ? 0.f : (q > top ? top : q);
}

__device__ __forceinline__ uint32_t seg_of(const SegDev* __restrict__ segs, uint32_t nsegs, uint32_t pos) {
    uint32_t lo = 0, hi = nsegs;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (segs[mid].prim_begin <= pos) lo = mid; else hi = mid;
    }
    return lo;
}

// Karras 2012 over one segment's sorted codes (local indices, so a segment's
// hierarchy is the one a standalone build of that scene gives); equal keys
// fall back to the index bits, 64 + clz(i ^ j).
template <class K>
__device__ __forceinline__ int kdelta(const K* __restrict__ k, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    const unsigned long long a = (unsigned long long)k[i], b = (unsigned long long)k[j];
    if (a != b) return __clzll((long long)(a ^ b));
    return 64 + __clz(i ^ j);
}

// One thread per node slot.  Slot P + i (i < n - 1) of a segment starting at
// P with n primitives is its internal node i; a one-primitive segment puts its
// leaf in both child slots of node P (marked for the refit by parent -2).
template <class K>
__global__ void k_karras(const K* __restrict__ codes, const SegDev* __restrict__ segs, uint32_t nsegs, uint32_t ntot,
                         float4* __restrict__ nodes, int* __restrict__ parent_leaf, int* __restrict__ parent_int) {
    const uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= ntot) return;
    const SegDev sg = segs[seg_of(segs, nsegs, slot)];
    const int n = int(sg.prim_count);
    const int i = int(slot - sg.prim_begin);
    const int P = int(sg.prim_begin);
    if (n == 1) {
        nodes[4 * size_t(P) + 3] = make_float4(__int_as_float(~P), __int_as_float(~P), 0.f, 0.f);
        parent_leaf[P] = -2;
        parent_int[P] = -1;
        return;
    }
    if (i >= n - 1) return;   // the spare slot of the segment
    const K* k = codes + P;
    const int d = (kdelta(k, n, i, i + 1) - kdelta(k, n, i, i - 1)) >= 0 ? 1 : -1;
    const int dmin = kdelta(k, n, i, i - d);
    int lmax = 2;
    while (kdelta(k, n, i, i + lmax * d) > dmin) lmax <<= 1;
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
        if (kdelta(k, n, i, i + (l + t) * d) > dmin) l += t;
    const int j = i + l * d;
    const int dnode = kdelta(k, n, i, j);
    int s = 0;
    int t = l;
    do {
        t = (t + 1) >> 1;
        if (kdelta(k, n, i, i + (s + t) * d) > dnode) s += t;
    } while (t > 1);
    const int gamma = i + s * d + (d < 0 ? -1 : 0);
    const int lo = min(i, j), hi = max(i, j);
    const int left = (lo == gamma) ? ~(P + gamma) : P + gamma;
    const int right = (hi == gamma + 1) ? ~(P + gamma + 1) : P + gamma + 1;
    nodes[4 * size_t(P + i) + 3] = make_float4(__int_as_float(left), __int_as_float(right), 0.f, 0.f);
    if (left < 0) parent_leaf[~left] = P + i; else parent_int[left] = P + i;
    if (right < 0) parent_leaf[~right] = P + i; else parent_int[right] = P + i;
    if (i == 0) parent_int[P] = -1;
}

}  // namespace
}  // namespace rt
