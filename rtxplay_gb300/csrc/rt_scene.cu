// rt_scene.cu -- scene construction: tessellation, flattening, LBVH build and refit.
//
// Replaces Sphere (optx/sphere.cxx:17-106), Scene::add / set / get / build /
// update (optx/scene.cxx:38-294) and the closed optixAccelBuild with GPU
// kernels.  HBM layout after a build: primitive records in leaf order (48 B
// each, three float4), internal nodes holding both child boxes (64 B each),
// a 48-byte optics record per thing.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <numeric>
#include <memory>
#include <vector>

#include "rt_scene.h"
#include "rt_lbvh.cuh"

namespace rt {
namespace {

constexpr int kThreads = 256;

inline unsigned grid_for(uint64_t n, int threads = kThreads) { return unsigned((n + threads - 1) / threads); }

// ------------------------------------------------------------ tessellation
// One thread per leaf triangle of the 4-way subdivision, walking the path of
// pumpup (optx/sphere.cxx:51-66) from its base face: the midpoints are the
// same operations on the same operands as the recursion, hence the same bits.
__global__ void k_tess_leaves(float radius, uint32_t ndiv, uint32_t ntri, float3* __restrict__ out) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntri) return;
    // optx/sphere.cxx:34-46: regular tetrahedron, midsphere radius m
    const float m = .57735026919f;
    const float3 v00 = mk(m, m, m), v01 = mk(m, -m, -m), v02 = mk(-m, -m, m), v03 = mk(-m, m, -m);
    const uint32_t face = t >> (2 * ndiv);
    float3 a, b, c;
    switch (face) {
        case 0: a = v00; b = v01; c = v02; break;
        case 1: a = v00; b = v02; c = v03; break;
        case 2: a = v00; b = v03; c = v01; break;
        default: a = v03; b = v02; c = v01; break;
    }
    for (int k = int(ndiv) - 1; k >= 0; --k) {
        const uint32_t digit = (t >> (2 * k)) & 3u;
        const float3 ab = unitV(mul(.5f, add(a, b)));
        const float3 bc = unitV(mul(.5f, add(b, c)));
        const float3 ca = unitV(mul(.5f, add(c, a)));
        switch (digit) {
            case 0: b = ab; c = ca; break;                 // (a, ab, ca)
            case 1: a = ab; c = bc; break;                 // (ab, b, bc)
            case 2: a = ca; b = bc; break;                 // (ca, bc, c)
            default: a = ab; b = bc; c = ca; break;        // (ab, bc, ca)
        }
    }
    out[3 * t] = mul(radius, a);
    out[3 * t + 1] = mul(radius, b);
    out[3 * t + 2] = mul(radius, c);
}

// IEEE order-preserving map float -> u32 (-0 folded onto +0 first, as the
// reference's comparator treats them as equal).
__device__ __forceinline__ uint32_t f2o(float f) {
    const uint32_t b = __float_as_uint(f + 0.0f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

__global__ void k_iota(uint32_t* __restrict__ v, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) v[i] = i;
}

__global__ void k_axis_keys(const float3* __restrict__ pts, const uint32_t* __restrict__ idx, uint32_t n, int axis,
                            uint32_t* __restrict__ keys) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float3 p = pts[idx[i]];
    keys[i] = f2o(axis == 0 ? p.x : axis == 1 ? p.y : p.z);
}

__global__ void k_run_heads(const float3* __restrict__ pts, const uint32_t* __restrict__ idx, uint32_t n,
                            uint32_t* __restrict__ head) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t h = 1;
    if (i > 0) {
        const float3 a = pts[idx[i]], b = pts[idx[i - 1]];
        h = (a.x != b.x || a.y != b.y || a.z != b.z) ? 1u : 0u;
    }
    head[i] = h;
}

// run[i] = (exclusive scan of heads)[i] + head[i] - 1; the head of a run is
// its first occurrence in generation order (stable sort keeps that order).
__global__ void k_mark_heads(const uint32_t* __restrict__ idx, const uint32_t* __restrict__ head,
                             const uint32_t* __restrict__ head_scan, uint32_t n, uint32_t* __restrict__ head_orig,
                             uint32_t* __restrict__ run_of_orig, uint32_t* __restrict__ mark) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t run = head_scan[i] + head[i] - 1u;
    const uint32_t orig = idx[i];
    run_of_orig[orig] = run;
    if (head[i]) {
        head_orig[run] = orig;
        mark[orig] = 1u;
    }
}

__global__ void k_emit_mesh(const float3* __restrict__ pts, const uint32_t* __restrict__ head_orig,
                            const uint32_t* __restrict__ run_of_orig, const uint32_t* __restrict__ mark,
                            const uint32_t* __restrict__ vid, uint32_t n, float3* __restrict__ vces,
                            uint32_t* __restrict__ ices) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const uint32_t h = head_orig[run_of_orig[p]];
    const uint32_t id = vid[h];
    ices[p] = id;
    if (mark[p]) vces[id] = pts[p];
}

// ------------------------------------------------------------- flattening
// Mesh of the bottom level: its object-space triangles are records
// [begin, begin + n) of the bottom level, one segment per mesh.
struct BlasMesh {
    const float3* v;
    const uint3* idx;
    uint32_t begin, n;
};

// One thread per bottom-level record: object-space triangle of an instanced
// mesh, local index in a.w.
__global__ void k_flatten_bottom(const BlasMesh* __restrict__ meshes, uint32_t nmeshes, uint32_t nrec,
                                 float4* __restrict__ out, uint32_t* __restrict__ prim_seg) {
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrec) return;
    uint32_t lo = 0, hi = nmeshes;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (meshes[mid].begin <= r) lo = mid; else hi = mid;
    }
    const BlasMesh m = meshes[lo];
    const uint32_t local = r - m.begin;
    const uint3 tri = m.idx[local];
    const float3 A = m.v[tri.x], B = m.v[tri.y], C = m.v[tri.z];
    float4* o = out + 3 * size_t(r);
    o[0] = make_float4(A.x, A.y, A.z, __uint_as_float(local));
    o[1] = make_float4(B.x, B.y, B.z, 0.f);
    o[2] = make_float4(C.x, C.y, C.z, __uint_as_float(kPrimTriangle));
    if (prim_seg) prim_seg[r] = lo;
}

// One thread per top-level record: the owning thing is the last one whose
// top_offset <= r.  Analytic spheres and flattened mesh triangles (world
// space, xform_point) as in a flat hierarchy; an instanced thing's record
// holds the world box of its bottom-level root box under the instance
// transform (the same monotone rounding as the vertices, so it is exact).
__global__ void k_flatten_top(const FlatDesc* __restrict__ desc, uint32_t nthings, uint32_t nrec,
                              const float4* __restrict__ bnodes, float4* __restrict__ out,
                              uint32_t* __restrict__ prim_seg) {
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrec) return;
    uint32_t lo = 0, hi = nthings;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (desc[mid].top_offset <= r) lo = mid; else hi = mid;
    }
    const FlatDesc& d = desc[lo];
    const uint32_t thing = lo;
    if (prim_seg) prim_seg[r] = d.seg;
    float4* o = out + 3 * size_t(r);
    if (d.analytic) {
        o[0] = make_float4(d.sphere.x, d.sphere.y, d.sphere.z, __uint_as_float(thing));
        o[1] = make_float4(d.sphere.w, 0.f, 0.f, __uint_as_float(d.prim_offset));
        o[2] = make_float4(0.f, 0.f, 0.f, __uint_as_float(kPrimSphere));
        return;
    }
    if (d.instanced) {
        const float4* n = bnodes + 4 * size_t(d.blas_root);
        const float4 n0 = n[0], n1 = n[1], n2 = n[2];
        const float sc[3] = {d.T[0], d.T[5], d.T[10]}, tr[3] = {d.T[3], d.T[7], d.T[11]};
        const float blo[3] = {fminf(n0.x, n1.x), fminf(n0.z, n1.z), fminf(n2.x, n2.z)};
        const float bhi[3] = {fmaxf(n0.y, n1.y), fmaxf(n0.w, n1.w), fmaxf(n2.y, n2.w)};
        float wlo[3], whi[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float p = blo[k] * sc[k] + tr[k], q = bhi[k] * sc[k] + tr[k];
            wlo[k] = fminf(p, q);
            whi[k] = fmaxf(p, q);
        }
        o[0] = make_float4(wlo[0], wlo[1], wlo[2], __uint_as_float(thing));
        o[1] = make_float4(whi[0], whi[1], whi[2], 0.f);
        o[2] = make_float4(0.f, 0.f, 0.f, __uint_as_float(kPrimInstance));
        return;
    }
    const uint32_t pid = d.prim_offset + (r - d.top_offset);
    float4 a, b, c;
    world_prim(desc, thing, pid, a, b, c);
    o[0] = a;
    o[1] = b;
    o[2] = c;
}

// ------------------------------------------------------------------- LBVH
__global__ void k_init_bounds(uint32_t* b, uint32_t nsegs) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 6 * nsegs) return;
    b[i] = (i % 6) < 3 ? 0xFFFFFFFFu : 0u;   // min slots start high, max slots low
}

// Centroid bounds per segment: a warp whose primitives share one segment
// reduces in registers; the warps of a block that share a segment merge in
// shared memory and issue six atomics per block; a mixed warp (segment
// border) issues them per lane.
__global__ void __launch_bounds__(kThreads)
    k_centroid_bounds(const float4* __restrict__ prims, const uint32_t* __restrict__ prim_seg, uint32_t n,
                      uint32_t* __restrict__ bounds, int by_thing) {
    __shared__ uint32_t s_v[kThreads / 32][6];
    __shared__ uint32_t s_seg[kThreads / 32];
    __shared__ int s_uni[kThreads / 32];
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t warp = threadIdx.x >> 5;
    const bool valid = i < n;
    uint32_t v[6] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0u, 0u, 0u};
    uint32_t seg = 0;
    if (valid) {
        const float3 c = centroid(prim_box(prims + 3 * size_t(i)));
        v[0] = v[3] = ford(c.x);
        v[1] = v[4] = ford(c.y);
        v[2] = v[5] = ford(c.z);
        seg = by_thing ? __float_as_uint(prims[3 * size_t(i)].w) : (prim_seg ? prim_seg[i] : 0u);
    }
    const uint32_t vmask = __ballot_sync(0xFFFFFFFFu, valid);
    const uint32_t seg0 = vmask ? __shfl_sync(0xFFFFFFFFu, seg, __ffs(vmask) - 1) : 0u;
    const bool uniform = vmask && __all_sync(0xFFFFFFFFu, !valid || seg == seg0);
    if (uniform) {
        for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
            for (int k = 0; k < 6; ++k) {
                const uint32_t w = __shfl_down_sync(0xFFFFFFFFu, v[k], o);
                v[k] = k < 3 ? min(v[k], w) : max(v[k], w);
            }
        }
    } else if (valid) {
        uint32_t* b = bounds + 6 * seg;
        atomicMin(&b[0], v[0]); atomicMin(&b[1], v[1]); atomicMin(&b[2], v[2]);
        atomicMax(&b[3], v[3]); atomicMax(&b[4], v[4]); atomicMax(&b[5], v[5]);
    }
    if ((threadIdx.x & 31u) == 0) {
        s_uni[warp] = uniform ? 1 : 0;
        s_seg[warp] = seg0;
#pragma unroll
        for (int k = 0; k < 6; ++k) s_v[warp][k] = v[k];
    }
    __syncthreads();
    if (threadIdx.x < 6) {   // thread k merges value k over runs of warps with one segment
        const uint32_t k = threadIdx.x;
        uint32_t cur = 0xFFFFFFFFu, acc = 0;
        for (uint32_t w = 0; w <= kThreads / 32; ++w) {
            const bool end = w == kThreads / 32;
            if (!end && !s_uni[w]) continue;
            if (end || s_seg[w] != cur) {
                if (cur != 0xFFFFFFFFu) {
                    if (k < 3) atomicMin(&bounds[6 * size_t(cur) + k], acc);
                    else atomicMax(&bounds[6 * size_t(cur) + k], acc);
                }
                if (end) break;
                cur = s_seg[w];
                acc = s_v[w][k];
            } else {
                acc = k < 3 ? min(acc, s_v[w][k]) : max(acc, s_v[w][k]);
            }
        }
    }
}

template <class K>
__global__ void k_morton(const float4* __restrict__ prims, const uint32_t* __restrict__ prim_seg, uint32_t n,
                         const uint32_t* __restrict__ bounds, K* __restrict__ codes, uint32_t* __restrict__ ids) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t* b = bounds + 6 * (prim_seg ? prim_seg[i] : 0u);
    const float3 lo = mk(fdeord(b[0]), fdeord(b[1]), fdeord(b[2]));
    const float3 hi = mk(fdeord(b[3]), fdeord(b[4]), fdeord(b[5]));
    const float3 ext = sub(hi, lo);
    const float3 c = centroid(prim_box(prims + 3 * size_t(i)));
    if (sizeof(K) == 4) {
        const uint32_t qx = uint32_t(quantf(c.x, lo.x, ext.x, 1024.f));
        const uint32_t qy = uint32_t(quantf(c.y, lo.y, ext.y, 1024.f));
        const uint32_t qz = uint32_t(quantf(c.z, lo.z, ext.z, 1024.f));
        codes[i] = K((expand10(qx) << 2) | (expand10(qy) << 1) | expand10(qz));
    } else {
        const unsigned long long qx = (unsigned long long)(quantf(c.x, lo.x, ext.x, 1048576.f));
        const unsigned long long qy = (unsigned long long)(quantf(c.y, lo.y, ext.y, 1048576.f));
        const unsigned long long qz = (unsigned long long)(quantf(c.z, lo.z, ext.z, 1048576.f));
        codes[i] = K((expand20(qx) << 2) | (expand20(qy) << 1) | expand20(qz));
    }
    ids[i] = i;
}

// Things-grouped hierarchy (a flat, world-space LBVH with the shape of a
// two-level one).  Primitives are keyed (thing << 30) | (30-bit Morton code of
// the centroid inside the thing's centroid bounds); a Karras hierarchy per
// thing (segments = things) gives each thing its subtree; the things of a
// scene are sorted by a 60-bit code of their centre in the scene's bounds and
// get a Karras hierarchy of their own, whose internal nodes are stitched into
// the spare node slot of each thing (a thing of n primitives uses n - 1 of its
// n slots).  Splits therefore never mix two things below the thing level.
__global__ void k_thing_codes(const uint32_t* __restrict__ tbounds, const FlatDesc* __restrict__ desc,
                              const uint32_t* __restrict__ sbounds, uint32_t nthings,
                              unsigned long long* __restrict__ codes, uint32_t* __restrict__ ids) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nthings) return;
    const uint32_t* tb = tbounds + 6 * size_t(t);
    const float3 c = centroid(Box3{mk(fdeord(tb[0]), fdeord(tb[1]), fdeord(tb[2])),
                                   mk(fdeord(tb[3]), fdeord(tb[4]), fdeord(tb[5]))});
    const uint32_t* b = sbounds + 6 * size_t(desc[t].seg);
    const float3 lo = mk(fdeord(b[0]), fdeord(b[1]), fdeord(b[2]));
    const float3 hi = mk(fdeord(b[3]), fdeord(b[4]), fdeord(b[5]));
    const float3 ext = sub(hi, lo);
    const unsigned long long qx = (unsigned long long)(quantf(c.x, lo.x, ext.x, 1048576.f));
    const unsigned long long qy = (unsigned long long)(quantf(c.y, lo.y, ext.y, 1048576.f));
    const unsigned long long qz = (unsigned long long)(quantf(c.z, lo.z, ext.z, 1048576.f));
    codes[t] = (expand20(qx) << 2) | (expand20(qy) << 1) | expand20(qz);
    ids[t] = t;
}

__global__ void k_morton_grouped(const float4* __restrict__ prims, uint32_t n, const uint32_t* __restrict__ tbounds,
                                 unsigned long long* __restrict__ codes, uint32_t* __restrict__ ids) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t t = __float_as_uint(prims[3 * size_t(i)].w);
    const uint32_t* tb = tbounds + 6 * size_t(t);
    const float3 lo = mk(fdeord(tb[0]), fdeord(tb[1]), fdeord(tb[2]));
    const float3 hi = mk(fdeord(tb[3]), fdeord(tb[4]), fdeord(tb[5]));
    const float3 ext = sub(hi, lo);
    const float3 c = centroid(prim_box(prims + 3 * size_t(i)));
    const uint32_t qx = uint32_t(quantf(c.x, lo.x, ext.x, 1024.f));
    const uint32_t qy = uint32_t(quantf(c.y, lo.y, ext.y, 1024.f));
    const uint32_t qz = uint32_t(quantf(c.z, lo.z, ext.z, 1024.f));
    codes[i] = ((unsigned long long)t << 30) | ((expand10(qx) << 2) | (expand10(qy) << 1) | expand10(qz));
    ids[i] = i;
}

// Spare node slot of thing t (its last slot; a thing of n records has n - 1 internal nodes).
__device__ __forceinline__ int spare_slot(const SegDev* __restrict__ tsegs, uint32_t t) {
    return int(tsegs[t].prim_begin + tsegs[t].prim_count) - 1;
}

// One thread per top-level (thing-tree) slot j: the thing tree's internal node
// j of a scene with at least two things moves to the spare slot of thing j;
// its children are remapped (internal -> their spare slots, thing leaf -> the
// thing's subtree root, or its single record) and their parents set.
__global__ void k_stitch(const float4* __restrict__ tnodes, const SegDev* __restrict__ scene_things, uint32_t nsegs,
                         const uint32_t* __restrict__ sorted_things, const SegDev* __restrict__ tsegs, uint32_t nthings,
                         float4* __restrict__ nodes, int* __restrict__ parent_leaf, int* __restrict__ parent_int) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nthings) return;
    const SegDev sc = scene_things[seg_of(scene_things, nsegs, j)];
    if (sc.prim_count < 2 || j - sc.prim_begin >= sc.prim_count - 1) return;
    const int D = spare_slot(tsegs, j);
    const float4 n3 = tnodes[4 * size_t(j) + 3];
    int ref[2];
    const int child[2] = {__float_as_int(n3.x), __float_as_int(n3.y)};
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        const int c = child[k];
        if (c >= 0) {
            ref[k] = spare_slot(tsegs, uint32_t(c));
            parent_int[ref[k]] = D;
        } else {
            const uint32_t t = sorted_things[~c];
            const SegDev ts = tsegs[t];
            if (ts.prim_count >= 2) {
                ref[k] = int(ts.prim_begin);
                parent_int[ts.prim_begin] = D;
            } else {
                ref[k] = ~int(ts.prim_begin);
                parent_leaf[ts.prim_begin] = D;
            }
        }
    }
    nodes[4 * size_t(D) + 3] = make_float4(__int_as_float(ref[0]), __int_as_float(ref[1]), 0.f, 0.f);
    if (j == sc.prim_begin) parent_int[D] = -1;   // the scene's root
}

// Segment ids of the code-sorted primitives, and the identity permutation.
__global__ void k_seg_keys(const uint32_t* __restrict__ prim_seg, const uint32_t* __restrict__ ids, uint32_t n,
                           uint32_t* __restrict__ keys, uint32_t* __restrict__ perm) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    keys[i] = prim_seg[ids[i]];
    perm[i] = i;
}

template <class K>
__global__ void k_permute(const K* __restrict__ codes_in, const uint32_t* __restrict__ ids_in,
                          const uint32_t* __restrict__ perm, uint32_t n, K* __restrict__ codes_out,
                          uint32_t* __restrict__ ids_out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    codes_out[i] = codes_in[perm[i]];
    ids_out[i] = ids_in[perm[i]];
}

// Records in leaf order, and their traversal form: a triangle as (A, B - A,
// C - A), the edges rounded as the triangle test rounds them, other records
// as they are.
__global__ void k_gather_prims(const float4* __restrict__ flat, const uint32_t* __restrict__ ids, uint32_t n,
                               float4* __restrict__ out, float4* __restrict__ out_e) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4* s = flat + 3 * size_t(ids[i]);
    const float4 a = s[0], b = s[1], c = s[2];
    float4* o = out + 3 * size_t(i);
    o[0] = a;
    o[1] = b;
    o[2] = c;
    float4* e = out_e + 3 * size_t(i);
    e[0] = a;
    if (__float_as_uint(c.w) == kPrimTriangle) {
        e[1] = make_float4(b.x - a.x, b.y - a.y, b.z - a.z, b.w);
        e[2] = make_float4(c.x - a.x, c.y - a.y, c.z - a.z, c.w);
    } else {
        e[1] = b;
        e[2] = c;
    }
}

__device__ __forceinline__ void write_child_box(float4* node, int slot, const Box3& b) {
    float* f = reinterpret_cast<float*>(node);
    if (slot == 0) {
        f[0] = b.lo.x; f[1] = b.hi.x; f[2] = b.lo.y; f[3] = b.hi.y;   // n0
        f[8] = b.lo.z; f[9] = b.hi.z;                                   // n2.xy
    } else {
        f[4] = b.lo.x; f[5] = b.hi.x; f[6] = b.lo.y; f[7] = b.hi.y;   // n1
        f[10] = b.lo.z; f[11] = b.hi.z;                                 // n2.zw
    }
}

// Bottom-up refit: every leaf writes its box into its parent's slot; the
// second thread to arrive at a node (atomic counter) unites both child boxes
// and climbs on.  No thread ever waits, so the kernel cannot stall.
__global__ void k_refit(const float4* __restrict__ prims, uint32_t n, float4* nodes, const int* __restrict__ parent_leaf,
                        const int* __restrict__ parent_int, uint32_t* flags) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Box3 b = prim_box(prims + 3 * size_t(i));
    int p = parent_leaf[i];
    if (p == -2) {   // one-primitive segment: the root holds the leaf twice
        write_child_box(nodes + 4 * size_t(i), 0, b);
        write_child_box(nodes + 4 * size_t(i), 1, b);
        float* f = reinterpret_cast<float*>(nodes + 4 * size_t(i) + 3);
        f[2] = f[3] = prims[3 * size_t(i) + 2].w;
        return;
    }
    int child = ~int(i);
    // the leaf's record kind goes next to its child reference (n3.z / n3.w),
    // so traversal knows an instance from a primitive without loading the record
    const uint32_t kind = __float_as_uint(prims[3 * size_t(i) + 2].w);
    {
        const float4 n3 = __ldcg(nodes + 4 * size_t(p) + 3);
        float* f = reinterpret_cast<float*>(nodes + 4 * size_t(p) + 3);
        f[(__float_as_int(n3.x) == child) ? 2 : 3] = __uint_as_float(kind);
    }
    while (p >= 0) {
        const float4 n3 = __ldcg(nodes + 4 * size_t(p) + 3);
        const int slot = (__float_as_int(n3.x) == child) ? 0 : 1;
        write_child_box(nodes + 4 * size_t(p), slot, b);
        __threadfence();
        const uint32_t old = atomicAdd(&flags[p], 1u);
        if (old == 0u) return;   // first arrival: the sibling finishes the node
        __threadfence();
        const float4 n0 = __ldcg(nodes + 4 * size_t(p));
        const float4 n1 = __ldcg(nodes + 4 * size_t(p) + 1);
        const float4 n2 = __ldcg(nodes + 4 * size_t(p) + 2);
        b.lo = mk(fminf(n0.x, n1.x), fminf(n0.z, n1.z), fminf(n2.x, n2.z));
        b.hi = mk(fmaxf(n0.y, n1.y), fmaxf(n0.w, n1.w), fmaxf(n2.y, n2.w));
        child = p;
        p = parent_int[p];
    }
}

// Albedos of all things from a device array (3 floats per thing), for
// optimisers that keep their parameters on the device.
__global__ void k_set_albedos(ThingDev* __restrict__ things, const float* __restrict__ albedo, uint32_t n) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    float4 a = things[t].albedo_type;
    a.x = albedo[3 * size_t(t)];
    a.y = albedo[3 * size_t(t) + 1];
    a.z = albedo[3 * size_t(t) + 2];
    things[t].albedo_type = a;
}

__global__ void k_lbvh_snapshot_codes32(const uint32_t* __restrict__ c, uint32_t n, unsigned long long* __restrict__ o) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) o[i] = c[i];
}

// ------------------------------------------------------------- host side
void check_optics(const rt_optics* o) {
    RT_REQUIRE(o != nullptr, "optics is NULL");
    RT_REQUIRE(o->type >= RT_OPTICS_DIFFUSE && o->type <= RT_OPTICS_REFRACT, "unknown optics type");
}

void check_transform(const float* t) {
    RT_REQUIRE(t != nullptr, "transform is NULL");
    for (int k = 0; k < 12; ++k) RT_REQUIRE(std::isfinite(t[k]), "transform has a non-finite entry");
}

inline float int_bits_as_float(int i) {
    float f;
    std::memcpy(&f, &i, 4);
    return f;
}

ThingDev thing_dev(const ThingHost& th) {
    ThingDev d;
    const float3 c = th.mesh < 0 ? th.center : make_float3(th.T[3], th.T[7], th.T[11]);
    d.albedo_type = make_float4(th.optics.albedo.x, th.optics.albedo.y, th.optics.albedo.z,
                                int_bits_as_float(th.optics.type));
    d.center_fuzz = make_float4(c.x, c.y, c.z, th.optics.fuzz);
    d.index_pad = make_float4(th.optics.index, 0.f, 0.f, 0.f);
    return d;
}

// In the instanced layout a mesh thing is instanced (one top-level record
// over a bottom-level hierarchy of its mesh) when its transform is diagonal
// with +0 off-diagonal entries, so the on-the-fly world vertices and boxes
// round exactly like the flat layout's, and its mesh is large enough for a
// hierarchy of its own to pay.
constexpr uint32_t kInstanceMinTris = 16;

bool diagonal_pos0(const float* T) {
    const int off[6] = {1, 2, 4, 6, 8, 9};
    for (int k : off) {
        uint32_t b;
        std::memcpy(&b, &T[k], 4);
        if (b != 0u) return false;
    }
    return true;
}

bool instance_thing(const ThingHost& th, const Scene& sc, int layout) {
    if (layout != RT_LAYOUT_INSTANCED || th.mesh < 0) return false;
    return diagonal_pos0(th.T) && sc.meshes[th.mesh].ni >= kInstanceMinTris;
}

// Host plan of a geometry: per-thing descriptors, optics, instance data and
// the bottom-level mesh table.
struct Plan {
    std::vector<FlatDesc> desc;
    std::vector<ThingDev> td;
    std::vector<InstDev> inst;
    std::vector<BlasMesh> meshes;
    std::vector<SegDev> top_segs, bottom_segs;
    std::vector<uint32_t> thing_begin;
    std::vector<int> inst_class;
    uint64_t nprims = 0, ntop = 0, nbottom = 0;
    uint32_t ninstances = 0;
};

Plan make_plan(const std::vector<Scene*>& scenes, int layout) {
    Plan P;
    P.thing_begin.assign(scenes.size(), 0);
    P.top_segs.assign(scenes.size(), SegDev{0, 0});
    for (size_t si = 0; si < scenes.size(); ++si) {
        const Scene& sc = *scenes[si];
        P.thing_begin[si] = uint32_t(P.desc.size());
        P.top_segs[si].prim_begin = uint32_t(P.ntop);
        std::vector<int> mesh_seg(sc.meshes.size(), -1);   // bottom-level segment of each mesh of this scene
        for (const ThingHost& th : sc.things) {
            FlatDesc d;
            std::memset(&d, 0, sizeof(d));
            d.prim_offset = uint32_t(P.nprims);
            d.seg = uint32_t(si);
            d.top_offset = uint32_t(P.ntop);
            d.blas_root = -1;
            InstDev in;
            std::memset(&in, 0, sizeof(in));
            if (th.mesh < 0) {
                d.analytic = 1;
                d.nprims = 1;
                d.ntop = 1;
                d.sphere = make_float4(th.center.x, th.center.y, th.center.z, th.radius);
            } else {
                const MeshDev& m = sc.meshes[th.mesh];
                d.v = m.v.as<float3>();
                d.idx = m.i.as<uint3>();
                d.nprims = m.ni;
                std::memcpy(d.T, th.T, sizeof(d.T));
                if (instance_thing(th, sc, layout)) {
                    if (mesh_seg[th.mesh] < 0) {
                        mesh_seg[th.mesh] = int(P.meshes.size());
                        P.meshes.push_back(BlasMesh{d.v, d.idx, uint32_t(P.nbottom), m.ni});
                        P.bottom_segs.push_back(SegDev{uint32_t(P.nbottom), m.ni});
                        P.nbottom += m.ni;
                        RT_REQUIRE(P.nbottom < (uint64_t(1) << 31), "too many bottom-level triangles (>= 2^31)");
                    }
                    const SegDev& bs = P.bottom_segs[mesh_seg[th.mesh]];
                    d.instanced = 1;
                    d.ntop = 1;
                    d.blas_seg = uint32_t(mesh_seg[th.mesh]);
                    d.blas_root = int(bs.prim_begin);   // a segment's root is its first node slot
                    in.a = make_float4(th.T[0], th.T[5], th.T[10], th.T[3]);
                    uint32_t po = d.prim_offset;
                    float pof, rootf;
                    std::memcpy(&pof, &po, 4);
                    std::memcpy(&rootf, &d.blas_root, 4);
                    in.b = make_float4(th.T[7], th.T[11], pof, rootf);
                    P.ninstances += 1;
                } else {
                    d.ntop = m.ni;
                }
            }
            P.nprims += d.nprims;
            P.ntop += d.ntop;
            RT_REQUIRE(P.nprims < (uint64_t(1) << 31), "too many primitives (>= 2^31)");
            RT_REQUIRE(P.ntop < (uint64_t(1) << 31), "too many top-level records (>= 2^31)");
            P.inst_class.push_back(d.instanced);
            P.desc.push_back(d);
            P.td.push_back(thing_dev(th));
            P.inst.push_back(in);
        }
        P.top_segs[si].prim_count = uint32_t(P.ntop) - P.top_segs[si].prim_begin;
    }
    return P;
}

void upload_lbvh_segments(Lbvh& L, const std::vector<SegDev>& segs, uint64_t nrec, cudaStream_t s) {
    L.seg_host = segs;
    L.nsegs = uint32_t(segs.size());
    L.nprims = uint32_t(nrec);
    L.segs.reserve(std::max<size_t>(1, segs.size()) * sizeof(SegDev));
    if (!segs.empty())
        RT_CUDA(cudaMemcpyAsync(L.segs.p, segs.data(), segs.size() * sizeof(SegDev), cudaMemcpyHostToDevice, s));
    L.prims_flat.reserve(std::max<size_t>(1, nrec) * 48);
    if (L.nsegs > 1) L.prim_seg.reserve(std::max<size_t>(1, nrec) * 4);
}

// Uploads the plan (descriptors, optics, instance data, segment tables).
void upload_plan(Geometry& g, const Plan& P, size_t nscenes, cudaStream_t s) {
    g.nprims = uint32_t(P.nprims);
    g.nthings = uint32_t(P.desc.size());
    g.nsegs = uint32_t(nscenes);
    g.ninstances = P.ninstances;
    g.thing_begin = P.thing_begin;
    g.inst_class = P.inst_class;
    g.desc_host = P.desc;
    g.desc.reserve(std::max<size_t>(1, P.desc.size()) * sizeof(FlatDesc));
    g.things_dev.reserve(std::max<size_t>(1, P.td.size()) * sizeof(ThingDev));
    g.inst.reserve(std::max<size_t>(1, P.inst.size()) * sizeof(InstDev));
    if (!P.desc.empty()) {
        RT_CUDA(cudaMemcpyAsync(g.desc.p, P.desc.data(), P.desc.size() * sizeof(FlatDesc), cudaMemcpyHostToDevice, s));
        RT_CUDA(cudaMemcpyAsync(g.things_dev.p, P.td.data(), P.td.size() * sizeof(ThingDev), cudaMemcpyHostToDevice, s));
        RT_CUDA(cudaMemcpyAsync(g.inst.p, P.inst.data(), P.inst.size() * sizeof(InstDev), cudaMemcpyHostToDevice, s));
    }
    upload_lbvh_segments(g.top, P.top_segs, P.ntop, s);
    upload_lbvh_segments(g.blas, P.bottom_segs, P.nbottom, s);
}

void flatten_bottom(Geometry& g, const Plan& P, cudaStream_t s) {
    if (g.blas.nprims == 0) return;
    DevBuf meshes;
    meshes.reserve(P.meshes.size() * sizeof(BlasMesh));
    RT_CUDA(cudaMemcpyAsync(meshes.p, P.meshes.data(), P.meshes.size() * sizeof(BlasMesh), cudaMemcpyHostToDevice, s));
    k_flatten_bottom<<<grid_for(g.blas.nprims), kThreads, 0, s>>>(
        meshes.as<BlasMesh>(), uint32_t(P.meshes.size()), g.blas.nprims, g.blas.prims_flat.as<float4>(),
        g.blas.nsegs > 1 ? g.blas.prim_seg.as<uint32_t>() : nullptr);
    RT_CHECK_LAUNCH();
    RT_CUDA(cudaStreamSynchronize(s));   // `meshes` and the plan's host arrays must outlive the copies
}

void flatten_top(Geometry& g, cudaStream_t s) {
    if (g.top.nprims == 0) return;
    k_flatten_top<<<grid_for(g.top.nprims), kThreads, 0, s>>>(
        g.desc.as<FlatDesc>(), g.nthings, g.top.nprims, g.blas.nodes.p ? g.blas.nodes.as<float4>() : nullptr,
        g.top.prims_flat.as<float4>(), g.top.nsegs > 1 ? g.top.prim_seg.as<uint32_t>() : nullptr);
    RT_CHECK_LAUNCH();
}

void refit(Lbvh& L, cudaStream_t s) {
    const uint32_t n = L.nprims;
    if (n == 0) return;
    k_gather_prims<<<grid_for(n), kThreads, 0, s>>>(L.prims_flat.as<float4>(), L.ids.as<uint32_t>(), n,
                                                     L.prims.as<float4>(), L.prims_e.as<float4>());
    RT_CHECK_LAUNCH();
    int* parents = L.parents.as<int>();
    RT_CUDA(cudaMemsetAsync(L.flags.p, 0, size_t(n) * sizeof(uint32_t), s));
    k_refit<<<grid_for(n), kThreads, 0, s>>>(L.prims.as<float4>(), n, L.nodes.as<float4>(), parents, parents + n,
                                              L.flags.as<uint32_t>());
    RT_CHECK_LAUNCH();
}

template <class K>
void build_topology(Lbvh& L, cudaStream_t s) {
    const uint32_t n = L.nprims;
    L.codes.reserve(size_t(n) * sizeof(K));
    L.ids.reserve(size_t(n) * sizeof(uint32_t));
    K* codes = L.codes.as<K>();
    uint32_t* ids = L.ids.as<uint32_t>();
    const uint32_t* pseg = L.nsegs > 1 ? L.prim_seg.as<uint32_t>() : nullptr;
    int key_bits = L.morton_bits;
    if (L.grouped) {
        k_morton_grouped<<<grid_for(n), kThreads, 0, s>>>(L.prims_flat.as<float4>(), n, L.tbounds.as<uint32_t>(),
                                                           reinterpret_cast<unsigned long long*>(codes), ids);
        int thing_bits = 1;
        while ((uint64_t(1) << thing_bits) < L.nthings) ++thing_bits;
        key_bits = 30 + thing_bits;
    } else {
        k_morton<K><<<grid_for(n), kThreads, 0, s>>>(L.prims_flat.as<float4>(), pseg, n, L.bounds.as<uint32_t>(),
                                                      codes, ids);
    }
    RT_CHECK_LAUNCH();
    if (sizeof(K) == 4)
        radix_sort_pairs_u32(reinterpret_cast<uint32_t*>(codes), ids, n, key_bits, L.sort_tmp, s);
    else
        radix_sort_pairs_u64(reinterpret_cast<unsigned long long*>(codes), ids, n, key_bits, L.sort_tmp, s);
    if (L.nsegs > 1 && !L.grouped) {   // grouped keys are thing-major, hence segment-major already
        // stable second pass by segment: (segment, code) order
        int seg_bits = 1;
        while ((1u << seg_bits) < L.nsegs) ++seg_bits;
        const size_t kb = size_t(n) * sizeof(K);
        L.seg_tmp.reserve(2 * size_t(n) * 4 + kb + size_t(n) * 4);
        uint32_t* keys = L.seg_tmp.as<uint32_t>();
        uint32_t* perm = keys + n;
        K* codes2 = reinterpret_cast<K*>(perm + n);
        uint32_t* ids2 = reinterpret_cast<uint32_t*>(reinterpret_cast<char*>(codes2) + kb);
        k_seg_keys<<<grid_for(n), kThreads, 0, s>>>(pseg, ids, n, keys, perm);
        RT_CHECK_LAUNCH();
        radix_sort_pairs_u32(keys, perm, n, seg_bits, L.sort_tmp, s);
        k_permute<K><<<grid_for(n), kThreads, 0, s>>>(codes, ids, perm, n, codes2, ids2);
        RT_CHECK_LAUNCH();
        RT_CUDA(cudaMemcpyAsync(codes, codes2, kb, cudaMemcpyDeviceToDevice, s));
        RT_CUDA(cudaMemcpyAsync(ids, ids2, size_t(n) * 4, cudaMemcpyDeviceToDevice, s));
    }
    int* parents = L.parents.as<int>();
    if (L.grouped) {   // one hierarchy per thing now, the thing trees are stitched on top afterwards
        k_karras<K><<<grid_for(n), kThreads, 0, s>>>(codes, L.tsegs.as<SegDev>(), L.nthings, n, L.nodes.as<float4>(),
                                                      parents, parents + n);
    } else {
        k_karras<K><<<grid_for(n), kThreads, 0, s>>>(codes, L.segs.as<SegDev>(), L.nsegs, n, L.nodes.as<float4>(),
                                                      parents, parents + n);
    }
    RT_CHECK_LAUNCH();
}

// Largest cluster of the binned-SAH layout: kSahClusterMax, or RTX_SAH_CLUSTER
// (tests use small clusters to get deep split trees from small scenes).
uint32_t sah_cluster_max() {
    const char* v = std::getenv("RTX_SAH_CLUSTER");
    if (!v || !*v) return kSahClusterMax;
    const unsigned long x = std::strtoul(v, nullptr, 10);
    return x >= 1 && x <= (1u << 20) ? uint32_t(x) : kSahClusterMax;
}

// Morton codes (or things-grouped keys, for top-level records whose a.w is
// the thing), sort, hierarchy and refit of an LBVH whose records are in
// prims_flat.
void build_lbvh(Lbvh& L, int morton_bits, cudaStream_t s, const FlatDesc* desc = nullptr,
                const std::vector<FlatDesc>* desc_host = nullptr, const std::vector<uint32_t>* thing_begin = nullptr,
                bool sah = false) {
    L.morton_bits = morton_bits;
    const uint32_t nthings = desc_host ? uint32_t(desc_host->size()) : 0u;
    L.sah = sah && L.nprims > 0;
    L.grouped = !L.sah && desc != nullptr && nthings > 0 && L.nprims > 0;
    L.nclusters = L.sah_levels = 0;
    L.nthings = nthings;
    L.roots.clear();
    if (L.grouped) {
        // host tables: per-thing record range and scene, per-scene thing range and root
        std::vector<SegDev> tsegs(nthings), scene_things(L.nsegs);
        std::vector<uint32_t> tseg(nthings);
        for (uint32_t t = 0; t < nthings; ++t) {
            tsegs[t] = SegDev{(*desc_host)[t].top_offset, (*desc_host)[t].ntop};
            tseg[t] = (*desc_host)[t].seg;
        }
        L.roots.assign(L.nsegs, -1);
        for (uint32_t sg = 0; sg < L.nsegs; ++sg) {
            const uint32_t tb = (*thing_begin)[sg];
            const uint32_t te = sg + 1 < L.nsegs ? (*thing_begin)[sg + 1] : nthings;
            scene_things[sg] = SegDev{tb, te - tb};
            if (te - tb >= 2) L.roots[sg] = int(tsegs[tb].prim_begin + tsegs[tb].prim_count) - 1;
            else if (te - tb == 1) L.roots[sg] = int(tsegs[tb].prim_begin);
        }
        L.tsegs.reserve(size_t(nthings) * sizeof(SegDev));
        L.scene_things.reserve(std::max<size_t>(1, L.nsegs) * sizeof(SegDev));
        L.tseg.reserve(size_t(nthings) * 4);
        RT_CUDA(cudaMemcpyAsync(L.tsegs.p, tsegs.data(), tsegs.size() * sizeof(SegDev), cudaMemcpyHostToDevice, s));
        RT_CUDA(cudaMemcpyAsync(L.scene_things.p, scene_things.data(), scene_things.size() * sizeof(SegDev),
                                cudaMemcpyHostToDevice, s));
        RT_CUDA(cudaMemcpyAsync(L.tseg.p, tseg.data(), tseg.size() * 4, cudaMemcpyHostToDevice, s));
        RT_CUDA(cudaStreamSynchronize(s));   // the host tables must outlive the copies
    }
    const uint32_t n = L.nprims;
    L.prims.reserve(std::max<size_t>(1, n) * 48);
    L.prims_e.reserve(std::max<size_t>(1, n) * 48);
    L.nodes.reserve(std::max<size_t>(1, n) * 64);
    L.parents.reserve((size_t(n) * 2 + 1) * sizeof(int));
    L.flags.reserve(std::max<size_t>(1, n) * sizeof(uint32_t));
    L.bounds.reserve(std::max<size_t>(1, L.nsegs) * 6 * sizeof(uint32_t));
    if (n == 0) return;
    k_init_bounds<<<grid_for(6 * L.nsegs), kThreads, 0, s>>>(L.bounds.as<uint32_t>(), L.nsegs);
    RT_CHECK_LAUNCH();
    k_centroid_bounds<<<grid_for(n), kThreads, 0, s>>>(L.prims_flat.as<float4>(),
                                                        L.nsegs > 1 ? L.prim_seg.as<uint32_t>() : nullptr, n,
                                                        L.bounds.as<uint32_t>(), 0);
    RT_CHECK_LAUNCH();
    if (L.sah) {
        NvtxRange nvtx("rt build: binned SAH");
        build_sah_topology(L, sah_cluster_max(), s);
    } else if (L.grouped) {
        const uint32_t T = nthings;
        L.tbounds.reserve(size_t(T) * 6 * sizeof(uint32_t));
        L.tcodes.reserve(size_t(T) * 8 * 2);
        L.tids.reserve(size_t(T) * 4 * 2);
        L.ttmp.reserve(size_t(T) * 64 + size_t(T) * 8 + 64);
        k_init_bounds<<<grid_for(6 * T), kThreads, 0, s>>>(L.tbounds.as<uint32_t>(), T);
        RT_CHECK_LAUNCH();
        k_centroid_bounds<<<grid_for(n), kThreads, 0, s>>>(L.prims_flat.as<float4>(), nullptr, n,
                                                            L.tbounds.as<uint32_t>(), 1);
        RT_CHECK_LAUNCH();
        // thing subtrees (segments = things)
        build_topology<unsigned long long>(L, s);
        // the things of each scene in 60-bit code order, scene-major
        unsigned long long* tc = L.tcodes.as<unsigned long long>();
        uint32_t* tid = L.tids.as<uint32_t>();
        k_thing_codes<<<grid_for(T), kThreads, 0, s>>>(L.tbounds.as<uint32_t>(), desc, L.bounds.as<uint32_t>(), T, tc,
                                                        tid);
        RT_CHECK_LAUNCH();
        radix_sort_pairs_u64(tc, tid, T, 60, L.sort_tmp, s);
        if (L.nsegs > 1) {
            int seg_bits = 1;
            while ((1u << seg_bits) < L.nsegs) ++seg_bits;
            L.seg_tmp.reserve(size_t(T) * 8);
            uint32_t* keys = L.seg_tmp.as<uint32_t>();
            uint32_t* perm = keys + T;
            unsigned long long* tc2 = tc + T;
            uint32_t* tid2 = tid + T;
            k_seg_keys<<<grid_for(T), kThreads, 0, s>>>(L.tseg.as<uint32_t>(), tid, T, keys, perm);
            RT_CHECK_LAUNCH();
            radix_sort_pairs_u32(keys, perm, T, seg_bits, L.sort_tmp, s);
            k_permute<unsigned long long><<<grid_for(T), kThreads, 0, s>>>(tc, tid, perm, T, tc2, tid2);
            RT_CHECK_LAUNCH();
            RT_CUDA(cudaMemcpyAsync(tc, tc2, size_t(T) * 8, cudaMemcpyDeviceToDevice, s));
            RT_CUDA(cudaMemcpyAsync(tid, tid2, size_t(T) * 4, cudaMemcpyDeviceToDevice, s));
        }
        // the thing tree of each scene, into scratch, then stitched into the spare slots
        float4* tnodes = L.ttmp.as<float4>();
        int* tpar = reinterpret_cast<int*>(tnodes + 4 * size_t(T));
        k_karras<unsigned long long><<<grid_for(T), kThreads, 0, s>>>(tc, L.scene_things.as<SegDev>(), L.nsegs, T,
                                                                       tnodes, tpar, tpar + T);
        RT_CHECK_LAUNCH();
        int* parents = L.parents.as<int>();
        k_stitch<<<grid_for(T), kThreads, 0, s>>>(tnodes, L.scene_things.as<SegDev>(), L.nsegs, tid,
                                                  L.tsegs.as<SegDev>(), T, L.nodes.as<float4>(), parents, parents + n);
        RT_CHECK_LAUNCH();
    } else if (morton_bits == 30) {
        build_topology<uint32_t>(L, s);
    } else {
        build_topology<unsigned long long>(L, s);
    }
    refit(L, s);
}

}  // namespace

// Bottom-level roots of the instanced things, read from the built bottom
// level (a binned-SAH hierarchy's root is not its segment's first slot).
void set_blas_roots(const Lbvh& blas, std::vector<FlatDesc>& desc, std::vector<InstDev>& inst) {
    for (size_t t = 0; t < desc.size(); ++t) {
        if (!desc[t].instanced) continue;
        const int r = blas.root(desc[t].blas_seg);
        desc[t].blas_root = r;
        float rootf;
        std::memcpy(&rootf, &r, 4);
        inst[t].b.w = rootf;
    }
}

void build_geometry(Geometry& g, const std::vector<Scene*>& scenes, int morton_bits, int layout, cudaStream_t s) {
    NvtxRange nvtx("rt build");
    RT_REQUIRE(morton_bits == 0 || morton_bits == 30 || morton_bits == 60, "morton_bits must be 0, 30 or 60");
    RT_REQUIRE(layout >= RT_LAYOUT_AUTO && layout <= RT_LAYOUT_SAH, "unknown layout");
    RT_REQUIRE(!scenes.empty(), "no scenes to build");
    g.morton_bits = morton_bits == 0 ? 60 : morton_bits;
    g.layout_req = layout;
    cudaEvent_t e0, e1;
    RT_CUDA(cudaEventCreate(&e0));
    RT_CUDA(cudaEventCreate(&e1));
    RT_CUDA(cudaEventRecord(e0, s));
    const Plan P = make_plan(scenes, layout);
    upload_plan(g, P, scenes.size(), s);
    g.layout = P.ninstances                                           ? RT_LAYOUT_INSTANCED
               : (layout == RT_LAYOUT_AUTO || layout == RT_LAYOUT_SAH) ? RT_LAYOUT_SAH
               : layout == RT_LAYOUT_GROUPED                          ? RT_LAYOUT_GROUPED
                                                                      : RT_LAYOUT_FLAT;
    g.optics_seen.assign(scenes.size(), 0);
    for (size_t si = 0; si < scenes.size(); ++si) g.optics_seen[si] = scenes[si]->optics_version;
    g.misc.reserve(256);
    flatten_bottom(g, P, s);
    // object space, before the instance boxes are taken; binned SAH per mesh
    build_lbvh(g.blas, g.morton_bits, s, nullptr, nullptr, nullptr, g.layout == RT_LAYOUT_INSTANCED);
    std::vector<InstDev> inst = P.inst;
    if (P.ninstances) {   // the bottom roots are known now
        set_blas_roots(g.blas, g.desc_host, inst);
        RT_CUDA(cudaMemcpyAsync(g.desc.p, g.desc_host.data(), g.desc_host.size() * sizeof(FlatDesc),
                                cudaMemcpyHostToDevice, s));
        RT_CUDA(cudaMemcpyAsync(g.inst.p, inst.data(), inst.size() * sizeof(InstDev), cudaMemcpyHostToDevice, s));
    }
    flatten_top(g, s);
    const bool grouped = g.layout == RT_LAYOUT_GROUPED;
    build_lbvh(g.top, g.morton_bits, s, grouped ? g.desc.as<FlatDesc>() : nullptr, grouped ? &g.desc_host : nullptr,
               &g.thing_begin, g.layout == RT_LAYOUT_SAH || g.layout == RT_LAYOUT_INSTANCED);
    RT_CUDA(cudaEventRecord(e1, s));
    RT_CUDA(cudaEventSynchronize(e1));
    RT_CUDA(cudaEventElapsedTime(&g.build_ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
}

void refit_geometry(Geometry& g, const std::vector<Scene*>& scenes, cudaStream_t s) {
    NvtxRange nvtx("rt refit");
    const Plan P = make_plan(scenes, g.layout_req);
    if (P.inst_class != g.inst_class || P.ntop != g.top.nprims || P.nbottom != g.blas.nprims) {
        // a thing changed between instanced and flattened: the hierarchy changes
        build_geometry(g, scenes, g.morton_bits, g.layout_req, s);
        g.refit_ms = g.build_ms;
        return;
    }
    cudaEvent_t e0, e1;
    RT_CUDA(cudaEventCreate(&e0));
    RT_CUDA(cudaEventCreate(&e1));
    RT_CUDA(cudaEventRecord(e0, s));
    // transforms only reach the descriptors, instance data and the top level;
    // the bottom level is in object space and stays as built
    g.desc_host = P.desc;
    std::vector<InstDev> inst = P.inst;
    set_blas_roots(g.blas, g.desc_host, inst);
    RT_CUDA(cudaMemcpyAsync(g.desc.p, g.desc_host.data(), g.desc_host.size() * sizeof(FlatDesc),
                            cudaMemcpyHostToDevice, s));
    RT_CUDA(cudaMemcpyAsync(g.things_dev.p, P.td.data(), P.td.size() * sizeof(ThingDev), cudaMemcpyHostToDevice, s));
    RT_CUDA(cudaMemcpyAsync(g.inst.p, inst.data(), inst.size() * sizeof(InstDev), cudaMemcpyHostToDevice, s));
    for (size_t si = 0; si < scenes.size(); ++si) g.optics_seen[si] = scenes[si]->optics_version;
    flatten_top(g, s);
    refit(g.top, s);
    RT_CUDA(cudaEventRecord(e1, s));
    RT_CUDA(cudaEventSynchronize(e1));   // the plan's host arrays must outlive the copies
    RT_CUDA(cudaEventElapsedTime(&g.refit_ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
}

void set_albedos_device(Geometry& g, const std::vector<Scene*>& scenes, const float* albedo, cudaStream_t s) {
    RT_REQUIRE(albedo != nullptr, "albedo is NULL");
    sync_optics(g, scenes, s);   // pending host-side optics first, so they cannot overwrite these later
    if (g.nthings == 0) return;
    k_set_albedos<<<grid_for(g.nthings), kThreads, 0, s>>>(g.things_dev.as<ThingDev>(), albedo, g.nthings);
    RT_CHECK_LAUNCH();
}

void sync_optics(Geometry& g, const std::vector<Scene*>& scenes, cudaStream_t s) {
    RT_REQUIRE(scenes.size() == g.optics_seen.size(), "scene list differs from the built geometry");
    bool stale = false;
    for (size_t si = 0; si < scenes.size(); ++si) stale = stale || scenes[si]->optics_version != g.optics_seen[si];
    if (!stale) return;
    RT_REQUIRE(!stream_capturing(s), "optics changed on the host since the last launch: upload them with a "
                                     "launch outside the stream capture first");
    g.things_host.clear();
    for (size_t si = 0; si < scenes.size(); ++si) {
        for (const ThingHost& th : scenes[si]->things) g.things_host.push_back(thing_dev(th));
        g.optics_seen[si] = scenes[si]->optics_version;
    }
    RT_REQUIRE(g.things_host.size() == g.nthings, "thing count changed since the build");
    if (g.nthings)
        RT_CUDA(cudaMemcpyAsync(g.things_dev.p, g.things_host.data(), g.things_host.size() * sizeof(ThingDev),
                                cudaMemcpyHostToDevice, s));
    RT_CUDA(cudaStreamSynchronize(s));
}

size_t Lbvh::device_bytes() const {
    return segs.bytes + prim_seg.bytes + prims_flat.bytes + prims.bytes + prims_e.bytes + nodes.bytes + codes.bytes + ids.bytes +
           parents.bytes + flags.bytes + bounds.bytes + sort_tmp.bytes + seg_tmp.bytes + tbounds.bytes + tcodes.bytes +
           tids.bytes + tsegs.bytes + scene_things.bytes + tseg.bytes + ttmp.bytes;
}

size_t Geometry::device_bytes() const {
    return things_dev.bytes + desc.bytes + inst.bytes + misc.bytes + top.device_bytes() + blas.device_bytes();
}

GeoView Geometry::view() const {
    GeoView v;
    v.tnodes = top.nodes.as<float4>();
    v.tprims = top.prims.as<float4>();
    v.tedges = top.prims_e.as<float4>();
    v.bnodes = blas.nodes.as<float4>();
    v.bprims = blas.prims.as<float4>();
    v.inst = inst.as<InstDev>();
    v.desc = desc.as<FlatDesc>();
    v.instanced = ninstances > 0 ? 1 : 0;
    v.ntnodes = uint32_t(top.nodes.bytes / 64);
    v.ntprims = uint32_t(top.prims.bytes / 48);
    v.nbnodes = uint32_t(blas.nodes.bytes / 64);
    v.nbprims = uint32_t(blas.prims.bytes / 48);
    v.nthings = nthings;
    v.err = nullptr;   // set by each launch
    return v;
}

size_t Scene::device_bytes() const {
    size_t b = geo.device_bytes();
    for (const auto& m : meshes) b += m.v.bytes + m.i.bytes;
    return b;
}

Scene* scene_from(rt_scene h) {
    RT_REQUIRE(h != nullptr, "scene handle is NULL");
    return reinterpret_cast<Scene*>(h);
}

namespace {

// The device arrays of the last scene destroyed on this host thread, kept for
// the next scene the thread builds: a hierarchy's arrays (1.8 GB for the
// 8 M-triangle C1 scene) are handed on instead of freed and allocated again
// (a new C1 scene per frame: 1.6 ms of cudaFree per destroy and 0.6 ms of
// cudaMalloc per build).  rt_scene_destroy(NULL) frees them.
struct SpareGeometry {
    int dev = -1;
    std::unique_ptr<Geometry> geo;
};
SpareGeometry& spare_geometry() {
    static thread_local SpareGeometry sp;
    return sp;
}

void scene_build(Scene& sc, int morton_bits, cudaStream_t s) {
    sc.built = false;   // a build that fails half way leaves no renderable scene behind
    if (!sc.geo.top.nodes.p) {   // a first build: take the spare arrays of this device, if any
        SpareGeometry& sp = spare_geometry();
        int dev = 0;
        RT_CUDA(cudaGetDevice(&dev));
        if (sp.geo && sp.dev == dev) {
            // records this scene will have (a sphere or instance is one, a
            // flattened mesh thing its triangles): arrays sized for more than
            // twice as many are freed rather than held by a smaller scene
            uint64_t recs = 0;
            for (const ThingHost& th : sc.things)
                recs += th.mesh >= 0 && size_t(th.mesh) < sc.meshes.size() ? sc.meshes[size_t(th.mesh)].ni : 1u;
            if (uint64_t(sp.geo->top.nprims) <= 2 * recs + 65536) sc.geo = std::move(*sp.geo);
            sp.geo.reset();
        }
    }
    build_geometry(sc.geo, {&sc}, morton_bits, sc.layout, s);
    sc.built = true;
    sc.topology_dirty = false;
    sc.xf_dirty = false;
}

void scene_update(Scene& sc, cudaStream_t s) {
    if (!sc.built) throw Error(RT_ERR_NOT_BUILT, "rt_scene_update before rt_scene_build");
    if (sc.topology_dirty) throw Error(RT_ERR_NOT_BUILT, "things were added since the last build; rebuild");
    refit_geometry(sc.geo, {&sc}, s);
    sc.xf_dirty = false;
}

void tessellate(Scene& sc, float radius, uint32_t ndiv, cudaStream_t s, uint32_t* mesh_id) {
    RT_REQUIRE(ndiv <= 10, "ndiv must be <= 10");
    RT_REQUIRE(std::isfinite(radius), "radius must be finite");
    const uint32_t ntri = 4u << (2 * ndiv);
    const uint32_t m = 3 * ntri;   // vertex instances in generation order
    DevBuf pts, idx, keys, head, head_scan, head_orig, run_of_orig, mark, vid, scan_tmp, sort_tmp;
    pts.reserve(size_t(m) * sizeof(float3));
    idx.reserve(size_t(m) * 4);
    keys.reserve(size_t(m) * 4);
    head.reserve(size_t(m) * 4);
    head_scan.reserve(size_t(m) * 4);
    head_orig.reserve(size_t(m) * 4);
    run_of_orig.reserve(size_t(m) * 4);
    mark.reserve(size_t(m) * 4);
    vid.reserve(size_t(m) * 4);
    k_tess_leaves<<<grid_for(ntri), kThreads, 0, s>>>(radius, ndiv, ntri, pts.as<float3>());
    RT_CHECK_LAUNCH();
    k_iota<<<grid_for(m), kThreads, 0, s>>>(idx.as<uint32_t>(), m);
    RT_CHECK_LAUNCH();
    // lexicographic (x, y, z) stable sort as three stable passes z, y, x
    for (int axis = 2; axis >= 0; --axis) {
        k_axis_keys<<<grid_for(m), kThreads, 0, s>>>(pts.as<float3>(), idx.as<uint32_t>(), m, axis, keys.as<uint32_t>());
        RT_CHECK_LAUNCH();
        radix_sort_pairs_u32(keys.as<uint32_t>(), idx.as<uint32_t>(), m, 32, sort_tmp, s);
    }
    k_run_heads<<<grid_for(m), kThreads, 0, s>>>(pts.as<float3>(), idx.as<uint32_t>(), m, head.as<uint32_t>());
    RT_CHECK_LAUNCH();
    scan_exclusive_u32(head.as<uint32_t>(), head_scan.as<uint32_t>(), m, scan_tmp, s);
    RT_CUDA(cudaMemsetAsync(mark.p, 0, size_t(m) * 4, s));
    k_mark_heads<<<grid_for(m), kThreads, 0, s>>>(idx.as<uint32_t>(), head.as<uint32_t>(), head_scan.as<uint32_t>(), m,
                                                  head_orig.as<uint32_t>(), run_of_orig.as<uint32_t>(),
                                                  mark.as<uint32_t>());
    RT_CHECK_LAUNCH();
    scan_exclusive_u32(mark.as<uint32_t>(), vid.as<uint32_t>(), m, scan_tmp, s);
    uint32_t last_vid = 0, last_mark = 0;
    RT_CUDA(cudaMemcpyAsync(&last_vid, vid.as<uint32_t>() + (m - 1), 4, cudaMemcpyDeviceToHost, s));
    RT_CUDA(cudaMemcpyAsync(&last_mark, mark.as<uint32_t>() + (m - 1), 4, cudaMemcpyDeviceToHost, s));
    RT_CUDA(cudaStreamSynchronize(s));
    const uint32_t nv = last_vid + last_mark;
    MeshDev mesh;
    mesh.v.reserve(size_t(nv) * sizeof(float3));
    mesh.i.reserve(size_t(ntri) * sizeof(uint3));
    mesh.nv = nv;
    mesh.ni = ntri;
    k_emit_mesh<<<grid_for(m), kThreads, 0, s>>>(pts.as<float3>(), head_orig.as<uint32_t>(),
                                                 run_of_orig.as<uint32_t>(), mark.as<uint32_t>(), vid.as<uint32_t>(), m,
                                                 mesh.v.as<float3>(), mesh.i.as<uint32_t>());
    RT_CHECK_LAUNCH();
    RT_CUDA(cudaStreamSynchronize(s));
    sc.meshes.push_back(std::move(mesh));
    *mesh_id = uint32_t(sc.meshes.size() - 1);
}

}  // namespace
}  // namespace rt

using namespace rt;

extern "C" {

rt_status rt_scene_create(rt_scene* out) {
    return guarded([&] {
        RT_REQUIRE(out != nullptr, "out is NULL");
        *out = reinterpret_cast<rt_scene>(new Scene());
    });
}

rt_status rt_scene_destroy(rt_scene scene) {
    return guarded([&] {
        SpareGeometry& sp = spare_geometry();
        if (!scene) {   // frees the arrays kept from the last destroyed scene
            sp.geo.reset();
            sp.dev = -1;
            return;
        }
        std::unique_ptr<Scene> sc(reinterpret_cast<Scene*>(scene));
        int dev = 0;
        // as cudaFree would, wait for every launch that may still read the arrays
        if (sc->geo.top.nodes.p && cudaGetDevice(&dev) == cudaSuccess && cudaDeviceSynchronize() == cudaSuccess) {
            sp.geo.reset();   // the previous spare's arrays are freed here
            sp.geo = std::make_unique<Geometry>(std::move(sc->geo));
            sp.dev = dev;
        }
    });
}

rt_status rt_scene_add_mesh(rt_scene scene, const rt_float3* vces, unsigned int nv, const rt_uint3* ices,
                            unsigned int ni, unsigned int* mesh_id) {
    return guarded([&] {
        Scene* sc = scene_from(scene);
        RT_REQUIRE(mesh_id != nullptr, "mesh_id is NULL");
        RT_REQUIRE(nv > 0 && ni > 0 && vces && ices, "mesh needs vertices and triangles");
        for (unsigned int k = 0; k < ni; ++k)
            RT_REQUIRE(ices[k].x < nv && ices[k].y < nv && ices[k].z < nv, "triangle index out of range");
        MeshDev m;
        m.v.reserve(size_t(nv) * sizeof(float3));
        m.i.reserve(size_t(ni) * sizeof(uint3));
        RT_CUDA(cudaMemcpy(m.v.p, vces, size_t(nv) * sizeof(float3), cudaMemcpyHostToDevice));
        RT_CUDA(cudaMemcpy(m.i.p, ices, size_t(ni) * sizeof(uint3), cudaMemcpyHostToDevice));
        m.nv = nv;
        m.ni = ni;
        sc->meshes.push_back(std::move(m));
        *mesh_id = unsigned(sc->meshes.size() - 1);
    });
}

rt_status rt_scene_add_sphere_mesh(rt_scene scene, float radius, unsigned int ndiv, unsigned int* mesh_id) {
    return guarded([&] {
        Scene* sc = scene_from(scene);
        RT_REQUIRE(mesh_id != nullptr, "mesh_id is NULL");
        tessellate(*sc, radius, ndiv, nullptr, mesh_id);
    });
}

rt_status rt_scene_get_mesh(rt_scene scene, unsigned int mesh_id, rt_float3* vces, unsigned int* nv, rt_uint3* ices,
                            unsigned int* ni) {
    return guarded([&] {
        Scene* sc = scene_from(scene);
        RT_REQUIRE(mesh_id < sc->meshes.size(), "bad mesh id");
        const MeshDev& m = sc->meshes[mesh_id];
        if (nv) *nv = m.nv;
        if (ni) *ni = m.ni;
        if (vces) RT_CUDA(cudaMemcpy(vces, m.v.p, size_t(m.nv) * sizeof(float3), cudaMemcpyDeviceToHost));
        if (ices) RT_CUDA(cudaMemcpy(ices, m.i.p, size_t(m.ni) * sizeof(uint3), cudaMemcpyDeviceToHost));
    });
}

rt_status rt_scene_add_thing(rt_scene scene, const rt_optics* optics, unsigned int mesh_id, const float transform[12],
                             unsigned int* thing_id) {
    return guarded([&] {
        Scene* sc = scene_from(scene);
        check_optics(optics);
        check_transform(transform);
        RT_REQUIRE(thing_id != nullptr, "thing_id is NULL");
        RT_REQUIRE(mesh_id < sc->meshes.size(), "bad mesh id");
        ThingHost th;
        th.optics = *optics;
        th.mesh = int(mesh_id);
        std::memcpy(th.T, transform, sizeof(th.T));
        sc->things.push_back(th);
        sc->topology_dirty = true;
        *thing_id = unsigned(sc->things.size() - 1);
    });
}

rt_status rt_scene_add_things(rt_scene scene, unsigned int n, const rt_optics* optics, const unsigned int* mesh_ids,
                              const float* transforms, unsigned int* first_id) {
    return guarded([&] {
        Scene* sc = scene_from(scene);
        RT_REQUIRE(first_id != nullptr, "first_id is NULL");
        RT_REQUIRE(n == 0 || (optics && mesh_ids && transforms), "optics/mesh_ids/transforms is NULL");
        for (unsigned k = 0; k < n; ++k) {
            check_optics(optics + k);
            check_transform(transforms + 12 * size_t(k));
            RT_REQUIRE(mesh_ids[k] < sc->meshes.size(), "bad mesh id");
        }
        *first_id = unsigned(sc->things.size());
        sc->things.reserve(sc->things.size() + n);
        for (unsigned k = 0; k < n; ++k) {
            ThingHost th;
            th.optics = optics[k];
            th.mesh = int(mesh_ids[k]);
            std::memcpy(th.T, transforms + 12 * size_t(k), sizeof(th.T));
            sc->things.push_back(th);
        }
        if (n) sc->topology_dirty = true;
    });
}

rt_status rt_scene_add_analytic_sphere(rt_scene scene, rt_float3 center, float radius, const rt_optics* optics,
                                       unsigned int* thing_id) {
    return guarded([&] {
        Scene* sc = scene_from(scene);
        check_optics(optics);
        RT_REQUIRE(thing_id != nullptr, "thing_id is NULL");
        RT_REQUIRE(std::isfinite(radius) && radius > 0.f, "radius must be positive");
        ThingHost th;
        th.optics = *optics;
        th.mesh = -1;
        th.center = make_float3(center.x, center.y, center.z);
        th.radius = radius;
        const float T[12] = {radius, 0, 0, center.x, 0, radius, 0, center.y, 0, 0, radius, center.z};
        std::memcpy(th.T, T, sizeof(T));
        sc->things.push_back(th);
        sc->topology_dirty = true;
        *thing_id = unsigned(sc->things.size() - 1);
    });
}

rt_status rt_scene_set_transform(rt_scene scene, unsigned int thing_id, const float transform[12]) {
    return guarded([&] {
        Scene* sc = scene_from(scene);
        RT_REQUIRE(thing_id < sc->things.size(), "bad thing id");
        check_transform(transform);
        ThingHost& th = sc->things[thing_id];
        std::memcpy(th.T, transform, sizeof(th.T));
        if (th.mesh < 0) {   // analytic sphere: translation and the x scale
            th.center = make_float3(transform[3], transform[7], transform[11]);
            th.radius = transform[0];
        }
        sc->xf_dirty = true;
    });
}

rt_status rt_scene_get_transform(rt_scene scene, unsigned int thing_id, float transform[12]) {
    return guarded([&] {
        Scene* sc = scene_from(scene);
        RT_REQUIRE(thing_id < sc->things.size(), "bad thing id");
        RT_REQUIRE(transform != nullptr, "transform is NULL");
        std::memcpy(transform, sc->things[thing_id].T, 12 * sizeof(float));
    });
}

rt_status rt_scene_set_optics(rt_scene scene, unsigned int thing_id, const rt_optics* optics) {
    return guarded([&] {
        Scene* sc = scene_from(scene);
        RT_REQUIRE(thing_id < sc->things.size(), "bad thing id");
        check_optics(optics);
        sc->things[thing_id].optics = *optics;
        sc->optics_version += 1;   // takes effect at the next launch, no refit
    });
}

rt_status rt_scene_set_layout(rt_scene scene, int layout) {
    return guarded([&] {
        RT_REQUIRE(layout >= RT_LAYOUT_AUTO && layout <= RT_LAYOUT_SAH, "unknown layout");
        Scene* sc = scene_from(scene);
        if (sc->layout != layout) sc->topology_dirty = true;
        sc->layout = layout;
    });
}

rt_status rt_scene_set_albedos(rt_scene scene, const float* albedo, void* stream) {
    return guarded([&] {
        Scene* sc = scene_from(scene);
        if (!sc->built || sc->topology_dirty) throw Error(RT_ERR_NOT_BUILT, "scene not built (call rt_scene_build)");
        set_albedos_device(sc->geo, {sc}, albedo, as_stream(stream));
    });
}

rt_status rt_scene_build(rt_scene scene, unsigned int morton_bits, void* stream) {
    return guarded([&] { scene_build(*scene_from(scene), int(morton_bits), as_stream(stream)); });
}

rt_status rt_scene_update(rt_scene scene, void* stream) {
    return guarded([&] { scene_update(*scene_from(scene), as_stream(stream)); });
}

rt_status rt_scene_info_get(rt_scene scene, rt_scene_info* info) {
    return guarded([&] {
        Scene* sc = scene_from(scene);
        RT_REQUIRE(info != nullptr, "info is NULL");
        info->n_meshes = unsigned(sc->meshes.size());
        info->n_things = unsigned(sc->things.size());
        info->n_prims = sc->geo.nprims;
        info->morton_bits = unsigned(sc->geo.morton_bits);
        info->device_bytes = sc->device_bytes();
        info->build_ms = sc->geo.build_ms;
        info->refit_ms = sc->geo.refit_ms;
        info->layout = unsigned(sc->geo.layout);
        info->n_instances = sc->geo.ninstances;
        info->n_top_records = sc->geo.top.nprims;
        info->n_bottom_records = sc->geo.blas.nprims;
    });
}

rt_status rt_scene_get_lbvh(rt_scene scene, unsigned long long* codes, unsigned int* ids, int* left, int* right,
                            float* boxes) {
    return guarded([&] {
        Scene* sc = scene_from(scene);
        if (!sc->built) throw Error(RT_ERR_NOT_BUILT, "scene not built");
        const Lbvh& g = sc->geo.top;
        const uint32_t n = g.nprims;
        if (n == 0) return;
        if (codes) {
            if (g.morton_bits == 30) {
                DevBuf tmp;
                tmp.reserve(size_t(n) * 8);
                k_lbvh_snapshot_codes32<<<grid_for(n), kThreads>>>(g.codes.as<uint32_t>(), n,
                                                                    tmp.as<unsigned long long>());
                RT_CHECK_LAUNCH();
                RT_CUDA(cudaMemcpy(codes, tmp.p, size_t(n) * 8, cudaMemcpyDeviceToHost));
            } else {
                RT_CUDA(cudaMemcpy(codes, g.codes.p, size_t(n) * 8, cudaMemcpyDeviceToHost));
            }
        }
        if (ids) RT_CUDA(cudaMemcpy(ids, g.ids.p, size_t(n) * 4, cudaMemcpyDeviceToHost));
        if (n < 2) return;
        std::vector<float4> nodes(size_t(n - 1) * 4);
        RT_CUDA(cudaMemcpy(nodes.data(), g.nodes.p, nodes.size() * sizeof(float4), cudaMemcpyDeviceToHost));
        for (uint32_t i = 0; i + 1 < n; ++i) {
            const float4 n0 = nodes[4 * i], n1 = nodes[4 * i + 1], n2 = nodes[4 * i + 2], n3 = nodes[4 * i + 3];
            int l, r;
            std::memcpy(&l, &n3.x, 4);
            std::memcpy(&r, &n3.y, 4);
            if (left) left[i] = l;
            if (right) right[i] = r;
            if (boxes) {
                float* o = boxes + 12 * size_t(i);
                o[0] = n0.x; o[1] = n0.z; o[2] = n2.x;   // lo0
                o[3] = n0.y; o[4] = n0.w; o[5] = n2.y;   // hi0
                o[6] = n1.x; o[7] = n1.z; o[8] = n2.z;   // lo1
                o[9] = n1.y; o[10] = n1.w; o[11] = n2.w; // hi1
            }
        }
    });
}

rt_status rt_radix_sort_pairs(void* keys, unsigned int* vals, unsigned int n, unsigned int key_bits, void* stream) {
    return guarded([&] {
        RT_REQUIRE(keys != nullptr && vals != nullptr, "keys/vals are NULL");
        RT_REQUIRE(key_bits >= 1 && key_bits <= 64, "key_bits must be 1..64");
        DevBuf tmp;
        cudaStream_t s = as_stream(stream);
        if (key_bits <= 32) radix_sort_pairs_u32(static_cast<uint32_t*>(keys), vals, n, int(key_bits), tmp, s);
        else radix_sort_pairs_u64(static_cast<unsigned long long*>(keys), vals, n, int(key_bits), tmp, s);
        RT_CUDA(cudaStreamSynchronize(s));
    });
}

}  // extern "C"
