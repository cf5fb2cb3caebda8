// rt_device.cuh -- device-side core of the GB300 path tracer.
//
// Vector maths in the operation order of optx/v.h:26-78, the counter RNG,
// the rejection samplers of optx/v.h:66-76, the primitive and node layouts in
// HBM and the closest-hit traversal shared by the first-hit and wavefront
// extend kernels.  Everything here is compiled with --fmad=false: products
// and sums are never fused behind the source's back, so results are the same
// bits as the binary32 CPU restatement of the same formulas.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "rt_api.h"

namespace rt {

// ------------------------------------------------------------------ vectors
__host__ __device__ __forceinline__ float3 mk(float x, float y, float z) { return make_float3(x, y, z); }
__host__ __device__ __forceinline__ float3 add(float3 a, float3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
__host__ __device__ __forceinline__ float3 sub(float3 a, float3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
__host__ __device__ __forceinline__ float3 neg(float3 a) { return mk(-a.x, -a.y, -a.z); }
__host__ __device__ __forceinline__ float3 mul(float s, float3 a) { return mk(s * a.x, s * a.y, s * a.z); }
__host__ __device__ __forceinline__ float3 mulv(float3 a, float3 b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }
__host__ __device__ __forceinline__ float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__host__ __device__ __forceinline__ float3 cross(float3 a, float3 b) {
    return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__host__ __device__ __forceinline__ float len(float3 v) { return sqrtf(dot(v, v)); }
// optx/v.h:576: unitV(v) = 1/len(v) * v
__host__ __device__ __forceinline__ float3 unitV(float3 v) { return mul(1.f / len(v), v); }
// optx/v.h:578 (kNear0 = 1e-8)
__host__ __device__ __forceinline__ bool near0(float3 v) {
    return fabsf(v.x) < 1e-8f && fabsf(v.y) < 1e-8f && fabsf(v.z) < 1e-8f;
}
__host__ __device__ __forceinline__ bool isnull(float3 v) { return v.x == 0.f && v.y == 0.f && v.z == 0.f; }
__host__ __device__ __forceinline__ float3 xyz(float4 a) { return mk(a.x, a.y, a.z); }

// ------------------------------------------------------------------ Philox
// Philox4x32-10 counter-based generator (Salmon, Moraes, Dror, Shaw, SC'11).
struct U4 {
    uint32_t x, y, z, w;
};

__device__ __forceinline__ U4 philox10(U4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        // one 32x32 -> 64-bit product per multiplier gives both halves
        const unsigned long long p0 = 0xD2511F53ull * c.x, p1 = 0xCD9E8D57ull * c.z;
        const uint32_t hi0 = uint32_t(p0 >> 32), lo0 = uint32_t(p0);
        const uint32_t hi1 = uint32_t(p1 >> 32), lo1 = uint32_t(p1);
        c = U4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return c;
}

// 24 high bits -> [0, 1), exact in binary32.
__host__ __device__ __forceinline__ float u01(uint32_t x) { return float(x >> 8) * (1.0f / 16777216.0f); }

// The draws of one bounce of one path: key = (seed, scene), counter =
// (pixel, sample, bounce, draw / 4); draw k is lane k % 4 of block k / 4.
// Bounce 0 is the camera (jitter and lens), bounce b >= 1 the scatter at the
// hit of the b-th ray.  Any path segment can be replayed from its ids alone.
struct Stream {
    uint32_t k0, k1, pixel, sample, bounce;
    uint32_t n;
    U4 buf;
    __device__ __forceinline__ Stream(uint32_t seed, uint32_t scene, uint32_t pix, uint32_t smp, uint32_t bnc)
        : k0(seed), k1(scene), pixel(pix), sample(smp), bounce(bnc), n(0), buf{0, 0, 0, 0} {}
    __device__ __forceinline__ float next() {
        const uint32_t lane = n & 3u;
        if (lane == 0) buf = philox10(U4{pixel, sample, bounce, n >> 2}, k0, k1);
        ++n;
        const uint32_t x = lane == 0 ? buf.x : lane == 1 ? buf.y : lane == 2 ? buf.z : buf.w;
        return u01(x);
    }
    // optx/util_gpu.h:28: rnd(min, max) = min + rnd * (max - min)
    __device__ __forceinline__ float next(float lo, float hi) { return lo + next() * (hi - lo); }
};

constexpr int kMaxRejections = 64;   // probability of reaching it < 1e-20

// optx/v.h:72: rejection sample of the unit ball; draws x, y, z in order.
__device__ __forceinline__ float3 rndVin1sphere(Stream& s) {
    for (int i = 0; i < kMaxRejections; ++i) {
        const float x = s.next(-1.f, 1.f);
        const float y = s.next(-1.f, 1.f);
        const float z = s.next(-1.f, 1.f);
        const float3 v = mk(x, y, z);
        if (1.f > dot(v, v)) return v;
    }
    return mk(0.f, 0.f, .5f);
}
// optx/v.h:73
__device__ __forceinline__ float3 rndVon1sphere(Stream& s) { return unitV(rndVin1sphere(s)); }
// optx/v.h:75: rejection sample of the unit disk; draws x then y.
__device__ __forceinline__ float3 rndVin1disk(Stream& s) {
    for (int i = 0; i < kMaxRejections; ++i) {
        const float x = s.next(-1.f, 1.f);
        const float y = s.next(-1.f, 1.f);
        const float3 v = mk(x, y, 0.f);
        if (1.f > dot(v, v)) return v;
    }
    return mk(0.f, 0.f, 0.f);
}

// ------------------------------------------------------------------ camera
struct CamDev {
    float3 eye, u, v, w, hvec, wvec, dvec;
    float aperture;
};

// optx/camera.h:67-77 with the pixel jitter of optx/camera_i.cu:61-65, or
// with rtow's mapping over w - 1 and h - 1 (rtow.cxx:112-113) when rtow_px.
__device__ __forceinline__ void camera_ray(const CamDev& c, uint32_t x, uint32_t y, uint32_t W, uint32_t H,
                                           bool rtow_px, Stream& s, float3& ori, float3& dir) {
    const float jx = s.next();
    const float jy = s.next();
    const float dw = rtow_px ? float(W - 1) : float(W);
    const float dh = rtow_px ? float(H - 1) : float(H);
    const float sx = 2.f * (float(x) + jx) / dw - 1.f;
    const float ty = 2.f * (float(y) + jy) / dh - 1.f;
    const float3 r = mul(c.aperture / 2.f, rndVin1disk(s));
    const float3 o = add(mul(r.x, c.u), mul(r.y, c.v));
    ori = add(c.eye, o);
    dir = sub(sub(add(mul(sx, c.wvec), mul(ty, c.hvec)), c.dvec), o);
}

// ------------------------------------------------------------------ layouts
// Primitive record, 48 bytes (three float4), in LBVH leaf order:
//   triangle (world):  a = (v0, thing id bits), b = (v1, prim id bits), c = (v2, 0)
//   sphere:            a = (centre, thing id bits), b = (radius, 0, 0, prim id bits), c = (0, 0, 0, 1)
//   instance (top):    a = (world box lo, thing id bits), b = (world box hi, -), c = (0, 0, 0, 2)
//   triangle (object, bottom level): a = (v0, local index bits), b = (v1, -), c = (v2, 0)
// `prim id` is the global id in thing-insertion order (the id parity tests and
// the picker report); a bottom-level triangle's global id is the instance's
// first primitive + its local index.
constexpr uint32_t kPrimTriangle = 0u;
constexpr uint32_t kPrimSphere = 1u;
constexpr uint32_t kPrimInstance = 2u;

// Internal node, 64 bytes (four float4), both child boxes held by the parent:
//   n0 = (c0.lo.x, c0.hi.x, c0.lo.y, c0.hi.y)
//   n1 = (c1.lo.x, c1.hi.x, c1.lo.y, c1.hi.y)
//   n2 = (c0.lo.z, c0.hi.z, c1.lo.z, c1.hi.z)
//   n3 = (child0 bits, child1 bits, 0, 0); child >= 0 internal node, < 0 leaf ~child
struct ThingDev {       // 48 bytes
    float4 albedo_type; // albedo.xyz, optics type (int bits)
    float4 center_fuzz; // instance centre (transform translation), fuzz
    float4 index_pad;   // refraction index, -, -, -
};

// Per-thing descriptor: where the thing's primitives come from (mesh arrays
// and transform, or an analytic sphere) and where they went in the two
// levels.  The build and every kernel that rebuilds a hit primitive's
// world-space record read it.
struct FlatDesc {
    const float3* v;
    const uint3* idx;
    uint32_t prim_offset;   // global first primitive (thing-insertion order)
    uint32_t nprims;
    int analytic;
    uint32_t seg;           // segment (scene) of the thing
    float T[12];            // 3x4 row-major object-to-world transform
    float4 sphere;          // centre, radius
    uint32_t top_offset;    // first top-level record of the thing
    uint32_t ntop;          // top-level records: 1 (sphere or instance) or nprims (flattened mesh)
    int instanced;          // 1: one instance record over a bottom-level hierarchy
    int blas_root;          // bottom-level root node (instanced only)
    uint32_t blas_seg;      // bottom-level segment of the thing's mesh (instanced only)
    uint32_t pad[3];
};

// Instance data of an instanced thing (diagonal transforms only): scale
// (sx, sy, sz), translation (tx, ty, tz), global first primitive, bottom root.
struct InstDev {
    float4 a;   // sx, sy, sz, tx
    float4 b;   // ty, tz, prim_offset (bits), blas_root (bits)
};

// Device view of a built geometry.
struct GeoView {
    const float4* tnodes;     // top level
    const float4* tprims;
    const float4* tedges;     // top level records for traversal: triangles as (A, B - A, C - A)
    const float4* bnodes;     // bottom level (instanced meshes, object space)
    const float4* bprims;
    const InstDev* inst;      // per thing
    const FlatDesc* desc;     // per thing
    int instanced;            // the top level has instance records
    // array lengths and the launch's error word, read by the bounds-checked
    // build only (RT_CHECKS)
    uint32_t ntnodes, ntprims, nbnodes, nbprims, nthings;
    uint32_t* err;
};

// Bounds-checked debug build (-DRT_CHECKS; compute-sanitizer is not
// available): every node, record, instance and thing index that traversal
// and shading take from memory is checked against its array.  A bad index
// sets kErrBounds in the launch's error word and ends the ray instead of
// reading out of bounds (no trap); the call then fails with RT_ERR_INTERNAL.
constexpr uint32_t kErrBounds = 4u;
#ifdef RT_CHECKS
__device__ __forceinline__ bool rt_in_bounds(bool ok, uint32_t* err) {
    if (!ok && err) atomicOr(err, kErrBounds);
    return ok;
}
#else
__device__ __forceinline__ bool rt_in_bounds(bool, uint32_t*) { return true; }
#endif

// Object-to-world transform of one vertex, in the reference's operation
// order (optx/optics_i.cu:46-62), row-major 3x4.
__host__ __device__ __forceinline__ float3 xform_point(const float* t, float3 a) {
    return mk(a.x * t[0] + a.y * t[1] + a.z * t[2] + t[3], a.x * t[4] + a.y * t[5] + a.z * t[6] + t[7],
              a.x * t[8] + a.y * t[9] + a.z * t[10] + t[11]);
}

// The same transform for a diagonal matrix whose off-diagonal entries are +0:
// the zero products are kept, so the result has the same bits as xform_point.
__device__ __forceinline__ float3 xform_diag(float3 sc, float3 tr, float3 a) {
    const float z = 0.f;
    return mk(a.x * sc.x + a.y * z + a.z * z + tr.x, a.x * z + a.y * sc.y + a.z * z + tr.y,
              a.x * z + a.y * z + a.z * sc.z + tr.z);
}

// World-space record of global primitive `id` of thing `thing`, bit for bit
// the record the flat layout stores (triangles transformed with
// xform_point; spheres from the descriptor).
__device__ __forceinline__ void world_prim(const FlatDesc* __restrict__ desc, uint32_t thing, uint32_t id,
                                           float4& a, float4& b, float4& c) {
    const FlatDesc& d = desc[thing];
    if (d.analytic) {
        a = make_float4(d.sphere.x, d.sphere.y, d.sphere.z, __uint_as_float(thing));
        b = make_float4(d.sphere.w, 0.f, 0.f, __uint_as_float(id));
        c = make_float4(0.f, 0.f, 0.f, __uint_as_float(kPrimSphere));
        return;
    }
    const uint3 tri = d.idx[id - d.prim_offset];
    float T[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) T[k] = d.T[k];
    const float3 A = xform_point(T, d.v[tri.x]), B = xform_point(T, d.v[tri.y]), C = xform_point(T, d.v[tri.z]);
    a = make_float4(A.x, A.y, A.z, __uint_as_float(thing));
    b = make_float4(B.x, B.y, B.z, __uint_as_float(id));
    c = make_float4(C.x, C.y, C.z, __uint_as_float(kPrimTriangle));
}

constexpr float kTmin = 1e-3f;   // optx/camera_i.cu:81
constexpr float kTmax = 1e16f;   // optx/camera_i.cu:82
// Conservative slab test: relative slack 2^-12 on the exit distance, so a
// box is never culled by rounding while a hit inside it is in range.  Every
// ancestor's box holds a record's own box (an exact union), and the rounded
// distances are monotone in the planes, so the closest hit is the closest over
// the records whose own box passes the test, whatever the hierarchy.  For
// triangles that is brute force over all records (tested).  A binary32 sphere
// root can lie outside the sphere's box: a ray leaving the r = 1000 ground
// sphere from 4e-5 inside it gets the exit root 1.04e-3 (the exact one, 6.9e-4,
// is below kTmin), a point above the box's top; the box test drops it, where
// brute force would take it (3 of 65,536 pixels of the final scene as spheres,
// 256x256 at 64 spp).  The oracle applies the same rule.
constexpr float kSlack = 1.f + 1.f / 4096.f;

__device__ __forceinline__ float safe_inv(float d) {
    const float dd = fabsf(d) < 1e-20f ? copysignf(1e-20f, d) : d;
    return 1.f / dd;
}

// Moller-Trumbore from a vertex and the two edges e1 = B - A, e2 = C - A
// (rounded differences of the vertices, so precomputed edges give the same
// bits), t >= tmin.
__device__ __forceinline__ bool tri_test_e(float3 A, float3 e1, float3 e2, float3 o, float3 d, float& t, float& u,
                                           float& v) {
    const float3 pv = cross(d, e2);
    const float det = dot(e1, pv);
    if (det == 0.f) return false;
    const float inv = 1.f / det;
    const float3 tv = sub(o, A);
    const float uu = dot(tv, pv) * inv;
    if (uu < 0.f || uu > 1.f) return false;
    const float3 qv = cross(tv, e1);
    const float vv = dot(d, qv) * inv;
    if (vv < 0.f || uu + vv > 1.f) return false;
    const float tt = dot(e2, qv) * inv;
    if (!(tt >= kTmin)) return false;
    t = tt;
    u = uu;
    v = vv;
    return true;
}

__device__ __forceinline__ bool tri_test(float3 A, float3 B, float3 C, float3 o, float3 d, float& t, float& u,
                                         float& v) {
    return tri_test_e(A, sub(B, A), sub(C, A), o, d, t, u, v);
}

// rtow's Sphere::hit (sphere.h:20-38) in binary32: nearest root in range.
__device__ __forceinline__ bool sph_test(float3 c, float r, float3 o, float3 d, float& t) {
    const float3 oc = sub(o, c);
    const float a = dot(d, d);
    const float b = dot(d, oc);
    const float cc = dot(oc, oc) - r * r;
    const float disc = b * b - a * cc;
    if (0.f > disc) return false;
    const float x = sqrtf(disc);
    float tt = (-b - x) / a;
    if (kTmin > tt || !(tt <= kTmax)) {
        tt = (-b + x) / a;
        if (kTmin > tt || !(tt <= kTmax)) return false;
    }
    t = tt;
    return true;
}

struct HitRec {
    float t, u, v;
    int hit;        // 1 on a hit, 0 on a miss
    uint32_t id;    // global primitive id of the hit
    uint32_t thing; // thing of the hit
    int leaf;       // top-level record of the hit, -1 for a bottom-level (instanced) triangle
    bool overflow;  // the traversal stack was full: a subtree was skipped
};

// The traversal stack lives in per-thread local memory (cached in L1).  A
// short stack in shared memory (the top 4, 8 or 16 entries of every thread in
// a ring, deeper ones spilled to local memory) measured 7 % slower on C1 at
// 64 spp (2139 / 2163 / 2164 against 2317 Mrays/s): the ring bookkeeping
// costs more issue slots and spills than the pops' local-memory latency.
// Keeping each pushed node's entry distance beside it (8-B entries) and
// skipping a popped node entered beyond the closest hit so far cut node
// visits by 7.5 % (37.1 -> 34.3 per ray, hits unchanged) but measured 10 %
// slower (2545 against 2841 Mrays/s): twice the stack traffic, more spills.
constexpr int kStackSize = 64;   // > the depth of the hierarchies in practice (50 at 8M flat triangles)
constexpr int kInstMarker = int(0x80000000u);   // stack entry: leave the current instance

// Traversal state of one ray: closest hit so far, current node, stack depth,
// and the instance being traversed (the stack itself is a separate
// per-thread array, so this state can stay in registers).
struct Trav {
    float3 o, d, inv;
    float best;
    HitRec h;
    int node;
    int sp;
    bool in_inst;            // the current node is a bottom-level node
    float3 isc, itr;         // instance scale, translation
    uint32_t ioff, ithing;   // instance first primitive, thing
};

__device__ __forceinline__ void trav_init(Trav& s, float3 o, float3 d, int root) {
    s.o = o;
    s.d = d;
    s.inv = mk(safe_inv(d.x), safe_inv(d.y), safe_inv(d.z));
    s.best = kTmax;
    s.h = HitRec{0.f, 0.f, 0.f, 0, 0u, 0u, -1, false};
    s.node = root;
    s.sp = 0;
    s.in_inst = false;
}

// Keeps a hit if it is the closest so far (smallest t, equal t -> larger
// primitive id).
__device__ __forceinline__ void trav_keep(Trav& s, float t, float u, float v, uint32_t id, uint32_t thing, int leaf) {
    if (t > s.best) return;
    if (!s.h.hit || t < s.h.t || (t == s.h.t && id > s.h.id)) {
        s.h.t = t; s.h.u = u; s.h.v = v; s.h.hit = 1; s.h.id = id; s.h.thing = thing; s.h.leaf = leaf;
        s.best = t;
    }
}

// Tests top-level primitive record li (a world-space triangle or a sphere).
template <bool kCount>
__device__ __forceinline__ void trav_leaf_top(Trav& s, const GeoView& g, int li, uint32_t& ntest) {
    if (kCount) ++ntest;
    if (!rt_in_bounds(uint32_t(li) < g.ntprims, g.err)) return;
    // the traversal form of the record: a triangle's edges come precomputed
    // (C1, 500 spp: traversal 350.7 -> 347.4 ms per frame)
    const float4 a = __ldg(g.tedges + 3 * li);
    const float4 b = __ldg(g.tedges + 3 * li + 1);
    const float4 c = __ldg(g.tedges + 3 * li + 2);
    float t, u, v;
    bool hit;
    if (__float_as_uint(c.w) == kPrimTriangle) {
        hit = tri_test_e(xyz(a), xyz(b), xyz(c), s.o, s.d, t, u, v);
    } else {
        u = v = 0.f;
        hit = sph_test(xyz(a), b.x, s.o, s.d, t);
    }
    if (hit) trav_keep(s, t, u, v, __float_as_uint(b.w), __float_as_uint(a.w), li);
}

// Tests bottom-level (object-space) triangle li of the current instance in
// world space: its vertices are transformed exactly as the flat layout
// transforms them, so the test is the flat layout's test bit for bit.
template <bool kCount>
__device__ __forceinline__ void trav_leaf_bottom(Trav& s, const GeoView& g, int li, uint32_t& ntest) {
    if (kCount) ++ntest;
    if (!rt_in_bounds(uint32_t(li) < g.nbprims, g.err)) return;
    const float4 a = __ldg(g.bprims + 3 * li);
    const float4 b = __ldg(g.bprims + 3 * li + 1);
    const float4 c = __ldg(g.bprims + 3 * li + 2);
    const float3 A = xform_diag(s.isc, s.itr, xyz(a));
    const float3 B = xform_diag(s.isc, s.itr, xyz(b));
    const float3 C = xform_diag(s.isc, s.itr, xyz(c));
    float t, u, v;
    if (tri_test(A, B, C, s.o, s.d, t, u, v)) trav_keep(s, t, u, v, s.ioff + __float_as_uint(a.w), s.ithing, -1);
}

// Enters instance record li of the top level: the stack gets a marker that
// leaves the instance when popped, traversal continues at the bottom root.
__device__ __forceinline__ void trav_enter(Trav& s, int* stack, const GeoView& g, int li) {
    const uint32_t thing = __float_as_uint(__ldg(g.tprims + 3 * li).w);
    if (!rt_in_bounds(uint32_t(li) < g.ntprims && thing < g.nthings, g.err)) {
        s.h.overflow = true;   // ends the traversal
        return;
    }
    const InstDev in = g.inst[thing];
    if (s.sp < kStackSize) stack[s.sp++] = kInstMarker;
    else { s.h.overflow = true; return; }
    s.in_inst = true;
    s.isc = mk(in.a.x, in.a.y, in.a.z);
    s.itr = mk(in.a.w, in.b.x, in.b.y);
    s.ioff = __float_as_uint(in.b.z);
    s.ithing = thing;
    s.node = __float_as_int(in.b.w);
}

// World slab of a bottom-level child box under the instance's diagonal
// transform: each bound goes through the same rounded operations as the
// vertices (fl(fl(s x) + t), monotone in x), so the slab holds the
// transformed triangles exactly.  A negative scale swaps the two bounds, which
// the slab test does not mind (it takes the min and max of both distances).
__device__ __forceinline__ void xbox(float lo, float hi, float sc, float tr, float& wlo, float& whi) {
    wlo = lo * sc + tr;
    whi = hi * sc + tr;
}

// One 64-B node slot as two 256-bit read-only loads (`ld.global.nc.v8.f32`,
// sm_100 and later) instead of four 128-bit ones: half the load instructions
// and L1 requests per step.  Node slots start at 64-B multiples of their own
// cudaMalloc allocation, so every half is 32-B aligned as the load requires.
// Measured on C1 at 64 spp: 2251 -> 2301 Mrays/s.  (Keeping the stack's top
// entry in a register, so that a pop's node fetch need not wait for a
// local-memory load, measured 1.5 % slower: 2291 against 2327, more spills
// at 48 registers.  With the wave queues evict-first, an L1 evict-last
// priority on node loads made no difference and an L2 evict-last cache
// policy cost 3 %.)
__device__ __forceinline__ void ld_node(const float4* p, float4& n0, float4& n1, float4& n2, float4& n3) {
    asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=f"(n0.x), "=f"(n0.y), "=f"(n0.z), "=f"(n0.w), "=f"(n1.x), "=f"(n1.y), "=f"(n1.z), "=f"(n1.w)
        : "l"(p));
    asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=f"(n2.x), "=f"(n2.y), "=f"(n2.z), "=f"(n2.w), "=f"(n3.x), "=f"(n3.y), "=f"(n3.z), "=f"(n3.w)
        : "l"(p + 2));
}

// Next node from the stack (markers leave instances, a negative top-level
// entry is an instance to enter).  Returns false when the stack is empty.
__device__ __forceinline__ bool trav_pop(Trav& s, int* stack, const GeoView& g) {
    while (true) {
        if (s.sp == 0) return false;
        const int v = stack[--s.sp];
        if (v == kInstMarker) {
            s.in_inst = false;
            continue;
        }
        if (!s.in_inst && v < 0) {
            trav_enter(s, stack, g, ~v);
            if (s.h.overflow) return false;
        } else {
            s.node = v;
        }
        return true;
    }
}

// One node of the traversal: both child boxes are tested; hit primitive
// leaves are tested at once, internal children (and, with kInst, instances)
// are descended near first (the far one is pushed).  Returns false when the
// ray is finished.  kInst = false is the flat layout's step (no instances, no
// transforms); kInst = true handles both levels.  The slab distances are
// (b - o) * (1/d): a fused fma(b, 1/d, -o/d) form needs an absolute slack that
// grows with |o/d| and measured 3x slower on the C1 scene (culling lost for
// rays with a near-zero direction component).  Kept per axis (widened
// per-ray offsets) and with three-input min/max, the fused form measured
// within 0.5 % of this one (C1, 64 spp) when held to 48 registers and slower
// at the 53 it takes otherwise: the step is latency-bound, not ALU-bound.
template <bool kCount, bool kInst>
__device__ __forceinline__ bool trav_step(Trav& s, int* stack, const GeoView& g, uint32_t& nvis, uint32_t& ntest) {
    if (kCount) ++nvis;
    const bool bottom = kInst && s.in_inst;
    const float4* nodes = bottom ? g.bnodes : g.tnodes;
    const int node = s.node;
    if (!rt_in_bounds(uint32_t(node) < (bottom ? g.nbnodes : g.ntnodes), g.err)) return false;
    float4 n0, n1, n2, n3;
    ld_node(nodes + 4 * node, n0, n1, n2, n3);
    if (bottom) {
        xbox(n0.x, n0.y, s.isc.x, s.itr.x, n0.x, n0.y);
        xbox(n0.z, n0.w, s.isc.y, s.itr.y, n0.z, n0.w);
        xbox(n1.x, n1.y, s.isc.x, s.itr.x, n1.x, n1.y);
        xbox(n1.z, n1.w, s.isc.y, s.itr.y, n1.z, n1.w);
        xbox(n2.x, n2.y, s.isc.z, s.itr.z, n2.x, n2.y);
        xbox(n2.z, n2.w, s.isc.z, s.itr.z, n2.z, n2.w);
    }
    const float3 o = s.o, inv = s.inv;
    // child 0
    float a0 = (n0.x - o.x) * inv.x, b0 = (n0.y - o.x) * inv.x;
    float a1 = (n0.z - o.y) * inv.y, b1 = (n0.w - o.y) * inv.y;
    float a2 = (n2.x - o.z) * inv.z, b2 = (n2.y - o.z) * inv.z;
    const float tn0 = fmaxf(fmaxf(fminf(a0, b0), fminf(a1, b1)), fmaxf(fminf(a2, b2), kTmin));
    const float tf0 = fminf(fminf(fmaxf(a0, b0), fmaxf(a1, b1)), fminf(fmaxf(a2, b2), s.best));
    // child 1
    a0 = (n1.x - o.x) * inv.x; b0 = (n1.y - o.x) * inv.x;
    a1 = (n1.z - o.y) * inv.y; b1 = (n1.w - o.y) * inv.y;
    a2 = (n2.z - o.z) * inv.z; b2 = (n2.w - o.z) * inv.z;
    const float tn1 = fmaxf(fmaxf(fminf(a0, b0), fminf(a1, b1)), fmaxf(fminf(a2, b2), kTmin));
    const float tf1 = fminf(fminf(fmaxf(a0, b0), fmaxf(a1, b1)), fminf(fmaxf(a2, b2), s.best));
    bool h0 = tn0 <= tf0 * kSlack;
    bool h1 = tn1 <= tf1 * kSlack;
    int c0 = __float_as_int(n3.x), c1 = __float_as_int(n3.y);
    uint32_t k0 = __float_as_uint(n3.z), k1 = __float_as_uint(n3.w);   // leaf kinds (written by the refit)
    if (h0 && h1 && tn1 < tn0) {
        const int tc = c0; c0 = c1; c1 = tc;
        const uint32_t tk = k0; k0 = k1; k1 = tk;
    }
    if (!h0 && h1) {   // only child 1 hit: treat it as the near child
        c0 = c1;
        k0 = k1;
        h0 = true;
        h1 = false;
    }
    // h0: c0 hit; h1: c1 hit too (c0 nearer).  Primitive leaves are tested
    // now; what stays hit is descended (an internal node, or an instance).
    // (One loop over both leaves, so that lanes with a near and lanes with a
    // far leaf share the test's code, measured 2 % slower on C1.)
    if (bottom) {
        if (h0 && c0 < 0) { trav_leaf_bottom<kCount>(s, g, ~c0, ntest); h0 = false; }
        if (h1 && c1 < 0) { trav_leaf_bottom<kCount>(s, g, ~c1, ntest); h1 = false; }
    } else {
        if (h0 && c0 < 0 && (!kInst || k0 != kPrimInstance)) { trav_leaf_top<kCount>(s, g, ~c0, ntest); h0 = false; }
        if (h1 && c1 < 0 && (!kInst || k1 != kPrimInstance)) { trav_leaf_top<kCount>(s, g, ~c1, ntest); h1 = false; }
    }
    if (h0 && h1) {
        if (s.sp < kStackSize) stack[s.sp++] = c1;   // a top-level instance stays negative (~record)
        else s.h.overflow = true;
    } else if (!h0 && h1) {
        c0 = c1;
        h0 = true;
    }
    if (h0) {
        if (!kInst || c0 >= 0) {
            s.node = c0;
        } else {   // only the top level has descendable leaves
            trav_enter(s, stack, g, ~c0);
            if (s.h.overflow) return false;
        }
        return true;
    }
    if (!kInst) {
        if (s.sp == 0) return false;
        s.node = stack[--s.sp];
        return true;
    }
    return trav_pop(s, stack, g);
}

// Closest hit below `root` for one ray (loop over trav_step); root < 0 is an
// empty scene.
template <bool kCount, bool kInst>
__device__ __forceinline__ HitRec closest_hit(const GeoView& g, int root, float3 o, float3 d, uint32_t& nvis,
                                              uint32_t& ntest) {
    Trav s;
    int stack[kStackSize];
    trav_init(s, o, d, root);
    if (root < 0) return s.h;
    while (trav_step<kCount, kInst>(s, stack, g, nvis, ntest)) {
    }
    return s.h;
}

// Dispatch on the geometry's layout (for kernels that serve both).
template <bool kCount>
__device__ __forceinline__ HitRec closest_hit_any(const GeoView& g, int root, float3 o, float3 d, uint32_t& nvis,
                                                  uint32_t& ntest) {
    if (g.instanced) return closest_hit<kCount, true>(g, root, o, d, nvis, ntest);
    return closest_hit<kCount, false>(g, root, o, d, nvis, ntest);
}

// Result of a scatter event at a hit (the closest-hit programs of
// optx/optics_i.cu:23-288): geometry, the outgoing direction and the random
// choices that fixed it (kept for the adjoint's path replay).
struct ScatterOut {
    float3 p, N;      // hit point, unit normal facing the incoming ray
    float3 dir;       // outgoing direction (when cont)
    float3 albedo;    // throughput factor: albedo, or (1,1,1) for glass
    float3 v;         // diffuse: unit random vector; metal: in-ball vector
    float ratio;      // glass: index ratio
    int type;         // optics type
    int branch;       // diffuse: 1 = near-zero fallback; glass: 0 reflect, 1 refract
    bool front;       // ray hits the outside
    bool cont;        // false: absorbed (metal below the surface)
    bool guide;       // diffuse and metal set the guide layers
};

// Geometry at a hit (optx/optics_i.cu:40-82 for triangles, sphere.h:40-46
// for spheres): hit point, unit normal facing the incoming ray, and whether
// the ray hits the outside (triangles: against the thing's centre,
// optx/optics_i.cu:259-267).  (pa, pb, pc) is the hit primitive's world-space
// record.
struct HitGeo {
    float3 p, N;
    bool front;
};

__device__ __forceinline__ HitGeo hit_geometry(float4 pa, float4 pb, float4 pc, float3 center, float3 o, float3 d,
                                               float t, float u, float v) {
    HitGeo g;
    if (__float_as_uint(pc.w) == kPrimTriangle) {
        const float3 A = xyz(pa), B = xyz(pb), C = xyz(pc);
        const float w = 1.f - u - v;
        g.p = add(add(mul(w, A), mul(u, B)), mul(v, C));
        float3 N = unitV(cross(sub(B, A), sub(C, A)));
        if (dot(d, N) > 0.f) N = neg(N);
        g.N = N;
        g.front = 0.f > dot(d, sub(g.p, center));
    } else {
        g.p = add(o, mul(t, d));
        const float3 outward = mul(1.f / pb.x, sub(g.p, xyz(pa)));
        g.front = 0.f > dot(d, outward);
        g.N = g.front ? outward : neg(outward);
    }
    return g;
}

// The Lambertian / fuzzy-metal / dielectric scatter at a hit of geometry g
// on a thing of optics th (optx/optics_i.cu:87-96, :168-190, :254-283;
// near-zero fallback of optics.h:17-18; Schlick's pow 5 as products).
__device__ __forceinline__ ScatterOut scatter_at(const HitGeo& g, const ThingDev& th, float3 d, Stream& s) {
    ScatterOut r;
    r.type = __float_as_int(th.albedo_type.w);
    r.albedo = xyz(th.albedo_type);
    r.branch = 0;
    r.ratio = 1.f;
    r.v = mk(0.f, 0.f, 0.f);
    r.cont = true;
    r.guide = r.type != RT_OPTICS_REFRACT;
    r.p = g.p;
    r.N = g.N;
    r.front = g.front;
    const float3 N = r.N;
    if (r.type == RT_OPTICS_DIFFUSE) {
        const float3 u = rndVon1sphere(s);
        float3 dir = add(N, u);
        r.v = u;
        if (near0(dir)) {
            dir = N;
            r.branch = 1;
        }
        r.dir = dir;
    } else if (r.type == RT_OPTICS_REFLECT) {
        const float3 d1V = unitV(d);
        const float3 refl = sub(d1V, mul(2.f * dot(d1V, N), N));
        const float3 v = rndVin1sphere(s);
        r.v = v;
        r.dir = add(refl, mul(th.center_fuzz.w, v));
        r.cont = dot(r.dir, N) > 0.f;
    } else {
        r.albedo = mk(1.f, 1.f, 1.f);
        const float3 d1V = unitV(d);
        const float cos_theta = fminf(dot(neg(d1V), N), 1.f);
        const float sin_theta = sqrtf(1.f - cos_theta * cos_theta);
        const float index = th.index_pad.x;
        const float ratio = r.front ? 1.f / index : index;
        r.ratio = ratio;
        const bool cannot = ratio * sin_theta > 1.f;
        float r0 = (1.f - ratio) / (1.f + ratio);
        r0 = r0 * r0;
        const float om = 1.f - cos_theta;
        const float pow5 = ((om * om) * (om * om)) * om;
        const float schlick = r0 + (1.f - r0) * pow5;
        if (cannot || schlick > s.next()) {
            r.dir = sub(d1V, mul(2.f * dot(d1V, N), N));
        } else {
            const float theta = fminf(dot(neg(d1V), N), 1.f);
            const float3 perpen = mul(ratio, add(d1V, mul(theta, N)));
            const float3 parall = mul(-sqrtf(fabsf(1.f - dot(perpen, perpen))), N);
            r.dir = add(perpen, parall);
            r.branch = 1;
        }
    }
    return r;
}

// Geometry and scatter of a hit on world-space record (pa, pb, pc); h4 = (t, u, v, -).
__device__ __forceinline__ ScatterOut scatter(float4 pa, float4 pb, float4 pc, const ThingDev* __restrict__ things,
                                              float3 o, float3 d, float4 h4, Stream& s) {
    const ThingDev th = things[__float_as_uint(pa.w)];
    const HitGeo g = hit_geometry(pa, pb, pc, xyz(th.center_fuzz), o, d, h4.x, h4.y, h4.z);
    return scatter_at(g, th, d, s);
}

// optx/camera_i.cu:133-139: sky gradient from white to ambient.
__device__ __forceinline__ float3 sky(float3 d, float3 ambient, float3 white) {
    const float3 unit = unitV(d);
    const float t = .5f * (unit.y + 1.f);
    return add(mul(1.f - t, white), mul(t, ambient));
}

}  // namespace rt
