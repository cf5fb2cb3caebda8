// CPU oracle for the GB300 path tracer -- TEST INFRASTRUCTURE ONLY.
//
// A plain C++ restatement of the reference's render path.  Only tests/,
// __graft_entry__.smoke() and bench.py's CPU-baseline leg use it, to check
// the product against; the product library never links or calls it.
//
// Parity is pinned by golden vectors made from the reference's own code
// (tests/golden/make_golden.py: optx/sphere.cxx tessellation bits, rtow.cxx
// scene list, glibc rand() stream) and by the published Philox4x32-10
// known-answer vectors.  The reference's OptiX traversal is closed and cannot
// run here, so closest-hit and image parity are defined by this restatement.
//
// Arithmetic: IEEE binary32, no FMA contraction (-ffp-contract=off), the same
// operation order as the CUDA kernels; per-pixel sample sums in 64-bit fixed
// point (see fx_add).  Pow-5 in Schlick's term is written as
// products (((x*x)*(x*x))*x) on both sides so CPU and GPU agree bit for bit.

#include "rt_oracle.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <map>
#include <numeric>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---------------------------------------------------------------- vectors --
// optx/v.h:26-78: float3 operators, evaluated left to right.
struct F3 {
    float x, y, z;
};
inline F3 mk(float x, float y, float z) { return F3{x, y, z}; }
inline F3 add(F3 a, F3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
inline F3 sub(F3 a, F3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
inline F3 neg(F3 a) { return mk(-a.x, -a.y, -a.z); }
inline F3 mul(float s, F3 a) { return mk(s * a.x, s * a.y, s * a.z); }
inline F3 mulv(F3 a, F3 b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }
inline float dot(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline F3 cross(F3 a, F3 b) {
    return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline float len(F3 v) { return sqrtf(dot(v, v)); }
// optx/v.h:576: unitV(v) = 1/len(v) * v
inline F3 unitV(F3 v) { return mul(1.f / len(v), v); }
// optx/v.h:578 / v.h:425 near-zero test with kNear0 = 1e-8
inline bool near0(F3 v) { return fabsf(v.x) < 1e-8f && fabsf(v.y) < 1e-8f && fabsf(v.z) < 1e-8f; }
inline bool isnull(F3 v) { return v.x == 0.f && v.y == 0.f && v.z == 0.f; }
inline F3 ld3(const float* p) { return mk(p[0], p[1], p[2]); }
inline void st3(float* p, F3 v) { p[0] = v.x; p[1] = v.y; p[2] = v.z; }

// ------------------------------------------------------------- Philox RNG --
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11).
constexpr uint32_t kPhiloxM0 = 0xD2511F53u, kPhiloxM1 = 0xCD9E8D57u;
constexpr uint32_t kPhiloxW0 = 0x9E3779B9u, kPhiloxW1 = 0xBB67AE85u;

inline void philox(const uint32_t in[4], const uint32_t k[2], uint32_t out[4]) {
    uint32_t c0 = in[0], c1 = in[1], c2 = in[2], c3 = in[3];
    uint32_t k0 = k[0], k1 = k[1];
    for (int r = 0; r < 10; ++r) {
        const uint64_t p0 = uint64_t(kPhiloxM0) * c0;
        const uint64_t p1 = uint64_t(kPhiloxM1) * c2;
        const uint32_t hi0 = uint32_t(p0 >> 32), lo0 = uint32_t(p0);
        const uint32_t hi1 = uint32_t(p1 >> 32), lo1 = uint32_t(p1);
        c0 = hi1 ^ c1 ^ k0;
        c1 = lo1;
        c2 = hi0 ^ c3 ^ k1;
        c3 = lo0;
        k0 += kPhiloxW0;
        k1 += kPhiloxW1;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

// 24 high bits -> [0,1): exact in binary32.
inline float u01(uint32_t x) { return float(x >> 8) * (1.0f / 16777216.0f); }

// Per-bounce draw stream: key = (seed, scene), counter = (pixel, sample,
// bounce, draw/4).  Draw k of a bounce is lane k%4 of block k/4.
struct Stream {
    uint32_t key[2];
    uint32_t ctr[4];
    uint32_t buf[4];
    uint32_t n = 0;
    Stream(uint32_t seed, uint32_t scene, uint32_t pixel, uint32_t sample, uint32_t bounce) {
        key[0] = seed; key[1] = scene;
        ctr[0] = pixel; ctr[1] = sample; ctr[2] = bounce; ctr[3] = 0;
    }
    float next() {
        if ((n & 3u) == 0) {
            ctr[3] = n >> 2;
            philox(ctr, key, buf);
        }
        return u01(buf[(n++) & 3u]);
    }
    // optx/util_gpu.h:28: rnd(min,max) = min + rnd*(max-min)
    float next(float lo, float hi) { return lo + next() * (hi - lo); }
};

constexpr int kMaxRejections = 64;

// optx/v.h:72 (rndVin1sphere), draws x, y, z in that order.
inline F3 rndVin1sphere(Stream& s) {
    for (int i = 0; i < kMaxRejections; ++i) {
        const float x = s.next(-1.f, 1.f);
        const float y = s.next(-1.f, 1.f);
        const float z = s.next(-1.f, 1.f);
        const F3 v = mk(x, y, z);
        if (1.f > dot(v, v)) return v;
    }
    return mk(0.f, 0.f, .5f);
}
// optx/v.h:73 (rndVon1sphere)
inline F3 rndVon1sphere(Stream& s) { return unitV(rndVin1sphere(s)); }
// optx/v.h:75 (rndVin1disk), draws x then y.
inline F3 rndVin1disk(Stream& s) {
    for (int i = 0; i < kMaxRejections; ++i) {
        const float x = s.next(-1.f, 1.f);
        const float y = s.next(-1.f, 1.f);
        const F3 v = mk(x, y, 0.f);
        if (1.f > dot(v, v)) return v;
    }
    return mk(0.f, 0.f, 0.f);
}

// ------------------------------------------------------ glibc rand() TYPE_3 --
// Additive feedback generator of glibc random_r(3) (degree 31, separation 3),
// seeded by the Park-Miller minimal standard LCG and warmed up by 310 draws.
struct GlibcRand {
    int32_t st[31];
    int fi = 3, ri = 0;
    explicit GlibcRand(uint32_t seed) {
        if (seed == 0) seed = 1;
        st[0] = int32_t(seed);
        for (int i = 1; i < 31; ++i) {
            // Schrage's method for 16807 * x mod (2^31 - 1)
            const int32_t hi = st[i - 1] / 127773;
            const int32_t lo = st[i - 1] % 127773;
            int32_t word = 16807 * lo - 2836 * hi;
            if (word < 0) word += 2147483647;
            st[i] = word;
        }
        fi = 3;
        ri = 0;
        for (int i = 0; i < 310; ++i) step();
    }
    uint32_t step() {
        st[fi] = int32_t(uint32_t(st[fi]) + uint32_t(st[ri]));
        const uint32_t result = uint32_t(st[fi]) >> 1;
        if (++fi >= 31) fi = 0;
        if (++ri >= 31) ri = 0;
        return result;
    }
    int32_t next() { return int32_t(step()); }
};

// ---------------------------------------------------------------- camera --
struct Cam {
    F3 eye, u, v, w, hvec, wvec, dvec;
    float aperture;
    bool rtow_px = false;   // rtow's pixel mapping (rtow.cxx:112-113)
};

// optx/camera.h:67-77 plus the jitter of optx/camera_i.cu:61-65; with
// rtow_px the jittered pixel maps over w - 1 and h - 1 as rtow.cxx:112-113.
inline void camera_ray(const Cam& c, unsigned x, unsigned y, unsigned W, unsigned H, Stream& s,
                       F3& ori, F3& dir) {
    const float jx = s.next();
    const float jy = s.next();
    const float dw = c.rtow_px ? float(W - 1) : float(W);
    const float dh = c.rtow_px ? float(H - 1) : float(H);
    const float sx = 2.f * (float(x) + jx) / dw - 1.f;
    const float ty = 2.f * (float(y) + jy) / dh - 1.f;
    const F3 r = mul(c.aperture / 2.f, rndVin1disk(s));
    const F3 o = add(mul(r.x, c.u), mul(r.y, c.v));
    ori = add(c.eye, o);
    dir = sub(sub(add(mul(sx, c.wvec), mul(ty, c.hvec)), c.dvec), o);
}

// ------------------------------------------------------------- primitives --
enum { OPT_DIFFUSE = 0, OPT_REFLECT = 1, OPT_REFRACT = 2 };

struct Thing {
    int type;       // optics type
    F3 albedo;
    float fuzz;
    float index;
    int mesh;       // -1: analytic sphere
    float T[12];    // 3x4 row-major object-to-world transform
    F3 center;      // analytic sphere centre
    float radius;   // analytic sphere radius
    uint32_t prim_offset = 0;
};

struct Mesh {
    std::vector<float> v;      // 3 per vertex
    std::vector<uint32_t> i;   // 3 per triangle
};

struct Prim {
    int kind;      // 0 triangle, 1 sphere
    F3 a, b, c;    // triangle vertices, or a = centre
    float r;       // sphere radius
    int thing;
    uint32_t id;   // global primitive id
};

constexpr float kTmin = 1e-3f;   // optx/camera_i.cu:81
constexpr float kTmax = 1e16f;   // optx/camera_i.cu:82

struct Hit {
    float t = 0.f, u = 0.f, v = 0.f;
    int prim = -1;   // index into prims (prim-id order)
};

// Moller-Trumbore, edges formed from the stored vertices.
inline bool tri_test(const Prim& p, F3 o, F3 d, float tmin, float& t, float& u, float& v) {
    const F3 e1 = sub(p.b, p.a);
    const F3 e2 = sub(p.c, p.a);
    const F3 pv = cross(d, e2);
    const float det = dot(e1, pv);
    if (det == 0.f) return false;
    const float inv = 1.f / det;
    const F3 tv = sub(o, p.a);
    const float uu = dot(tv, pv) * inv;
    if (uu < 0.f || uu > 1.f) return false;
    const F3 qv = cross(tv, e1);
    const float vv = dot(d, qv) * inv;
    if (vv < 0.f || uu + vv > 1.f) return false;
    const float tt = dot(e2, qv) * inv;
    if (!(tt >= tmin)) return false;
    t = tt; u = uu; v = vv;
    return true;
}

// sphere.h:20-38 in binary32: nearest root in range.
inline bool sph_test(const Prim& p, F3 o, F3 d, float tmin, float& t) {
    const F3 oc = sub(o, p.a);
    const float a = dot(d, d);
    const float b = dot(d, oc);
    const float c = dot(oc, oc) - p.r * p.r;
    const float disc = b * b - a * c;
    if (0.f > disc) return false;
    const float x = sqrtf(disc);
    float tt = (-b - x) / a;
    if (tmin > tt || !(tt <= kTmax)) {
        tt = (-b + x) / a;
        if (tmin > tt || !(tt <= kTmax)) return false;
    }
    t = tt;
    return true;
}

// Closest-hit rule: smallest t; equal t -> larger primitive id.
inline bool better(float t, uint32_t id, float bt, uint32_t bid, bool have) {
    if (!have) return true;
    return t < bt || (t == bt && id > bid);
}

// ------------------------------------------------------------------ LBVH --
inline uint32_t expand10(uint32_t x) {
    x = (x * 0x00010001u) & 0xFF0000FFu;
    x = (x * 0x00000101u) & 0x0F00F00Fu;
    x = (x * 0x00000011u) & 0xC30C30C3u;
    x = (x * 0x00000005u) & 0x49249249u;
    return x;
}

inline uint32_t quant10(float c, float lo, float ext) {
    const float f = ext > 0.f ? (c - lo) / ext : 0.f;
    float q = f * 1024.f;
    q = q < 0.f ? 0.f : (q > 1023.f ? 1023.f : q);
    return uint32_t(q);
}

inline int clz32(uint32_t x) { return x == 0 ? 32 : __builtin_clz(x); }
inline int clz64(uint64_t x) { return x == 0 ? 64 : __builtin_clzll(x); }

// 20-bit spread into every third bit of a 60-bit code.
inline uint64_t expand20(uint64_t x) {
    x &= 0xFFFFFull;
    x = (x | x << 32) & 0x001F00000000FFFFull;
    x = (x | x << 16) & 0x001F0000FF0000FFull;
    x = (x | x << 8) & 0x100F00F00F00F00Full;
    x = (x | x << 4) & 0x10C30C30C30C30C3ull;
    x = (x | x << 2) & 0x1249249249249249ull;
    return x;
}

inline uint64_t quant20(float c, float lo, float ext) {
    const float f = ext > 0.f ? (c - lo) / ext : 0.f;
    float q = f * 1048576.f;
    q = q < 0.f ? 0.f : (q > 1048575.f ? 1048575.f : q);
    return uint64_t(q);
}

// Karras 2012 delta over 64-bit keys; equal keys fall back to the index bits
// (64 + clz(i^j) is above every key-derived value, also for 30-bit codes).
inline int kdelta(const uint64_t* k, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    const uint64_t a = k[i], b = k[j];
    if (a != b) return clz64(a ^ b);
    return 64 + clz32(uint32_t(i) ^ uint32_t(j));
}

void karras(const uint64_t* k, int n, int32_t* left, int32_t* right) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n - 1; ++i) {
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
        const int lo = i < j ? i : j, hi = i < j ? j : i;
        left[i] = (lo == gamma) ? ~gamma : gamma;
        right[i] = (hi == gamma + 1) ? ~(gamma + 1) : gamma + 1;
    }
}

struct Box {
    F3 lo, hi;
};
inline Box prim_box(const Prim& p) {
    if (p.kind == 0) {
        return Box{mk(fminf(fminf(p.a.x, p.b.x), p.c.x), fminf(fminf(p.a.y, p.b.y), p.c.y),
                      fminf(fminf(p.a.z, p.b.z), p.c.z)),
                   mk(fmaxf(fmaxf(p.a.x, p.b.x), p.c.x), fmaxf(fmaxf(p.a.y, p.b.y), p.c.y),
                      fmaxf(fmaxf(p.a.z, p.b.z), p.c.z))};
    }
    return Box{mk(p.a.x - p.r, p.a.y - p.r, p.a.z - p.r), mk(p.a.x + p.r, p.a.y + p.r, p.a.z + p.r)};
}
inline Box unite(const Box& a, const Box& b) {
    return Box{mk(fminf(a.lo.x, b.lo.x), fminf(a.lo.y, b.lo.y), fminf(a.lo.z, b.lo.z)),
               mk(fmaxf(a.hi.x, b.hi.x), fmaxf(a.hi.y, b.hi.y), fmaxf(a.hi.z, b.hi.z))};
}

// Conservative slab test: relative slack 2^-12 so a box is never culled by
// rounding while a hit inside it is in range.  Ancestor boxes hold a record's
// own box, so the closest hit is the closest over the records whose own box
// passes the test, for any hierarchy: brute force for triangles; a binary32
// sphere root outside the sphere's box (a ray leaving the r = 1000 ground
// sphere from just inside it) is dropped, as the product drops it.
constexpr float kSlack = 1.f + 1.f / 4096.f;
inline bool slab(const Box& b, F3 o, F3 inv, float tmin, float tmax, float& tnear) {
    const float tx0 = (b.lo.x - o.x) * inv.x, tx1 = (b.hi.x - o.x) * inv.x;
    const float ty0 = (b.lo.y - o.y) * inv.y, ty1 = (b.hi.y - o.y) * inv.y;
    const float tz0 = (b.lo.z - o.z) * inv.z, tz1 = (b.hi.z - o.z) * inv.z;
    const float tn = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fmaxf(fminf(tz0, tz1), tmin));
    const float tf = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fminf(fmaxf(tz0, tz1), tmax));
    tnear = tn;
    return tn <= tf * kSlack;
}
inline float safe_inv(float d) {
    const float dd = fabsf(d) < 1e-20f ? copysignf(1e-20f, d) : d;
    return 1.f / dd;
}

}  // namespace

// ================================================================ world ====
struct orc_world {
    std::vector<Mesh> meshes;
    std::vector<Thing> things;
    std::vector<Prim> prims;           // prim-id order
    // LBVH
    std::vector<uint64_t> codes;         // sorted Morton codes
    std::vector<uint32_t> order;         // sorted prim ids
    int morton_bits = 60;
    bool grouped = false;                // things-grouped keys (rank of the thing, then a code inside it)
    unsigned sah_cluster = 0;            // > 0: binned-SAH hierarchy with clusters of at most this many records
    std::vector<int32_t> left, right;
    std::vector<Box> cbox0, cbox1;       // per internal node: child boxes
    F3 clo{0, 0, 0}, chi{0, 0, 0};
    int32_t root = 0;                    // ~0 when a single leaf
    bool built = false;
};

namespace {

void flatten(orc_world& w) {
    w.prims.clear();
    for (size_t k = 0; k < w.things.size(); ++k) {
        Thing& th = w.things[k];
        th.prim_offset = uint32_t(w.prims.size());
        if (th.mesh < 0) {
            Prim p{};
            p.kind = 1; p.a = th.center; p.r = th.radius; p.thing = int(k);
            p.id = uint32_t(w.prims.size());
            w.prims.push_back(p);
            continue;
        }
        const Mesh& m = w.meshes[th.mesh];
        const float* t = th.T;
        auto xf = [&](uint32_t vi) {
            const float ax = m.v[3 * vi], ay = m.v[3 * vi + 1], az = m.v[3 * vi + 2];
            // optx/optics_i.cu:46-62: object-to-world transform, left to right
            return mk(ax * t[0] + ay * t[1] + az * t[2] + t[3],
                      ax * t[4] + ay * t[5] + az * t[6] + t[7],
                      ax * t[8] + ay * t[9] + az * t[10] + t[11]);
        };
        const size_t nt = m.i.size() / 3;
        for (size_t i = 0; i < nt; ++i) {
            Prim p{};
            p.kind = 0;
            p.a = xf(m.i[3 * i]); p.b = xf(m.i[3 * i + 1]); p.c = xf(m.i[3 * i + 2]);
            p.thing = int(k);
            p.id = uint32_t(w.prims.size());
            w.prims.push_back(p);
        }
    }
}

void build_lbvh_topology(orc_world& w, const std::vector<Box>& pb, const std::vector<F3>& cen, F3 lo, F3 hi);
void refit_tree(orc_world& w, const std::vector<Box>& pb);

// ---- binned-SAH hierarchy (the product's RT_LAYOUT_SAH, rt_sah.cu) --------
// Top-down over record positions: a node of more than cluster_max records is
// binned (32 bins per axis over its centroid bounds: bin = int((c - lo) *
// (32 / extent)) clamped to [0, 31]), split at the border of least cost
// A(left) * n(left) + A(right) * n(right) (A = 2 (dx dy + dy dz + dz dx);
// ties: the lower axis, then the lower border; no border with records on
// both sides, or depth >= 64: the median position) and partitioned stably.
// Smaller nodes are clusters: keys cluster << 30 | 30-bit Morton code inside
// the cluster's centroid bounds, a Karras hierarchy per cluster, and each
// split node in slot split - 1 (the spare slot of the cluster ending there).
constexpr int kSahBins = 32;
constexpr int kSahMaxLevels = 64;

inline float sah_area(const Box& b) {
    const float dx = fmaxf(b.hi.x - b.lo.x, 0.f), dy = fmaxf(b.hi.y - b.lo.y, 0.f), dz = fmaxf(b.hi.z - b.lo.z, 0.f);
    return 2.f * (dx * dy + dy * dz + dz * dx);
}

inline int sah_bin(float c, float lo, float scale) {
    const float f = (c - lo) * scale;
    if (!(f > 0.f)) return 0;
    if (f >= float(kSahBins)) return kSahBins - 1;
    return int(f);
}

struct SahBuild {
    const std::vector<Box>& pb;
    const std::vector<F3>& cen;
    std::vector<uint32_t> perm;          // record ids by position
    unsigned cluster_max;
    struct Split { int start, split, end, child[2]; };
    struct Cluster { int start, count; F3 lo, hi; };
    std::vector<Split> splits;
    std::vector<Cluster> clusters;

    void bounds(int b, int e, F3& lo, F3& hi) const {
        const float inf = std::numeric_limits<float>::infinity();
        lo = mk(inf, inf, inf);
        hi = mk(-inf, -inf, -inf);
        for (int i = b; i < e; ++i) {
            const F3 c = cen[perm[i]];
            lo = mk(fminf(lo.x, c.x), fminf(lo.y, c.y), fminf(lo.z, c.z));
            hi = mk(fmaxf(hi.x, c.x), fmaxf(hi.y, c.y), fmaxf(hi.z, c.z));
        }
    }

    // Returns the child reference of node [b, b + count): split index (>= 0)
    // or ~cluster index.
    int node(int b, int count, int level) {
        F3 lo, hi;
        bounds(b, b + count, lo, hi);
        if (unsigned(count) <= cluster_max) {
            clusters.push_back(Cluster{b, count, lo, hi});
            return ~int(clusters.size() - 1);
        }
        const float clo[3] = {lo.x, lo.y, lo.z}, chi[3] = {hi.x, hi.y, hi.z};
        float scale[3];
        for (int a = 0; a < 3; ++a) {
            const float ext = chi[a] - clo[a];
            scale[a] = ext > 0.f ? float(kSahBins) / ext : 0.f;
        }
        int axis = -1, border = 0, nleft = count / 2;
        if (level < kSahMaxLevels) {
            float best = std::numeric_limits<float>::infinity();
            const float inf = std::numeric_limits<float>::infinity();
            for (int a = 0; a < 3; ++a) {
                Box bb[kSahBins];
                int cnt[kSahBins] = {};
                for (int k = 0; k < kSahBins; ++k) bb[k] = Box{mk(inf, inf, inf), mk(-inf, -inf, -inf)};
                for (int i = b; i < b + count; ++i) {
                    const uint32_t r = perm[i];
                    const float c = a == 0 ? cen[r].x : a == 1 ? cen[r].y : cen[r].z;
                    const int k = sah_bin(c, clo[a], scale[a]);
                    bb[k] = unite(bb[k], pb[r]);
                    cnt[k] += 1;
                }
                Box pre[kSahBins], suf[kSahBins];
                int pc[kSahBins], sc[kSahBins];
                for (int k = 0; k < kSahBins; ++k) {
                    pre[k] = k ? unite(pre[k - 1], bb[k]) : bb[k];
                    pc[k] = (k ? pc[k - 1] : 0) + cnt[k];
                }
                for (int k = kSahBins - 1; k >= 0; --k) {
                    suf[k] = k + 1 < kSahBins ? unite(suf[k + 1], bb[k]) : bb[k];
                    sc[k] = (k + 1 < kSahBins ? sc[k + 1] : 0) + cnt[k];
                }
                for (int k = 0; k + 1 < kSahBins; ++k) {   // border k + 1
                    if (pc[k] == 0 || sc[k + 1] == 0) continue;
                    const float cost = sah_area(pre[k]) * float(pc[k]) + sah_area(suf[k + 1]) * float(sc[k + 1]);
                    if (cost < best) {
                        best = cost;
                        axis = a;
                        border = k + 1;
                        nleft = pc[k];
                    }
                }
            }
        }
        if (axis >= 0) {   // stable partition by bin < border
            std::vector<uint32_t> L, R;
            for (int i = b; i < b + count; ++i) {
                const uint32_t r = perm[i];
                const float c = axis == 0 ? cen[r].x : axis == 1 ? cen[r].y : cen[r].z;
                (sah_bin(c, clo[axis], scale[axis]) < border ? L : R).push_back(r);
            }
            std::copy(L.begin(), L.end(), perm.begin() + b);
            std::copy(R.begin(), R.end(), perm.begin() + b + int(L.size()));
        }
        const int id = int(splits.size());
        splits.push_back(Split{b, b + nleft, b + count, {0, 0}});
        const int c0 = node(b, nleft, level + 1);
        const int c1 = node(b + nleft, count - nleft, level + 1);
        splits[id].child[0] = c0;
        splits[id].child[1] = c1;
        return id;
    }
};

void build_sah(orc_world& w, const std::vector<Box>& pb, const std::vector<F3>& cen) {
    const int n = int(pb.size());
    SahBuild sb{pb, cen, {}, w.sah_cluster, {}, {}};
    sb.perm.resize(n);
    std::iota(sb.perm.begin(), sb.perm.end(), 0u);
    const int top = n ? sb.node(0, n, 0) : ~0;
    // clusters in position order; keys cluster << 30 | local Morton code; stable sort
    std::vector<int> rank(sb.clusters.size());
    std::vector<int> by_pos(sb.clusters.size());
    std::iota(by_pos.begin(), by_pos.end(), 0);
    std::sort(by_pos.begin(), by_pos.end(), [&](int x, int y) { return sb.clusters[x].start < sb.clusters[y].start; });
    for (size_t r = 0; r < by_pos.size(); ++r) rank[by_pos[r]] = int(r);
    std::vector<uint64_t> code(n);
    std::vector<uint32_t> ids(n);
    for (const auto& c : sb.clusters) {
        const F3 e = sub(c.hi, c.lo);
        const int r = rank[&c - &sb.clusters[0]];
        for (int i = c.start; i < c.start + c.count; ++i) {
            const F3 q = cen[sb.perm[i]];
            const uint32_t qx = quant10(q.x, c.lo.x, e.x), qy = quant10(q.y, c.lo.y, e.y), qz = quant10(q.z, c.lo.z, e.z);
            code[i] = (uint64_t(r) << 30) | ((expand10(qx) << 2) | (expand10(qy) << 1) | expand10(qz));
            ids[i] = sb.perm[i];
        }
    }
    orc_stable_sort_pairs64(code.data(), ids.data(), unsigned(n));
    w.codes = code;
    w.order = ids;
    w.left.assign(n > 1 ? n - 1 : 0, 0);
    w.right.assign(n > 1 ? n - 1 : 0, 0);
    std::vector<int32_t> L, R;
    for (const auto& c : sb.clusters) {   // Karras per cluster, slots start + i
        if (c.count < 2) continue;
        L.assign(c.count - 1, 0);
        R.assign(c.count - 1, 0);
        karras(code.data() + c.start, c.count, L.data(), R.data());
        auto g = [&](int32_t x) { return x >= 0 ? c.start + x : ~(c.start + ~x); };
        for (int i = 0; i < c.count - 1; ++i) {
            w.left[c.start + i] = g(L[i]);
            w.right[c.start + i] = g(R[i]);
        }
    }
    auto ref = [&](int x) {   // split -> its slot; cluster -> its root slot, or its single record
        if (x >= 0) return sb.splits[x].split - 1;
        const auto& c = sb.clusters[~x];
        return c.count >= 2 ? c.start : ~c.start;
    };
    for (const auto& sp : sb.splits) {
        w.left[sp.split - 1] = ref(sp.child[0]);
        w.right[sp.split - 1] = ref(sp.child[1]);
    }
    w.root = n > 1 ? ref(top) : ~0;
}

void build_lbvh(orc_world& w) {
    const int n = int(w.prims.size());
    std::vector<Box> pb(n);
    std::vector<F3> cen(n);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        pb[i] = prim_box(w.prims[i]);
        cen[i] = mul(0.5f, add(pb[i].lo, pb[i].hi));
    }
    F3 lo = cen.empty() ? mk(0, 0, 0) : cen[0], hi = lo;
    for (int i = 0; i < n; ++i) {
        lo = mk(fminf(lo.x, cen[i].x), fminf(lo.y, cen[i].y), fminf(lo.z, cen[i].z));
        hi = mk(fmaxf(hi.x, cen[i].x), fmaxf(hi.y, cen[i].y), fmaxf(hi.z, cen[i].z));
    }
    w.clo = lo; w.chi = hi;
    if (w.sah_cluster > 0) {
        build_sah(w, pb, cen);
    } else {
        build_lbvh_topology(w, pb, cen, lo, hi);
    }
    refit_tree(w, pb);
    w.built = true;
}

void build_lbvh_topology(orc_world& w, const std::vector<Box>& pb, const std::vector<F3>& cen, F3 lo, F3 hi) {
    const int n = int(pb.size());
    std::vector<uint64_t> code(n);
    std::vector<uint32_t> ids(n);
    const float lo3[3] = {lo.x, lo.y, lo.z}, hi3[3] = {hi.x, hi.y, hi.z};
    // things-grouped hierarchy (see below): per-thing centroid bounds
    const size_t nt = w.things.size();
    std::vector<F3> tlo, thi;
    if (w.grouped) {
        const float inf = std::numeric_limits<float>::infinity();
        tlo.assign(nt, mk(inf, inf, inf));
        thi.assign(nt, mk(-inf, -inf, -inf));
        for (int i = 0; i < n; ++i) {
            const int t = w.prims[i].thing;
            tlo[t] = mk(fminf(tlo[t].x, cen[i].x), fminf(tlo[t].y, cen[i].y), fminf(tlo[t].z, cen[i].z));
            thi[t] = mk(fmaxf(thi[t].x, cen[i].x), fmaxf(thi[t].y, cen[i].y), fmaxf(thi[t].z, cen[i].z));
        }
        // key = thing << 30 | 30-bit Morton code inside the thing's centroid bounds
        for (int i = 0; i < n; ++i) {
            const int t = w.prims[i].thing;
            const F3 e = sub(thi[t], tlo[t]);
            const uint32_t qx = quant10(cen[i].x, tlo[t].x, e.x);
            const uint32_t qy = quant10(cen[i].y, tlo[t].y, e.y);
            const uint32_t qz = quant10(cen[i].z, tlo[t].z, e.z);
            code[i] = (uint64_t(t) << 30) | ((expand10(qx) << 2) | (expand10(qy) << 1) | expand10(qz));
        }
    } else if (w.morton_bits == 30) {
        std::vector<uint32_t> c32(n);
        orc_morton30(&cen[0].x, unsigned(n), lo3, hi3, c32.data());
        for (int i = 0; i < n; ++i) code[i] = c32[i];
    } else {
        orc_morton60(&cen[0].x, unsigned(n), lo3, hi3, code.data());
    }
    std::iota(ids.begin(), ids.end(), 0u);
    orc_stable_sort_pairs64(code.data(), ids.data(), unsigned(n));
    w.codes = code;
    w.order = ids;
    w.left.assign(n > 1 ? n - 1 : 0, 0);
    w.right.assign(n > 1 ? n - 1 : 0, 0);
    if (n > 1 && !w.grouped) karras(code.data(), n, w.left.data(), w.right.data());
    w.root = n > 1 ? 0 : ~0;
    if (n > 1 && w.grouped) {
        // Things-grouped hierarchy: a Karras hierarchy per thing over its keys
        // (node slots b + i of a thing whose records start at b), then one over
        // the things sorted by a 60-bit code of their centroid-bounds centre;
        // internal node j of the thing tree lives in the spare slot of thing j
        // (b_j + n_j - 1), a thing leaf points at the thing's subtree root (or
        // its single record).
        std::vector<uint32_t> tb(nt), tn(nt, 0);
        for (size_t t = 0; t < nt; ++t) tb[t] = w.things[t].prim_offset;
        for (int i = 0; i < n; ++i) tn[w.prims[i].thing] += 1;
        std::vector<int32_t> L, R;
        for (size_t t = 0; t < nt; ++t) {
            const int m = int(tn[t]);
            if (m < 2) continue;
            L.assign(m - 1, 0);
            R.assign(m - 1, 0);
            karras(code.data() + tb[t], m, L.data(), R.data());
            const int b0 = int(tb[t]);
            auto g = [&](int32_t x) { return x >= 0 ? b0 + x : ~(b0 + ~x); };
            for (int i = 0; i < m - 1; ++i) {
                w.left[b0 + i] = g(L[i]);
                w.right[b0 + i] = g(R[i]);
            }
        }
        if (nt == 1) {
            w.root = 0;   // n > 1 records of the one thing
        } else {
            std::vector<float> tc(3 * nt);
            for (size_t t = 0; t < nt; ++t) st3(&tc[3 * t], mul(0.5f, add(tlo[t], thi[t])));
            std::vector<uint64_t> tcode(nt);
            std::vector<uint32_t> tsorted(nt);
            orc_morton60(tc.data(), unsigned(nt), lo3, hi3, tcode.data());
            std::iota(tsorted.begin(), tsorted.end(), 0u);
            orc_stable_sort_pairs64(tcode.data(), tsorted.data(), unsigned(nt));
            L.assign(nt - 1, 0);
            R.assign(nt - 1, 0);
            karras(tcode.data(), int(nt), L.data(), R.data());
            auto spare = [&](size_t t) { return int(tb[t] + tn[t]) - 1; };
            auto ref = [&](int32_t x) {
                if (x >= 0) return spare(size_t(x));
                const uint32_t t = tsorted[~x];
                return tn[t] >= 2 ? int(tb[t]) : ~int(tb[t]);
            };
            for (size_t j = 0; j + 1 < nt; ++j) {
                w.left[spare(j)] = ref(L[j]);
                w.right[spare(j)] = ref(R[j]);
            }
            w.root = spare(0);
        }
    }
}

// Bottom-up refit of the child boxes (post order, iterative).
void refit_tree(orc_world& w, const std::vector<Box>& pb) {
    const int n = int(pb.size());
    w.cbox0.assign(n > 1 ? n - 1 : 0, Box{});
    w.cbox1.assign(n > 1 ? n - 1 : 0, Box{});
    if (n > 1) {
        std::vector<Box> nb(n - 1);
        std::vector<int> parent(n - 1, -1);
        for (int i = 0; i < n - 1; ++i) {
            if (w.left[i] >= 0) parent[w.left[i]] = i;
            if (w.right[i] >= 0) parent[w.right[i]] = i;
        }
        // children of a Karras node always have larger or smaller index ranges;
        // a DFS post-order is the safe order.
        std::vector<int> stack{w.root}, post;
        post.reserve(n - 1);
        while (!stack.empty()) {
            const int i = stack.back();
            stack.pop_back();
            post.push_back(i);
            if (w.left[i] >= 0) stack.push_back(w.left[i]);
            if (w.right[i] >= 0) stack.push_back(w.right[i]);
        }
        for (auto it = post.rbegin(); it != post.rend(); ++it) {
            const int i = *it;
            const Box b0 = w.left[i] >= 0 ? nb[w.left[i]] : pb[w.order[~w.left[i]]];
            const Box b1 = w.right[i] >= 0 ? nb[w.right[i]] : pb[w.order[~w.right[i]]];
            w.cbox0[i] = b0;
            w.cbox1[i] = b1;
            nb[i] = unite(b0, b1);
        }
    }
}

inline bool prim_hit(const Prim& p, F3 o, F3 d, float& t, float& u, float& v) {
    if (p.kind == 0) return tri_test(p, o, d, kTmin, t, u, v);
    u = v = 0.f;
    return sph_test(p, o, d, kTmin, t);
}

Hit closest_brute(const orc_world& w, F3 o, F3 d) {
    Hit h;
    bool have = false;
    for (size_t i = 0; i < w.prims.size(); ++i) {
        float t, u, v;
        if (!prim_hit(w.prims[i], o, d, t, u, v) || t > kTmax) continue;
        if (better(t, w.prims[i].id, h.t, have ? w.prims[h.prim].id : 0, have)) {
            h.t = t; h.u = u; h.v = v; h.prim = int(i); have = true;
        }
    }
    return h;
}

Hit closest_bvh(const orc_world& w, F3 o, F3 d) {
    Hit h;
    bool have = false;
    float best = kTmax;
    const F3 inv = mk(safe_inv(d.x), safe_inv(d.y), safe_inv(d.z));
    auto leaf = [&](int li) {
        const Prim& p = w.prims[w.order[li]];
        float t, u, v;
        if (!prim_hit(p, o, d, t, u, v) || t > best) return;
        if (better(t, p.id, h.t, have ? w.prims[h.prim].id : 0, have)) {
            h.t = t; h.u = u; h.v = v; h.prim = int(p.id); have = true; best = t;
        }
    };
    if (w.prims.empty()) return h;
    if (w.root < 0) {
        leaf(~w.root);
        return h;
    }
    int stack[128];
    int sp = 0;
    int node = w.root;
    while (true) {
        float tn0, tn1;
        const bool h0 = slab(w.cbox0[node], o, inv, kTmin, best, tn0);
        const bool h1 = slab(w.cbox1[node], o, inv, kTmin, best, tn1);
        int next = -1;
        const int c0 = w.left[node], c1 = w.right[node];
        int first = c0, second = c1;
        bool hf = h0, hs = h1;
        if (h0 && h1 && tn1 < tn0) { first = c1; second = c0; hf = h1; hs = h0; }
        // leaves are tested at once; internal children are descended near first
        if (hf && first < 0) { leaf(~first); hf = false; }
        if (hs && second < 0) { leaf(~second); hs = false; }
        if (hf && hs) { stack[sp++] = second; next = first; }
        else if (hf) next = first;
        else if (hs) next = second;
        if (next < 0) {
            if (sp == 0) break;
            next = stack[--sp];
        }
        node = next;
    }
    return h;
}

// Brute force over the records whose own box passes the slab test (with the
// far limit at kTmax): the hit set the hierarchy's rule implies, since every
// ancestor box holds a record's box.
Hit closest_brute_boxed(const orc_world& w, F3 o, F3 d) {
    Hit h;
    bool have = false;
    const F3 inv = mk(safe_inv(d.x), safe_inv(d.y), safe_inv(d.z));
    for (size_t i = 0; i < w.prims.size(); ++i) {
        float tn;
        if (!slab(prim_box(w.prims[i]), o, inv, kTmin, kTmax, tn)) continue;
        float t, u, v;
        if (!prim_hit(w.prims[i], o, d, t, u, v) || t > kTmax) continue;
        if (better(t, w.prims[i].id, h.t, have ? w.prims[h.prim].id : 0, have)) {
            h.t = t; h.u = u; h.v = v; h.prim = int(i); have = true;
        }
    }
    return h;
}

inline Hit closest(const orc_world& w, F3 o, F3 d, int use_bvh) {
    return use_bvh ? closest_bvh(w, o, d) : closest_brute(w, o, d);
}

// FP64 distance from (FP32) ray to a given primitive; NaN when it misses.
double t64_of(const Prim& p, F3 of, F3 df) {
    const double o[3] = {of.x, of.y, of.z}, d[3] = {df.x, df.y, df.z};
    auto sub3 = [](const double* a, const double* b, double* r) {
        r[0] = a[0] - b[0]; r[1] = a[1] - b[1]; r[2] = a[2] - b[2];
    };
    auto cr = [](const double* a, const double* b, double* r) {
        r[0] = a[1] * b[2] - a[2] * b[1];
        r[1] = a[2] * b[0] - a[0] * b[2];
        r[2] = a[0] * b[1] - a[1] * b[0];
    };
    auto dt = [](const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; };
    if (p.kind == 0) {
        const double A[3] = {p.a.x, p.a.y, p.a.z}, B[3] = {p.b.x, p.b.y, p.b.z},
                     C[3] = {p.c.x, p.c.y, p.c.z};
        double e1[3], e2[3], pv[3], tv[3], qv[3];
        sub3(B, A, e1); sub3(C, A, e2); cr(d, e2, pv);
        const double det = dt(e1, pv);
        if (det == 0.0) return NAN;
        sub3(o, A, tv); cr(tv, e1, qv);
        return dt(e2, qv) / det;
    }
    const double c[3] = {p.a.x, p.a.y, p.a.z};
    double oc[3];
    sub3(o, c, oc);
    const double a = dt(d, d), b = dt(d, oc), cc = dt(oc, oc) - double(p.r) * p.r;
    const double disc = b * b - a * cc;
    if (disc < 0) return NAN;
    const double x = std::sqrt(disc);
    double t = (-b - x) / a;
    if (t < kTmin) t = (-b + x) / a;
    return t;
}

struct ShadeIn {
    F3 p;      // hit point
    F3 N;      // unit normal facing against the ray
    bool front;
};

// Geometry at a hit: optx/optics_i.cu:40-82 (triangles), sphere.h:40-46 (spheres).
inline ShadeIn hit_geometry(const orc_world& w, const Hit& h, F3 o, F3 d) {
    const Prim& p = w.prims[h.prim];
    ShadeIn s;
    if (p.kind == 0) {
        const float ww = 1.f - h.u - h.v;
        s.p = add(add(mul(ww, p.a), mul(h.u, p.b)), mul(h.v, p.c));
        F3 N = unitV(cross(sub(p.b, p.a), sub(p.c, p.a)));
        if (dot(d, N) > 0.f) N = neg(N);
        s.N = N;
        const Thing& th = w.things[p.thing];
        const F3 center = mk(th.T[3], th.T[7], th.T[11]);
        s.front = 0.f > dot(d, sub(s.p, center));  // optx/optics_i.cu:259-267
    } else {
        s.p = add(o, mul(h.t, d));
        const F3 outward = mul(1.f / p.r, sub(s.p, p.a));
        s.front = 0.f > dot(d, outward);
        s.N = s.front ? outward : neg(outward);
    }
    return s;
}

struct PathOut {
    F3 color;
    F3 normal, albedo;
    uint32_t rays;
};

// One scattering vertex of a recorded path (for the adjoint): the incoming
// ray, the hit and the random choices that fix the outgoing direction.
struct Vtx {
    int prim, thing, type;
    F3 o, d;        // incoming ray
    float t;        // hit distance along d
    F3 p, N;        // hit point, normal facing the incoming ray
    bool front;
    F3 v;           // diffuse: unit random vector; metal: in-sphere vector
    int branch;     // diffuse: 1 = near-zero fallback; glass: 0 reflect, 1 refract
    float ratio;    // glass: index ratio
};

struct PathRec {
    std::vector<Vtx> vtx;
    bool miss = false;   // ended by a miss (sky), not absorbed / depth limit
    F3 d_last{0, 0, 0};  // direction of the missing ray
};

inline F3 sky(F3 d, F3 ambient, F3 white) {
    // optx/camera_i.cu:133-139
    const F3 unit = unitV(d);
    const float t = .5f * (unit.y + 1.f);
    return add(mul(1.f - t, white), mul(t, ambient));
}

PathOut trace_path(const orc_world& w, const Cam& cam, unsigned x, unsigned y, unsigned W,
                   unsigned H, unsigned depth, uint32_t seed, uint32_t scene, uint32_t sample,
                   F3 ambient, F3 white, PathRec* rec = nullptr, int fthing = -1, float fuzz = 0.f) {
    const uint32_t pix = W * y + x;
    PathOut out{mk(1.f, 1.f, 1.f), mk(0, 0, 0), mk(0, 0, 0), 0};
    F3 o, d;
    {
        Stream s(seed, scene, pix, sample, 0);
        camera_ray(cam, x, y, W, H, s, o, d);
    }
    if (rec) { rec->vtx.clear(); rec->miss = false; }
    for (uint32_t k = 0;; ++k) {
        out.rays++;
        const Hit h = closest_bvh(w, o, d);
        if (h.prim < 0) {
            out.color = mulv(out.color, sky(d, ambient, white));
            if (rec) { rec->miss = true; rec->d_last = d; }
            break;
        }
        if (k + 1 >= depth) {  // black at the depth limit (optx/optics_r.cu:34-42)
            out.color = mk(0.f, 0.f, 0.f);
            break;
        }
        const ShadeIn g = hit_geometry(w, h, o, d);
        const Thing& th = w.things[w.prims[h.prim].thing];
        Stream s(seed, scene, pix, sample, k + 1);
        Vtx vx{h.prim, w.prims[h.prim].thing, th.type, o, d, h.t, g.p, g.N, g.front, mk(0, 0, 0), 0, 1.f};
        if (th.type == OPT_DIFFUSE) {
            // optx/optics_i.cu:87-96 with the near-zero fallback of optics.h:17-18
            const F3 u = rndVon1sphere(s);
            F3 dir = add(g.N, u);
            vx.v = u;
            if (near0(dir)) { dir = g.N; vx.branch = 1; }
            out.color = mulv(out.color, th.albedo);
            if (isnull(out.normal)) out.normal = g.N;
            if (isnull(out.albedo)) out.albedo = th.albedo;
            o = g.p; d = dir;
        } else if (th.type == OPT_REFLECT) {
            // optx/optics_i.cu:168-190
            const F3 d1V = unitV(d);
            const F3 refl = sub(d1V, mul(2.f * dot(d1V, g.N), g.N));
            const F3 v = rndVin1sphere(s);
            const F3 dir = add(refl, mul(w.prims[h.prim].thing == fthing ? fuzz : th.fuzz, v));
            vx.v = v;
            if (isnull(out.normal)) out.normal = g.N;
            if (isnull(out.albedo)) out.albedo = th.albedo;
            if (dot(dir, g.N) > 0.f) {
                out.color = mulv(out.color, th.albedo);
                o = g.p; d = dir;
            } else {
                out.color = mk(0.f, 0.f, 0.f);
                if (rec) rec->vtx.push_back(vx);
                break;
            }
        } else {
            // optx/optics_i.cu:254-283
            const F3 d1V = unitV(d);
            const float cos_theta = fminf(dot(neg(d1V), g.N), 1.f);
            const float sin_theta = sqrtf(1.f - cos_theta * cos_theta);
            const float ratio = g.front ? 1.f / th.index : th.index;
            const bool cannot = ratio * sin_theta > 1.f;
            float r0 = (1.f - ratio) / (1.f + ratio);
            r0 = r0 * r0;
            const float om = 1.f - cos_theta;
            const float pow5 = ((om * om) * (om * om)) * om;
            const float schlick = r0 + (1.f - r0) * pow5;
            F3 dir;
            vx.ratio = ratio;
            if (cannot || schlick > s.next()) {
                dir = sub(d1V, mul(2.f * dot(d1V, g.N), g.N));
                vx.branch = 0;
            } else {
                const float theta = fminf(dot(neg(d1V), g.N), 1.f);
                const F3 perpen = mul(ratio, add(d1V, mul(theta, g.N)));
                const F3 parall = mul(-sqrtf(fabsf(1.f - dot(perpen, perpen))), g.N);
                dir = add(perpen, parall);
                vx.branch = 1;
            }
            o = g.p; d = dir;
        }
        if (rec) rec->vtx.push_back(vx);
    }
    return out;
}

// trace_path with the fuzz of thing `fthing` replaced by `fuzz` (the world is
// not modified, so threads can trace different values at once).
inline PathOut trace_path_fuzz(const orc_world& w, const Cam& cam, unsigned x, unsigned y, unsigned W,
                               unsigned H, unsigned depth, uint32_t seed, uint32_t scene, uint32_t sample,
                               F3 ambient, F3 white, int fthing, float fuzz, PathRec* rec) {
    return trace_path(w, cam, x, y, W, H, depth, seed, scene, sample, ambient, white, rec, fthing, fuzz);
}

// ------------------------------------------------------------- adjoint --
// Double-precision tangent of the path below a perturbation (do, dd) of the
// ray leaving vertex k0: the same hits and branches as the primal path
// (visibility is held fixed), differentiated vertex by vertex.
struct D3 {
    double x, y, z;
};
inline D3 dd3(F3 a) { return D3{a.x, a.y, a.z}; }
inline D3 operator+(D3 a, D3 b) { return D3{a.x + b.x, a.y + b.y, a.z + b.z}; }
inline D3 operator-(D3 a, D3 b) { return D3{a.x - b.x, a.y - b.y, a.z - b.z}; }
inline D3 operator*(double s, D3 a) { return D3{s * a.x, s * a.y, s * a.z}; }
inline double ddot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline double dlen(D3 a) { return std::sqrt(ddot(a, a)); }

// derivative of unit(d) along dd
inline D3 dunit(D3 d, D3 dd) {
    const double l = dlen(d);
    const D3 u = (1.0 / l) * d;
    return (1.0 / l) * (dd - ddot(u, dd) * u);
}

// Propagates (dO, dD) of the ray entering vertex m through vertices m..end;
// returns d(sky colour)/d(perturbation) of the final miss, per channel.
D3 tangent_to_sky(const orc_world& w, const PathRec& rec, size_t m, D3 dO, D3 dD, F3 ambient, F3 white) {
    for (size_t k = m; k < rec.vtx.size(); ++k) {
        const Vtx& v = rec.vtx[k];
        const Prim& pr = w.prims[v.prim];
        const D3 d = dd3(v.d), N = dd3(v.N);
        const double t = v.t;
        // hit point on the (fixed) surface: dp = q - d (n.q)/(n.d), q = dO + t dD
        const D3 q = dO + t * dD;
        D3 n;
        if (pr.kind == 0) n = N; else n = dd3(v.p) - dd3(pr.a);
        const double nd = ddot(n, d);
        const D3 dp = nd != 0.0 ? q - (ddot(n, q) / nd) * d : q;
        D3 dN{0, 0, 0};
        if (pr.kind == 1) {   // sphere: N = +-(p - c)/r
            const double sgn = v.front ? 1.0 : -1.0;
            dN = (sgn / double(pr.r)) * dp;
        }
        D3 dOut;
        if (v.type == OPT_DIFFUSE) {
            dOut = dN;   // d' = N + u (or N)
        } else {
            const D3 d1 = (1.0 / dlen(d)) * d;
            const D3 dd1 = dunit(d, dD);
            const bool refl = v.type == OPT_REFLECT || v.branch == 0;
            if (refl) {
                const double c = ddot(d1, N);
                const double dc = ddot(dd1, N) + ddot(d1, dN);
                dOut = dd1 - 2.0 * ((dc * N) + c * dN);
            } else {
                const double ratio = v.ratio;
                const double raw = -ddot(d1, N);
                const double cth = raw < 1.0 ? raw : 1.0;
                const double dcth = raw < 1.0 ? -(ddot(dd1, N) + ddot(d1, dN)) : 0.0;
                const D3 perp = ratio * (d1 + cth * N);
                const D3 dperp = ratio * (dd1 + (dcth * N) + cth * dN);
                const double qq = ddot(perp, perp);
                const double sroot = std::sqrt(std::fabs(1.0 - qq));
                const double dq = 2.0 * ddot(perp, dperp);
                const double ds = sroot > 0.0 ? ((1.0 - qq) >= 0.0 ? -dq : dq) / (2.0 * sroot) : 0.0;
                dOut = dperp - ((ds * N) + sroot * dN);
            }
        }
        dO = dp;
        dD = dOut;
    }
    // miss: sky = (1 - s) white + s ambient, s = .5 (unit(d).y + 1)
    const D3 du = dunit(dd3(rec.d_last), dD);
    const double ds = 0.5 * du.y;
    return D3{ds * (double(ambient.x) - white.x), ds * (double(ambient.y) - white.y),
              ds * (double(ambient.z) - white.z)};
}

// 64-bit fixed-point sample sums: q(x) = round-half-even(x * 2^32) (exact in
// binary32 up to the final rounding); mean = (double)sum * 2^-32 / spp rounded
// to binary32.
inline int64_t fx_q(float x) { return int64_t(llrintf(x * 4294967296.0f)); }
inline void fx_add(int64_t s[3], F3 v) {
    s[0] += fx_q(v.x);
    s[1] += fx_q(v.y);
    s[2] += fx_q(v.z);
}
inline float fx_div(int64_t s, unsigned spp) { return float(double(s) * 0x1p-32 / double(spp)); }
inline F3 fx_mean(const int64_t s[3], unsigned spp) { return mk(fx_div(s[0], spp), fx_div(s[1], spp), fx_div(s[2], spp)); }

Cam to_cam(const orc_camera* c) {
    Cam k;
    k.eye = ld3(c->eye); k.u = ld3(c->u); k.v = ld3(c->v); k.w = ld3(c->w);
    k.hvec = ld3(c->hvec); k.wvec = ld3(c->wvec); k.dvec = ld3(c->dvec);
    k.aperture = c->aperture;
    k.rtow_px = c->rtow_pixels != 0;
    return k;
}

// Tessellation: optx/sphere.cxx:51-66 (pumpup) restated.
void pumpup(F3 a, F3 b, F3 c, unsigned n, float radius, std::vector<F3>& out) {
    if (n > 0) {
        const F3 ab = unitV(mul(.5f, add(a, b)));
        const F3 bc = unitV(mul(.5f, add(b, c)));
        const F3 ca = unitV(mul(.5f, add(c, a)));
        pumpup(a, ab, ca, n - 1, radius, out);
        pumpup(ab, b, bc, n - 1, radius, out);
        pumpup(ca, bc, c, n - 1, radius, out);
        pumpup(ab, bc, ca, n - 1, radius, out);
    } else {
        out.push_back(mul(radius, a));
        out.push_back(mul(radius, b));
        out.push_back(mul(radius, c));
    }
}

}  // namespace

// ============================================================ C exports ====
extern "C" {

void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    philox(ctr, key, out);
}

float orc_u01(uint32_t x) { return u01(x); }

void orc_glibc_rand(uint32_t seed, int n, int32_t* out) {
    GlibcRand g(seed);
    for (int i = 0; i < n; ++i) out[i] = g.next();
}

int orc_scene_rtow(int rng_kind, uint32_t seed, int half_extent, int cap, float* centers,
                   float* radii, int* types, float* albedos, float* fuzz, float* index) {
    int n = 0;
    auto put = [&](double cx, double cy, double cz, double r, int type, double ar, double ag,
                   double ab, double fz, double ix) {
        if (n >= cap) return;
        centers[3 * n] = float(cx); centers[3 * n + 1] = float(cy); centers[3 * n + 2] = float(cz);
        radii[n] = float(r); types[n] = type;
        albedos[3 * n] = float(ar); albedos[3 * n + 1] = float(ag); albedos[3 * n + 2] = float(ab);
        fuzz[n] = float(fz); index[n] = float(ix);
        ++n;
    };
    if (rng_kind == 0) {
        // rtow.cxx:51-80 in double precision with glibc rand(); arguments of one
        // constructor call are drawn last-to-first (g++ order: z, y, x).
        GlibcRand g(seed);
        auto rnd = [&]() { return double(g.next()) / (2147483647.0 + 1.0); };
        auto rndr = [&](double lo, double hi) { return lo + rnd() * (hi - lo); };
        put(0, -1000, 0, 1000, OPT_DIFFUSE, .5, .5, .5, 0, 0);
        for (int a = -half_extent; a < half_extent; ++a) {
            for (int b = -half_extent; b < half_extent; ++b) {
                const double select = rnd();
                const double rz = rnd();
                const double rx = rnd();
                const double cx = a + .9 * rx, cy = .2, cz = b + .9 * rz;
                const double dx = cx - 4, dy = cy - .2, dz = cz - 0;
                if (std::sqrt(dx * dx + dy * dy + dz * dz) > .9) {
                    if (select < .8) {
                        double f1[3], f2[3];
                        for (int i = 2; i >= 0; --i) f1[i] = rnd();
                        for (int i = 2; i >= 0; --i) f2[i] = rnd();
                        put(cx, cy, cz, .2, OPT_DIFFUSE, f1[0] * f2[0], f1[1] * f2[1],
                            f1[2] * f2[2], 0, 0);
                    } else if (select < .95) {
                        double al[3];
                        for (int i = 2; i >= 0; --i) al[i] = rndr(.5, 1.);
                        const double fz = rndr(0, .5);
                        put(cx, cy, cz, .2, OPT_REFLECT, al[0], al[1], al[2], fz, 0);
                    } else {
                        put(cx, cy, cz, .2, OPT_REFRACT, 0, 0, 0, 0, 1.5);
                    }
                }
            }
        }
    } else if (rng_kind == 1) {
        // Same recipe in binary32 with the counter RNG: draw k of the scene
        // stream is lane k%4 of Philox(ctr=(k/4, 0, 0, 0x5343454E), key=(seed, 0)).
        uint32_t k = 0;
        uint32_t buf[4];
        auto rnd = [&]() {
            if ((k & 3u) == 0) {
                const uint32_t ctr[4] = {k >> 2, 0u, 0u, 0x5343454Eu};
                const uint32_t key[2] = {seed, 0u};
                philox(ctr, key, buf);
            }
            return u01(buf[(k++) & 3u]);
        };
        auto rndr = [&](float lo, float hi) { return lo + rnd() * (hi - lo); };
        put(0, -1000, 0, 1000, OPT_DIFFUSE, .5, .5, .5, 0, 0);
        for (int a = -half_extent; a < half_extent; ++a) {
            for (int b = -half_extent; b < half_extent; ++b) {
                const float select = rnd();
                const float rx = rnd();
                const float rz = rnd();
                const F3 c = mk(float(a) + .9f * rx, .2f, float(b) + .9f * rz);
                if (len(sub(c, mk(4.f, .2f, 0.f))) > .9f) {
                    if (select < .8f) {
                        float f1[3], f2[3];
                        for (int i = 0; i < 3; ++i) f1[i] = rnd();
                        for (int i = 0; i < 3; ++i) f2[i] = rnd();
                        put(c.x, c.y, c.z, .2f, OPT_DIFFUSE, f1[0] * f2[0], f1[1] * f2[1],
                            f1[2] * f2[2], 0, 0);
                    } else if (select < .95f) {
                        float al[3];
                        for (int i = 0; i < 3; ++i) al[i] = rndr(.5f, 1.f);
                        const float fz = rndr(0.f, .5f);
                        put(c.x, c.y, c.z, .2f, OPT_REFLECT, al[0], al[1], al[2], fz, 0);
                    } else {
                        put(c.x, c.y, c.z, .2f, OPT_REFRACT, 0, 0, 0, 0, 1.5f);
                    }
                }
            }
        }
    } else {
        return -1;
    }
    put(0, 1, 0, 1, OPT_REFRACT, 0, 0, 0, 0, 1.5);
    put(-4, 1, 0, 1, OPT_DIFFUSE, .4, .2, .1, 0, 0);
    put(4, 1, 0, 1, OPT_REFLECT, .7, .6, .5, 0, 0);
    return n;
}

void orc_tessellate_counts(unsigned ndiv, unsigned* nv, unsigned* ni) {
    const unsigned t = 4u << (2 * ndiv);
    *ni = t;
    *nv = t / 2 + 2;  // Euler: V = F/2 + 2 for a closed triangulated sphere
}

int orc_tessellate(float radius, unsigned ndiv, float* vces, unsigned* ices) {
    // optx/sphere.cxx:34-46 (regular tetrahedron, m = .57735026919f)
    const float m = .57735026919f;
    const F3 v00 = mk(m, m, m), v01 = mk(m, -m, -m), v02 = mk(-m, -m, m), v03 = mk(-m, m, -m);
    std::vector<F3> tmp;
    tmp.reserve(size_t(12) << (2 * ndiv));
    pumpup(v00, v01, v02, ndiv, radius, tmp);
    pumpup(v00, v02, v03, ndiv, radius, tmp);
    pumpup(v00, v03, v01, ndiv, radius, tmp);
    pumpup(v03, v02, v01, ndiv, radius, tmp);
    // Vertex dedup numbered in first-seen order (optx/sphere.cxx:68-106),
    // done as a stable sort by (x, y, z): the head of every run of equal
    // vertices is its first occurrence.
    const size_t n = tmp.size();
    std::vector<uint32_t> idx(n);
    std::iota(idx.begin(), idx.end(), 0u);
    auto lessv = [&](uint32_t a, uint32_t b) {
        const F3 &l = tmp[a], &r = tmp[b];
        if (l.x != r.x) return l.x < r.x;
        if (l.y != r.y) return l.y < r.y;
        return l.z < r.z;
    };
    std::stable_sort(idx.begin(), idx.end(), lessv);
    std::vector<uint32_t> head(n);  // per element: position of its first occurrence
    for (size_t s = 0; s < n;) {
        size_t e = s + 1;
        while (e < n && !lessv(idx[s], idx[e])) ++e;
        for (size_t j = s; j < e; ++j) head[idx[j]] = idx[s];
        s = e;
    }
    std::vector<uint32_t> id(n, 0xFFFFFFFFu);
    uint32_t next = 0;
    for (size_t i = 0; i < n; ++i) {
        if (head[i] == i) {
            id[i] = next;
            st3(vces + 3 * size_t(next), tmp[i]);
            ++next;
        }
    }
    for (size_t i = 0; i < n; ++i) ices[i] = id[head[i]];
    return int(next);
}

void orc_camera_set(const float eye[3], const float pat[3], const float vup[3], float fov,
                    float aspratio, float aperture, float fostance, float out[18]) {
    (void)aperture;
    // optx/camera.h:30-48
    const F3 E = ld3(eye), P = ld3(pat), U = ld3(vup);
    const F3 w = unitV(sub(E, P));
    const F3 u = unitV(cross(U, w));
    const F3 v = cross(w, u);
    const float kPi = 3.14159265358979323846f;
    const float h = 2.f * tanf(.5f * (fov * kPi / 180.f));
    const float wd = h * aspratio;
    const F3 hvec = mul(fostance * h / 2.f, v);
    const F3 wvec = mul(fostance * wd / 2.f, u);
    const F3 dvec = mul(fostance, w);
    st3(out, u); st3(out + 3, v); st3(out + 6, w);
    st3(out + 9, hvec); st3(out + 12, wvec); st3(out + 15, dvec);
}

void orc_morton30(const float* c, unsigned n, const float lo[3], const float hi[3], uint32_t* codes) {
    const float ex = hi[0] - lo[0], ey = hi[1] - lo[1], ez = hi[2] - lo[2];
#pragma omp parallel for schedule(static)
    for (long i = 0; i < long(n); ++i) {
        const uint32_t qx = quant10(c[3 * i], lo[0], ex);
        const uint32_t qy = quant10(c[3 * i + 1], lo[1], ey);
        const uint32_t qz = quant10(c[3 * i + 2], lo[2], ez);
        codes[i] = (expand10(qx) << 2) | (expand10(qy) << 1) | expand10(qz);
    }
}

void orc_morton60(const float* c, unsigned n, const float lo[3], const float hi[3], uint64_t* codes) {
    const float ex = hi[0] - lo[0], ey = hi[1] - lo[1], ez = hi[2] - lo[2];
#pragma omp parallel for schedule(static)
    for (long i = 0; i < long(n); ++i) {
        const uint64_t qx = quant20(c[3 * i], lo[0], ex);
        const uint64_t qy = quant20(c[3 * i + 1], lo[1], ey);
        const uint64_t qz = quant20(c[3 * i + 2], lo[2], ez);
        codes[i] = (expand20(qx) << 2) | (expand20(qy) << 1) | expand20(qz);
    }
}

void orc_stable_sort_pairs64(uint64_t* keys, uint32_t* vals, unsigned n) {
    std::vector<std::pair<uint64_t, uint32_t>> kv(n);
    for (unsigned i = 0; i < n; ++i) kv[i] = {keys[i], vals[i]};
    std::stable_sort(kv.begin(), kv.end(),
                     [](const std::pair<uint64_t, uint32_t>& a, const std::pair<uint64_t, uint32_t>& b) {
                         return a.first < b.first;
                     });
    for (unsigned i = 0; i < n; ++i) {
        keys[i] = kv[i].first;
        vals[i] = kv[i].second;
    }
}

void orc_stable_sort_pairs(uint32_t* keys, uint32_t* vals, unsigned n) {
    std::vector<std::pair<uint32_t, uint32_t>> kv(n);
    for (unsigned i = 0; i < n; ++i) kv[i] = {keys[i], vals[i]};
    std::stable_sort(kv.begin(), kv.end(),
                     [](const std::pair<uint32_t, uint32_t>& a, const std::pair<uint32_t, uint32_t>& b) {
                         return a.first < b.first;
                     });
    for (unsigned i = 0; i < n; ++i) {
        keys[i] = kv[i].first;
        vals[i] = kv[i].second;
    }
}

void orc_karras(const uint64_t* sorted_codes, unsigned n, int32_t* left, int32_t* right) {
    if (n > 1) karras(sorted_codes, int(n), left, right);
}

orc_world* orc_world_new(void) { return new orc_world(); }
void orc_world_free(orc_world* w) { delete w; }

int orc_world_add_mesh(orc_world* w, const float* vces, unsigned nv, const unsigned* ices, unsigned ni) {
    Mesh m;
    m.v.assign(vces, vces + 3 * size_t(nv));
    m.i.assign(ices, ices + 3 * size_t(ni));
    for (uint32_t x : m.i)
        if (x >= nv) return -1;
    w->meshes.push_back(std::move(m));
    return int(w->meshes.size()) - 1;
}

int orc_world_add_thing(orc_world* w, int type, const float albedo[3], float fuzz, float index,
                        int mesh, const float transform[12]) {
    if (mesh < 0 || mesh >= int(w->meshes.size())) return -1;
    Thing t{};
    t.type = type; t.albedo = ld3(albedo); t.fuzz = fuzz; t.index = index; t.mesh = mesh;
    memcpy(t.T, transform, sizeof(t.T));
    t.center = mk(transform[3], transform[7], transform[11]);
    w->things.push_back(t);
    w->built = false;
    return int(w->things.size()) - 1;
}

int orc_world_add_sphere(orc_world* w, int type, const float albedo[3], float fuzz, float index,
                         const float center[3], float radius) {
    Thing t{};
    t.type = type; t.albedo = ld3(albedo); t.fuzz = fuzz; t.index = index; t.mesh = -1;
    t.center = ld3(center); t.radius = radius;
    const float T[12] = {radius, 0, 0, center[0], 0, radius, 0, center[1], 0, 0, radius, center[2]};
    memcpy(t.T, T, sizeof(T));
    w->things.push_back(t);
    w->built = false;
    return int(w->things.size()) - 1;
}

int orc_world_set_transform(orc_world* w, int thing, const float transform[12]) {
    if (thing < 0 || thing >= int(w->things.size())) return -1;
    Thing& t = w->things[thing];
    memcpy(t.T, transform, sizeof(t.T));
    t.center = mk(transform[3], transform[7], transform[11]);
    w->built = false;
    return 0;
}

int orc_world_build(orc_world* w, int morton_bits) {
    if (morton_bits != 30 && morton_bits != 60) return -1;
    w->morton_bits = morton_bits;
    w->grouped = false;
    w->sah_cluster = 0;
    flatten(*w);
    build_lbvh(*w);
    return 0;
}

int orc_world_build_grouped(orc_world* w) {
    w->morton_bits = 60;
    w->grouped = true;
    w->sah_cluster = 0;
    flatten(*w);
    build_lbvh(*w);
    return 0;
}

int orc_world_build_sah(orc_world* w, unsigned cluster_max) {
    if (cluster_max < 1) return -1;
    w->morton_bits = 60;
    w->grouped = false;
    w->sah_cluster = cluster_max;
    flatten(*w);
    build_lbvh(*w);
    return 0;
}

unsigned orc_world_nprims(const orc_world* w) { return unsigned(w->prims.size()); }

void orc_world_lbvh(const orc_world* w, uint64_t* codes, uint32_t* ids, int32_t* left,
                    int32_t* right, float* boxes, float* clo, float* chi) {
    const size_t n = w->prims.size();
    if (codes) std::copy(w->codes.begin(), w->codes.end(), codes);
    if (ids) std::copy(w->order.begin(), w->order.end(), ids);
    if (left) std::copy(w->left.begin(), w->left.end(), left);
    if (right) std::copy(w->right.begin(), w->right.end(), right);
    if (boxes) {
        for (size_t i = 0; i + 1 < n; ++i) {
            const Box& a = w->cbox0[i];
            const Box& b = w->cbox1[i];
            float* o = boxes + 12 * i;
            st3(o, a.lo); st3(o + 3, a.hi); st3(o + 6, b.lo); st3(o + 9, b.hi);
        }
    }
    if (clo) st3(clo, w->clo);
    if (chi) st3(chi, w->chi);
}

void orc_world_triangles(const orc_world* w, float* tris) {
    for (size_t i = 0; i < w->prims.size(); ++i) {
        const Prim& p = w->prims[i];
        st3(tris + 9 * i, p.a); st3(tris + 9 * i + 3, p.b); st3(tris + 9 * i + 6, p.c);
    }
}

void orc_first_hit(const orc_world* wd, const orc_camera* cam, unsigned w, unsigned h,
                   uint32_t seed, uint32_t scene, uint32_t sample, int use_bvh, int32_t* prim,
                   int32_t* thing, float* t, float* u, float* v, double* t64, int nthreads) {
    const Cam c = to_cam(cam);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
#pragma omp parallel for schedule(dynamic, 64)
    for (long p = 0; p < long(w) * long(h); ++p) {
        const unsigned x = unsigned(p % w), y = unsigned(p / w);
        Stream s(seed, scene, uint32_t(p), sample, 0);
        F3 o, d;
        camera_ray(c, x, y, w, h, s, o, d);
        const Hit hh = closest(*wd, o, d, use_bvh);
        if (hh.prim < 0) {
            prim[p] = -1; thing[p] = -1; t[p] = 0.f; u[p] = 0.f; v[p] = 0.f;
            if (t64) t64[p] = NAN;
        } else {
            const Prim& pr = wd->prims[hh.prim];
            prim[p] = int32_t(pr.id); thing[p] = pr.thing;
            t[p] = hh.t; u[p] = hh.u; v[p] = hh.v;
            if (t64) t64[p] = t64_of(pr, o, d);
        }
    }
}

void orc_closest(const orc_world* wd, unsigned n, const float* o, const float* d, int mode, int32_t* prim,
                 float* t, int nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
#pragma omp parallel for schedule(dynamic, 256)
    for (long k = 0; k < long(n); ++k) {
        const F3 oo = mk(o[3 * k], o[3 * k + 1], o[3 * k + 2]), dd = mk(d[3 * k], d[3 * k + 1], d[3 * k + 2]);
        const Hit hh = mode == 1 ? closest_bvh(*wd, oo, dd) : mode == 2 ? closest_brute_boxed(*wd, oo, dd)
                                                            : closest_brute(*wd, oo, dd);
        prim[k] = hh.prim < 0 ? -1 : int32_t(wd->prims[hh.prim].id);
        t[k] = hh.prim < 0 ? 0.f : hh.t;
    }
}

uint64_t orc_render(const orc_world* wd, const orc_camera* cam, unsigned w, unsigned h,
                    unsigned spp, unsigned depth, uint32_t seed, uint32_t scene,
                    const float ambient[3], const float white[3], const uint32_t* pixels,
                    unsigned npixels, float* rawRGB, uint32_t* rpp, float* normals,
                    float* albedos, int nthreads) {
    const Cam c = to_cam(cam);
    const F3 amb = ld3(ambient), wht = ld3(white);
    const long count = pixels ? long(npixels) : long(w) * long(h);
    std::atomic<uint64_t> total{0};
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
#pragma omp parallel
    {
        uint64_t mine = 0;
#pragma omp for schedule(dynamic, 16)
        for (long q = 0; q < count; ++q) {
            const uint32_t pix = pixels ? pixels[q] : uint32_t(q);
            const unsigned x = pix % w, y = pix / w;
            // Per-pixel sums in 64-bit fixed point (2^-32 units): every sample
            // adds round(x * 2^32), an integer sum that is exact and does not
            // depend on the order in which samples finish.
            int64_t sc[3] = {0, 0, 0}, sn[3] = {0, 0, 0}, sa[3] = {0, 0, 0};
            uint32_t rays = 0;
            for (unsigned s = 0; s < spp; ++s) {
                const PathOut po = trace_path(*wd, c, x, y, w, h, depth, seed, scene, s, amb, wht);
                fx_add(sc, po.color);   // optx/camera_i.cu:95
                fx_add(sn, po.normal);
                fx_add(sa, po.albedo);
                rays += po.rays;
            }
            // optx/camera_i.cu:105-113: mean over spp, clamped to [0,1]
            auto cl = [](float x) { return 0.f > x ? 0.f : (x > 1.f ? 1.f : x); };
            const F3 mean = fx_mean(sc, spp);
            st3(rawRGB + 3 * q, mk(cl(mean.x), cl(mean.y), cl(mean.z)));
            if (rpp) rpp[q] = rays;
            if (normals) st3(normals + 3 * q, fx_mean(sn, spp));
            if (albedos) st3(albedos + 3 * q, fx_mean(sa, spp));
            mine += rays;
        }
        total += mine;
    }
    return total.load();
}

unsigned orc_world_nthings(const orc_world* w) { return unsigned(w->things.size()); }

// Per-path check of the fuzz tangent: for every path of the image that
// reflects off `thing`, d(colour)/d(fuzz) from tangent_to_sky against a
// central difference of the same path (same random numbers) -- counted only
// where both perturbed paths keep the hit sequence and branches (no
// visibility change).  out[0] = paths compared, out[1] = paths skipped,
// out[2] = max |adj - fd| / max(|fd|, floor), out[3] = sum |fd|, out[4] =
// paths with a relative error above 5%, out[5] / out[6] = sum of adj / fd
// over the compared paths (all channels).
void orc_fuzz_path_check(orc_world* wd, const orc_camera* cam, unsigned w, unsigned h, unsigned spp,
                         unsigned depth, uint32_t seed, int thing, float step, const float ambient[3],
                         const float white[3], double* out) {
    const Cam c = to_cam(cam);
    const F3 amb = ld3(ambient), wht = ld3(white);
    Thing& th = wd->things[thing];
    const float f0 = th.fuzz;
    double compared = 0, skipped = 0, maxrel = 0, sumfd = 0, outliers = 0, sadj = 0, sfd = 0;
    PathRec r0, rp, rm;
    auto same = [](const PathRec& a, const PathRec& b) {
        if (a.miss != b.miss || a.vtx.size() != b.vtx.size()) return false;
        for (size_t k = 0; k < a.vtx.size(); ++k)
            if (a.vtx[k].prim != b.vtx[k].prim || a.vtx[k].branch != b.vtx[k].branch) return false;
        return true;
    };
    for (unsigned pix = 0; pix < w * h; ++pix) {
        for (unsigned smp = 0; smp < spp; ++smp) {
            th.fuzz = f0;
            const PathOut p0 = trace_path(*wd, c, pix % w, pix / w, w, h, depth, seed, 0, smp, amb, wht, &r0);
            if (!r0.miss) continue;
            bool touches = false;
            for (const Vtx& v : r0.vtx) touches |= (v.thing == thing && v.type == OPT_REFLECT);
            if (!touches) continue;
            th.fuzz = f0 + step;
            const PathOut pp = trace_path(*wd, c, pix % w, pix / w, w, h, depth, seed, 0, smp, amb, wht, &rp);
            th.fuzz = f0 - step;
            const PathOut pm = trace_path(*wd, c, pix % w, pix / w, w, h, depth, seed, 0, smp, amb, wht, &rm);
            th.fuzz = f0;
            if (!same(r0, rp) || !same(r0, rm)) { skipped += 1; continue; }
            // tangent: sum over the events on `thing`
            D3 thr{1, 1, 1};
            for (const Vtx& v : r0.vtx)
                if (v.type != OPT_REFRACT) {
                    const F3 a = wd->things[v.thing].albedo;
                    thr = D3{thr.x * a.x, thr.y * a.y, thr.z * a.z};
                }
            D3 adj{0, 0, 0};
            for (size_t k = 0; k < r0.vtx.size(); ++k) {
                const Vtx& v = r0.vtx[k];
                if (v.thing != thing || v.type != OPT_REFLECT) continue;
                const D3 ds = tangent_to_sky(*wd, r0, k + 1, D3{0, 0, 0}, dd3(v.v), amb, wht);
                adj = adj + D3{thr.x * ds.x, thr.y * ds.y, thr.z * ds.z};
            }
            const D3 fd = (1.0 / (2.0 * step)) * (dd3(pp.color) - dd3(pm.color));
            const double den = std::max(1e-3, std::max(std::fabs(fd.x), std::max(std::fabs(fd.y), std::fabs(fd.z))));
            const double err = std::max(std::fabs(adj.x - fd.x), std::max(std::fabs(adj.y - fd.y), std::fabs(adj.z - fd.z)));
            maxrel = std::max(maxrel, err / den);
            if (err / den > 0.05) outliers += 1;
            sumfd += std::fabs(fd.x) + std::fabs(fd.y) + std::fabs(fd.z);
            sadj += adj.x + adj.y + adj.z;
            sfd += fd.x + fd.y + fd.z;
            compared += 1;
            (void)p0;
        }
    }
    out[0] = compared; out[1] = skipped; out[2] = maxrel; out[3] = sumfd;
    out[4] = outliers; out[5] = sadj; out[6] = sfd;
}

// Colour of recorded path `rec` replayed in double precision with its
// visibility held fixed and metal `fthing`'s fuzz replaced by `fuzz`: the
// same random numbers, the same primitive at every vertex (the ray meets the
// recorded triangle's plane -- Moller-Trumbore without the barycentric
// bounds -- or the recorded sphere's root chosen by the same rule), the
// recorded facing, branches and near-zero fallbacks.  This is the function
// whose derivative the adjoint forms (the tangent differentiates it
// analytically), so a central difference of it at image level checks the
// fuzz gradient without the hit-sequence changes that a plain re-render
// mixes in; double precision lets the step be small enough to follow the
// steep near-silhouette paths.  Returns false when a replayed vertex is
// degenerate (a ray parallel to a recorded plane, or missing a recorded
// sphere).
static bool replay_held(const orc_world& w, const Cam& cam, const PathRec& rec, unsigned x, unsigned y, unsigned W,
                        unsigned H, uint32_t seed, uint32_t scene, uint32_t sample, F3 ambient, F3 white, int fthing,
                        double fuzz, D3& color, PathRec* out = nullptr) {
    auto cr = [](D3 a, D3 b) { return D3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; };
    auto unit = [](D3 a) { return (1.0 / dlen(a)) * a; };
    auto mv = [](D3 a, D3 b) { return D3{a.x * b.x, a.y * b.y, a.z * b.z}; };
    const uint32_t pix = W * y + x;
    D3 o, d;
    {
        F3 of, df;
        Stream s(seed, scene, pix, sample, 0);
        camera_ray(cam, x, y, W, H, s, of, df);
        o = dd3(of);
        d = dd3(df);
    }
    auto f3 = [](D3 a) { return mk(float(a.x), float(a.y), float(a.z)); };
    if (out) { *out = rec; }
    D3 thr{1, 1, 1};
    for (size_t k = 0; k < rec.vtx.size(); ++k) {
        const Vtx& v = rec.vtx[k];
        const Prim& p = w.prims[v.prim];
        const D3 o_in = o, d_in = d;
        D3 hp, N;
        if (p.kind == 0) {
            const D3 A = dd3(p.a), e1 = dd3(p.b) - A, e2 = dd3(p.c) - A;
            const D3 pv = cr(d, e2);
            const double det = ddot(e1, pv);
            if (det == 0.0) return false;
            const D3 tv = o - A, qv = cr(tv, e1);
            const double u = ddot(tv, pv) / det, vv = ddot(d, qv) / det;
            hp = A + u * e1 + vv * e2;
            N = unit(cr(e1, e2));
            if (ddot(d, N) > 0.0) N = -1.0 * N;
        } else {
            const D3 c = dd3(p.a), oc = o - c;
            const double a = ddot(d, d), b = ddot(d, oc), cc = ddot(oc, oc) - double(p.r) * double(p.r);
            const double disc = b * b - a * cc;
            if (disc < 0.0) return false;
            const double xs = std::sqrt(disc);
            double t = (-b - xs) / a;
            if (t < double(kTmin)) t = (-b + xs) / a;
            if (t < double(kTmin)) return false;
            hp = o + t * d;
            const D3 outward = (1.0 / double(p.r)) * (hp - c);
            N = v.front ? outward : -1.0 * outward;   // facing held as recorded
        }
        if (out) {   // the replayed vertex, for a tangent evaluated on this trajectory
            Vtx& r = out->vtx[k];
            r.o = f3(o_in); r.d = f3(d_in); r.p = f3(hp); r.N = f3(N);
            r.t = float(ddot(hp - o_in, d_in) / ddot(d_in, d_in));
        }
        const Thing& th = w.things[v.thing];
        Stream s(seed, scene, pix, sample, uint32_t(k + 1));
        if (v.type == OPT_DIFFUSE) {
            const D3 u = dd3(rndVon1sphere(s));
            d = v.branch ? N : N + u;
            thr = mv(thr, dd3(th.albedo));
        } else if (v.type == OPT_REFLECT) {
            const D3 d1 = unit(d);
            const D3 refl = d1 - (2.0 * ddot(d1, N)) * N;
            const D3 vv = dd3(rndVin1sphere(s));
            const double fz = int(v.thing) == fthing ? fuzz : double(th.fuzz);
            d = refl + fz * vv;
            thr = mv(thr, dd3(th.albedo));
        } else {
            const D3 d1 = unit(d);
            const double ratio = v.front ? 1.0 / double(th.index) : double(th.index);
            if (v.branch == 0) {
                d = d1 - (2.0 * ddot(d1, N)) * N;
            } else {
                const double theta = std::min(ddot(-1.0 * d1, N), 1.0);
                const D3 perpen = ratio * (d1 + theta * N);
                d = perpen + (-std::sqrt(std::fabs(1.0 - ddot(perpen, perpen)))) * N;
            }
        }
        o = hp;
    }
    if (out) out->d_last = f3(d);
    const D3 u = unit(d);
    const double sv = 0.5 * (u.y + 1.0);
    color = mv(thr, D3{(1.0 - sv) * white.x + sv * ambient.x, (1.0 - sv) * white.y + sv * ambient.y,
                       (1.0 - sv) * white.z + sv * ambient.z});
    return true;
}

// Image-level central difference of the fuzz of metal `thing` with
// visibility held fixed: for every path that ends in the sky and reflects off
// `thing`, its colour replayed with fuzz f0 + step and f0 - step
// (replay_held); delta_plus / delta_minus (w*h*3 doubles) receive the per-pixel
// change of the mean over spp.  out[0] = paths replayed, out[1] = paths with a
// degenerate replay (left out), out[2] = paths whose plain re-render at
// f0 +- step changes its hit sequence or branches (the paths a whole-image
// difference of re-renders would see jump), out[3] = (with image and
// grad_image given) the adjoint's fuzz gradient over the same paths, its
// tangent evaluated on the replayed double-precision trajectory -- the
// trajectory the difference follows, which on chaotic paths (chains of
// reflections off small spheres) drifts from the binary32 one.
void orc_fuzz_held_delta(const orc_world* wd, const orc_camera* cam, unsigned w, unsigned h, unsigned spp,
                         unsigned depth, uint32_t seed, uint32_t scene, int thing, double step,
                         const float ambient[3], const float white[3], const float* image, const float* grad_image,
                         double* delta_plus, double* delta_minus, double* out, int nthreads) {
    const Cam c = to_cam(cam);
    const F3 amb = ld3(ambient), wht = ld3(white);
    const double f0 = wd->things[thing].fuzz;
    const double fp = f0 + step, fm = f0 - step;
    std::fill(delta_plus, delta_plus + size_t(w) * h * 3, 0.0);
    std::fill(delta_minus, delta_minus + size_t(w) * h * 3, 0.0);
    double replayed = 0, degenerate = 0, changed = 0, adj = 0;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
#pragma omp parallel reduction(+ : replayed, degenerate, changed, adj)
    {
        PathRec r0, rr;
#pragma omp for schedule(dynamic, 16)
        for (long pix = 0; pix < long(w) * long(h); ++pix) {
            const unsigned x = unsigned(pix % w), y = unsigned(pix / w);
            for (unsigned smp = 0; smp < spp; ++smp) {
                trace_path(*wd, c, x, y, w, h, depth, seed, scene, smp, amb, wht, &r0);
                if (!r0.miss) continue;
                bool touches = false;
                for (const Vtx& v : r0.vtx) touches |= (v.thing == thing && v.type == OPT_REFLECT);
                if (!touches) continue;
                D3 c0, cp, cm;
                if (!replay_held(*wd, c, r0, x, y, w, h, seed, scene, smp, amb, wht, thing, f0, c0, &rr) ||
                    !replay_held(*wd, c, r0, x, y, w, h, seed, scene, smp, amb, wht, thing, fp, cp) ||
                    !replay_held(*wd, c, r0, x, y, w, h, seed, scene, smp, amb, wht, thing, fm, cm)) {
                    degenerate += 1;
                    continue;
                }
                replayed += 1;
                const double inv = 1.0 / double(spp);
                if (image && grad_image) {   // the adjoint's term of this path, on the replayed trajectory
                    double g[3];
                    for (int ch = 0; ch < 3; ++ch) {
                        const float I = image[3 * pix + ch];
                        g[ch] = (I > 0.f && I < 1.f) ? double(grad_image[3 * pix + ch]) * inv : 0.0;
                    }
                    D3 thr{1, 1, 1};
                    for (const Vtx& v : rr.vtx)
                        if (v.type != OPT_REFRACT) {
                            const F3 a = wd->things[v.thing].albedo;
                            thr = D3{thr.x * a.x, thr.y * a.y, thr.z * a.z};
                        }
                    for (size_t k = 0; k < rr.vtx.size(); ++k) {
                        const Vtx& v = rr.vtx[k];
                        if (v.thing != thing || v.type != OPT_REFLECT) continue;
                        const D3 ds = tangent_to_sky(*wd, rr, k + 1, D3{0, 0, 0}, dd3(v.v), amb, wht);
                        adj += g[0] * thr.x * ds.x + g[1] * thr.y * ds.y + g[2] * thr.z * ds.z;
                    }
                }
                delta_plus[3 * pix + 0] += (cp.x - c0.x) * inv;
                delta_plus[3 * pix + 1] += (cp.y - c0.y) * inv;
                delta_plus[3 * pix + 2] += (cp.z - c0.z) * inv;
                delta_minus[3 * pix + 0] += (cm.x - c0.x) * inv;
                delta_minus[3 * pix + 1] += (cm.y - c0.y) * inv;
                delta_minus[3 * pix + 2] += (cm.z - c0.z) * inv;
                // would a plain re-render see this path jump?
                PathRec rp;
                for (float f : {float(fp), float(fm)}) {
                    trace_path_fuzz(*wd, c, x, y, w, h, depth, seed, scene, smp, amb, wht, thing, f, &rp);
                    bool same = rp.miss == r0.miss && rp.vtx.size() == r0.vtx.size();
                    for (size_t k = 0; same && k < rp.vtx.size(); ++k)
                        same = rp.vtx[k].prim == r0.vtx[k].prim && rp.vtx[k].branch == r0.vtx[k].branch;
                    if (!same) { changed += 1; break; }
                }
            }
        }
    }
    out[0] = replayed;
    out[1] = degenerate;
    out[2] = changed;
    out[3] = adj;
}

int orc_world_set_optics(orc_world* w, int thing, int type, const float albedo[3], float fuzz, float index) {
    if (thing < 0 || thing >= int(w->things.size())) return -1;
    Thing& t = w->things[thing];
    t.type = type; t.albedo = ld3(albedo); t.fuzz = fuzz; t.index = index;
    return 0;   // optics do not change the geometry: no rebuild needed
}

void orc_world_get_optics(const orc_world* w, int* types, float* albedos, float* fuzz, float* index) {
    for (size_t k = 0; k < w->things.size(); ++k) {
        const Thing& t = w->things[k];
        types[k] = t.type;
        st3(albedos + 3 * k, t.albedo);
        fuzz[k] = t.fuzz;
        index[k] = t.index;
    }
}

// Gradients of a scalar image loss L(I) given dL/dI (grad_image, w*h*3):
// per thing d/d albedo (3), d/d fuzz, and d/d ambient (3), d/d white (3).
// Each path is replayed exactly as rendered; visibility is held fixed.
void orc_adjoint(const orc_world* wd, const orc_camera* cam, unsigned w, unsigned h, unsigned spp,
                 unsigned depth, uint32_t seed, uint32_t scene, const float ambient[3],
                 const float white[3], const float* image, const float* grad_image,
                 double* grad_albedo, double* grad_fuzz, double* grad_sky, int nthreads) {
    const Cam c = to_cam(cam);
    const F3 amb = ld3(ambient), wht = ld3(white);
    const size_t nt = wd->things.size();
    std::fill(grad_albedo, grad_albedo + 3 * nt, 0.0);
    std::fill(grad_fuzz, grad_fuzz + nt, 0.0);
    std::fill(grad_sky, grad_sky + 6, 0.0);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
#pragma omp parallel
    {
        std::vector<double> ga(3 * nt, 0.0), gf(nt, 0.0), gs(6, 0.0);
        PathRec rec;
#pragma omp for schedule(dynamic, 16)
        for (long pix = 0; pix < long(w) * long(h); ++pix) {
            const unsigned x = unsigned(pix % w), y = unsigned(pix / w);
            double g[3];
            for (int ch = 0; ch < 3; ++ch) {
                const float I = image[3 * pix + ch];
                const double mask = (I > 0.f && I < 1.f) ? 1.0 : 0.0;   // clamp to [0,1]
                g[ch] = double(grad_image[3 * pix + ch]) * mask / double(spp);
            }
            if (g[0] == 0.0 && g[1] == 0.0 && g[2] == 0.0) continue;
            for (unsigned smp = 0; smp < spp; ++smp) {
                trace_path(*wd, c, x, y, w, h, depth, seed, scene, smp, amb, wht, &rec);
                if (!rec.miss) continue;   // absorbed or depth-limited: black, no gradient
                const size_t ne = rec.vtx.size();
                // albedo factors per event (glass: 1)
                std::vector<D3> a(ne);
                for (size_t k = 0; k < ne; ++k) {
                    const Vtx& v = rec.vtx[k];
                    a[k] = v.type == OPT_REFRACT ? D3{1, 1, 1} : dd3(wd->things[v.thing].albedo);
                }
                const D3 u = (1.0 / dlen(dd3(rec.d_last))) * dd3(rec.d_last);
                const double sv = 0.5 * (u.y + 1.0);
                const double skyc[3] = {(1.0 - sv) * wht.x + sv * amb.x, (1.0 - sv) * wht.y + sv * amb.y,
                                        (1.0 - sv) * wht.z + sv * amb.z};
                // prefix / suffix products of the albedos
                std::vector<D3> pre(ne + 1, D3{1, 1, 1}), suf(ne + 1, D3{1, 1, 1});
                for (size_t k = 0; k < ne; ++k)
                    pre[k + 1] = D3{pre[k].x * a[k].x, pre[k].y * a[k].y, pre[k].z * a[k].z};
                for (size_t k = ne; k-- > 0;)
                    suf[k] = D3{suf[k + 1].x * a[k].x, suf[k + 1].y * a[k].y, suf[k + 1].z * a[k].z};
                const D3 thr = pre[ne];
                const double th3[3] = {thr.x, thr.y, thr.z};
                for (int ch = 0; ch < 3; ++ch) {
                    gs[ch] += g[ch] * th3[ch] * sv;            // ambient
                    gs[3 + ch] += g[ch] * th3[ch] * (1.0 - sv); // white
                }
                for (size_t k = 0; k < ne; ++k) {
                    const Vtx& v = rec.vtx[k];
                    if (v.type == OPT_REFRACT) continue;
                    const double o3[3] = {pre[k].x * suf[k + 1].x, pre[k].y * suf[k + 1].y,
                                          pre[k].z * suf[k + 1].z};
                    for (int ch = 0; ch < 3; ++ch) ga[3 * size_t(v.thing) + ch] += g[ch] * o3[ch] * skyc[ch];
                    if (v.type == OPT_REFLECT) {
                        const D3 ds = tangent_to_sky(*wd, rec, k + 1, D3{0, 0, 0}, dd3(v.v), amb, wht);
                        gf[size_t(v.thing)] += g[0] * th3[0] * ds.x + g[1] * th3[1] * ds.y + g[2] * th3[2] * ds.z;
                    }
                }
            }
        }
#pragma omp critical
        {
            for (size_t i = 0; i < 3 * nt; ++i) grad_albedo[i] += ga[i];
            for (size_t i = 0; i < nt; ++i) grad_fuzz[i] += gf[i];
            for (int i = 0; i < 6; ++i) grad_sky[i] += gs[i];
        }
    }
}

// optx/postproc.cu:2-16: sRGB transfer curve, then x255 truncated.
void orc_pp_srgb(const float* src, uint8_t* dst, int w, int h) {
    auto curve = [](float x) { return x < .0031308f ? 12.92f * x : 1.055f * powf(x, 1.f / 2.4f) - .055f; };
    for (long p = 0; p < long(w) * h; ++p) {
        for (int k = 0; k < 3; ++k) dst[4 * p + k] = static_cast<unsigned char>(curve(src[3 * p + k]) * 255);
        dst[4 * p + 3] = 255;
    }
}

// optx/postproc.cu:18-34
void orc_pp_none(const float* src, uint8_t* dst, int w, int h) {
    for (long p = 0; p < long(w) * h; ++p) {
        for (int k = 0; k < 3; ++k) dst[4 * p + k] = static_cast<unsigned char>(src[3 * p + k] * 255);
        dst[4 * p + 3] = 255;
    }
}

// rtow.cxx:6-21: gamma 2 (square root), int(256 * clamp(x, 0, .999)), in binary32.
void orc_pp_gamma2(const float* src, uint8_t* dst, int w, int h) {
    for (long p = 0; p < long(w) * h; ++p) {
        for (int k = 0; k < 3; ++k) {
            float x = sqrtf(src[3 * p + k]);
            x = 0.f > x ? 0.f : (x > .999f ? .999f : x);
            dst[4 * p + k] = static_cast<unsigned char>(int(256.f * x));
        }
        dst[4 * p + 3] = 255;
    }
}

}  // extern "C"
