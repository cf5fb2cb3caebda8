// rt_render.cu -- wavefront path tracer, first-hit/picker kernels, post-processing.
//
// Replaces Launcher::ignite + optixLaunch (optx/launcher.cxx:49-77) and the
// OptiX programs __raygen__camera / __miss__ambient (optx/camera_i.cu:24-141)
// and __closesthit__diffuse/reflect/refract (optx/optics_i.cu:23-288), plus
// pp_sRGB / pp_none (optx/postproc.cu).
//
// Design: paths are numbered pid = sample_in_chunk * npix + pixel.  A wave
// queue of W rays (SoA float4 arrays) is traversed by `extend` (one thread per
// ray, closest hit over the LBVH) and resolved by `shade` (miss/sky, depth
// limit, Lambertian / metal / dielectric scatter).  A path that ends writes
// its colour and ray count to its own slot of a per-chunk result buffer and is
// replaced in the same thread by the next camera path (one atomic per warp);
// continuing and new rays are appended to the next queue with a warp ballot
// and one atomic per warp.  After a chunk of samples drains, `accumulate` adds
// each pixel's samples in sample order, so the image does not depend on the
// order in which paths finished and equals the sequential CPU sum bit for bit.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "rt_scene.h"

namespace rt {
namespace {

constexpr int kThreads = 256;
inline unsigned grid_for(uint64_t n, int threads = kThreads) { return unsigned((n + threads - 1) / threads); }

struct WaveState {
    uint32_t count[2];       // rays in queue 0 / 1
    uint32_t next_path;      // next path id to start (chunk-relative)
    uint32_t err;            // nonzero: a traversal stack overflowed
    uint32_t fetch[2];       // next ray of queue 0 / 1 to hand to a persistent traversal lane
    unsigned long long nodes, prims, rays;
};

struct RenderArgs {
    CamDev cam;
    uint32_t W, H, npix;
    uint32_t spp, depth, seed, scene_id;
    uint32_t sample_base;    // first sample of this chunk
    uint32_t npaths;         // paths in this chunk
    float3 ambient, white;
    int guides;
};

struct Queue {
    float4* ori;   // origin.xyz, path id
    float4* dir;   // direction.xyz, bounce
    float4* thr;   // throughput.rgb
    float4* gn;    // guide normal (guides only)
    float4* ga;    // guide albedo (guides only)
};

struct Results {
    float4* col;   // colour.rgb, rays (as float)
    float4* gn;
    float4* ga;
};

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }

// Camera path pid of the chunk: primary ray + queue entry.
__device__ __forceinline__ void make_camera_ray(const RenderArgs& a, uint32_t pid, float3& o, float3& d) {
    const uint32_t pixel = pid % a.npix;
    const uint32_t sample = a.sample_base + pid / a.npix;
    Stream s(a.seed, a.scene_id, pixel, sample, 0);
    camera_ray(a.cam, pixel % a.W, pixel / a.W, a.W, a.H, s, o, d);
}

__global__ void __launch_bounds__(kThreads) k_generate(RenderArgs a, Queue q, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float3 o, d;
    make_camera_ray(a, i, o, d);
    q.ori[i] = make_float4(o.x, o.y, o.z, __uint_as_float(i));
    q.dir[i] = make_float4(d.x, d.y, d.z, __uint_as_float(0u));
    q.thr[i] = make_float4(1.f, 1.f, 1.f, 0.f);
    if (a.guides) {
        q.gn[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        q.ga[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
}

__global__ void k_set_state(WaveState* st, uint32_t n0) {
    st->count[0] = n0;
    st->count[1] = 0;
    st->next_path = n0;
    st->fetch[0] = 0;
    st->fetch[1] = 0;
}

// Persistent traversal: a grid sized to the resident blocks; every lane that
// finishes its ray takes the next one of the queue, so lanes do not idle while
// the rest of their warp is still traversing.  A warp looks for new rays every
// kInner traversal steps and refills once at least kRefill lanes are free
// (one atomic per warp per refill).
template <bool kCount, int kInner, int kRefill>
__global__ void __launch_bounds__(kThreads)
    k_extend_p(const float4* __restrict__ q_ori, const float4* __restrict__ q_dir, float4* __restrict__ hits,
               WaveState* st, int cur, const float4* __restrict__ nodes, const float4* __restrict__ prims,
               uint32_t nprims) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        st->count[cur ^ 1] = 0;   // the next queue starts empty
        st->fetch[cur ^ 1] = 0;
    }
    const uint32_t n = *((volatile uint32_t*)&st->count[cur]);
    const uint32_t lane = lane_id();
    const uint32_t lanemask_lt = (1u << lane) - 1u;
    Trav s;
    int stack[kStackSize];
    int ray = -1;
    bool exhausted = false;   // warp-uniform: the queue has no rays left to hand out
    uint32_t nvis = 0, ntest = 0;
    while (true) {
        const uint32_t idle = __ballot_sync(0xFFFFFFFFu, ray < 0);
        if (!exhausted && (idle == 0xFFFFFFFFu || __popc(idle) >= kRefill)) {
            const int leader = __ffs(idle) - 1;
            uint32_t base = 0;
            if (int(lane) == leader) base = atomicAdd(&st->fetch[cur], uint32_t(__popc(idle)));
            base = __shfl_sync(0xFFFFFFFFu, base, leader);
            if (base + uint32_t(__popc(idle)) >= n) exhausted = true;
            if (ray < 0) {
                const uint32_t idx = base + __popc(idle & lanemask_lt);
                if (idx < n) {
                    ray = int(idx);
                    const float4 o4 = q_ori[idx], d4 = q_dir[idx];
                    trav_init(s, xyz(o4), xyz(d4));
                }
            }
        }
        if (__ballot_sync(0xFFFFFFFFu, ray >= 0) == 0) break;
        if (ray >= 0) {
            for (int k = 0; k < kInner; ++k) {
                if (nprims == 0 || !trav_step<kCount>(s, stack, nodes, prims, nvis, ntest)) {
                    hits[ray] = make_float4(s.h.t, s.h.u, s.h.v, __int_as_float(s.h.leaf));
                    if (s.h.overflow) atomicOr(&st->err, 1u);
                    ray = -1;
                    break;
                }
            }
        }
    }
    if (kCount) {
        for (int o = 16; o > 0; o >>= 1) {
            nvis += __shfl_down_sync(0xFFFFFFFFu, nvis, o);
            ntest += __shfl_down_sync(0xFFFFFFFFu, ntest, o);
        }
        if (lane == 0 && (nvis | ntest)) {
            atomicAdd(&st->nodes, (unsigned long long)nvis);
            atomicAdd(&st->prims, (unsigned long long)ntest);
        }
    }
}

// One thread per queued ray.
template <bool kCount>
__global__ void __launch_bounds__(kThreads)
    k_extend(const float4* __restrict__ q_ori, const float4* __restrict__ q_dir, float4* __restrict__ hits,
             WaveState* st, int cur, const float4* __restrict__ nodes, const float4* __restrict__ prims,
             uint32_t nprims) {
    if (blockIdx.x == 0 && threadIdx.x == 0) st->count[cur ^ 1] = 0;   // the next queue starts empty
    const uint32_t n = *((volatile uint32_t*)&st->count[cur]);
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t nvis = 0, ntest = 0;
    if (i < n) {
        const float4 o4 = q_ori[i], d4 = q_dir[i];
        const HitRec h = closest_hit<kCount>(nodes, prims, nprims, xyz(o4), xyz(d4), nvis, ntest);
        hits[i] = make_float4(h.t, h.u, h.v, __int_as_float(h.leaf));
        if (h.overflow) atomicOr(&st->err, 1u);
    }
    if (kCount) {
        for (int o = 16; o > 0; o >>= 1) {
            nvis += __shfl_down_sync(0xFFFFFFFFu, nvis, o);
            ntest += __shfl_down_sync(0xFFFFFFFFu, ntest, o);
        }
        if (lane_id() == 0 && (nvis | ntest)) {
            atomicAdd(&st->nodes, (unsigned long long)nvis);
            atomicAdd(&st->prims, (unsigned long long)ntest);
        }
    }
}

// Traversal kernel variants, chosen per launch by name (RTX_EXTEND) or the
// default; each has a plain and a counting instantiation.
using ExtendFn = void (*)(const float4*, const float4*, float4*, WaveState*, int, const float4*, const float4*,
                          uint32_t);
struct ExtendVariant {
    const char* name;
    ExtendFn fn[2];     // [counting]
    bool persistent;
};
// Measured on C1 (1200x800, 64 spp): plain 1194-1241 Mrays/s; persistent
// lanes raise the active lanes per instruction from 12.0 to 16.6 of 32 but add
// 35% instructions to an issue-bound kernel (1172 Mrays/s, refill 8, 1 step).
const ExtendVariant kExtendVariants[] = {
    {"plain", {k_extend<false>, k_extend<true>}, false},
    {"persistent", {k_extend_p<false, 4, 16>, k_extend_p<true, 4, 16>}, true},
};
constexpr int kNumExtendVariants = int(sizeof(kExtendVariants) / sizeof(kExtendVariants[0]));
constexpr int kDefaultExtend = 0;

__device__ __forceinline__ float3 sky(float3 d, float3 ambient, float3 white) {
    // optx/camera_i.cu:133-139
    const float3 unit = unitV(d);
    const float t = .5f * (unit.y + 1.f);
    return add(mul(1.f - t, white), mul(t, ambient));
}

__global__ void __launch_bounds__(kThreads) k_shade(RenderArgs a, Queue cur, Queue nxt, const float4* __restrict__ hits,
                                                    WaveState* st, int ci, const float4* __restrict__ prims,
                                                    const ThingDev* __restrict__ things, Results res) {
    const uint32_t n = *((volatile uint32_t*)&st->count[ci]);
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t lane = lane_id();
    if (i - lane >= n) return;   // whole warp past the queue end
    const bool active = i < n;

    bool cont = false, ended = false;
    float3 no{}, nd{}, nthr{};
    float3 gN{}, gA{};
    uint32_t pid = 0, bounce = 0;
    if (active) {
        const float4 o4 = cur.ori[i], d4 = cur.dir[i], t4 = cur.thr[i], h4 = hits[i];
        pid = __float_as_uint(o4.w);
        bounce = __float_as_uint(d4.w);
        const float3 o = xyz(o4), d = xyz(d4);
        float3 thr = xyz(t4);
        if (a.guides) {
            gN = xyz(cur.gn[i]);
            gA = xyz(cur.ga[i]);
        }
        const int leaf = __float_as_int(h4.w);
        float3 color = mk(0.f, 0.f, 0.f);
        if (leaf < 0) {
            color = mulv(thr, sky(d, a.ambient, a.white));
            ended = true;
        } else if (bounce + 1 >= a.depth) {
            ended = true;   // black at the depth limit (optx/optics_r.cu:34-42)
        } else {
            const float4 pa = __ldg(prims + 3 * leaf), pb = __ldg(prims + 3 * leaf + 1), pc = __ldg(prims + 3 * leaf + 2);
            const uint32_t thing = __float_as_uint(pa.w);
            const ThingDev th = things[thing];
            const int type = __float_as_int(th.albedo_type.w);
            const float3 albedo = xyz(th.albedo_type);
            // hit geometry: optx/optics_i.cu:40-82 (triangles), sphere.h:40-46 (spheres)
            float3 p, N;
            bool front;
            if (__float_as_uint(pc.w) == kPrimTriangle) {
                const float3 A = xyz(pa), B = xyz(pb), C = xyz(pc);
                const float u = h4.y, v = h4.z;
                const float w = 1.f - u - v;
                p = add(add(mul(w, A), mul(u, B)), mul(v, C));
                N = unitV(cross(sub(B, A), sub(C, A)));
                if (dot(d, N) > 0.f) N = neg(N);
                front = 0.f > dot(d, sub(p, xyz(th.center_fuzz)));   // optx/optics_i.cu:259-267
            } else {
                p = add(o, mul(h4.x, d));
                const float3 outward = mul(1.f / pb.x, sub(p, xyz(pa)));
                front = 0.f > dot(d, outward);
                N = front ? outward : neg(outward);
            }
            const uint32_t pixel = pid % a.npix;
            const uint32_t sample = a.sample_base + pid / a.npix;
            Stream s(a.seed, a.scene_id, pixel, sample, bounce + 1);
            if (type == RT_OPTICS_DIFFUSE) {
                // optx/optics_i.cu:87-96, near-zero fallback of optics.h:17-18
                float3 dir = add(N, rndVon1sphere(s));
                if (near0(dir)) dir = N;
                thr = mulv(thr, albedo);
                if (isnull(gN)) gN = N;
                if (isnull(gA)) gA = albedo;
                no = p; nd = dir; nthr = thr; cont = true;
            } else if (type == RT_OPTICS_REFLECT) {
                // optx/optics_i.cu:168-190
                const float3 d1V = unitV(d);
                const float3 refl = sub(d1V, mul(2.f * dot(d1V, N), N));
                const float3 dir = add(refl, mul(th.center_fuzz.w, rndVin1sphere(s)));
                if (isnull(gN)) gN = N;
                if (isnull(gA)) gA = albedo;
                if (dot(dir, N) > 0.f) {
                    thr = mulv(thr, albedo);
                    no = p; nd = dir; nthr = thr; cont = true;
                } else {
                    ended = true;   // absorbed: black
                }
            } else {
                // optx/optics_i.cu:254-283, Schlick's pow 5 as products
                const float3 d1V = unitV(d);
                const float cos_theta = fminf(dot(neg(d1V), N), 1.f);
                const float sin_theta = sqrtf(1.f - cos_theta * cos_theta);
                const float index = th.index_pad.x;
                const float ratio = front ? 1.f / index : index;
                const bool cannot = ratio * sin_theta > 1.f;
                float r0 = (1.f - ratio) / (1.f + ratio);
                r0 = r0 * r0;
                const float om = 1.f - cos_theta;
                const float pow5 = ((om * om) * (om * om)) * om;
                const float schlick = r0 + (1.f - r0) * pow5;
                float3 dir;
                if (cannot || schlick > s.next()) {
                    dir = sub(d1V, mul(2.f * dot(d1V, N), N));
                } else {
                    const float theta = fminf(dot(neg(d1V), N), 1.f);
                    const float3 perpen = mul(ratio, add(d1V, mul(theta, N)));
                    const float3 parall = mul(-sqrtf(fabsf(1.f - dot(perpen, perpen))), N);
                    dir = add(perpen, parall);
                }
                no = p; nd = dir; nthr = thr; cont = true;
            }
        }
        if (ended) {
            const uint32_t slot = pid;   // chunk-relative path id
            res.col[slot] = make_float4(color.x, color.y, color.z, float(bounce + 1));
            if (a.guides) {
                res.gn[slot] = make_float4(gN.x, gN.y, gN.z, 0.f);
                res.ga[slot] = make_float4(gA.x, gA.y, gA.z, 0.f);
            }
        }
    }

    // regenerate: every ended path is replaced by the next camera path
    const uint32_t want = __ballot_sync(0xFFFFFFFFu, ended);
    uint32_t new_pid = 0xFFFFFFFFu;
    if (want) {
        uint32_t base = 0;
        if (lane == uint32_t(__ffs(want) - 1)) base = atomicAdd(&st->next_path, uint32_t(__popc(want)));
        base = __shfl_sync(0xFFFFFFFFu, base, __ffs(want) - 1);
        if (ended) {
            const uint32_t cand = base + __popc(want & ((1u << lane) - 1u));
            if (cand < a.npaths) new_pid = cand;
        }
    }
    bool fresh = false;
    if (new_pid != 0xFFFFFFFFu) {
        make_camera_ray(a, new_pid, no, nd);
        nthr = mk(1.f, 1.f, 1.f);
        gN = mk(0.f, 0.f, 0.f);
        gA = mk(0.f, 0.f, 0.f);
        pid = new_pid;
        bounce = 0;
        fresh = true;
    } else if (cont) {
        bounce += 1;
    }
    const bool push = cont || fresh;
    const uint32_t pm = __ballot_sync(0xFFFFFFFFu, push);
    if (pm) {
        uint32_t base = 0;
        if (lane == uint32_t(__ffs(pm) - 1)) base = atomicAdd(&st->count[ci ^ 1], uint32_t(__popc(pm)));
        base = __shfl_sync(0xFFFFFFFFu, base, __ffs(pm) - 1);
        if (push) {
            const uint32_t slot = base + __popc(pm & ((1u << lane) - 1u));
            nxt.ori[slot] = make_float4(no.x, no.y, no.z, __uint_as_float(pid));
            nxt.dir[slot] = make_float4(nd.x, nd.y, nd.z, __uint_as_float(bounce));
            nxt.thr[slot] = make_float4(nthr.x, nthr.y, nthr.z, 0.f);
            if (a.guides) {
                nxt.gn[slot] = make_float4(gN.x, gN.y, gN.z, 0.f);
                nxt.ga[slot] = make_float4(gA.x, gA.y, gA.z, 0.f);
            }
        }
    }
}

// Adds the chunk's samples of every pixel in sample order (optx/camera_i.cu:95-101).
__global__ void __launch_bounds__(kThreads) k_accumulate(Results res, uint32_t npix, uint32_t nsamples, int first,
                                                         int guides, float4* __restrict__ acc,
                                                         uint32_t* __restrict__ acc_rays, float4* __restrict__ acc_n,
                                                         float4* __restrict__ acc_a) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npix) return;
    float3 c = first ? mk(0.f, 0.f, 0.f) : xyz(acc[p]);
    uint32_t rays = first ? 0u : acc_rays[p];
    float3 gn = mk(0.f, 0.f, 0.f), ga = mk(0.f, 0.f, 0.f);
    if (guides && !first) {
        gn = xyz(acc_n[p]);
        ga = xyz(acc_a[p]);
    }
    for (uint32_t s = 0; s < nsamples; ++s) {
        const size_t slot = size_t(s) * npix + p;
        const float4 r = res.col[slot];
        c = add(c, xyz(r));
        rays += uint32_t(r.w);
        if (guides) {
            gn = add(gn, xyz(res.gn[slot]));
            ga = add(ga, xyz(res.ga[slot]));
        }
    }
    acc[p] = make_float4(c.x, c.y, c.z, 0.f);
    acc_rays[p] = rays;
    if (guides) {
        acc_n[p] = make_float4(gn.x, gn.y, gn.z, 0.f);
        acc_a[p] = make_float4(ga.x, ga.y, ga.z, 0.f);
    }
}

__device__ __forceinline__ float clamp01(float x) { return 0.f > x ? 0.f : (x > 1.f ? 1.f : x); }

// optx/camera_i.cu:104-113: mean = 1/spp * sum clamped to [0,1]; rpp; guides.
__global__ void __launch_bounds__(kThreads) k_finalize(const float4* __restrict__ acc, const uint32_t* __restrict__ acc_rays,
                                                       const float4* __restrict__ acc_n, const float4* __restrict__ acc_a,
                                                       uint32_t npix, uint32_t spp, rt_float3* rawRGB, uint32_t* rpp,
                                                       rt_float3* normals, rt_float3* albedos, WaveState* st) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long r = 0;
    if (p < npix) {
        const float inv = 1.f / float(spp);
        const float3 m = mul(inv, xyz(acc[p]));
        rawRGB[p] = rt_float3{clamp01(m.x), clamp01(m.y), clamp01(m.z)};
        r = acc_rays[p];
        if (rpp) rpp[p] = acc_rays[p];
        if (normals) {
            const float3 n = mul(inv, xyz(acc_n[p]));
            normals[p] = rt_float3{n.x, n.y, n.z};
        }
        if (albedos) {
            const float3 al = mul(inv, xyz(acc_a[p]));
            albedos[p] = rt_float3{al.x, al.y, al.z};
        }
    }
    for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xFFFFFFFFu, r, o);
    if (lane_id() == 0 && r) atomicAdd(&st->rays, r);
}

// FP64 distance from the (binary32) ray to the selected primitive: the
// binary32 Moller-Trumbore t loses digits on grazing hits (its error grows
// like 1/sin of the grazing angle), so the reported distance re-evaluates the
// winner in double precision; the selection itself stays binary32.
__device__ double dist64(const float4* __restrict__ rec, float3 of, float3 df) {
    const float4 a = __ldg(rec), b = __ldg(rec + 1), c = __ldg(rec + 2);
    const double o[3] = {of.x, of.y, of.z}, d[3] = {df.x, df.y, df.z};
    if (__float_as_uint(c.w) == kPrimTriangle) {
        const double A[3] = {a.x, a.y, a.z}, B[3] = {b.x, b.y, b.z}, C[3] = {c.x, c.y, c.z};
        const double e1[3] = {B[0] - A[0], B[1] - A[1], B[2] - A[2]};
        const double e2[3] = {C[0] - A[0], C[1] - A[1], C[2] - A[2]};
        const double pv[3] = {d[1] * e2[2] - d[2] * e2[1], d[2] * e2[0] - d[0] * e2[2], d[0] * e2[1] - d[1] * e2[0]};
        const double det = e1[0] * pv[0] + e1[1] * pv[1] + e1[2] * pv[2];
        if (det == 0.0) return __longlong_as_double(0x7FF8000000000000ll);
        const double tv[3] = {o[0] - A[0], o[1] - A[1], o[2] - A[2]};
        const double qv[3] = {tv[1] * e1[2] - tv[2] * e1[1], tv[2] * e1[0] - tv[0] * e1[2],
                              tv[0] * e1[1] - tv[1] * e1[0]};
        return (e2[0] * qv[0] + e2[1] * qv[1] + e2[2] * qv[2]) / det;
    }
    const double oc[3] = {o[0] - a.x, o[1] - a.y, o[2] - a.z};
    const double qa = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    const double qb = d[0] * oc[0] + d[1] * oc[1] + d[2] * oc[2];
    const double qc = (oc[0] * oc[0] + oc[1] * oc[1] + oc[2] * oc[2]) - double(b.x) * b.x;
    const double disc = qb * qb - qa * qc;
    if (disc < 0.0) return __longlong_as_double(0x7FF8000000000000ll);
    const double x = sqrt(disc);
    double t = (-qb - x) / qa;
    if (t < double(kTmin)) t = (-qb + x) / qa;
    return t;
}

// Primary-ray closest hit of one sample for a pixel rectangle.
__global__ void __launch_bounds__(kThreads) k_first_hit(RenderArgs a, uint32_t sample, uint32_t x0, uint32_t y0,
                                                        uint32_t nx, uint32_t ny, const float4* __restrict__ nodes,
                                                        const float4* __restrict__ prims, uint32_t nprims, int* prim,
                                                        int* thing, float* t, float* u, float* v, double* t64,
                                                        uint32_t* err) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nx * ny) return;
    const uint32_t x = x0 + k % nx, y = y0 + k / nx;
    const uint32_t pixel = a.W * y + x;
    Stream s(a.seed, a.scene_id, pixel, sample, 0);
    float3 o, d;
    camera_ray(a.cam, x, y, a.W, a.H, s, o, d);
    uint32_t nv = 0, nt = 0;
    const HitRec h = closest_hit<false>(nodes, prims, nprims, o, d, nv, nt);
    if (h.overflow) atomicOr(err, 1u);
    if (h.leaf < 0) {
        prim[k] = -1;
        if (thing) thing[k] = -1;
        if (t) t[k] = 0.f;
        if (u) u[k] = 0.f;
        if (v) v[k] = 0.f;
        if (t64) t64[k] = __longlong_as_double(0x7FF8000000000000ll);
        return;
    }
    prim[k] = int(h.id);
    if (thing) thing[k] = int(__float_as_uint(__ldg(prims + 3 * h.leaf).w));
    if (t) t[k] = h.t;
    if (u) u[k] = h.u;
    if (v) v[k] = h.v;
    if (t64) t64[k] = dist64(prims + 3 * h.leaf, o, d);
}

// ------------------------------------------------------------ post-process
__device__ __forceinline__ unsigned char to_byte(float c) {
    const float s = c * 255;
    return static_cast<unsigned char>(s < 0.f ? 0.f : (s > 255.f ? 255.f : s));
}

// optx/postproc.cu:2-16: sRGB curve (exponent 1/2.4), x255 truncated.
__device__ __forceinline__ float srgb_curve(float x) {
    return x < .0031308f ? 12.92f * x : 1.055f * powf(x, 1.f / 2.4f) - .055f;
}

__global__ void k_pp(const rt_float3* __restrict__ src, rt_uchar4* __restrict__ dst, int n, int mode) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const rt_float3 s = src[p];
    rt_uchar4 o;
    if (mode == 0) {          // none: optx/postproc.cu:18-34
        o = rt_uchar4{to_byte(s.x), to_byte(s.y), to_byte(s.z), 255};
    } else if (mode == 1) {   // sRGB: optx/postproc.cu:36-47
        o = rt_uchar4{to_byte(srgb_curve(s.x)), to_byte(srgb_curve(s.y)), to_byte(srgb_curve(s.z)), 255};
    } else {                  // gamma 2: rtow.cxx:6-21
        auto g = [](float x) {
            float r = sqrtf(x);
            r = 0.f > r ? 0.f : (r > .999f ? .999f : r);
            return static_cast<unsigned char>(int(256.f * r));
        };
        o = rt_uchar4{g(s.x), g(s.y), g(s.z), 255};
    }
    dst[p] = o;
}

// -------------------------------------------------------------- host side
CamDev cam_dev(const rt_camera& c) {
    CamDev d;
    d.eye = make_float3(c.eye.x, c.eye.y, c.eye.z);
    d.u = make_float3(c.u.x, c.u.y, c.u.z);
    d.v = make_float3(c.v.x, c.v.y, c.v.z);
    d.w = make_float3(c.w.x, c.w.y, c.w.z);
    d.hvec = make_float3(c.hvec.x, c.hvec.y, c.hvec.z);
    d.wvec = make_float3(c.wvec.x, c.wvec.y, c.wvec.z);
    d.dvec = make_float3(c.dvec.x, c.dvec.y, c.dvec.z);
    d.aperture = c.aperture;
    return d;
}

void check_params(const rt_launch_params* p) {
    RT_REQUIRE(p != nullptr, "params is NULL");
    RT_REQUIRE(p->image_w > 0 && p->image_h > 0, "image size must be positive");
    RT_REQUIRE(uint64_t(p->image_w) * p->image_h <= (uint64_t(1) << 28), "image has more than 2^28 pixels");
    RT_REQUIRE(p->spp >= 1, "spp must be >= 1");
    RT_REQUIRE(p->depth >= 1 && p->depth <= 255, "depth must be 1..255");
}

RenderArgs make_args(const rt_camera& cam, const rt_launch_params& p) {
    RenderArgs a{};
    a.cam = cam_dev(cam);
    a.W = p.image_w;
    a.H = p.image_h;
    a.npix = p.image_w * p.image_h;
    a.spp = p.spp;
    a.depth = p.depth;
    a.seed = p.seed;
    a.scene_id = 0;
    a.ambient = make_float3(p.ambient.x, p.ambient.y, p.ambient.z);
    a.white = make_float3(p.white.x, p.white.y, p.white.z);
    a.guides = (p.flags & RT_FLAG_GUIDES) ? 1 : 0;
    return a;
}

uint32_t env_u32(const char* name, uint32_t dflt) {
    const char* v = std::getenv(name);
    if (!v || !*v) return dflt;
    const unsigned long x = std::strtoul(v, nullptr, 10);
    return x ? uint32_t(x) : dflt;
}

// Per-thread render workspace (queues, results, accumulators), grow-only.
struct Workspace {
    DevBuf q[2][5];
    DevBuf hits, res_col, res_gn, res_ga, acc, acc_rays, acc_n, acc_a, state;
    uint32_t* host_count = nullptr;   // pinned
    std::vector<cudaEvent_t> events;
    ~Workspace() {
        if (host_count) cudaFreeHost(host_count);
        for (auto e : events) cudaEventDestroy(e);
    }
    cudaEvent_t event(size_t k) {
        while (events.size() <= k) {
            cudaEvent_t e;
            RT_CUDA(cudaEventCreate(&e));
            events.push_back(e);
        }
        return events[k];
    }
};

Workspace& workspace() {
    static thread_local Workspace ws;
    return ws;
}

// Resident blocks of a traversal kernel on this device (persistent grids).
unsigned resident_grid(ExtendFn fn) {
    int per_sm = 0;
    RT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kThreads, 0));
    return unsigned(std::max(1, per_sm) * sm_count());
}

// Traversal variant of this process: RTX_EXTEND=<name> or the default.
int extend_variant() {
    static int v = -1;
    if (v < 0) {
        v = kDefaultExtend;
        const char* e = std::getenv("RTX_EXTEND");
        for (int k = 0; e && k < kNumExtendVariants; ++k)
            if (std::strcmp(e, kExtendVariants[k].name) == 0) v = k;
    }
    return v;
}

void render(Scene& sc, const rt_camera& cam, const rt_launch_params& p, const rt_frame& f, cudaStream_t s,
            rt_launch_stats* stats) {
    check_params(&p);
    RT_REQUIRE(f.rawRGB != nullptr, "frame.rawRGB is NULL");
    const bool guides = (p.flags & RT_FLAG_GUIDES) != 0;
    RT_REQUIRE(!guides || (f.normals && f.albedos), "RT_FLAG_GUIDES needs frame.normals and frame.albedos");
    if (!sc.built || sc.topology_dirty) throw Error(RT_ERR_NOT_BUILT, "scene not built (call rt_scene_build)");
    if (sc.xf_dirty) throw Error(RT_ERR_NOT_BUILT, "transforms changed; call rt_scene_update");
    const bool timing = (p.flags & RT_FLAG_STAGE_TIMING) != 0;
    const bool count = (p.flags & RT_FLAG_COUNT_VISITS) != 0;

    Workspace& ws = workspace();
    RenderArgs a = make_args(cam, p);
    const uint32_t npix = a.npix;
    // chunk of samples whose per-path results fit the result budget
    const uint64_t budget = uint64_t(env_u32("RTX_RESULT_MB", 1024)) << 20;
    const uint64_t per_sample = uint64_t(npix) * 16u * (guides ? 3u : 1u);
    uint32_t chunk = uint32_t(std::max<uint64_t>(1, budget / per_sample));
    chunk = std::min(chunk, p.spp);
    chunk = uint32_t(std::min<uint64_t>(chunk, (uint64_t(1) << 31) / npix));
    chunk = std::max(chunk, 1u);
    const uint64_t max_paths = uint64_t(npix) * chunk;
    const uint32_t W = uint32_t(std::min<uint64_t>(env_u32("RTX_WAVE", 1u << 21), max_paths));

    for (int b = 0; b < 2; ++b) {
        for (int k = 0; k < 3; ++k) ws.q[b][k].reserve(size_t(W) * 16);
        if (guides) for (int k = 3; k < 5; ++k) ws.q[b][k].reserve(size_t(W) * 16);
    }
    ws.hits.reserve(size_t(W) * 16);
    ws.res_col.reserve(size_t(max_paths) * 16);
    if (guides) {
        ws.res_gn.reserve(size_t(max_paths) * 16);
        ws.res_ga.reserve(size_t(max_paths) * 16);
        ws.acc_n.reserve(size_t(npix) * 16);
        ws.acc_a.reserve(size_t(npix) * 16);
    }
    ws.acc.reserve(size_t(npix) * 16);
    ws.acc_rays.reserve(size_t(npix) * 4);
    ws.state.reserve(sizeof(WaveState));
    if (!ws.host_count) RT_CUDA(cudaMallocHost(&ws.host_count, 64));

    Queue q[2];
    for (int b = 0; b < 2; ++b) {
        q[b].ori = ws.q[b][0].as<float4>();
        q[b].dir = ws.q[b][1].as<float4>();
        q[b].thr = ws.q[b][2].as<float4>();
        q[b].gn = guides ? ws.q[b][3].as<float4>() : nullptr;
        q[b].ga = guides ? ws.q[b][4].as<float4>() : nullptr;
    }
    Results res{ws.res_col.as<float4>(), guides ? ws.res_gn.as<float4>() : nullptr,
                guides ? ws.res_ga.as<float4>() : nullptr};
    WaveState* st = ws.state.as<WaveState>();
    RT_CUDA(cudaMemsetAsync(st, 0, sizeof(WaveState), s));

    const float4* nodes = sc.nodes.as<float4>();
    const float4* prims = sc.prims.as<float4>();
    const ThingDev* things = sc.things_dev.as<ThingDev>();
    uint32_t launches = 1, waves = 0, ext_launches = 0;
    size_t ev = 0;
    std::vector<std::pair<size_t, int>> timed;   // (event index, 0 extend / 1 shade)
    const unsigned qgrid = grid_for(W);
    const uint32_t kBatch = 8;
    const ExtendVariant& xv = kExtendVariants[extend_variant()];
    const ExtendFn ext_fn = xv.fn[count ? 1 : 0];
    const unsigned ext_grid = xv.persistent ? std::min<unsigned>(qgrid, resident_grid(ext_fn)) : qgrid;
    float4* hits_buf = ws.hits.as<float4>();
    uint32_t nprims = sc.nprims;

    for (uint32_t s0 = 0; s0 < p.spp; s0 += chunk) {
        const uint32_t ns = std::min(chunk, p.spp - s0);
        a.sample_base = s0;
        a.npaths = npix * ns;
        const uint32_t n0 = std::min<uint32_t>(W, a.npaths);
        k_set_state<<<1, 1, 0, s>>>(st, n0);
        k_generate<<<grid_for(n0), kThreads, 0, s>>>(a, q[0], n0);
        RT_CHECK_LAUNCH();
        launches += 2;
        // wave loop bound: while paths remain to start the queue holds n0 rays,
        // and a path is queued at most `depth` times, so the loop ends within
        // npaths*depth/n0 + depth iterations
        const uint64_t max_iters = uint64_t(a.npaths) * a.depth / n0 + a.depth + 2 * kBatch;
        uint32_t it = 0;
        while (true) {
            for (uint32_t b = 0; b < kBatch; ++b, ++it) {
                const int ci = int(it & 1u);
                if (timing) {
                    RT_CUDA(cudaEventRecord(ws.event(ev), s));
                    timed.push_back({ev, 0});
                    ev += 2;
                }
                {
                    const float4* qo = q[ci].ori;
                    const float4* qd = q[ci].dir;
                    int cur = ci;
                    void* args[] = {&qo, &qd, &hits_buf, &st, &cur, &nodes, &prims, &nprims};
                    RT_CUDA(cudaLaunchKernel(reinterpret_cast<const void*>(ext_fn), dim3(ext_grid), dim3(kThreads),
                                             args, 0, s));
                }
                if (timing) {
                    RT_CUDA(cudaEventRecord(ws.event(ev - 1), s));
                    RT_CUDA(cudaEventRecord(ws.event(ev), s));
                    timed.push_back({ev, 1});
                    ev += 2;
                }
                k_shade<<<qgrid, kThreads, 0, s>>>(a, q[ci], q[ci ^ 1], ws.hits.as<float4>(), st, ci, prims, things, res);
                if (timing) RT_CUDA(cudaEventRecord(ws.event(ev - 1), s));
                RT_CHECK_LAUNCH();
                launches += 2;
                ext_launches += 1;
            }
            RT_CUDA(cudaMemcpyAsync(ws.host_count, &st->count[it & 1u], 4, cudaMemcpyDeviceToHost, s));
            RT_CUDA(cudaStreamSynchronize(s));
            if (*ws.host_count == 0) break;
            if (it > max_iters) throw Error(RT_ERR_LIMIT, "wave loop did not drain");
        }
        waves += it;
        k_accumulate<<<grid_for(npix), kThreads, 0, s>>>(res, npix, ns, s0 == 0 ? 1 : 0, guides ? 1 : 0,
                                                          ws.acc.as<float4>(), ws.acc_rays.as<uint32_t>(),
                                                          guides ? ws.acc_n.as<float4>() : nullptr,
                                                          guides ? ws.acc_a.as<float4>() : nullptr);
        RT_CHECK_LAUNCH();
        launches += 1;
    }
    k_finalize<<<grid_for(npix), kThreads, 0, s>>>(ws.acc.as<float4>(), ws.acc_rays.as<uint32_t>(),
                                                    guides ? ws.acc_n.as<float4>() : nullptr,
                                                    guides ? ws.acc_a.as<float4>() : nullptr, npix, p.spp, f.rawRGB,
                                                    f.rpp, guides ? f.normals : nullptr, guides ? f.albedos : nullptr,
                                                    st);
    RT_CHECK_LAUNCH();
    launches += 1;
    WaveState hs;
    RT_CUDA(cudaMemcpyAsync(&hs, st, sizeof(hs), cudaMemcpyDeviceToHost, s));
    RT_CUDA(cudaStreamSynchronize(s));
    if (hs.err) throw Error(RT_ERR_LIMIT, "traversal stack overflow (LBVH deeper than the stack)");
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        stats->rays = hs.rays;
        stats->paths = uint64_t(npix) * p.spp;
        stats->node_visits = hs.nodes;
        stats->prim_tests = hs.prims;
        stats->waves = waves;
        stats->kernel_launches = launches;
        stats->extend_launches = ext_launches;
        stats->wave_capacity = W;
        if (timing) {
            for (auto& tv : timed) {
                float ms = 0.f;
                RT_CUDA(cudaEventElapsedTime(&ms, ws.event(tv.first), ws.event(tv.first + 1)));
                (tv.second == 0 ? stats->extend_ms : stats->shade_ms) += ms;
            }
        }
    }
}

void first_hit_rect(Scene& sc, const rt_camera& cam, const rt_launch_params& p, uint32_t sample, uint32_t x0,
                    uint32_t y0, uint32_t nx, uint32_t ny, int* prim, int* thing, float* t, float* u, float* v,
                    double* t64, cudaStream_t s) {
    check_params(&p);
    if (!sc.built || sc.topology_dirty || sc.xf_dirty) throw Error(RT_ERR_NOT_BUILT, "scene not built or not updated");
    RT_REQUIRE(prim != nullptr, "prim is NULL");
    const RenderArgs a = make_args(cam, p);
    uint32_t* err = sc.misc.as<uint32_t>();
    RT_CUDA(cudaMemsetAsync(err, 0, 4, s));
    k_first_hit<<<grid_for(uint64_t(nx) * ny), kThreads, 0, s>>>(a, sample, x0, y0, nx, ny, sc.nodes.as<float4>(),
                                                                  sc.prims.as<float4>(), sc.nprims, prim, thing, t, u, v,
                                                                  t64, err);
    RT_CHECK_LAUNCH();
    uint32_t herr = 0;
    RT_CUDA(cudaMemcpyAsync(&herr, err, 4, cudaMemcpyDeviceToHost, s));
    RT_CUDA(cudaStreamSynchronize(s));
    if (herr) throw Error(RT_ERR_LIMIT, "traversal stack overflow (LBVH deeper than the stack)");
}

void postproc(const rt_float3* src, rt_uchar4* dst, int w, int h, int mode, cudaStream_t s) {
    RT_REQUIRE(src != nullptr && dst != nullptr, "src/dst is NULL");
    RT_REQUIRE(w > 0 && h > 0, "w and h must be positive");
    const int n = w * h;
    k_pp<<<grid_for(uint64_t(n)), kThreads, 0, s>>>(src, dst, n, mode);
    RT_CHECK_LAUNCH();
}

struct Launcher {
    uint32_t w = 0, h = 0;
    DevBuf raw, rpp, nrm, alb, img, pick;
    void resize(uint32_t W, uint32_t H) {
        RT_REQUIRE(W > 0 && H > 0, "launcher size must be positive");
        const size_t n = size_t(W) * H;
        raw.reserve(n * 12);
        rpp.reserve(n * 4);
        nrm.reserve(n * 12);
        alb.reserve(n * 12);
        img.reserve(n * 4);
        pick.reserve(4);
        w = W;
        h = H;
    }
};

Launcher* launcher_from(rt_launcher l) {
    RT_REQUIRE(l != nullptr, "launcher handle is NULL");
    return reinterpret_cast<Launcher*>(l);
}

}  // namespace
}  // namespace rt

using namespace rt;

extern "C" {

rt_status rt_launch(rt_scene scene, const rt_camera* cam, const rt_launch_params* params, const rt_frame* frame,
                    void* stream) {
    return guarded([&] {
        RT_REQUIRE(cam && params && frame, "cam/params/frame is NULL");
        render(*scene_from(scene), *cam, *params, *frame, as_stream(stream), nullptr);
    });
}

rt_status rt_launch_ex(rt_scene scene, const rt_camera* cam, const rt_launch_params* params, const rt_frame* frame,
                       void* stream, rt_launch_stats* stats) {
    return guarded([&] {
        RT_REQUIRE(cam && params && frame && stats, "cam/params/frame/stats is NULL");
        render(*scene_from(scene), *cam, *params, *frame, as_stream(stream), stats);
    });
}

rt_status rt_first_hit(rt_scene scene, const rt_camera* cam, const rt_launch_params* params, unsigned int sample,
                       int* prim, int* thing, float* t, float* u, float* v, double* t64, void* stream) {
    return guarded([&] {
        RT_REQUIRE(cam && params, "cam/params is NULL");
        first_hit_rect(*scene_from(scene), *cam, *params, sample, 0, 0, params->image_w, params->image_h, prim, thing,
                       t, u, v, t64, as_stream(stream));
    });
}

rt_status rt_pick(rt_scene scene, const rt_camera* cam, const rt_launch_params* params, unsigned int x, unsigned int y,
                  unsigned int* thing_id, void* stream) {
    return guarded([&] {
        RT_REQUIRE(cam && params && thing_id, "cam/params/thing_id is NULL");
        RT_REQUIRE(x < params->image_w && y < params->image_h, "pick position outside the image");
        DevBuf buf;
        buf.reserve(8);
        cudaStream_t s = as_stream(stream);
        first_hit_rect(*scene_from(scene), *cam, *params, 0, x, y, 1, 1, buf.as<int>(), buf.as<int>() + 1, nullptr,
                       nullptr, nullptr, nullptr, s);
        int host[2];
        RT_CUDA(cudaMemcpyAsync(host, buf.p, 8, cudaMemcpyDeviceToHost, s));
        RT_CUDA(cudaStreamSynchronize(s));
        *thing_id = host[0] < 0 ? 0xFFFFFFFFu : unsigned(host[1]);
    });
}

rt_status rt_postproc_srgb(const rt_float3* src, rt_uchar4* dst, int w, int h, void* stream) {
    return guarded([&] { postproc(src, dst, w, h, 1, as_stream(stream)); });
}
rt_status rt_postproc_none(const rt_float3* src, rt_uchar4* dst, int w, int h, void* stream) {
    return guarded([&] { postproc(src, dst, w, h, 0, as_stream(stream)); });
}
rt_status rt_postproc_gamma2(const rt_float3* src, rt_uchar4* dst, int w, int h, void* stream) {
    return guarded([&] { postproc(src, dst, w, h, 2, as_stream(stream)); });
}

rt_status rt_launcher_create(rt_launcher* out, unsigned int w, unsigned int h) {
    return guarded([&] {
        RT_REQUIRE(out != nullptr, "out is NULL");
        auto* l = new Launcher();
        try {
            l->resize(w, h);
        } catch (...) {
            delete l;
            throw;
        }
        *out = reinterpret_cast<rt_launcher>(l);
    });
}

rt_status rt_launcher_destroy(rt_launcher l) {
    return guarded([&] {
        if (l) delete reinterpret_cast<Launcher*>(l);
    });
}

rt_status rt_launcher_resize(rt_launcher l, unsigned int w, unsigned int h) {
    return guarded([&] { launcher_from(l)->resize(w, h); });
}

rt_status rt_launcher_ignite(rt_launcher l, rt_scene scene, const rt_camera* cam, const rt_launch_params* params,
                             void* stream, int once, unsigned int pick_x, unsigned int pick_y, rt_launch_stats* stats) {
    return guarded([&] {
        Launcher* L = launcher_from(l);
        RT_REQUIRE(cam && params, "cam/params is NULL");
        RT_REQUIRE(params->image_w == L->w && params->image_h == L->h, "params size differs from the launcher size");
        Scene& sc = *scene_from(scene);
        cudaStream_t s = as_stream(stream);
        if (once) {
            RT_REQUIRE(pick_x < L->w && pick_y < L->h, "pick position outside the image");
            DevBuf buf;
            buf.reserve(8);
            first_hit_rect(sc, *cam, *params, 0, pick_x, pick_y, 1, 1, buf.as<int>(), buf.as<int>() + 1, nullptr,
                           nullptr, nullptr, nullptr, s);
            int host[2];
            RT_CUDA(cudaMemcpyAsync(host, buf.p, 8, cudaMemcpyDeviceToHost, s));
            RT_CUDA(cudaStreamSynchronize(s));
            const unsigned id = host[0] < 0 ? 0xFFFFFFFFu : unsigned(host[1]);
            RT_CUDA(cudaMemcpy(L->pick.p, &id, 4, cudaMemcpyHostToDevice));
            return;
        }
        rt_frame f{L->raw.as<rt_float3>(), L->rpp.as<unsigned>(), L->nrm.as<rt_float3>(), L->alb.as<rt_float3>()};
        render(sc, *cam, *params, f, s, stats);
        postproc(L->raw.as<rt_float3>(), L->img.as<rt_uchar4>(), int(L->w), int(L->h), 1, s);
        RT_CUDA(cudaStreamSynchronize(s));
    });
}

rt_status rt_launcher_frame(rt_launcher l, rt_frame* frame, rt_uchar4** image, unsigned int** pick_id) {
    return guarded([&] {
        Launcher* L = launcher_from(l);
        if (frame) *frame = rt_frame{L->raw.as<rt_float3>(), L->rpp.as<unsigned>(), L->nrm.as<rt_float3>(),
                                     L->alb.as<rt_float3>()};
        if (image) *image = L->img.as<rt_uchar4>();
        if (pick_id) *pick_id = L->pick.as<unsigned>();
    });
}

rt_status rt_launcher_download(rt_launcher l, rt_float3* rawRGB, unsigned int* rpp, rt_float3* normals,
                               rt_float3* albedos, rt_uchar4* image, unsigned int* pick_id) {
    return guarded([&] {
        Launcher* L = launcher_from(l);
        const size_t n = size_t(L->w) * L->h;
        if (rawRGB) RT_CUDA(cudaMemcpy(rawRGB, L->raw.p, n * 12, cudaMemcpyDeviceToHost));
        if (rpp) RT_CUDA(cudaMemcpy(rpp, L->rpp.p, n * 4, cudaMemcpyDeviceToHost));
        if (normals) RT_CUDA(cudaMemcpy(normals, L->nrm.p, n * 12, cudaMemcpyDeviceToHost));
        if (albedos) RT_CUDA(cudaMemcpy(albedos, L->alb.p, n * 12, cudaMemcpyDeviceToHost));
        if (image) RT_CUDA(cudaMemcpy(image, L->img.p, n * 4, cudaMemcpyDeviceToHost));
        if (pick_id) RT_CUDA(cudaMemcpy(pick_id, L->pick.p, 4, cudaMemcpyDeviceToHost));
    });
}

}  // extern "C"
