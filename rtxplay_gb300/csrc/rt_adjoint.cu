// rt_adjoint.cu -- adjoint path replay: gradients of an image loss with
// respect to per-thing albedo, metal fuzz and the two sky colours.
//
// The reference has no derivative path; this is the differentiable launch
// beside the forward renderer of rt_render.cu.  Method: path replay
// backpropagation (Vicini, Speierer, Jakob 2021): a path is not stored by the
// forward pass but replayed from its counter-based random stream, which
// reproduces the rendered path bit for bit (same camera ray, same closest
// hits, same scatter code); visibility is held fixed.
//
// Loss model: L = sum over pixels and channels of f(clamp(I, 0, 1)) where I
// is the rendered image; the caller passes dL/dI' (grad_image, with respect
// to the clamped image) and I itself.  A pixel channel on or beyond the clamp
// (I <= 0 or I >= 1) passes no gradient.  I = (1/spp) sum_s c_s, and a path
// contributes c = (prod_k a_k) * sky(d_last) only when it ends in a miss
// (absorbed and depth-limited paths are black).  Per path, with
// g = grad_image * mask / spp (one value per channel):
//   d/d albedo_k   = g * (prod_{i != k} a_i) * sky        (prefix x suffix products)
//   d/d ambient    = g * prod a * s,  d/d white = g * prod a * (1 - s),
//                    s = (unit(d_last).y + 1) / 2           (optx/camera_i.cu:133-139)
//   d/d fuzz_k     = g * prod a * d sky / d fuzz_k, a forward tangent from the
//                    metal vertex k (outgoing direction refl + fuzz v moves
//                    by v) through every later vertex to the miss: hit points
//                    move on the fixed surface, sphere normals turn with the
//                    hit point, reflection / refraction directions are
//                    differentiated, diffuse directions follow the normal.
// Each path's terms are binary32 products in the operation order of the FP64
// CPU restatement of the method (oracle/rt_oracle.cpp, orc_adjoint); a block
// sums them in binary32 in shared memory and adds its sums to double-precision
// totals.  GB300's FP64 rate made the all-double form of these terms the
// adjoint's bound (FP64 pipe 64 % busy); the totals agree with the FP64
// restatement to single precision.  The fuzz tangent keeps two double-precision
// steps where grazing geometry cancels digits (see tangent_to_sky).
#include <algorithm>
#include <cstring>
#include <vector>

#include "rt_scene.h"

namespace rt {
namespace {

constexpr int kAdjThreads = 128;
constexpr uint32_t kAdjPathsPerThread = 4;                     // paths per thread, block-strided
constexpr uint32_t kAdjPathsPerBlock = kAdjThreads * kAdjPathsPerThread;
constexpr uint32_t kAdjMaxDepth = 16;                          // at most 15 scatter vertices per path
constexpr uint32_t kAdjShThings = 1024;                        // per-block shared accumulators up to this many things

struct AdjJob {
    CamDev cam;
    float3 ambient, white;
    uint32_t W, H, npix, spp, depth, seed, key1;
    int root;
    int rtow_px;             // RT_FLAG_RTOW_PIXELS
    uint32_t thing_begin, nthings;
    unsigned long long path_offset;
    uint32_t pix_offset;     // first pixel of the job in the per-pixel gradient array
    const rt_float3* image;
    const rt_float3* grad_image;
};

struct D3 {
    double x, y, z;
};
__device__ __forceinline__ D3 dd3(float3 a) { return D3{double(a.x), double(a.y), double(a.z)}; }
__device__ __forceinline__ D3 operator+(D3 a, D3 b) { return D3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ D3 operator-(D3 a, D3 b) { return D3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ D3 operator*(double s, D3 a) { return D3{s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ double ddot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ double dlen(D3 a) { return sqrt(ddot(a, a)); }

// derivative of unit(d) along dd
__device__ __forceinline__ D3 dunit(D3 d, D3 dd) {
    const double l = dlen(d);
    const D3 u = (1.0 / l) * d;
    return (1.0 / l) * (dd - ddot(u, dd) * u);
}

// One scatter vertex of a replayed path.
struct AdjVtx {
    float3 d;        // incoming direction
    float t;         // hit distance
    float3 p, N;     // hit point, normal facing the incoming ray
    float3 v;        // metal: in-ball vector of the fuzz
    float ratio;     // glass: index ratio
    uint32_t thing;  // global thing (sphere centre / radius for the tangent)
    uint32_t bits;   // type | branch << 2 | front << 3
    float3 pre;      // product of the albedos before this vertex
};

// Forward tangent (dO, dD) of the ray entering vertex m, carried through
// vertices m..ne-1 to the miss direction d_last; returns d(unit(d_last).y)/d(.)
// (the sky's derivative is 0.5 times this times (ambient - white) per
// channel).  Mostly binary32 (GB300's FP64 rate made an all-double version 45 %
// of the adjoint's time); the two places where grazing geometry cancels
// digits stay in double: the projection onto the surface plane (n.q / n.d,
// with n = p - c exact for spheres) and the refraction branch (1 - |perp|^2
// near total internal reflection).
__device__ float tangent_to_sky(const AdjVtx* V, uint32_t m, uint32_t ne, const FlatDesc* __restrict__ desc, float3 dO,
                                float3 dD, float3 d_last) {
    for (uint32_t k = m; k < ne; ++k) {
        const AdjVtx& v = V[k];
        const FlatDesc& fd = desc[v.thing];
        const bool sphere = fd.analytic != 0;
        const int type = int(v.bits & 3u);
        const int branch = int((v.bits >> 2) & 1u);
        const bool front = ((v.bits >> 3) & 1u) != 0;
        const float3 d = v.d, N = v.N;
        // hit point on the fixed surface: dp = q - d (n.q)/(n.d), q = dO + t dD
        const float3 q = add(dO, mul(v.t, dD));
        const D3 n = sphere ? dd3(v.p) - dd3(xyz(fd.sphere)) : dd3(N);
        const double nd = ddot(n, dd3(d));   // both dot products exact to double rounding,
        const double nq = ddot(n, dd3(q));   // their quotient then needs single precision only
        const float3 dp = nd != 0.0 ? sub(q, mul(float(nq) / float(nd), d)) : q;
        float3 dN = mk(0.f, 0.f, 0.f);
        if (sphere) dN = mul((front ? 1.f : -1.f) / fd.sphere.w, dp);   // N = +-(p - c) / r
        float3 dOut;
        if (type == RT_OPTICS_DIFFUSE) {
            dOut = dN;   // d' = N + u, or N
        } else {
            const float il = 1.f / sqrtf(dot(d, d));
            const float3 d1 = mul(il, d);
            const float3 dd1 = mul(il, sub(dD, mul(dot(d1, dD), d1)));
            const bool refl = type == RT_OPTICS_REFLECT || branch == 0;
            if (refl) {
                const float c = dot(d1, N);
                const float dc = dot(dd1, N) + dot(d1, dN);
                dOut = sub(dd1, mul(2.f, add(mul(dc, N), mul(c, dN))));
            } else {
                const D3 dd = dd3(d), DN = dd3(N), dDd = dd3(dD), dNd = dd3(dN);
                const D3 e1 = (1.0 / dlen(dd)) * dd;
                const D3 de1 = dunit(dd, dDd);
                const double ratio = v.ratio;
                const double raw = -ddot(e1, DN);
                const double cth = raw < 1.0 ? raw : 1.0;
                const double dcth = raw < 1.0 ? -(ddot(de1, DN) + ddot(e1, dNd)) : 0.0;
                const D3 perp = ratio * (e1 + cth * DN);
                const D3 dperp = ratio * (de1 + (dcth * DN) + cth * dNd);
                const double qq = ddot(perp, perp);
                const double sroot = sqrt(fabs(1.0 - qq));
                const double dq = 2.0 * ddot(perp, dperp);
                const double ds = sroot > 0.0 ? ((1.0 - qq) >= 0.0 ? -dq : dq) / (2.0 * sroot) : 0.0;
                const D3 o = dperp - ((ds * DN) + sroot * dNd);
                dOut = mk(float(o.x), float(o.y), float(o.z));
            }
        }
        dO = dp;
        dD = dOut;
    }
    const float il = 1.f / sqrtf(dot(d_last, d_last));
    const float3 u = mul(il, d_last);
    return il * (dD.y - dot(u, dD) * u.y);
}

__device__ __forceinline__ uint32_t adj_job_of(const AdjJob* __restrict__ jobs, uint32_t nj, unsigned long long g) {
    uint32_t lo = 0, hi = nj;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (jobs[mid].path_offset <= g) lo = mid; else hi = mid;
    }
    return lo;
}

// Gradient sinks of one block: per-thing sums of the block's first job in
// shared memory (4 floats per thing: albedo rgb, fuzz), everything else in
// the global double sums G (4 per global thing, then 6 sky values per job).
struct Sink {
    float* sh;          // shared sums of job j0, or nullptr
    uint32_t j0;
    double* G;
    uint32_t nthings_total;
    __device__ __forceinline__ void add(uint32_t jx, const AdjJob& j, uint32_t thing, int c, float x) const {
        if (x == 0.f) return;
        if (sh && jx == j0) atomicAdd(sh + 4 * (thing - j.thing_begin) + c, x);
        else atomicAdd(G + 4 * size_t(thing) + c, double(x));
    }
};

// Replays global path `path` and adds its gradient terms.  Returns 1 when the
// traversal stack overflowed.
__device__ uint32_t adjoint_path(const AdjJob* __restrict__ jobs, uint32_t nj, unsigned long long path, const GeoView& geo,
                                 const ThingDev* __restrict__ things, const float* __restrict__ gpix, const Sink& sink,
                                 float gsky[6]) {
    const uint32_t jx = adj_job_of(jobs, nj, path);
    const AdjJob& j = jobs[jx];
    const uint32_t pid = uint32_t(path - j.path_offset);
    const uint32_t pix = pid / j.spp, smp = pid % j.spp;   // pixel-major, as the forward wavefront
    float g[3];
    {
        const float* gp = gpix + 3 * (size_t(j.pix_offset) + pix);
        g[0] = gp[0];
        g[1] = gp[1];
        g[2] = gp[2];
    }
    if (g[0] == 0.f && g[1] == 0.f && g[2] == 0.f) return 0;

    float3 o, d;
    {
        Stream s(j.seed, j.key1, pix, smp, 0);
        camera_ray(j.cam, pix % j.W, pix / j.W, j.W, j.H, j.rtow_px != 0, s, o, d);
    }
    AdjVtx V[kAdjMaxDepth - 1];
    uint32_t ne = 0;
    bool miss = false;
    float3 pre = mk(1.f, 1.f, 1.f);
    for (uint32_t k = 0;; ++k) {
        uint32_t nv = 0, nt = 0;
        const HitRec h = closest_hit_any<false>(geo, j.root, o, d, nv, nt);
        if (h.overflow) return 1;
        if (!h.hit) {
            miss = true;
            break;
        }
        if (k + 1 >= j.depth) break;   // black at the depth limit
        Stream s(j.seed, j.key1, pix, smp, k + 1);
        const float4 h4 = make_float4(h.t, h.u, h.v, 0.f);
        float4 pa, pb, pc;
        world_prim(geo.desc, h.thing, h.id, pa, pb, pc);
        const ScatterOut so = scatter(pa, pb, pc, things, o, d, h4, s);
        AdjVtx& v = V[ne];
        v.d = d;
        v.t = h.t;
        v.p = so.p;
        v.N = so.N;
        v.v = so.v;
        v.ratio = so.ratio;
        v.thing = h.thing;
        v.bits = uint32_t(so.type) | (uint32_t(so.branch) << 2) | (uint32_t(so.front) << 3);
        v.pre = pre;
        const float3 a = so.type == RT_OPTICS_REFRACT ? mk(1.f, 1.f, 1.f) : xyz(things[v.thing].albedo_type);
        pre = mulv(pre, a);
        ++ne;
        if (!so.cont) break;   // absorbed
        o = so.p;
        d = so.dir;
    }
    if (!miss) return 0;   // absorbed or depth-limited: black, no gradient

    const float3 u = mul(1.f / len(d), d);
    const float sv = .5f * (u.y + 1.f);
    const float skyc[3] = {(1.f - sv) * j.white.x + sv * j.ambient.x, (1.f - sv) * j.white.y + sv * j.ambient.y,
                           (1.f - sv) * j.white.z + sv * j.ambient.z};
    const float th3[3] = {pre.x, pre.y, pre.z};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        gsky[c] += g[c] * th3[c] * sv;              // ambient
        gsky[3 + c] += g[c] * th3[c] * (1.f - sv);  // white
    }
    float3 suf = mk(1.f, 1.f, 1.f);
    for (uint32_t k = ne; k-- > 0;) {
        const AdjVtx& v = V[k];
        const int type = int(v.bits & 3u);
        if (type == RT_OPTICS_REFRACT) continue;   // albedo factor 1: suffix unchanged
        const float3 o3 = mulv(v.pre, suf);
        sink.add(jx, j, v.thing, 0, g[0] * o3.x * skyc[0]);
        sink.add(jx, j, v.thing, 1, g[1] * o3.y * skyc[1]);
        sink.add(jx, j, v.thing, 2, g[2] * o3.z * skyc[2]);
        if (type == RT_OPTICS_REFLECT) {
            const float duy = tangent_to_sky(V, k + 1, ne, geo.desc, mk(0.f, 0.f, 0.f), v.v, d);
            const float ds = .5f * duy;
            const float3 dsc = mk(ds * (j.ambient.x - j.white.x), ds * (j.ambient.y - j.white.y),
                                  ds * (j.ambient.z - j.white.z));
            sink.add(jx, j, v.thing, 3, g[0] * th3[0] * dsc.x + g[1] * th3[1] * dsc.y + g[2] * th3[2] * dsc.z);
        }
        suf = mulv(suf, xyz(things[v.thing].albedo_type));
    }
    return 0;
}

// Per pixel and channel, the loss gradient each of the pixel's paths carries:
// g = dL/dI' * [0 < I < 1] / spp (once per pixel instead of once per path).
__global__ void k_adjoint_pixel_g(const AdjJob* __restrict__ jobs, uint32_t nj, uint32_t total_pix,
                                  float* __restrict__ gpix) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= total_pix) return;
    uint32_t lo = 0, hi = nj;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (jobs[mid].pix_offset <= p) lo = mid; else hi = mid;
    }
    const AdjJob& j = jobs[lo];
    const uint32_t pix = p - j.pix_offset;
    const rt_float3 I = j.image[pix], GI = j.grad_image[pix];
    const float Ic[3] = {I.x, I.y, I.z}, Gc[3] = {GI.x, GI.y, GI.z};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const double mask = (Ic[c] > 0.f && Ic[c] < 1.f) ? 1.0 : 0.0;   // clamp to [0, 1]
        gpix[3 * size_t(p) + c] = float(double(Gc[c]) * mask / double(j.spp));
    }
}

// One block: kAdjPathsPerBlock consecutive global paths, thread-strided.
// Four resident blocks per SM cap the registers at 128 per thread.  Lanes
// claiming their warp's next path from a shared counter as soon as they finish
// (instead of the fixed stride) measured 2 % slower (3.60 vs 3.52 ms, C3).
__global__ void __launch_bounds__(kAdjThreads, 4)
    k_adjoint(const AdjJob* __restrict__ jobs, uint32_t nj, unsigned long long total, GeoView geo,
              const ThingDev* __restrict__ things, const float* __restrict__ gpix, double* G, uint32_t nthings_total,
              uint32_t sh_things, uint32_t* err) {
    extern __shared__ float sh[];   // [4 * sh_things] + [6]
    const unsigned long long base = (unsigned long long)blockIdx.x * kAdjPathsPerBlock;
    const uint32_t j0 = adj_job_of(jobs, nj, base);
    const bool use_sh = jobs[j0].nthings <= sh_things;
    const uint32_t nsh = use_sh ? 4 * jobs[j0].nthings : 0;
    for (uint32_t i = threadIdx.x; i < nsh + 6; i += blockDim.x) sh[i] = 0.f;
    __syncthreads();
    Sink sink{use_sh ? sh : nullptr, j0, G, nthings_total};
    float gsky[6] = {0, 0, 0, 0, 0, 0};
    uint32_t my_err = 0;
    for (uint32_t c = 0; c < kAdjPathsPerThread; ++c) {
        const unsigned long long path = base + c * kAdjThreads + threadIdx.x;
        if (path >= total) break;
        const uint32_t jx = adj_job_of(jobs, nj, path);
        if (jx == j0) {
            my_err |= adjoint_path(jobs, nj, path, geo, things, gpix, sink, gsky);
        } else {   // a block that straddles two jobs: sky terms of the later job go straight to G
            float gs[6] = {0, 0, 0, 0, 0, 0};
            my_err |= adjoint_path(jobs, nj, path, geo, things, gpix, sink, gs);
            for (int k = 0; k < 6; ++k)
                if (gs[k] != 0.f) atomicAdd(G + 4 * size_t(nthings_total) + 6 * size_t(jx) + k, double(gs[k]));
        }
    }
    if (my_err) atomicOr(err, 1u);
    // sky sums of job j0: warp reduction, then one shared atomic per warp
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        float x = gsky[k];
        for (int off = 16; off > 0; off >>= 1) x += __shfl_down_sync(0xFFFFFFFFu, x, off);
        if ((threadIdx.x & 31u) == 0 && x != 0.f) atomicAdd(sh + nsh + k, x);
    }
    __syncthreads();
    const size_t tb = jobs[j0].thing_begin;
    for (uint32_t i = threadIdx.x; i < nsh; i += blockDim.x) {
        const float x = sh[i];
        if (x != 0.f) atomicAdd(G + 4 * tb + i, double(x));
    }
    if (threadIdx.x < 6) {
        const float x = sh[nsh + threadIdx.x];
        if (x != 0.f) atomicAdd(G + 4 * size_t(nthings_total) + 6 * size_t(j0) + threadIdx.x, double(x));
    }
}

struct AdjOut {
    double* albedo;   // [nthings x 3]
    double* fuzz;     // [nthings]
    double* sky;      // [6]
    uint32_t thing_begin, nthings;
};

// Scatters the global sums into each job's output arrays.
__global__ void k_adjoint_out(const double* __restrict__ G, uint32_t nthings_total, const AdjOut* __restrict__ outs,
                              uint32_t nj) {
    const uint32_t jx = blockIdx.y;
    if (jx >= nj) return;
    const AdjOut o = outs[jx];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < o.nthings; i += gridDim.x * blockDim.x) {
        const double* src = G + 4 * size_t(o.thing_begin + i);
        if (o.albedo) {
            o.albedo[3 * size_t(i)] = src[0];
            o.albedo[3 * size_t(i) + 1] = src[1];
            o.albedo[3 * size_t(i) + 2] = src[2];
        }
        if (o.fuzz) o.fuzz[i] = src[3];
    }
    if (blockIdx.x == 0 && threadIdx.x < 6 && o.sky)
        o.sky[threadIdx.x] = G[4 * size_t(nthings_total) + 6 * size_t(jx) + threadIdx.x];
}

// ORs the launch's error word into a caller's word (launches inside a stream
// capture, which read nothing back).
__global__ void k_or_error(const uint32_t* __restrict__ err, uint32_t* sticky) {
    if (*err) atomicOr(sticky, *err);
}

}  // namespace

struct AdjointWorkspace {
    DevBuf jobs, outs, G, err, gpix;
    std::vector<AdjJob> jobs_host, jobs_uploaded;
    std::vector<AdjOut> outs_host, outs_uploaded;
};

AdjointWorkspace* adjoint_workspace_new() { return new AdjointWorkspace(); }
void adjoint_workspace_free(AdjointWorkspace* ws) { delete ws; }

namespace {
AdjointWorkspace& adj_workspace() {
    static thread_local AdjointWorkspace ws;
    return ws;
}

template <class T>
bool same_table(const std::vector<T>& a, const std::vector<T>& b) {
    return a.size() == b.size() && std::memcmp(a.data(), b.data(), a.size() * sizeof(T)) == 0;
}
}  // namespace

// Inside a stream capture the adjoint enqueues its work without reading back:
// the job and output tables must be the ones the workspace already holds and
// no buffer may grow (both hold after the same call ran once outside the
// capture), and the error word is ORed into `sticky` for a later check.
void adjoint_jobs(const Geometry& g, const std::vector<AdjointJob>& jobs, cudaStream_t s, AdjointWorkspace* own,
                  uint32_t* sticky) {
    NvtxRange nvtx("rt adjoint");
    RT_REQUIRE(!jobs.empty(), "no adjoint jobs");
    RT_REQUIRE(jobs.size() < (1u << 24), "too many jobs (>= 2^24)");
    const bool capturing = stream_capturing(s);
    RT_REQUIRE(!capturing || sticky, "this adjoint cannot run inside a stream capture");
    CaptureNoAlloc no_alloc(capturing);
    AdjointWorkspace& ws = own ? *own : adj_workspace();
    const uint32_t nj = uint32_t(jobs.size());
    ws.jobs_host.resize(nj);
    ws.outs_host.resize(nj);
    unsigned long long total = 0;
    uint64_t total_pix = 0;
    uint32_t max_things = 0;
    for (uint32_t k = 0; k < nj; ++k) {
        const AdjointJob& a = jobs[k];
        check_params(&a.params);
        RT_REQUIRE(a.params.depth <= kAdjMaxDepth, "adjoint depth must be <= 16");
        RT_REQUIRE(a.image && a.grad_image, "image / grad_image is NULL");
        RT_REQUIRE(a.seg < g.nsegs, "job segment out of range");
        AdjJob& d = ws.jobs_host[k];
        std::memset(&d, 0, sizeof(d));
        d.cam = cam_dev(a.cam);
        d.ambient = make_float3(a.params.ambient.x, a.params.ambient.y, a.params.ambient.z);
        d.white = make_float3(a.params.white.x, a.params.white.y, a.params.white.z);
        d.W = a.params.image_w;
        d.H = a.params.image_h;
        d.npix = d.W * d.H;
        d.spp = a.params.spp;
        d.depth = a.params.depth;
        d.seed = a.params.seed;
        d.key1 = 0;
        d.root = g.root(a.seg);
        d.rtow_px = (a.params.flags & RT_FLAG_RTOW_PIXELS) ? 1 : 0;
        d.thing_begin = g.thing_begin[a.seg];
        d.nthings = (a.seg + 1 < g.nsegs ? g.thing_begin[a.seg + 1] : g.nthings) - d.thing_begin;
        d.path_offset = total;
        d.pix_offset = uint32_t(total_pix);
        d.image = a.image;
        d.grad_image = a.grad_image;
        total += (unsigned long long)d.npix * d.spp;
        total_pix += d.npix;
        max_things = std::max(max_things, d.nthings);
        ws.outs_host[k] = AdjOut{a.grad_albedo, a.grad_fuzz, a.grad_sky, d.thing_begin, d.nthings};
    }
    RT_REQUIRE(total_pix < (uint64_t(1) << 31), "too many pixels in one launch (>= 2^31)");
    const size_t gsize = (4 * size_t(g.nthings) + 6 * size_t(nj)) * sizeof(double);
    ws.gpix.reserve(std::max<size_t>(1, total_pix) * 3 * sizeof(float));
    ws.jobs.reserve(nj * sizeof(AdjJob));
    ws.outs.reserve(nj * sizeof(AdjOut));
    ws.G.reserve(gsize);
    ws.err.reserve(4);
    if (capturing) {
        RT_REQUIRE(same_table(ws.jobs_host, ws.jobs_uploaded) && same_table(ws.outs_host, ws.outs_uploaded),
                   "the adjoint's job table differs from the workspace's: make the same call once before capturing");
    } else {
        RT_CUDA(cudaMemcpyAsync(ws.jobs.p, ws.jobs_host.data(), nj * sizeof(AdjJob), cudaMemcpyHostToDevice, s));
        RT_CUDA(cudaMemcpyAsync(ws.outs.p, ws.outs_host.data(), nj * sizeof(AdjOut), cudaMemcpyHostToDevice, s));
        ws.jobs_uploaded = ws.jobs_host;
        ws.outs_uploaded = ws.outs_host;
    }
    RT_CUDA(cudaMemsetAsync(ws.G.p, 0, gsize, s));
    RT_CUDA(cudaMemsetAsync(ws.err.p, 0, 4, s));
    const uint32_t sh_things = std::min(max_things, kAdjShThings);
    const size_t shmem = (4 * size_t(sh_things) + 6) * sizeof(float);
    if (total) {
        k_adjoint_pixel_g<<<unsigned((total_pix + 255) / 256), 256, 0, s>>>(ws.jobs.as<AdjJob>(), nj,
                                                                           uint32_t(total_pix), ws.gpix.as<float>());
        RT_CHECK_LAUNCH();
        const unsigned grid = unsigned((total + kAdjPathsPerBlock - 1) / kAdjPathsPerBlock);
        GeoView gv = g.view();
        gv.err = ws.err.as<uint32_t>();
        k_adjoint<<<grid, kAdjThreads, shmem, s>>>(ws.jobs.as<AdjJob>(), nj, total, gv,
                                                   g.things_dev.as<ThingDev>(), ws.gpix.as<float>(),
                                                   ws.G.as<double>(), g.nthings, sh_things, ws.err.as<uint32_t>());
        RT_CHECK_LAUNCH();
    }
    const unsigned gx = std::max(1u, std::min(64u, (max_things + 255) / 256));
    k_adjoint_out<<<dim3(gx, nj), 256, 0, s>>>(ws.G.as<double>(), g.nthings, ws.outs.as<AdjOut>(), nj);
    RT_CHECK_LAUNCH();
    if (capturing) {
        k_or_error<<<1, 1, 0, s>>>(ws.err.as<uint32_t>(), sticky);
        RT_CHECK_LAUNCH();
        return;
    }
    uint32_t herr = 0;
    RT_CUDA(cudaMemcpyAsync(&herr, ws.err.p, 4, cudaMemcpyDeviceToHost, s));
    RT_CUDA(cudaStreamSynchronize(s));
    if (herr & kErrBounds) throw Error(RT_ERR_INTERNAL, "bounds check failed (RT_CHECKS build)");
    if (herr) throw Error(RT_ERR_LIMIT, "traversal stack overflow (LBVH deeper than the stack)");
}

}  // namespace rt

using namespace rt;

extern "C" {

rt_status rt_adjoint_launch(rt_scene scene, const rt_camera* cam, const rt_launch_params* params,
                            const rt_float3* image, const rt_float3* grad_image, double* grad_albedo,
                            double* grad_fuzz, double* grad_sky, void* stream) {
    return guarded([&] {
        RT_REQUIRE(cam && params, "cam/params is NULL");
        Scene& sc = *scene_from(scene);
        if (!sc.built || sc.topology_dirty) throw Error(RT_ERR_NOT_BUILT, "scene not built (call rt_scene_build)");
        if (sc.xf_dirty) throw Error(RT_ERR_NOT_BUILT, "transforms changed; call rt_scene_update");
        cudaStream_t s = as_stream(stream);
        sync_optics(sc.geo, {&sc}, s);
        std::vector<AdjointJob> jobs(1);
        jobs[0] = AdjointJob{0, *cam, *params, image, grad_image, grad_albedo, grad_fuzz, grad_sky};
        adjoint_jobs(sc.geo, jobs, s);
    });
}

}  // extern "C"
