// rt_render.cu -- wavefront path tracer over one or many scenes, first-hit /
// picker kernels, post-processing, launcher and batch ABI.
//
// Replaces Launcher::ignite + optixLaunch (optx/launcher.cxx:49-77) and the
// OptiX programs __raygen__camera / __miss__ambient (optx/camera_i.cu:24-141)
// and __closesthit__diffuse/reflect/refract (optx/optics_i.cu:23-288), plus
// pp_sRGB / pp_none (optx/postproc.cu).
//
// Design: a render is a list of jobs (a scene segment of a geometry, its
// camera, parameters and output frame); a single-scene launch is a list of
// one.  Paths are numbered globally (job after job, pixel-major inside a
// job).  A wave queue of W rays (SoA float4 arrays) is traversed by `extend`
// (closest hit over the job's LBVH) and resolved by `shade` (miss/sky, depth
// limit, Lambertian / metal / dielectric scatter).  A path that ends adds its
// colour and ray count to its pixel in 64-bit fixed point (integer atomics,
// so the sums do not depend on the order in which paths finish); continuing
// rays are appended to the front of the next queue (a warp ballot, one atomic
// per block), and `fill` starts the next paths in path order in the free slots
// behind them.  A one-thread `ctrl` kernel advances the path counter, flips
// the queues and decides whether another wave runs; the wave loop runs either
// from the host (a status read every 8 waves) or inside a CUDA graph as a
// conditional WHILE node.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <vector>

#include "rt_scene.h"

namespace rt {

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
    RT_REQUIRE(uint64_t(p->image_w) * p->image_h * p->spp <= 0xFFFFFFFFull, "w*h*spp must fit in 32 bits");
    RT_REQUIRE(p->depth >= 1 && p->depth <= 255, "depth must be 1..255");
    RT_REQUIRE((p->flags & ~(RT_FLAG_GUIDES | RT_FLAG_STAGE_TIMING | RT_FLAG_COUNT_VISITS | RT_FLAG_RTOW_PIXELS)) == 0,
               "unknown flags");
    if (p->flags & RT_FLAG_RTOW_PIXELS)
        RT_REQUIRE(p->image_w >= 2 && p->image_h >= 2, "RT_FLAG_RTOW_PIXELS needs an image of at least 2x2");
}

namespace {

constexpr int kThreads = 256;
inline unsigned grid_for(uint64_t n, int threads = kThreads) { return unsigned((n + threads - 1) / threads); }

// Wave queues and hit records pass through L2 once per wave (a 2^26-ray
// wave's queue is 3.2 GB against 126 MB of L2): their loads and stores are
// evict-first (.cs), so they displace less of the hierarchy the traversal
// keeps re-reading.  C1 frame: traversal 336.9 -> 335.2 ms, shading 66.9 ->
// 65.5 ms, 3130 -> 3153 Mrays/s.
__device__ __forceinline__ float4 qld(const float4* p) { return __ldcs(p); }
__device__ __forceinline__ void qst(float4* p, float4 v) { __stcs(p, v); }

struct JobDev {              // one render job on the device
    CamDev cam;
    float3 ambient, white;
    uint32_t W, H, npix, spp, depth, seed, key1;
    uint32_t first_sample;   // sample index of the job's first sample (progressive rendering)
    uint32_t mean_spp;       // samples per pixel in the sums (spp, or more when accumulating)
    int root;                // root node of the job's scene, -1: empty scene
    uint32_t pix_offset;     // first pixel of the job in the accumulators
    int guides;
    int rtow_px;             // RT_FLAG_RTOW_PIXELS
    unsigned long long path_offset;   // first global path of the job
    rt_float3* rawRGB;
    uint32_t* rpp;
    rt_float3* normals;
    rt_float3* albedos;
};

struct WaveState {
    uint32_t count[2];       // rays in queue 0 / 1
    uint32_t front[2];       // continuing rays, slots [0, front) of queue 0 / 1
    uint32_t back[2];        // fresh camera rays, slots [cap - back, cap) of queue 0 / 1
    uint32_t cap;            // queue capacity
    uint32_t cur;            // queue of the current wave
    uint32_t iter;           // waves run
    uint32_t max_iter;       // exact upper bound of the waves
    uint32_t err;            // 1: traversal stack overflow, 2: wave bound exceeded
    uint32_t ext_next[2];    // next unclaimed ray of queue 0 / 1 (persistent traversal)
    unsigned long long next_path, total_paths;
    unsigned long long nodes, prims, rays;
};

struct Queue {
    float4* ori;   // origin.xyz, job-local pixel
    float4* dir;   // direction.xyz, (job << 8) | bounce
    float4* thr;   // throughput.rgb, sample
    float4* gn;    // guide normal (guides only)
    float4* ga;    // guide albedo (guides only)
};
struct Queues {
    Queue q[2];
};

// Per-pixel sums, structure of arrays over the launch's pixels: colour
// channels in 64-bit fixed point (2^-32 units), rays as u32, guide layers
// (normal xyz, albedo xyz) in fixed point.
struct Acc {
    unsigned long long* col[3];
    uint32_t* rays;
    unsigned long long* gd[6];
};

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }

__device__ __forceinline__ Queue pick(const Queues& qs, uint32_t k) { return k ? qs.q[1] : qs.q[0]; }

// Job of a global path / global pixel (jobs are ordered by both offsets).
__device__ __forceinline__ uint32_t job_of_path(const JobDev* __restrict__ jobs, uint32_t nj, unsigned long long g) {
    uint32_t lo = 0, hi = nj;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (jobs[mid].path_offset <= g) lo = mid; else hi = mid;
    }
    return lo;
}
__device__ __forceinline__ uint32_t job_of_pixel(const JobDev* __restrict__ jobs, uint32_t nj, uint32_t p) {
    uint32_t lo = 0, hi = nj;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (jobs[mid].pix_offset <= p) lo = mid; else hi = mid;
    }
    return lo;
}

// Camera ray of a job's pixel and sample.  Paths are numbered pixel-major
// (path = pixel * spp + sample; the queues carry pixel and sample, so shading
// divides once per path, not once per ray).  Consecutive paths are samples of
// one pixel, so the fresh rays of a block
// start inside one pixel footprint and their bounces leave from nearby points:
// measured on C1 (64 spp) against sample-major numbering, traversal -16 % and
// shading -22 % (1888 vs 1566 Mrays/s); the image does not change (every
// random number is keyed by pixel and sample).
__device__ __forceinline__ void make_camera_ray(const JobDev& j, uint32_t pixel, uint32_t sample, float3& o,
                                                float3& d) {
    Stream s(j.seed, j.key1, pixel, sample, 0);
    camera_ray(j.cam, pixel % j.W, pixel / j.W, j.W, j.H, j.rtow_px != 0, s, o, d);
}

// Queue slot of the i-th ray of a wave: continuing rays first, then the fresh
// camera rays from the back of the queue (kept apart so that the pixel-
// coherent primary rays share warps with each other, not with bounces).
__device__ __forceinline__ uint32_t wave_slot(const WaveState* st, uint32_t cur, uint32_t i) {
    const uint32_t f = st->front[cur];
    return i < f ? i : st->cap - st->back[cur] + (i - f);
}

__global__ void k_init_state(WaveState* st, uint32_t n0, unsigned long long total, uint32_t max_iter, uint32_t cap) {
    st->count[0] = n0;
    st->count[1] = 0;
    st->front[0] = n0;
    st->front[1] = 0;
    st->back[0] = 0;
    st->back[1] = 0;
    st->cap = cap;
    st->cur = 0;
    st->iter = 0;
    st->max_iter = max_iter;
    st->err = 0;
    st->ext_next[0] = st->ext_next[1] = 0;
    st->next_path = n0;
    st->total_paths = total;
    st->nodes = st->prims = st->rays = 0;
}

__global__ void __launch_bounds__(kThreads) k_generate(const JobDev* __restrict__ jobs, uint32_t nj, Queue q,
                                                       uint32_t n, int any_guides) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t jx = job_of_path(jobs, nj, i);
    const JobDev& j = jobs[jx];
    const uint32_t pid = uint32_t(i - j.path_offset);
    const uint32_t pixel = pid / j.spp, sample = j.first_sample + pid % j.spp;
    float3 o, d;
    make_camera_ray(j, pixel, sample, o, d);
    q.ori[i] = make_float4(o.x, o.y, o.z, __uint_as_float(pixel));
    q.dir[i] = make_float4(d.x, d.y, d.z, __uint_as_float(jx << 8));
    q.thr[i] = make_float4(1.f, 1.f, 1.f, __uint_as_float(sample));
    if (any_guides) {
        q.gn[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        q.ga[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
}

// Fresh paths of the next wave: the queue's free slots behind the continuing
// rays (slots [front, cap)) take the next paths in path order, as many as
// remain.  Path order is pixel-major, so consecutive claims of the next
// traversal are samples of one pixel.  A fixed grid (a graph node needs a
// fixed shape) of a few blocks per SM strides over the fresh paths, so a wave
// that needs few pays for few; k_wave_ctrl then advances next_path by the
// same count.  Moving the start of new paths here from the shading kernel
// took the path counter's block-wide aggregation, the camera-ray work and most
// of its register spills out of it (shading 100.4 -> 78.3 ms per C1 frame).
__device__ __forceinline__ uint32_t fresh_count(const WaveState* st, uint32_t nxt) {
    const unsigned long long rem = st->total_paths - st->next_path;
    const uint32_t room = st->cap - st->front[nxt];
    return rem < room ? uint32_t(rem) : room;
}

__global__ void __launch_bounds__(kThreads) k_fill(const JobDev* __restrict__ jobs, uint32_t nj, Queues qs,
                                                   const WaveState* st, int any_guides) {
    const uint32_t nxt = (*((volatile const uint32_t*)&st->cur)) ^ 1u;
    const uint32_t n = fresh_count(st, nxt);
    const unsigned long long base = st->next_path;
    const uint32_t cap = st->cap;
    const Queue Q = nxt ? qs.q[1] : qs.q[0];
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const unsigned long long g = base + t;
        const uint32_t jx = job_of_path(jobs, nj, g);
        const JobDev& j = jobs[jx];
        const uint32_t pid = uint32_t(g - j.path_offset);
        const uint32_t pixel = pid / j.spp, sample = j.first_sample + pid % j.spp;
        float3 o, d;
        make_camera_ray(j, pixel, sample, o, d);
        const uint32_t slot = cap - n + t;
        qst(Q.ori + slot, make_float4(o.x, o.y, o.z, __uint_as_float(pixel)));
        qst(Q.dir + slot, make_float4(d.x, d.y, d.z, __uint_as_float(jx << 8)));
        qst(Q.thr + slot, make_float4(1.f, 1.f, 1.f, __uint_as_float(sample)));
        if (any_guides) {
            Q.gn[slot] = make_float4(0.f, 0.f, 0.f, 0.f);
            Q.ga[slot] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
    }
}

// Refill rule of the persistent traversal (rt_tuning: refill_below,
// steps_per_check); the counting pass takes it too, unused, so both kernels
// share one signature.
struct ExtTune {
    uint32_t refill_below;
    int steps;
};

// One thread per queued ray (the counting pass; rendering uses the persistent
// k_extend_p below); kInst selects the two-level traversal.  Warp-cooperative
// traversal with parked leaf tests measured slower (active lanes 9.6 -> 12.9,
// 30 % more instructions: 803 vs 993 Mrays/s instanced, 64 spp); an earlier
// persistent form that refilled lanes eagerly cost 35 % more instructions.
// Writing the hit geometry (point, normal, facing) here instead, so shading
// needs no gather of the primitive, measured slower on C1 (1146 vs 1216
// Mrays/s, 64 spp): the shading time did not drop and traversal grew.
template <bool kCount, bool kInst>
__global__ void __launch_bounds__(kThreads)
    k_extend(Queues qs, float4* __restrict__ hits, uint32_t* __restrict__ hthing, WaveState* st,
             const JobDev* __restrict__ jobs, GeoView g, ExtTune) {
    const uint32_t cur = *((volatile uint32_t*)&st->cur);
    if (blockIdx.x == 0 && threadIdx.x == 0) {   // the next queue starts empty
        st->count[cur ^ 1] = 0;
        st->front[cur ^ 1] = 0;
        st->back[cur ^ 1] = 0;
    }
    const uint32_t n = *((volatile uint32_t*)&st->count[cur]);
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t nvis = 0, ntest = 0;
    if (i < n) {
        const Queue Q = pick(qs, cur);
        const uint32_t q = wave_slot(st, cur, i);
        const float4 o4 = Q.ori[q], d4 = Q.dir[q];
        const int root = jobs[__float_as_uint(d4.w) >> 8].root;
        const HitRec h = closest_hit<kCount, kInst>(g, root, xyz(o4), xyz(d4), nvis, ntest);
        // hit reference: top-level record (>= 0), miss (-1), or an instanced
        // triangle's global id as -2 - id with its thing beside
        const int ref = !h.hit ? -1 : (h.leaf >= 0 ? h.leaf : -2 - int(h.id));
        hits[i] = make_float4(h.t, h.u, h.v, __int_as_float(ref));
        if (kInst && ref <= -2) hthing[i] = h.thing;
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

// Persistent traversal: a grid that fills the GPU once, each warp claiming
// rays of the wave from a counter.  A warp claims new rays for its idle lanes
// whenever at most kRefillBelow of its lanes are still traversing (checked
// every kStepsPerCheck steps), so lanes whose rays finish early do not wait
// for the warp's longest ray.  Same hits as k_extend.  Measured on C1 (64
// spp, binned-SAH layout, 2070 MHz): one thread per ray 2097 Mrays/s;
// persistent with (threshold, steps) = (16, 8) 2182, (8, 16) 2282, (12, 16)
// 2283, (16, 32) 2278, (4, 16) 2259, (24, 8) 2114, (28, 8) 2015 -- and
// 2135 at the 54 registers the kernel takes unbounded (5 blocks per SM at 48
// registers are worth a few spilled bytes).
constexpr uint32_t kRefillBelow = 12;
constexpr int kStepsPerCheck = 16;

// Flat layouts: 48 registers (five 256-thread blocks per SM) set as a register
// cap rather than as a minimum of resident blocks: the compiled kernel differs
// and measured 0.9 % faster (C1: traversal 335.8 -> 332.4 ms per frame); 192- or
// 224-thread blocks (42 warps per SM instead of 40) were 3-4 % slower.
template <bool kInst>
__global__ void __launch_bounds__(kThreads, kInst ? 4 : 1) __maxnreg__(kInst ? 64 : 48)
    k_extend_p(Queues qs, float4* __restrict__ hits, uint32_t* __restrict__ hthing, WaveState* st,
               const JobDev* __restrict__ jobs, GeoView g, ExtTune tn) {
    const uint32_t cur = *((volatile uint32_t*)&st->cur);
    if (blockIdx.x == 0 && threadIdx.x == 0) {   // the next queue starts empty
        st->count[cur ^ 1] = 0;
        st->front[cur ^ 1] = 0;
        st->back[cur ^ 1] = 0;
    }
    const uint32_t n = *((volatile uint32_t*)&st->count[cur]);
    const Queue Q = pick(qs, cur);
    const uint32_t lane = lane_id();
    Trav s;
    int stack[kStackSize];
    uint32_t i = 0, nvis = 0, ntest = 0;
    bool busy = false, drained = false;
    while (true) {
        uint32_t bm = __ballot_sync(0xFFFFFFFFu, busy);
        if (!drained && uint32_t(__popc(bm)) <= tn.refill_below) {
            const uint32_t idle = ~bm;
            uint32_t base = 0;
            if (lane == 0) base = atomicAdd(&st->ext_next[cur], uint32_t(__popc(idle)));
            base = __shfl_sync(0xFFFFFFFFu, base, 0);
            if (base + uint32_t(__popc(idle)) >= n) drained = true;
            if (!busy) {
                i = base + __popc(idle & ((1u << lane) - 1u));
                if (i < n) {
                    const uint32_t q = wave_slot(st, cur, i);
                    const float4 o4 = qld(Q.ori + q), d4 = qld(Q.dir + q);
                    const int root = jobs[__float_as_uint(d4.w) >> 8].root;
                    trav_init(s, xyz(o4), xyz(d4), root);
                    if (root >= 0) busy = true;
                    else qst(hits + i, make_float4(0.f, 0.f, 0.f, __int_as_float(-1)));   // empty scene: a miss
                }
            }
            bm = __ballot_sync(0xFFFFFFFFu, busy);
        }
        if (bm == 0) {
            if (drained) break;
            continue;
        }
        if (busy) {
#pragma unroll 1   // unrolled twice: 2.6 % slower (C1, 500 spp)
            for (int k = 0; k < tn.steps; ++k) {
                if (!trav_step<false, kInst>(s, stack, g, nvis, ntest)) {
                    const HitRec& h = s.h;
                    const int ref = !h.hit ? -1 : (h.leaf >= 0 ? h.leaf : -2 - int(h.id));
                    qst(hits + i, make_float4(h.t, h.u, h.v, __int_as_float(ref)));
                    if (kInst && ref <= -2) hthing[i] = h.thing;
                    if (h.overflow) atomicOr(&st->err, 1u);
                    busy = false;
                    break;
                }
            }
        }
    }
}

using ExtendFn = void (*)(Queues, float4*, uint32_t*, WaveState*, const JobDev*, GeoView, ExtTune);

// 64-bit fixed-point sample sums: round-half-even(x * 2^32) as two's
// complement, added with integer atomics (exact, order-free).
__device__ __forceinline__ unsigned long long fx_q(float x) {
    return (unsigned long long)__float2ll_rn(x * 4294967296.0f);
}

// kB threads per block (rt_tuning: shade_block), held to 64 registers, so two
// 512-thread blocks per SM; the grid is the resident blocks, each walking the
// wave in tiles of kB rays (one block per tile measured slower: 78.2 against
// 69.5 ms of shading per C1 frame, the empty blocks of short waves included).  One block-wide aggregation round (two barriers)
// for the continuing rays' queue offsets.  Measured without gain on C1 (64
// spp, within 0.3 %) when the kernel also started the fresh paths: one
// aggregation round for its three counters instead of two, and the hit's
// thing id written by k_extend so its optics load beside the primitive record
// (k_extend then needs 51 registers, 4 % slower overall unless held to 48);
// three 512-thread blocks per SM at 40 registers, with 408 B of spills, were
// slower on the full C1 frame (103.3 against 100.5 ms of shading per frame);
// without the fresh paths (40 registers, 256 B of spills) the same as two
// blocks (78.2 against 78.8 ms), 256-thread blocks 80.3 ms.
template <int kB>
__global__ void __launch_bounds__(kB, 1024 / kB)
    k_shade(Queues qs, const float4* __restrict__ hits, const uint32_t* __restrict__ hthing, WaveState* st,
            const JobDev* __restrict__ jobs, uint32_t nj, const float4* __restrict__ tprims,
            const FlatDesc* __restrict__ desc, const ThingDev* __restrict__ things, Acc acc, int any_guides,
            uint2 lim) {
    // per-warp counts, turned into block-exclusive offsets by thread 0, and the
    // block's base from one global atomic per block (not one per warp); two
    // buffers by tile parity, so that a tile's counts are written while slower
    // warps may still read the previous tile's offsets
    __shared__ uint32_t s_warp_buf[2][kB / 32];
    __shared__ unsigned long long s_base_buf[2];
    const uint32_t cur = *((volatile uint32_t*)&st->cur);
    const uint32_t n = *((volatile uint32_t*)&st->count[cur]);
    const uint32_t lane = lane_id(), warp = threadIdx.x >> 5;
    const Queue Q = pick(qs, cur), N = pick(qs, cur ^ 1);
    // a grid of resident blocks walks the wave in tiles of kB rays (the loop
    // condition is the same for the whole block, so every thread of the block
    // meets the barriers inside)
    uint32_t parity = 0;
    for (uint32_t tile = blockIdx.x; tile * kB < n; tile += gridDim.x, parity ^= 1u) {
        uint32_t* s_warp = s_warp_buf[parity];
        unsigned long long& s_base = s_base_buf[parity];
        const uint32_t i = tile * kB + threadIdx.x;
        const bool active = i < n;

        bool cont = false, ended = false;
        unsigned long long a_px = ~0ull, a_r = 0, a_g = 0, a_b = 0, a_n = 0;
        float3 no{}, nd{}, nthr{};
        float3 gN{}, gA{};
        uint32_t pixel = 0, sample = 0, bounce = 0, jx = 0;
        if (active) {
            const uint32_t q = wave_slot(st, cur, i);
            const float4 o4 = qld(Q.ori + q), d4 = qld(Q.dir + q), t4 = qld(Q.thr + q), h4 = qld(hits + i);
            pixel = __float_as_uint(o4.w);
            sample = __float_as_uint(t4.w);
            const uint32_t tag = __float_as_uint(d4.w);
            jx = tag >> 8;
            bounce = tag & 0xFFu;
            const JobDev& j = jobs[jx];
            const float3 o = xyz(o4), d = xyz(d4);
            float3 thr = xyz(t4);
            if (any_guides) {
                gN = xyz(Q.gn[q]);
                gA = xyz(Q.ga[q]);
            }
            const int ref = __float_as_int(h4.w);
            float3 color = mk(0.f, 0.f, 0.f);
            if (ref == -1) {
                color = mulv(thr, sky(d, j.ambient, j.white));
                ended = true;
            } else if (bounce + 1 >= j.depth) {
                ended = true;   // black at the depth limit (optx/optics_r.cu:34-42)
            } else {
                Stream s(j.seed, j.key1, pixel, sample, bounce + 1);
                float4 pa, pb, pc;
                bool ok = ref >= 0 ? rt_in_bounds(uint32_t(ref) < lim.x, &st->err)
                                   : rt_in_bounds(hthing[i] < lim.y, &st->err);
                if (ok) {
                    if (ref >= 0) {   // the world-space record itself
                        pa = __ldg(tprims + 3 * ref);
                        pb = __ldg(tprims + 3 * ref + 1);
                        pc = __ldg(tprims + 3 * ref + 2);
                    } else {          // an instanced triangle, rebuilt exactly as the flat layout stores it
                        world_prim(desc, hthing[i], uint32_t(-2 - ref), pa, pb, pc);
                    }
                    ok = rt_in_bounds(__float_as_uint(pa.w) < lim.y, &st->err);
                }
                const ScatterOut so = ok ? scatter(pa, pb, pc, things, o, d, h4, s) : ScatterOut{};
                if (so.guide) {
                    if (isnull(gN)) gN = so.N;
                    if (isnull(gA)) gA = so.albedo;
                }
                if (so.cont) {
                    thr = mulv(thr, so.albedo);   // glass: albedo (1,1,1), an exact no-op
                    no = so.p; nd = so.dir; nthr = thr; cont = true;
                } else {
                    ended = true;   // absorbed: black
                }
            }
            if (ended) {
                const size_t px = size_t(j.pix_offset) + pixel;
                a_px = px;
                a_r = fx_q(color.x);
                a_g = fx_q(color.y);
                a_b = fx_q(color.z);
                a_n = bounce + 1;
                if (j.guides) {
                    const float gv[6] = {gN.x, gN.y, gN.z, gA.x, gA.y, gA.z};
    #pragma unroll
                    for (int k = 0; k < 6; ++k) {
                        const unsigned long long q = fx_q(gv[k]);
                        if (q) atomicAdd(acc.gd[k] + px, q);
                    }
                }
            }
        }

        {   // pixel sums: one atomic per sum when every ended lane of the warp shares the pixel
            // (common with pixel-major path numbers), else one per lane
            const uint32_t em = __ballot_sync(0xFFFFFFFFu, ended);
            if (em) {
                const uint32_t grp = __match_any_sync(0xFFFFFFFFu, a_px);
                const uint32_t leader = __ffs(em) - 1;
                const bool uni = __shfl_sync(0xFFFFFFFFu, (grp & em) == em ? 1 : 0, leader) != 0;
                if (uni) {
                    for (int o = 16; o > 0; o >>= 1) {
                        a_r += __shfl_xor_sync(0xFFFFFFFFu, a_r, o);
                        a_g += __shfl_xor_sync(0xFFFFFFFFu, a_g, o);
                        a_b += __shfl_xor_sync(0xFFFFFFFFu, a_b, o);
                        a_n += __shfl_xor_sync(0xFFFFFFFFu, a_n, o);
                    }
                }
                if (ended && (!uni || lane == leader)) {
                    if (a_r) atomicAdd(acc.col[0] + a_px, a_r);
                    if (a_g) atomicAdd(acc.col[1] + a_px, a_g);
                    if (a_b) atomicAdd(acc.col[2] + a_px, a_b);
                    atomicAdd(acc.rays + a_px, uint32_t(a_n));
                }
            }
        }
        // continuing rays fill the next queue from the front (one atomic per
        // block); the fresh paths follow behind them (k_fill)
        if (cont) bounce += 1;
        const uint32_t pc = __ballot_sync(0xFFFFFFFFu, cont);
        if (lane == 0) s_warp[warp] = __popc(pc);
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t tc = 0;
            for (uint32_t w = 0; w < kB / 32; ++w) {
                const uint32_t c = s_warp[w];
                s_warp[w] = tc;
                tc += c;
            }
            s_base = tc ? (unsigned long long)atomicAdd(&st->front[cur ^ 1], tc) : 0ull;
        }
        __syncthreads();
        if (cont) {
            const uint32_t slot = uint32_t(s_base) + s_warp[warp] + __popc(pc & ((1u << lane) - 1u));
            qst(N.ori + slot, make_float4(no.x, no.y, no.z, __uint_as_float(pixel)));
            qst(N.dir + slot, make_float4(nd.x, nd.y, nd.z, __uint_as_float((jx << 8) | bounce)));
            qst(N.thr + slot, make_float4(nthr.x, nthr.y, nthr.z, __uint_as_float(sample)));
            if (any_guides) {
                N.gn[slot] = make_float4(gN.x, gN.y, gN.z, 0.f);
                N.ga[slot] = make_float4(gA.x, gA.y, gA.z, 0.f);
            }
        }
    }
}

// One thread: flips the queues and decides whether another wave runs; inside
// a graph it sets the WHILE condition.  The wave count is capped by an exact
// bound, past which the loop stops with an error flag.
__global__ void k_wave_ctrl(WaveState* st, cudaGraphConditionalHandle handle, int in_graph) {
    const uint32_t cur = st->cur;
    if (st->count[cur] != 0) st->iter += 1;   // a wave ran (the host loop may run empty ones)
    const uint32_t next = cur ^ 1u;
    const uint32_t nf = fresh_count(st, next);   // the paths k_fill started behind the continuing rays
    st->next_path += nf;
    st->back[next] = nf;
    st->cur = next;
    st->count[next] = st->front[next] + st->back[next];
    st->ext_next[next] = 0;
    bool more = st->count[next] != 0;
    if (more && st->iter >= st->max_iter) {
        st->err |= 2u;
        more = false;
    }
    if (in_graph) cudaGraphSetConditional(handle, more ? 1u : 0u);
}

__device__ __forceinline__ float clamp01(float x) { return 0.f > x ? 0.f : (x > 1.f ? 1.f : x); }
__device__ __forceinline__ float fx_mean(unsigned long long s, uint32_t spp) {
    return float(double((long long)s) * 0x1p-32 / double(spp));
}

// optx/camera_i.cu:104-113: mean over spp clamped to [0,1]; rpp; guides.
// With `sticky` (launches inside a stream capture, which read no state back)
// the launch's error bits are also ORed into that word for a later check.
__global__ void __launch_bounds__(kThreads) k_finalize(const JobDev* __restrict__ jobs, uint32_t nj, Acc acc,
                                                       uint32_t total_pix, WaveState* st, uint32_t* sticky) {
    const uint32_t gp = blockIdx.x * blockDim.x + threadIdx.x;
    if (sticky && gp == 0 && st->err) atomicOr(sticky, st->err);
    unsigned long long r = 0;
    if (gp < total_pix) {
        const JobDev& j = jobs[job_of_pixel(jobs, nj, gp)];
        const uint32_t p = gp - j.pix_offset;
        j.rawRGB[p] = rt_float3{clamp01(fx_mean(acc.col[0][gp], j.mean_spp)),
                                clamp01(fx_mean(acc.col[1][gp], j.mean_spp)),
                                clamp01(fx_mean(acc.col[2][gp], j.mean_spp))};
        r = acc.rays[gp];
        if (j.rpp) j.rpp[p] = acc.rays[gp];
        if (j.guides) {
            j.normals[p] = rt_float3{fx_mean(acc.gd[0][gp], j.spp), fx_mean(acc.gd[1][gp], j.spp),
                                     fx_mean(acc.gd[2][gp], j.spp)};
            j.albedos[p] = rt_float3{fx_mean(acc.gd[3][gp], j.spp), fx_mean(acc.gd[4][gp], j.spp),
                                     fx_mean(acc.gd[5][gp], j.spp)};
        }
    }
    for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xFFFFFFFFu, r, o);
    if (lane_id() == 0 && r) atomicAdd(&st->rays, r);
}

// An accumulator's sums as an image: the mean over `spp` samples clamped to
// [0, 1] and the rays per pixel (k_finalize for sums merged elsewhere).
__global__ void __launch_bounds__(kThreads) k_resolve(Acc acc, uint32_t npix, uint32_t spp, rt_float3* rawRGB,
                                                      uint32_t* rpp) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npix) return;
    rawRGB[p] = rt_float3{clamp01(fx_mean(acc.col[0][p], spp)), clamp01(fx_mean(acc.col[1][p], spp)),
                          clamp01(fx_mean(acc.col[2][p], spp))};
    if (rpp) rpp[p] = acc.rays[p];
}

// FP64 distance from the (binary32) ray to the selected primitive: the
// binary32 Moller-Trumbore t loses digits on grazing hits (its error grows
// like 1/sin of the grazing angle), so the reported distance re-evaluates the
// winner in double precision; the selection itself stays binary32.
__device__ double dist64(float4 a, float4 b, float4 c, float3 of, float3 df) {
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

struct FirstHitArgs {
    CamDev cam;
    uint32_t W, H, seed, key1, sample, x0, y0, nx, ny;
    int root;
    int rtow_px;
};

// Primary-ray closest hit of one sample for a pixel rectangle.
__global__ void __launch_bounds__(kThreads) k_first_hit(FirstHitArgs a, GeoView g, int* prim, int* thing, float* t,
                                                        float* u, float* v, double* t64, uint32_t* err) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= a.nx * a.ny) return;
    const uint32_t x = a.x0 + k % a.nx, y = a.y0 + k / a.nx;
    const uint32_t pixel = a.W * y + x;
    Stream s(a.seed, a.key1, pixel, a.sample, 0);
    float3 o, d;
    camera_ray(a.cam, x, y, a.W, a.H, a.rtow_px != 0, s, o, d);
    uint32_t nv = 0, nt = 0;
    const HitRec h = closest_hit_any<false>(g, a.root, o, d, nv, nt);
    if (h.overflow) atomicOr(err, 1u);
    if (!h.hit) {
        prim[k] = -1;
        if (thing) thing[k] = -1;
        if (t) t[k] = 0.f;
        if (u) u[k] = 0.f;
        if (v) v[k] = 0.f;
        if (t64) t64[k] = __longlong_as_double(0x7FF8000000000000ll);
        return;
    }
    prim[k] = int(h.id);
    if (thing) thing[k] = int(h.thing);
    if (t) t[k] = h.t;
    if (u) u[k] = h.u;
    if (v) v[k] = h.v;
    if (t64) {
        float4 pa, pb, pc;
        world_prim(g.desc, h.thing, h.id, pa, pb, pc);
        t64[k] = dist64(pa, pb, pc, o, d);
    }
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
uint32_t env_u32(const char* name, uint32_t dflt) {
    const char* v = std::getenv(name);
    if (!v || !*v) return dflt;
    const unsigned long x = std::strtoul(v, nullptr, 10);
    return x ? uint32_t(x) : dflt;
}

// Launch shape set by rt_tuning_set (process-wide; zero fields: defaults).
// The defaults come from the full C1 frame (1200x800, 500 spp, 7,979,008
// triangles): 512-thread shading blocks, and waves of 2^26 rays (7.7 GB of
// queues; fewer waves, so fewer traversal drains and launches per frame):
// 3019 / 3088 / 3117 / 3132 Mrays/s for 2^23 / 2^24 / 2^25 / 2^26.
constexpr uint32_t kWaveDefault = 1u << 26;
constexpr int kShadeBlockDefault = 512;
std::mutex g_tune_mu;
rt_tuning g_tune{};

struct LaunchShape {
    uint32_t wave;        // rays per wave queue
    int shade_block;      // threads per k_shade block
    uint32_t ext_bpsm;    // persistent traversal blocks per SM (0: all that fit)
    ExtTune ext;
};

LaunchShape launch_shape() {
    rt_tuning t;
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        t = g_tune;
    }
    LaunchShape r;
    r.wave = t.wave_log2 ? (1u << t.wave_log2) : env_u32("RTX_WAVE", kWaveDefault);
    r.shade_block = t.shade_block ? int(t.shade_block) : kShadeBlockDefault;
    r.ext_bpsm = t.extend_blocks_per_sm;
    r.ext.refill_below = t.refill_below ? t.refill_below : kRefillBelow;
    r.ext.steps = t.steps_per_check ? int(t.steps_per_check) : kStepsPerCheck;
    return r;
}

using ShadeFn = void (*)(Queues, const float4*, const uint32_t*, WaveState*, const JobDev*, uint32_t, const float4*,
                         const FlatDesc*, const ThingDev*, Acc, int, uint2);

ShadeFn shade_fn(int block) {
    return block == 128 ? k_shade<128> : block == 512 ? k_shade<512> : block == 1024 ? k_shade<1024> : k_shade<256>;
}

// The wave loop captured once as a graph: a conditional WHILE node whose body
// is extend -> shade -> fill -> ctrl; rebuilt whenever a baked-in pointer or launch
// shape changes.
struct WaveGraph {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    std::vector<const void*> key;
    void reset() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        exec = nullptr;
        graph = nullptr;
        key.clear();
    }
    ~WaveGraph() { reset(); }
};

// Per-thread render workspace (queues, accumulators, job table), grow-only.
struct Workspace {
    DevBuf q[2][5];
    DevBuf hits, hthing, acc, acc_gd, jobs, state;
    WaveState* host_state = nullptr;   // pinned
    std::vector<JobDev> jobs_host;
    std::vector<JobDev> jobs_uploaded;   // the job table in `jobs` (a capture may not upload one)
    std::vector<cudaEvent_t> events;
    WaveGraph graph;
    ~Workspace() {
        graph.reset();
        if (host_state) cudaFreeHost(host_state);
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

// Wave loop mode: graph (default) or host-driven (RTX_GRAPH=0, and always
// when per-kernel CUDA-event timing is requested).
bool graph_mode() {
    const char* e = std::getenv("RTX_GRAPH");
    return !(e && std::strcmp(e, "0") == 0);
}

struct WaveLaunch {
    ExtendFn ext_fn;
    unsigned egrid;    // extend grid (persistent: fills the GPU once)
    unsigned qgrid;    // one thread per wave slot, kThreads per block
    unsigned fgrid;    // k_fill: a few blocks per SM striding over the fresh paths
    ShadeFn shade;
    unsigned sgrid;    // shading grid, sblock threads per block
    int sblock;
    ExtTune tn;
    uint2 lim;         // record and thing counts (bounds-checked build)
    Queues qs;
    float4* hits;      // t, u, v, hit reference
    uint32_t* hthing;  // thing of an instanced hit
    WaveState* st;
    const JobDev* jobs;
    uint32_t nj;
    GeoView geo;
    const ThingDev* things;
    Acc acc;
    int any_guides;
};

// Blocks of a persistent extend kernel: resident blocks per SM (at most
// `bpsm` when nonzero) x SMs.  (A zero shared-memory carveout, all of the
// SM's unified storage as L1 for nodes and stacks, measured no change: C1 at
// 64 spp, 2302 against 2301.)
unsigned persistent_grid(ExtendFn fn, uint32_t bpsm) {
    int per_sm = 0;
    RT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, reinterpret_cast<const void*>(fn), kThreads, 0));
    per_sm = std::max(1, per_sm);
    if (bpsm) per_sm = std::min(per_sm, int(bpsm));
    return unsigned(per_sm * sm_count());
}

// Adds the wave loop to `graph` after `deps`: a conditional WHILE node (its
// condition set to 1 at every launch of the graph) whose body is extend ->
// shade -> fill -> ctrl; k_wave_ctrl clears the condition when the loop is done.
cudaGraphNode_t add_wave_loop(cudaGraph_t graph, const cudaGraphNode_t* deps, size_t ndeps, const WaveLaunch& L) {
    cudaGraphConditionalHandle handle;
    RT_CUDA(cudaGraphConditionalHandleCreate(&handle, graph, 1u, cudaGraphCondAssignDefault));
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = handle;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t cnode;
    RT_CUDA(cudaGraphAddNode(&cnode, graph, deps, nullptr, ndeps, &cp));
    cudaGraph_t body = cp.conditional.phGraph_out[0];

    WaveLaunch l = L;   // kernel arguments must stay addressable while the nodes are added
    cudaKernelNodeParams kp = {};
    cudaGraphNode_t n_ext, n_shade, n_ctrl;
    void* ext_args[] = {&l.qs, &l.hits, &l.hthing, &l.st, &l.jobs, &l.geo, &l.tn};
    kp.func = reinterpret_cast<void*>(l.ext_fn);
    kp.gridDim = dim3(l.egrid);
    kp.blockDim = dim3(kThreads);
    kp.kernelParams = ext_args;
    RT_CUDA(cudaGraphAddKernelNode(&n_ext, body, nullptr, 0, &kp));
    const float4* hits_c = l.hits;
    const uint32_t* hthing_c = l.hthing;
    const float4* tprims_c = l.geo.tprims;
    const FlatDesc* desc_c = l.geo.desc;
    void* shade_args[] = {&l.qs,      &hits_c, &hthing_c, &l.st,  &l.jobs,       &l.nj,
                          &tprims_c, &desc_c, &l.things, &l.acc, &l.any_guides, &l.lim};
    kp.func = reinterpret_cast<void*>(l.shade);
    kp.gridDim = dim3(l.sgrid);
    kp.blockDim = dim3(unsigned(l.sblock));
    kp.kernelParams = shade_args;
    RT_CUDA(cudaGraphAddKernelNode(&n_shade, body, &n_ext, 1, &kp));
    cudaGraphNode_t n_fill;
    const WaveState* st_c = l.st;
    void* fill_args[] = {&l.jobs, &l.nj, &l.qs, &st_c, &l.any_guides};
    kp.func = reinterpret_cast<void*>(k_fill);
    kp.gridDim = dim3(l.fgrid);
    kp.blockDim = dim3(kThreads);
    kp.kernelParams = fill_args;
    RT_CUDA(cudaGraphAddKernelNode(&n_fill, body, &n_shade, 1, &kp));
    int in_graph = 1;
    void* ctrl_args[] = {&l.st, &handle, &in_graph};
    kp.func = reinterpret_cast<void*>(k_wave_ctrl);
    kp.gridDim = dim3(1);
    kp.blockDim = dim3(1);
    kp.kernelParams = ctrl_args;
    RT_CUDA(cudaGraphAddKernelNode(&n_ctrl, body, &n_fill, 1, &kp));
    return cnode;
}

void build_wave_graph(Workspace& ws, const WaveLaunch& L) {
    WaveGraph& G = ws.graph;
    G.reset();
    RT_CUDA(cudaGraphCreate(&G.graph, 0));
    add_wave_loop(G.graph, nullptr, 0, L);
    RT_CUDA(cudaGraphInstantiate(&G.exec, G.graph, 0));
}

// Adds the wave loop to the graph that stream `s` is being captured into, after
// the work captured so far, and makes later captured work depend on it.
void capture_wave_loop(cudaStream_t s, const WaveLaunch& L) {
    cudaStreamCaptureStatus cs;
    cudaGraph_t graph;
    const cudaGraphNode_t* deps = nullptr;
    size_t ndeps = 0;
    RT_CUDA(cudaStreamGetCaptureInfo(s, &cs, nullptr, &graph, &deps, nullptr, &ndeps));
    RT_REQUIRE(cs == cudaStreamCaptureStatusActive, "stream is not capturing");
    const std::vector<cudaGraphNode_t> d(deps, deps + ndeps);   // valid until the next capture call
    cudaGraphNode_t loop = add_wave_loop(graph, d.data(), d.size(), L);
    RT_CUDA(cudaStreamUpdateCaptureDependencies(s, &loop, nullptr, 1, cudaStreamSetCaptureDependencies));
}

}  // namespace

namespace {

// The wavefront over all jobs with workspace `ws`.  Inside a stream capture
// (a caller capturing a whole iteration into one CUDA graph) the launch
// enqueues its work without reading anything back: the job table must be
// the one the workspace already holds and no buffer may grow (both hold
// after the same launch ran once outside the capture), the wave loop becomes
// a conditional node of the captured graph, no stats are filled in, and the
// launch's error bits are ORed into `sticky` for a later check.
void render_jobs_ws(const Geometry& g, const std::vector<Job>& jobs, cudaStream_t s, rt_launch_stats* stats,
                    AccumState* accum, Workspace& ws, uint32_t* sticky) {
    NvtxRange nvtx("rt render");
    const bool capturing = stream_capturing(s);
    RT_REQUIRE(!jobs.empty(), "no jobs to render");
    if (accum) {
        RT_REQUIRE(jobs.size() == 1, "an accumulator takes one job");
        const rt_launch_params& p = jobs[0].params;
        RT_REQUIRE(p.image_w == accum->W && p.image_h == accum->H, "image size differs from the accumulator's");
        RT_REQUIRE(!(p.flags & RT_FLAG_GUIDES), "RT_FLAG_GUIDES is not supported with an accumulator");
        // the per-pixel ray count is u32 and the RNG's sample index u32
        RT_REQUIRE((accum->samples + p.spp) * p.depth < (1ull << 32), "accumulator full (samples x depth >= 2^32)");
        RT_REQUIRE(accum->first + accum->samples + p.spp < (1ull << 32), "sample index beyond 2^32");
    }
    uint32_t flags_union = 0;
    for (const Job& j : jobs) {
        check_params(&j.params);
        RT_REQUIRE(j.frame.rawRGB != nullptr, "frame.rawRGB is NULL");
        if (j.params.flags & RT_FLAG_GUIDES)
            RT_REQUIRE(j.frame.normals && j.frame.albedos, "RT_FLAG_GUIDES needs frame.normals and frame.albedos");
        RT_REQUIRE(j.seg < g.nsegs, "job segment out of range");
        flags_union |= j.params.flags;
    }
    RT_REQUIRE(jobs.size() < (1u << 24), "too many jobs (>= 2^24)");
    const bool stage_timing = (flags_union & RT_FLAG_STAGE_TIMING) != 0;
    const bool count = (flags_union & RT_FLAG_COUNT_VISITS) != 0;
    const int any_guides = (flags_union & RT_FLAG_GUIDES) ? 1 : 0;
    const bool use_graph = graph_mode() && !stage_timing;
    if (capturing) {
        RT_REQUIRE(!stats && !accum && !stage_timing && !count,
                   "inside a stream capture: no stats, accumulator, stage timing or visit counting");
        RT_REQUIRE(use_graph, "inside a stream capture the wave loop must be a graph (RTX_GRAPH=0 is set)");
        RT_REQUIRE(sticky != nullptr, "this launch cannot run inside a stream capture");
    }
    CaptureNoAlloc no_alloc(capturing);

    const uint32_t nj = uint32_t(jobs.size());
    ws.jobs_host.resize(nj);
    unsigned long long total_paths = 0;
    uint64_t total_pix = 0;
    uint32_t max_depth = 1;
    for (uint32_t k = 0; k < nj; ++k) {
        const Job& jb = jobs[k];
        JobDev& d = ws.jobs_host[k];
        std::memset(&d, 0, sizeof(d));
        d.cam = cam_dev(jb.cam);
        d.ambient = make_float3(jb.params.ambient.x, jb.params.ambient.y, jb.params.ambient.z);
        d.white = make_float3(jb.params.white.x, jb.params.white.y, jb.params.white.z);
        d.W = jb.params.image_w;
        d.H = jb.params.image_h;
        d.npix = d.W * d.H;
        d.spp = jb.params.spp;
        d.depth = jb.params.depth;
        d.seed = jb.params.seed;
        d.key1 = 0;
        d.first_sample = accum ? uint32_t(accum->first + accum->samples) : 0u;
        d.mean_spp = accum ? uint32_t(accum->samples + d.spp) : d.spp;
        d.root = g.root(jb.seg);
        d.pix_offset = uint32_t(total_pix);
        d.guides = (jb.params.flags & RT_FLAG_GUIDES) ? 1 : 0;
        d.rtow_px = (jb.params.flags & RT_FLAG_RTOW_PIXELS) ? 1 : 0;
        d.path_offset = total_paths;
        d.rawRGB = jb.frame.rawRGB;
        d.rpp = jb.frame.rpp;
        d.normals = d.guides ? jb.frame.normals : nullptr;
        d.albedos = d.guides ? jb.frame.albedos : nullptr;
        total_paths += (unsigned long long)d.npix * d.spp;
        total_pix += d.npix;
        max_depth = std::max(max_depth, d.depth);
    }
    RT_REQUIRE(total_pix < (uint64_t(1) << 31), "too many pixels in one launch (>= 2^31)");
    // wave capacity (one-thread-per-ray traversal, C1 at 64 spp): 2^22: 1217, 2^21: 1210, 2^20: 1137,
    // 2^19: 1020 Mrays/s; the current default comes from the autotuner (see launch_shape)
    const LaunchShape shape = launch_shape();
    const uint32_t W = uint32_t(std::min<unsigned long long>(shape.wave, total_paths));
    // wave bound: the queue holds W rays while paths remain to start and a
    // path is queued at most max_depth times
    const uint64_t max_iter64 = total_paths * max_depth / W + max_depth + 8;
    RT_REQUIRE(max_iter64 < 0xFFFFFFFFull, "launch too large");

    for (int b = 0; b < 2; ++b) {
        for (int k = 0; k < 3; ++k) ws.q[b][k].reserve(size_t(W) * 16);
        if (any_guides) for (int k = 3; k < 5; ++k) ws.q[b][k].reserve(size_t(W) * 16);
    }
    ws.hits.reserve(size_t(W) * 16);
    ws.hthing.reserve(size_t(W) * 4);
    ws.acc.reserve(size_t(total_pix) * 28);   // 3 x u64 colour + u32 rays
    if (any_guides) ws.acc_gd.reserve(size_t(total_pix) * 48);
    ws.jobs.reserve(size_t(nj) * sizeof(JobDev));
    ws.state.reserve(sizeof(WaveState));
    if (!ws.host_state) {
        RT_REQUIRE(!capturing, "make the same launch once before capturing it");
        RT_CUDA(cudaMallocHost(&ws.host_state, sizeof(WaveState)));
    }

    WaveLaunch L;
    for (int b = 0; b < 2; ++b) {
        L.qs.q[b].ori = ws.q[b][0].as<float4>();
        L.qs.q[b].dir = ws.q[b][1].as<float4>();
        L.qs.q[b].thr = ws.q[b][2].as<float4>();
        L.qs.q[b].gn = any_guides ? ws.q[b][3].as<float4>() : nullptr;
        L.qs.q[b].ga = any_guides ? ws.q[b][4].as<float4>() : nullptr;
    }
    // the counting pass keeps one thread per ray (its counts are per-ray sums)
    L.ext_fn = g.ninstances ? (count ? k_extend<true, true> : k_extend_p<true>)
                            : (count ? k_extend<true, false> : k_extend_p<false>);
    L.qgrid = grid_for(W);
    L.fgrid = std::min(L.qgrid, unsigned(8 * sm_count()));
    L.egrid = count ? L.qgrid : persistent_grid(L.ext_fn, shape.ext_bpsm);
    L.sblock = shape.shade_block;
    L.shade = shade_fn(L.sblock);
    {   // shading: the resident blocks, walking the wave in tiles
        int per_sm = 0;
        RT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, reinterpret_cast<const void*>(L.shade),
                                                              L.sblock, 0));
        L.sgrid = std::min(grid_for(W, L.sblock), unsigned(std::max(1, per_sm) * sm_count()));
    }
    L.tn = shape.ext;
    L.hits = ws.hits.as<float4>();
    L.hthing = ws.hthing.as<uint32_t>();
    L.st = ws.state.as<WaveState>();
    L.jobs = ws.jobs.as<JobDev>();
    L.nj = nj;
    L.geo = g.view();
    L.geo.err = &L.st->err;   // the bounds-checked build reports there
    L.lim = make_uint2(L.geo.ntprims, L.geo.nthings);
    L.things = g.things_dev.as<ThingDev>();
    {
        unsigned long long* c = accum ? accum->sums.as<unsigned long long>() : ws.acc.as<unsigned long long>();
        for (int k = 0; k < 3; ++k) L.acc.col[k] = c + size_t(k) * total_pix;
        L.acc.rays = reinterpret_cast<uint32_t*>(c + 3 * size_t(total_pix));
        unsigned long long* gd = any_guides ? ws.acc_gd.as<unsigned long long>() : nullptr;
        for (int k = 0; k < 6; ++k) L.acc.gd[k] = gd ? gd + size_t(k) * total_pix : nullptr;
    }
    L.any_guides = any_guides;

    const bool same_jobs = ws.jobs_uploaded.size() == ws.jobs_host.size() &&
                           std::memcmp(ws.jobs_uploaded.data(), ws.jobs_host.data(), size_t(nj) * sizeof(JobDev)) == 0;
    if (capturing) {
        RT_REQUIRE(same_jobs, "the job table differs from the workspace's: make the same launch once before "
                              "capturing it");
    } else {
        RT_CUDA(cudaMemcpyAsync(ws.jobs.p, ws.jobs_host.data(), size_t(nj) * sizeof(JobDev), cudaMemcpyHostToDevice,
                                s));
        ws.jobs_uploaded = ws.jobs_host;
    }
    if (!accum) RT_CUDA(cudaMemsetAsync(ws.acc.p, 0, size_t(total_pix) * 28, s));
    if (any_guides) RT_CUDA(cudaMemsetAsync(ws.acc_gd.p, 0, size_t(total_pix) * 48, s));
    const uint32_t n0 = W;
    k_init_state<<<1, 1, 0, s>>>(L.st, n0, total_paths, uint32_t(max_iter64), W);
    k_generate<<<grid_for(n0), kThreads, 0, s>>>(L.jobs, nj, L.qs.q[0], n0, any_guides);
    RT_CHECK_LAUNCH();
    uint32_t launches = 2;
    std::vector<std::pair<size_t, int>> timed;   // (event index, 0 extend / 1 shade)

    if (capturing) {
        NvtxRange nvtx_loop("wave loop (captured)");
        capture_wave_loop(s, L);
    } else if (use_graph) {
        const std::vector<const void*> key = {
            reinterpret_cast<const void*>(L.ext_fn), reinterpret_cast<const void*>(uintptr_t(L.qgrid)),
            reinterpret_cast<const void*>(uintptr_t(L.egrid)), reinterpret_cast<const void*>(L.shade),
            reinterpret_cast<const void*>(uintptr_t(L.sgrid)), reinterpret_cast<const void*>(uintptr_t(L.tn.refill_below)),
            reinterpret_cast<const void*>(uintptr_t(L.tn.steps)),
            L.qs.q[0].ori, L.qs.q[0].gn, L.qs.q[1].ori, L.qs.q[1].gn, L.hits, L.hthing, L.st, L.jobs,
            reinterpret_cast<const void*>(uintptr_t(nj)), L.geo.tnodes, L.geo.tprims, L.geo.tedges, L.geo.bnodes,
            L.geo.bprims, reinterpret_cast<const void*>(uintptr_t(L.geo.ntnodes)),
            reinterpret_cast<const void*>(uintptr_t(L.geo.ntprims)), reinterpret_cast<const void*>(uintptr_t(L.geo.nbnodes)),
            reinterpret_cast<const void*>(uintptr_t(L.geo.nbprims)), reinterpret_cast<const void*>(uintptr_t(L.geo.nthings)),
            reinterpret_cast<const void*>(uintptr_t(L.geo.instanced)), reinterpret_cast<const void*>(uintptr_t(L.lim.x)),
            reinterpret_cast<const void*>(uintptr_t(L.lim.y)),
            L.geo.inst, L.geo.desc, L.things, L.acc.col[0], L.acc.gd[0], reinterpret_cast<const void*>(uintptr_t(total_pix)),
            reinterpret_cast<const void*>(uintptr_t(any_guides))};
        if (!ws.graph.exec || ws.graph.key != key) {
            build_wave_graph(ws, L);
            ws.graph.key = key;
        }
        NvtxRange nvtx_loop("wave loop (graph)");
        RT_CUDA(cudaGraphLaunch(ws.graph.exec, s));
    } else {
        size_t ev = 0;
        const uint32_t kBatch = 8;
        void* ext_args[] = {&L.qs, &L.hits, &L.hthing, &L.st, &L.jobs, &L.geo, &L.tn};
        const float4* hits_c = L.hits;
        const uint32_t* hthing_c = L.hthing;
        const float4* tprims_c = L.geo.tprims;
        const FlatDesc* desc_c = L.geo.desc;
        uint32_t nj_c = nj;
        void* shade_args[] = {&L.qs,      &hits_c, &hthing_c, &L.st,  &L.jobs,       &nj_c,
                              &tprims_c, &desc_c, &L.things, &L.acc, &L.any_guides, &L.lim};
        cudaGraphConditionalHandle no_handle = 0;
        while (true) {
            for (uint32_t b = 0; b < kBatch; ++b) {
                if (stage_timing) {
                    RT_CUDA(cudaEventRecord(ws.event(ev), s));
                    timed.push_back({ev, 0});
                    ev += 2;
                }
                {
                    NvtxRange r("wave: extend");
                    RT_CUDA(cudaLaunchKernel(reinterpret_cast<const void*>(L.ext_fn), dim3(L.egrid),
                                             dim3(kThreads), ext_args, 0, s));
                }
                if (stage_timing) {
                    RT_CUDA(cudaEventRecord(ws.event(ev - 1), s));
                    RT_CUDA(cudaEventRecord(ws.event(ev), s));
                    timed.push_back({ev, 1});
                    ev += 2;
                }
                {
                    NvtxRange r("wave: shade");
                    RT_CUDA(cudaLaunchKernel(reinterpret_cast<const void*>(L.shade), dim3(L.sgrid),
                                             dim3(unsigned(L.sblock)), shade_args, 0, s));
                }
                if (stage_timing) RT_CUDA(cudaEventRecord(ws.event(ev - 1), s));
                k_fill<<<L.fgrid, kThreads, 0, s>>>(L.jobs, nj, L.qs, L.st, L.any_guides);
                RT_CHECK_LAUNCH();
                k_wave_ctrl<<<1, 1, 0, s>>>(L.st, no_handle, 0);
                RT_CHECK_LAUNCH();
                launches += 4;
            }
            RT_CUDA(cudaMemcpyAsync(ws.host_state, L.st, sizeof(WaveState), cudaMemcpyDeviceToHost, s));
            RT_CUDA(cudaStreamSynchronize(s));
            const WaveState& hs = *ws.host_state;
            if (hs.count[hs.cur] == 0 || hs.err) break;
        }
    }
    k_finalize<<<grid_for(total_pix), kThreads, 0, s>>>(L.jobs, nj, L.acc, uint32_t(total_pix), L.st,
                                                        capturing ? sticky : nullptr);
    RT_CHECK_LAUNCH();
    launches += 1;
    if (capturing) return;
    RT_CUDA(cudaMemcpyAsync(ws.host_state, L.st, sizeof(WaveState), cudaMemcpyDeviceToHost, s));
    RT_CUDA(cudaStreamSynchronize(s));
    const WaveState hs = *ws.host_state;
    if (hs.err & kErrBounds) throw Error(RT_ERR_INTERNAL, "bounds check failed (RT_CHECKS build)");
    if (hs.err & 1u) throw Error(RT_ERR_LIMIT, "traversal stack overflow (LBVH deeper than the stack)");
    if (hs.err & 2u) throw Error(RT_ERR_LIMIT, "wave loop exceeded its bound");
    // with an accumulator the pixel sums (and so hs.rays) cover every sample so far
    unsigned long long launch_rays = hs.rays;
    if (accum) {
        launch_rays = hs.rays - accum->rays;
        accum->rays = hs.rays;
        accum->samples += jobs[0].params.spp;
    }
    if (use_graph) launches += 4 * hs.iter;
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        stats->rays = launch_rays;
        stats->paths = total_paths;
        stats->node_visits = hs.nodes;
        stats->prim_tests = hs.prims;
        stats->waves = hs.iter;
        stats->kernel_launches = launches;
        stats->extend_launches = hs.iter;
        stats->wave_capacity = W;
        for (auto& tv : timed) {
            float ms = 0.f;
            RT_CUDA(cudaEventElapsedTime(&ms, ws.event(tv.first), ws.event(tv.first + 1)));
            (tv.second == 0 ? stats->extend_ms : stats->shade_ms) += ms;
        }
        if (!timed.empty()) stats->extend_launches = uint32_t(timed.size() / 2);
    }
}

}  // namespace

void render_jobs(const Geometry& g, const std::vector<Job>& jobs, cudaStream_t s, rt_launch_stats* stats,
                 AccumState* accum) {
    render_jobs_ws(g, jobs, s, stats, accum, workspace(), nullptr);
}

namespace {

void first_hit_rect(Scene& sc, const rt_camera& cam, const rt_launch_params& p, uint32_t sample, uint32_t x0,
                    uint32_t y0, uint32_t nx, uint32_t ny, int* prim, int* thing, float* t, float* u, float* v,
                    double* t64, cudaStream_t s) {
    check_params(&p);
    if (!sc.built || sc.topology_dirty || sc.xf_dirty) throw Error(RT_ERR_NOT_BUILT, "scene not built or not updated");
    RT_REQUIRE(prim != nullptr, "prim is NULL");
    sync_optics(sc.geo, {&sc}, s);
    FirstHitArgs a{};
    a.cam = cam_dev(cam);
    a.W = p.image_w;
    a.H = p.image_h;
    a.seed = p.seed;
    a.key1 = 0;
    a.sample = sample;
    a.x0 = x0;
    a.y0 = y0;
    a.nx = nx;
    a.ny = ny;
    a.root = sc.geo.root(0);
    a.rtow_px = (p.flags & RT_FLAG_RTOW_PIXELS) ? 1 : 0;
    uint32_t* err = sc.geo.misc.as<uint32_t>();
    RT_CUDA(cudaMemsetAsync(err, 0, 4, s));
    GeoView gv = sc.geo.view();
    gv.err = err;
    k_first_hit<<<grid_for(uint64_t(nx) * ny), kThreads, 0, s>>>(a, gv, prim, thing, t, u, v, t64, err);
    RT_CHECK_LAUNCH();
    uint32_t herr = 0;
    RT_CUDA(cudaMemcpyAsync(&herr, err, 4, cudaMemcpyDeviceToHost, s));
    RT_CUDA(cudaStreamSynchronize(s));
    if (herr & kErrBounds) throw Error(RT_ERR_INTERNAL, "bounds check failed (RT_CHECKS build)");
    if (herr) throw Error(RT_ERR_LIMIT, "traversal stack overflow (LBVH deeper than the stack)");
}

void render_scene(Scene& sc, const rt_camera& cam, const rt_launch_params& p, const rt_frame& f, cudaStream_t s,
                  rt_launch_stats* stats, AccumState* accum = nullptr) {
    if (!sc.built || sc.topology_dirty) throw Error(RT_ERR_NOT_BUILT, "scene not built (call rt_scene_build)");
    if (sc.xf_dirty) throw Error(RT_ERR_NOT_BUILT, "transforms changed; call rt_scene_update");
    sync_optics(sc.geo, {&sc}, s);
    std::vector<Job> jobs(1);
    jobs[0].seg = 0;
    jobs[0].cam = cam;
    jobs[0].params = p;
    jobs[0].frame = f;
    render_jobs(sc.geo, jobs, s, stats, accum);
}

// Checkpoint bytes of an accumulator: a header, then the sums as on the device.
struct AccumHeader {
    char magic[8];   // "rtaccum2"
    uint32_t W, H;
    unsigned long long first, samples, rays;
    unsigned long long sum_bytes;
};

size_t accum_sum_bytes(const AccumState& a) { return size_t(a.W) * a.H * 28; }

AccumState* accum_from(rt_accum a) {
    RT_REQUIRE(a != nullptr, "accumulator handle is NULL");
    return reinterpret_cast<AccumState*>(a);
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

// Many scenes rendered by one wavefront over one segmented geometry.  A
// batch owns the workspaces of its launches and adjoints (queues, sums, job
// tables), so that a launch captured into a CUDA graph keeps pointing at
// buffers that no other launch reuses or regrows, and a device error word
// that launches inside a capture report to (rt_batch_status).
struct Batch {
    std::vector<Scene*> scenes;
    std::vector<Job> jobs;
    std::vector<AdjointJob> adj;   // per scene; grad_image NULL: not registered
    int layout = RT_LAYOUT_AUTO;
    Geometry geo;
    bool built = false;
    Workspace ws;
    std::unique_ptr<AdjointWorkspace, void (*)(AdjointWorkspace*)> adj_ws{adjoint_workspace_new(),
                                                                          adjoint_workspace_free};
    DevBuf sticky;                 // error bits of captured launches since the last rt_batch_status
};

Batch* batch_from(rt_batch b) {
    RT_REQUIRE(b != nullptr, "batch handle is NULL");
    return reinterpret_cast<Batch*>(b);
}

}  // namespace
}  // namespace rt

using namespace rt;

extern "C" {

rt_status rt_accum_create(rt_accum* out, unsigned int w, unsigned int h) {
    return guarded([&] {
        RT_REQUIRE(out != nullptr, "out is NULL");
        RT_REQUIRE(w > 0 && h > 0 && uint64_t(w) * h < (1ull << 31), "bad accumulator size");
        auto* a = new AccumState();
        try {
            a->W = w;
            a->H = h;
            a->sums.reserve(accum_sum_bytes(*a));
            RT_CUDA(cudaMemset(a->sums.p, 0, accum_sum_bytes(*a)));
        } catch (...) {
            delete a;
            throw;
        }
        *out = reinterpret_cast<rt_accum>(a);
    });
}

rt_status rt_accum_destroy(rt_accum acc) {
    return guarded([&] { delete reinterpret_cast<AccumState*>(acc); });
}

rt_status rt_accum_reset(rt_accum acc, void* stream) {
    return guarded([&] {
        AccumState* a = accum_from(acc);
        cudaStream_t s = as_stream(stream);
        RT_CUDA(cudaMemsetAsync(a->sums.p, 0, accum_sum_bytes(*a), s));
        RT_CUDA(cudaStreamSynchronize(s));
        a->first = 0;
        a->samples = 0;
        a->rays = 0;
    });
}

rt_status rt_accum_samples(rt_accum acc, unsigned long long* samples) {
    return guarded([&] {
        RT_REQUIRE(samples != nullptr, "samples is NULL");
        *samples = accum_from(acc)->samples;
    });
}

rt_status rt_launch_accum(rt_scene scene, const rt_camera* cam, const rt_launch_params* params, rt_accum acc,
                          const rt_frame* frame, void* stream, rt_launch_stats* stats) {
    return guarded([&] {
        RT_REQUIRE(cam && params && frame, "cam/params/frame is NULL");
        AccumState* a = accum_from(acc);
        render_scene(*scene_from(scene), *cam, *params, *frame, as_stream(stream), stats, a);
    });
}

rt_status rt_accum_state_size(rt_accum acc, size_t* bytes) {
    return guarded([&] {
        RT_REQUIRE(bytes != nullptr, "bytes is NULL");
        *bytes = sizeof(AccumHeader) + accum_sum_bytes(*accum_from(acc));
    });
}

rt_status rt_accum_save(rt_accum acc, void* host, size_t bytes, void* stream) {
    return guarded([&] {
        AccumState* a = accum_from(acc);
        RT_REQUIRE(host != nullptr, "host is NULL");
        RT_REQUIRE(bytes == sizeof(AccumHeader) + accum_sum_bytes(*a), "state size differs (rt_accum_state_size)");
        AccumHeader h{};
        std::memcpy(h.magic, "rtaccum2", 8);
        h.W = a->W;
        h.H = a->H;
        h.first = a->first;
        h.samples = a->samples;
        h.rays = a->rays;
        h.sum_bytes = accum_sum_bytes(*a);
        std::memcpy(host, &h, sizeof h);
        cudaStream_t s = as_stream(stream);
        RT_CUDA(cudaMemcpyAsync(static_cast<char*>(host) + sizeof h, a->sums.p, h.sum_bytes, cudaMemcpyDeviceToHost, s));
        RT_CUDA(cudaStreamSynchronize(s));
    });
}

rt_status rt_accum_load(rt_accum acc, const void* host, size_t bytes, void* stream) {
    return guarded([&] {
        AccumState* a = accum_from(acc);
        RT_REQUIRE(host != nullptr, "host is NULL");
        RT_REQUIRE(bytes >= sizeof(AccumHeader), "not an accumulator state (too short)");
        AccumHeader h;
        std::memcpy(&h, host, sizeof h);
        RT_REQUIRE(std::memcmp(h.magic, "rtaccum2", 8) == 0, "not an accumulator state");
        RT_REQUIRE(h.W == a->W && h.H == a->H,
                   "accumulator state of another image size (" + std::to_string(h.W) + "x" + std::to_string(h.H) +
                       ", not " + std::to_string(a->W) + "x" + std::to_string(a->H) + ")");
        RT_REQUIRE(h.sum_bytes == accum_sum_bytes(*a) && bytes == sizeof h + h.sum_bytes,
                   "accumulator state truncated or damaged");
        cudaStream_t s = as_stream(stream);
        RT_CUDA(cudaMemcpyAsync(a->sums.p, static_cast<const char*>(host) + sizeof h, h.sum_bytes,
                                cudaMemcpyHostToDevice, s));
        RT_CUDA(cudaStreamSynchronize(s));
        a->first = h.first;
        a->samples = h.samples;
        a->rays = h.rays;
    });
}

rt_status rt_accum_set_first_sample(rt_accum acc, unsigned long long first) {
    return guarded([&] {
        AccumState* a = accum_from(acc);
        RT_REQUIRE(a->samples == 0, "the accumulator holds samples (rt_accum_reset first)");
        RT_REQUIRE(first < (1ull << 32), "first sample beyond 2^32");
        a->first = first;
    });
}

rt_status rt_accum_device_sums(rt_accum acc, unsigned long long** red, unsigned long long** green,
                               unsigned long long** blue, unsigned int** rays) {
    return guarded([&] {
        AccumState* a = accum_from(acc);
        const size_t n = size_t(a->W) * a->H;
        unsigned long long* c = a->sums.as<unsigned long long>();
        if (red) *red = c;
        if (green) *green = c + n;
        if (blue) *blue = c + 2 * n;
        if (rays) *rays = reinterpret_cast<unsigned int*>(c + 3 * n);
    });
}

rt_status rt_accum_set_range(rt_accum acc, unsigned long long first, unsigned long long samples,
                             unsigned long long rays) {
    return guarded([&] {
        AccumState* a = accum_from(acc);
        RT_REQUIRE(first + samples < (1ull << 32), "sample range beyond 2^32");
        a->first = first;
        a->samples = samples;
        a->rays = rays;
    });
}

rt_status rt_accum_resolve(rt_accum acc, const rt_frame* frame, void* stream) {
    return guarded([&] {
        AccumState* a = accum_from(acc);
        RT_REQUIRE(frame != nullptr && frame->rawRGB != nullptr, "frame/rawRGB is NULL");
        RT_REQUIRE(a->samples > 0, "the accumulator holds no samples");
        const uint32_t n = a->W * a->H;
        unsigned long long* c = a->sums.as<unsigned long long>();
        Acc acc_v{};
        for (int k = 0; k < 3; ++k) acc_v.col[k] = c + size_t(k) * n;
        acc_v.rays = reinterpret_cast<uint32_t*>(c + 3 * size_t(n));
        k_resolve<<<grid_for(n), kThreads, 0, as_stream(stream)>>>(acc_v, n, uint32_t(a->samples), frame->rawRGB,
                                                                  frame->rpp);
        RT_CHECK_LAUNCH();
    });
}

rt_status rt_tuning_set(const rt_tuning* tuning) {
    return guarded([&] {
        rt_tuning t{};
        if (tuning) t = *tuning;
        RT_REQUIRE(t.wave_log2 == 0 || (t.wave_log2 >= 16 && t.wave_log2 <= 26), "wave_log2 outside 16..26");
        RT_REQUIRE(t.shade_block == 0 || t.shade_block == 128 || t.shade_block == 256 || t.shade_block == 512 ||
                       t.shade_block == 1024,
                   "shade_block must be 128, 256, 512 or 1024");
        RT_REQUIRE(t.extend_blocks_per_sm <= 32, "extend_blocks_per_sm outside 1..32");
        RT_REQUIRE(t.refill_below <= 31, "refill_below outside 1..31");
        RT_REQUIRE(t.steps_per_check <= 64, "steps_per_check outside 1..64");
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune = t;
    });
}

rt_status rt_tuning_get(rt_tuning* tuning) {
    return guarded([&] {
        RT_REQUIRE(tuning != nullptr, "tuning is NULL");
        rt_tuning t;
        {
            std::lock_guard<std::mutex> lk(g_tune_mu);
            t = g_tune;
        }
        const LaunchShape r = launch_shape();
        if (!t.wave_log2) {   // the default (or RTX_WAVE), rounded down to a power of two
            t.wave_log2 = 0;
            while ((2ull << t.wave_log2) <= r.wave) ++t.wave_log2;
        }
        t.shade_block = unsigned(r.shade_block);
        t.refill_below = r.ext.refill_below;
        t.steps_per_check = unsigned(r.ext.steps);
        *tuning = t;   // extend_blocks_per_sm stays 0 (all that fit) unless set
    });
}

rt_status rt_launch(rt_scene scene, const rt_camera* cam, const rt_launch_params* params, const rt_frame* frame,
                    void* stream) {
    return guarded([&] {
        RT_REQUIRE(cam && params && frame, "cam/params/frame is NULL");
        render_scene(*scene_from(scene), *cam, *params, *frame, as_stream(stream), nullptr);
    });
}

rt_status rt_launch_ex(rt_scene scene, const rt_camera* cam, const rt_launch_params* params, const rt_frame* frame,
                       void* stream, rt_launch_stats* stats) {
    return guarded([&] {
        RT_REQUIRE(cam && params && frame && stats, "cam/params/frame/stats is NULL");
        render_scene(*scene_from(scene), *cam, *params, *frame, as_stream(stream), stats);
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
        render_scene(sc, *cam, *params, f, s, stats);
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

rt_status rt_batch_create(rt_batch* out) {
    return guarded([&] {
        RT_REQUIRE(out != nullptr, "out is NULL");
        *out = reinterpret_cast<rt_batch>(new Batch());
    });
}

rt_status rt_batch_destroy(rt_batch b) {
    return guarded([&] {
        if (b) delete reinterpret_cast<Batch*>(b);
    });
}

rt_status rt_batch_add(rt_batch b, rt_scene scene, const rt_camera* cam, const rt_launch_params* params,
                       const rt_frame* frame, unsigned int* index) {
    return guarded([&] {
        Batch* B = batch_from(b);
        Scene* sc = scene_from(scene);
        RT_REQUIRE(cam && params && frame, "cam/params/frame is NULL");
        check_params(params);
        RT_REQUIRE(frame->rawRGB != nullptr, "frame.rawRGB is NULL");
        if (params->flags & RT_FLAG_GUIDES)
            RT_REQUIRE(frame->normals && frame->albedos, "RT_FLAG_GUIDES needs frame.normals and frame.albedos");
        Job j;
        j.seg = uint32_t(B->scenes.size());
        j.cam = *cam;
        j.params = *params;
        j.frame = *frame;
        B->scenes.push_back(sc);
        B->jobs.push_back(j);
        B->adj.push_back(AdjointJob{j.seg, j.cam, j.params, frame->rawRGB, nullptr, nullptr, nullptr, nullptr});
        B->built = false;
        if (index) *index = j.seg;
    });
}

rt_status rt_batch_set_layout(rt_batch b, int layout) {
    return guarded([&] {
        RT_REQUIRE(layout >= RT_LAYOUT_AUTO && layout <= RT_LAYOUT_SAH, "unknown layout");
        Batch* B = batch_from(b);
        if (B->layout != layout) B->built = false;
        B->layout = layout;
    });
}

rt_status rt_batch_build(rt_batch b, unsigned int morton_bits, void* stream) {
    return guarded([&] {
        Batch* B = batch_from(b);
        RT_REQUIRE(!B->scenes.empty(), "batch is empty");
        B->built = false;   // a build that fails half way leaves no launchable batch behind
        build_geometry(B->geo, B->scenes, int(morton_bits), B->layout, as_stream(stream));
        B->sticky.reserve(4);
        RT_CUDA(cudaMemset(B->sticky.p, 0, 4));
        B->built = true;
    });
}

rt_status rt_batch_launch(rt_batch b, void* stream, rt_launch_stats* stats) {
    return guarded([&] {
        Batch* B = batch_from(b);
        if (!B->built) throw Error(RT_ERR_NOT_BUILT, "batch not built (call rt_batch_build)");
        rt_launch_stats st{};
        cudaStream_t s = as_stream(stream);
        const bool capturing = stream_capturing(s);
        RT_REQUIRE(!capturing || !stats, "no stats from a launch inside a stream capture");
        sync_optics(B->geo, B->scenes, s);
        render_jobs_ws(B->geo, B->jobs, s, capturing ? nullptr : (stats ? stats : &st), nullptr, B->ws,
                       B->sticky.as<uint32_t>());
    });
}

rt_status rt_batch_status(rt_batch b, void* stream) {
    return guarded([&] {
        Batch* B = batch_from(b);
        if (!B->built) throw Error(RT_ERR_NOT_BUILT, "batch not built (call rt_batch_build)");
        cudaStream_t s = as_stream(stream);
        uint32_t err = 0;
        RT_CUDA(cudaMemcpyAsync(&err, B->sticky.p, 4, cudaMemcpyDeviceToHost, s));
        RT_CUDA(cudaMemsetAsync(B->sticky.p, 0, 4, s));
        RT_CUDA(cudaStreamSynchronize(s));
        if (err & kErrBounds) throw Error(RT_ERR_INTERNAL, "a captured launch failed a bounds check (RT_CHECKS build)");
        if (err & 1u) throw Error(RT_ERR_LIMIT, "a captured launch overflowed its traversal stack");
        if (err & 2u) throw Error(RT_ERR_LIMIT, "a captured launch exceeded its wave bound");
        if (err) throw Error(RT_ERR_INTERNAL, "a captured launch reported error bits " + std::to_string(err));
    });
}

rt_status rt_batch_set_albedos(rt_batch b, const float* albedo, void* stream) {
    return guarded([&] {
        Batch* B = batch_from(b);
        if (!B->built) throw Error(RT_ERR_NOT_BUILT, "batch not built (call rt_batch_build)");
        set_albedos_device(B->geo, B->scenes, albedo, as_stream(stream));
    });
}

rt_status rt_batch_set_adjoint(rt_batch b, unsigned int index, const rt_float3* grad_image, double* grad_albedo,
                               double* grad_fuzz, double* grad_sky) {
    return guarded([&] {
        Batch* B = batch_from(b);
        RT_REQUIRE(index < B->adj.size(), "bad batch index");
        AdjointJob& a = B->adj[index];
        a.grad_image = grad_image;
        a.grad_albedo = grad_albedo;
        a.grad_fuzz = grad_fuzz;
        a.grad_sky = grad_sky;
    });
}

rt_status rt_batch_adjoint(rt_batch b, void* stream) {
    return guarded([&] {
        Batch* B = batch_from(b);
        if (!B->built) throw Error(RT_ERR_NOT_BUILT, "batch not built (call rt_batch_build)");
        std::vector<AdjointJob> jobs;
        for (const AdjointJob& a : B->adj)
            if (a.grad_image) jobs.push_back(a);
        RT_REQUIRE(!jobs.empty(), "no scene of the batch has adjoint buffers (rt_batch_set_adjoint)");
        cudaStream_t s = as_stream(stream);
        sync_optics(B->geo, B->scenes, s);
        adjoint_jobs(B->geo, jobs, s, B->adj_ws.get(), B->sticky.as<uint32_t>());
    });
}

rt_status rt_batch_info(rt_batch b, unsigned int* n_scenes, unsigned int* n_prims, float* build_ms,
                        unsigned long long* device_bytes) {
    return guarded([&] {
        Batch* B = batch_from(b);
        if (n_scenes) *n_scenes = unsigned(B->scenes.size());
        if (n_prims) *n_prims = B->geo.nprims;
        if (build_ms) *build_ms = B->geo.build_ms;
        if (device_bytes) *device_bytes = B->geo.device_bytes();
    });
}

}  // extern "C"
