// rt_sah.cu -- binned-SAH hierarchy over the flattened world-space records.
//
// Replaces the closed optixAccelBuild of Scene::build (optx/scene.cxx:227-273)
// by a builder whose tree depends on the geometry, not on a space-filling
// curve alone.  Top-down, one level of the tree per pass over the records:
// every node of the level is binned (32 bins per axis over its centroid
// bounds), the split of least surface-area cost is taken (Wald 2007) and the
// node's records are partitioned stably; nodes of at most `cluster_max`
// records become clusters.  Each cluster then gets a Karras 2012 hierarchy over 30-bit
// Morton codes inside its own centroid bounds (keys cluster << 30 | code), and
// the split nodes above the clusters are stitched into the spare node slot of
// each cluster: a split whose left part ends at record position p lives in
// slot p - 1, the last slot of the cluster ending there, which that cluster's
// own n - 1 internal nodes leave free.
//
// Everything is a function of the records alone (child allocation order does
// not reach the result: slots follow from positions), so a rebuild gives the
// same tree.  The host reads two counters per level; no kernel waits on
// another block.
#include <algorithm>
#include <vector>

#include "rt_lbvh.cuh"

namespace rt {
namespace {

constexpr int kSahBins = 32;
constexpr uint32_t kSahChunk = 2048;   // records per binning / partition block
constexpr int kSahThreads = 256;
constexpr int kSahMaxLevels = 64;      // deeper levels split at the median position
constexpr int kBinWords = 7;           // count, box lo xyz, box hi xyz (orderable u32)

// A record on its way down: box and record id.
struct SahRec {
    float4 lo_id;   // box lo, record id (bits)
    float4 hi;      // box hi
};

// A node of the current level.
struct SahNode {
    uint32_t start, count;
    int parent;        // split node of the parent, -1 at a segment root
    uint32_t side;     // which child of the parent
    uint32_t seg;      // segment (scene) of the records
    uint32_t cb[6];    // centroid bounds, orderable u32 (lo xyz, hi xyz)
    uint32_t chunk0;   // first chunk of the node in the level's chunk table
    int axis;          // chosen split: axis (-1: median position), bin, left count
    int bin;
    uint32_t nleft;
    int child[2];      // >= 0: node of the next level; < 0: ~cluster
};

struct SahCluster {
    uint32_t start, count;
    uint32_t cb[6];
};

// A split node above the clusters: records [start, end), left part [start, split).
struct SahSplit {
    uint32_t start, split, end;
    int child[2];   // split node, or -1 where the part is a cluster
    int parent;
    uint32_t seg;
};

struct SahCounters {
    uint32_t nnext, ncl, nsplit, nchunks, err;
};

__device__ __forceinline__ uint32_t sah_bin(float c, float lo, float scale) {
    const int k = int((c - lo) * scale);
    return uint32_t(min(max(k, 0), kSahBins - 1));
}

// Bin origin and scale of a node's centroid bounds (0 scale: one bin).
__device__ __forceinline__ void sah_frame(const uint32_t* cb, float lo[3], float scale[3]) {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        lo[a] = fdeord(cb[a]);
        const float ext = fdeord(cb[3 + a]) - lo[a];
        scale[a] = ext > 0.f ? float(kSahBins) / ext : 0.f;
    }
}

__device__ __forceinline__ uint32_t node_of_chunk(const SahNode* __restrict__ nodes, uint32_t nact, uint32_t c) {
    uint32_t lo = 0, hi = nact;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (nodes[mid].chunk0 <= c) lo = mid; else hi = mid;
    }
    return lo;
}

__global__ void k_sah_records(const float4* __restrict__ prims, uint32_t n, SahRec* __restrict__ recs,
                              uint32_t* __restrict__ out_ids) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Box3 b = prim_box(prims + 3 * size_t(i));
    recs[i].lo_id = make_float4(b.lo.x, b.lo.y, b.lo.z, __uint_as_float(i));
    recs[i].hi = make_float4(b.hi.x, b.hi.y, b.hi.z, 0.f);
    out_ids[i] = i;
}

__global__ void k_sah_nchunks(const SahNode* __restrict__ nodes, uint32_t nact, uint32_t* __restrict__ nch) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nact) return;
    nch[i] = (nodes[i].count + kSahChunk - 1) / kSahChunk;
}

// chunk0 of every node from the scanned chunk counts; the total to the counters;
// the node's bins emptied.
__global__ void k_sah_prepare(SahNode* __restrict__ nodes, uint32_t nact, const uint32_t* __restrict__ chunk0,
                              SahCounters* __restrict__ ctr, uint32_t* __restrict__ bins) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nact) {
        nodes[i].chunk0 = chunk0[i];
        if (i == nact - 1) {
            ctr->nchunks = chunk0[i] + (nodes[i].count + kSahChunk - 1) / kSahChunk;
            ctr->nnext = 0;
        }
    }
    const size_t words = size_t(nact) * 3 * kSahBins * kBinWords;
    for (size_t w = i; w < words; w += size_t(gridDim.x) * blockDim.x) {
        const uint32_t k = uint32_t(w % kBinWords);
        bins[w] = (k >= 1 && k <= 3) ? 0xFFFFFFFFu : 0u;
    }
}

// One block per chunk of a node: per-axis bins of the chunk in shared memory
// (lanes of a warp that fall into one bin reduce first, their leader updates
// shared memory), then added to the node's bins; the chunk's bin counts are
// kept for the partition offsets.
__global__ void __launch_bounds__(kSahThreads)
    k_sah_bin(const SahRec* __restrict__ recs, const SahNode* __restrict__ nodes, uint32_t nact,
              uint32_t* __restrict__ bins, uint32_t* __restrict__ chunk_counts) {
    __shared__ uint32_t sb[3 * kSahBins * kBinWords];
    const uint32_t c = blockIdx.x;
    const uint32_t ni = node_of_chunk(nodes, nact, c);
    const SahNode& nd = nodes[ni];
    const uint32_t b = nd.start + (c - nd.chunk0) * kSahChunk;
    const uint32_t e = min(b + kSahChunk, nd.start + nd.count);
    for (uint32_t w = threadIdx.x; w < 3 * kSahBins * kBinWords; w += blockDim.x) {
        const uint32_t k = w % kBinWords;
        sb[w] = (k >= 1 && k <= 3) ? 0xFFFFFFFFu : 0u;
    }
    float lo[3], scale[3];
    sah_frame(nd.cb, lo, scale);
    __syncthreads();
    const uint32_t lane = threadIdx.x & 31u;
    for (uint32_t base = b; base < e; base += blockDim.x) {
        const uint32_t p = base + threadIdx.x;
        const bool valid = p < e;
        SahRec r{};
        if (valid) r = recs[p];
        const float cc[3] = {0.5f * (r.lo_id.x + r.hi.x), 0.5f * (r.lo_id.y + r.hi.y), 0.5f * (r.lo_id.z + r.hi.z)};
        const uint32_t box[6] = {ford(r.lo_id.x), ford(r.lo_id.y), ford(r.lo_id.z),
                                 ford(r.hi.x), ford(r.hi.y), ford(r.hi.z)};
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const uint32_t bin = valid ? sah_bin(cc[a], lo[a], scale[a]) : 0xFFFFu;
            const uint32_t g = __match_any_sync(0xFFFFFFFFu, bin);
            if (valid) {
                const uint32_t m0 = __reduce_min_sync(g, box[0]);
                const uint32_t m1 = __reduce_min_sync(g, box[1]);
                const uint32_t m2 = __reduce_min_sync(g, box[2]);
                const uint32_t x0 = __reduce_max_sync(g, box[3]);
                const uint32_t x1 = __reduce_max_sync(g, box[4]);
                const uint32_t x2 = __reduce_max_sync(g, box[5]);
                if (lane == uint32_t(__ffs(g) - 1)) {
                    uint32_t* s = sb + (a * kSahBins + bin) * kBinWords;
                    atomicAdd(&s[0], uint32_t(__popc(g)));
                    atomicMin(&s[1], m0); atomicMin(&s[2], m1); atomicMin(&s[3], m2);
                    atomicMax(&s[4], x0); atomicMax(&s[5], x1); atomicMax(&s[6], x2);
                }
            }
        }
    }
    __syncthreads();
    for (uint32_t t = threadIdx.x; t < 3 * kSahBins; t += blockDim.x) {
        const uint32_t* s = sb + t * kBinWords;
        chunk_counts[size_t(c) * 3 * kSahBins + t] = s[0];
        if (s[0]) {
            uint32_t* g = bins + (size_t(ni) * 3 * kSahBins + t) * kBinWords;
            atomicAdd(&g[0], s[0]);
            atomicMin(&g[1], s[1]); atomicMin(&g[2], s[2]); atomicMin(&g[3], s[3]);
            atomicMax(&g[4], s[4]); atomicMax(&g[5], s[5]); atomicMax(&g[6], s[6]);
        }
    }
}

__device__ __forceinline__ float box_area(float3 lo, float3 hi) {
    const float dx = fmaxf(hi.x - lo.x, 0.f), dy = fmaxf(hi.y - lo.y, 0.f), dz = fmaxf(hi.z - lo.z, 0.f);
    return 2.f * (dx * dy + dy * dz + dz * dx);
}

// One warp per node: the least-cost split over 3 x 31 bin borders (ties: the
// lower axis, then the lower border), the median position where no border
// separates records or the level cap is reached; children allocated, the
// split node recorded and linked to its parent, the chunks' left offsets.
__global__ void k_sah_split(SahNode* __restrict__ nodes, uint32_t nact, const uint32_t* __restrict__ bins,
                            const uint32_t* __restrict__ chunk_counts, uint32_t* __restrict__ chunk_left,
                            SahNode* __restrict__ next, SahCluster* __restrict__ clusters,
                            SahSplit* __restrict__ splits, SahCounters* __restrict__ ctr, uint32_t cluster_max,
                            int median_only) {
    const uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t lane = threadIdx.x & 31u;
    if (w >= nact) return;
    SahNode nd = nodes[w];
    float best = INFINITY;
    int axis = -1, bin = 0;
    uint32_t nleft = nd.count / 2;
    if (!median_only) {
        for (int a = 0; a < 3; ++a) {
            const uint32_t* g = bins + (size_t(w) * 3 * kSahBins + a * kSahBins + lane) * kBinWords;
            uint32_t cnt = g[0];
            float3 blo = cnt ? mk(fdeord(g[1]), fdeord(g[2]), fdeord(g[3])) : mk(INFINITY, INFINITY, INFINITY);
            float3 bhi = cnt ? mk(fdeord(g[4]), fdeord(g[5]), fdeord(g[6])) : mk(-INFINITY, -INFINITY, -INFINITY);
            // prefix (bins 0..lane) and suffix (bins lane..31)
            uint32_t pc = cnt, sc = cnt;
            float3 plo = blo, phi = bhi, slo = blo, shi = bhi;
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t uc = __shfl_up_sync(0xFFFFFFFFu, pc, o);
                const float3 ulo = mk(__shfl_up_sync(0xFFFFFFFFu, plo.x, o), __shfl_up_sync(0xFFFFFFFFu, plo.y, o),
                                      __shfl_up_sync(0xFFFFFFFFu, plo.z, o));
                const float3 uhi = mk(__shfl_up_sync(0xFFFFFFFFu, phi.x, o), __shfl_up_sync(0xFFFFFFFFu, phi.y, o),
                                      __shfl_up_sync(0xFFFFFFFFu, phi.z, o));
                const uint32_t dc = __shfl_down_sync(0xFFFFFFFFu, sc, o);
                const float3 dlo = mk(__shfl_down_sync(0xFFFFFFFFu, slo.x, o),
                                      __shfl_down_sync(0xFFFFFFFFu, slo.y, o),
                                      __shfl_down_sync(0xFFFFFFFFu, slo.z, o));
                const float3 dhi = mk(__shfl_down_sync(0xFFFFFFFFu, shi.x, o),
                                      __shfl_down_sync(0xFFFFFFFFu, shi.y, o),
                                      __shfl_down_sync(0xFFFFFFFFu, shi.z, o));
                if (lane >= uint32_t(o)) {
                    pc += uc;
                    plo = mk(fminf(plo.x, ulo.x), fminf(plo.y, ulo.y), fminf(plo.z, ulo.z));
                    phi = mk(fmaxf(phi.x, uhi.x), fmaxf(phi.y, uhi.y), fmaxf(phi.z, uhi.z));
                }
                if (lane + o < 32) {
                    sc += dc;
                    slo = mk(fminf(slo.x, dlo.x), fminf(slo.y, dlo.y), fminf(slo.z, dlo.z));
                    shi = mk(fmaxf(shi.x, dhi.x), fmaxf(shi.y, dhi.y), fmaxf(shi.z, dhi.z));
                }
            }
            // border lane + 1: left = bins 0..lane (own prefix), right = bins lane+1..31
            const uint32_t rc = __shfl_down_sync(0xFFFFFFFFu, sc, 1);
            const float3 rlo = mk(__shfl_down_sync(0xFFFFFFFFu, slo.x, 1), __shfl_down_sync(0xFFFFFFFFu, slo.y, 1),
                                  __shfl_down_sync(0xFFFFFFFFu, slo.z, 1));
            const float3 rhi = mk(__shfl_down_sync(0xFFFFFFFFu, shi.x, 1), __shfl_down_sync(0xFFFFFFFFu, shi.y, 1),
                                  __shfl_down_sync(0xFFFFFFFFu, shi.z, 1));
            float cost = INFINITY;
            if (lane < 31 && pc > 0 && rc > 0) cost = box_area(plo, phi) * float(pc) + box_area(rlo, rhi) * float(rc);
            // warp argmin (cost, lane)
            float bc = cost;
            uint32_t bl = lane;
            for (int o = 16; o > 0; o >>= 1) {
                const float oc = __shfl_xor_sync(0xFFFFFFFFu, bc, o);
                const uint32_t ol = __shfl_xor_sync(0xFFFFFFFFu, bl, o);
                if (oc < bc || (oc == bc && ol < bl)) { bc = oc; bl = ol; }
            }
            const uint32_t bpc = __shfl_sync(0xFFFFFFFFu, pc, bl);
            if (bc < best) {
                best = bc;
                axis = a;
                bin = int(bl) + 1;
                nleft = bpc;
            }
        }
    }
    const uint32_t nch = (nd.count + kSahChunk - 1) / kSahChunk;
    if (lane == 0) {
        const uint32_t sid = atomicAdd(&ctr->nsplit, 1u);
        SahSplit sp;
        sp.start = nd.start;
        sp.split = nd.start + nleft;
        sp.end = nd.start + nd.count;
        sp.child[0] = sp.child[1] = -1;
        sp.parent = nd.parent;
        sp.seg = nd.seg;
        for (int k = 0; k < 2; ++k) {
            const uint32_t cs = k ? nd.start + nleft : nd.start;
            const uint32_t cn = k ? nd.count - nleft : nleft;
            if (cn > cluster_max) {
                const uint32_t id = atomicAdd(&ctr->nnext, 1u);
                SahNode ch;
                ch.start = cs;
                ch.count = cn;
                ch.parent = int(sid);
                ch.side = uint32_t(k);
                ch.seg = nd.seg;
                ch.cb[0] = ch.cb[1] = ch.cb[2] = 0xFFFFFFFFu;
                ch.cb[3] = ch.cb[4] = ch.cb[5] = 0u;
                ch.chunk0 = 0;
                ch.axis = -1;
                ch.bin = 0;
                ch.nleft = 0;
                ch.child[0] = ch.child[1] = 0;
                next[id] = ch;
                nd.child[k] = int(id);
            } else {
                const uint32_t id = atomicAdd(&ctr->ncl, 1u);
                SahCluster cl;
                cl.start = cs;
                cl.count = cn;
                cl.cb[0] = cl.cb[1] = cl.cb[2] = 0xFFFFFFFFu;
                cl.cb[3] = cl.cb[4] = cl.cb[5] = 0u;
                clusters[id] = cl;
                nd.child[k] = ~int(id);
            }
        }
        splits[sid] = sp;
        if (nd.parent >= 0) splits[nd.parent].child[nd.side] = int(sid);
        nd.axis = axis;
        nd.bin = bin;
        nd.nleft = nleft;
        nodes[w] = nd;
    }
    // left records before each chunk of the node (stable partition offsets)
    uint32_t run = 0;
    for (uint32_t c0 = 0; c0 < nch; c0 += 32) {
        const uint32_t ci = c0 + lane;
        uint32_t l = 0;
        if (ci < nch) {
            if (axis >= 0) {
                const uint32_t* cc = chunk_counts + size_t(nd.chunk0 + ci) * 3 * kSahBins + axis * kSahBins;
                for (int k = 0; k < bin; ++k) l += cc[k];
            } else {
                const uint32_t first = ci * kSahChunk;
                const uint32_t len = min(kSahChunk, nd.count - first);
                l = nleft > first ? min(nleft - first, len) : 0u;
            }
        }
        uint32_t x = l;   // inclusive warp scan
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
            if (lane >= uint32_t(o)) x += y;
        }
        if (ci < nch) chunk_left[nd.chunk0 + ci] = run + x - l;
        run += __shfl_sync(0xFFFFFFFFu, x, 31);
    }
}

// One block per chunk: stable partition of the chunk's records into the two
// children (block-wide ranks from warp ballots), records of a cluster child
// also to their final position in out_ids; centroid bounds of both children
// accumulated.
__global__ void __launch_bounds__(kSahThreads)
    k_sah_partition(const SahRec* __restrict__ recs, SahRec* __restrict__ out, const SahNode* __restrict__ nodes,
                    uint32_t nact, const uint32_t* __restrict__ chunk_left, SahNode* __restrict__ next,
                    SahCluster* __restrict__ clusters, uint32_t* __restrict__ out_ids, SahCounters* __restrict__ ctr) {
    __shared__ uint32_t s_warp[kSahThreads / 32];
    __shared__ uint32_t s_cb[12];
    const uint32_t c = blockIdx.x;
    const uint32_t ni = node_of_chunk(nodes, nact, c);
    const SahNode& nd = nodes[ni];
    const uint32_t b = nd.start + (c - nd.chunk0) * kSahChunk;
    const uint32_t e = min(b + kSahChunk, nd.start + nd.count);
    const uint32_t left_base = chunk_left[c];
    const uint32_t before = b - nd.start;   // records of the node before this chunk
    const int axis = nd.axis;
    const uint32_t bin = uint32_t(nd.bin), nleft = nd.nleft;
    float lo[3], scale[3];
    sah_frame(nd.cb, lo, scale);
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    if (threadIdx.x < 12) s_cb[threadIdx.x] = (threadIdx.x % 6) < 3 ? 0xFFFFFFFFu : 0u;
    uint32_t acc[12];   // child 0 lo xyz, hi xyz, child 1 lo xyz, hi xyz
#pragma unroll
    for (int k = 0; k < 12; ++k) acc[k] = (k % 6) < 3 ? 0xFFFFFFFFu : 0u;
    uint32_t run = 0;   // left records of this chunk in earlier rounds
    for (uint32_t base = b; base < e; base += blockDim.x) {
        const uint32_t p = base + threadIdx.x;
        const bool valid = p < e;
        SahRec r{};
        if (valid) r = recs[p];
        const float cc[3] = {0.5f * (r.lo_id.x + r.hi.x), 0.5f * (r.lo_id.y + r.hi.y), 0.5f * (r.lo_id.z + r.hi.z)};
        bool left = false;
        if (valid) left = axis >= 0 ? sah_bin(cc[axis], lo[axis], scale[axis]) < bin : (p - nd.start) < nleft;
        const uint32_t ballot = __ballot_sync(0xFFFFFFFFu, left);
        if (lane == 0) s_warp[warp] = __popc(ballot);
        __syncthreads();
        uint32_t woff = 0, total = 0;
        for (uint32_t k = 0; k < blockDim.x / 32; ++k) {
            const uint32_t v = s_warp[k];
            woff += k < warp ? v : 0u;
            total += v;
        }
        if (valid) {
            const uint32_t lbefore = run + woff + __popc(ballot & ((1u << lane) - 1u));   // lefts before p in chunk
            const uint32_t pos_in_chunk = p - b;
            const uint32_t dest = left ? nd.start + left_base + lbefore
                                       : nd.start + nleft + (before - left_base) + (pos_in_chunk - lbefore);
            const int ch = nd.child[left ? 0 : 1];
            // the binning and this pass bin identically, so dest stays inside the
            // child; the check only guards the writes
            const uint32_t cb = left ? nd.start : nd.start + nleft;
            const uint32_t ce = left ? nd.start + nleft : nd.start + nd.count;
            if (dest < cb || dest >= ce) atomicOr(&ctr->err, 1u);
            else if (ch >= 0) out[dest] = r;
            else out_ids[dest] = __float_as_uint(r.lo_id.w);
            const int o = left ? 0 : 6;
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                const uint32_t v = ford(cc[a]);
                acc[o + a] = min(acc[o + a], v);
                acc[o + 3 + a] = max(acc[o + 3 + a], v);
            }
        }
        run += total;
        __syncthreads();   // s_warp is rewritten in the next round
    }
#pragma unroll
    for (int k = 0; k < 12; ++k) {
        const uint32_t v = (k % 6) < 3 ? __reduce_min_sync(0xFFFFFFFFu, acc[k]) : __reduce_max_sync(0xFFFFFFFFu, acc[k]);
        if (lane == 0) {
            if ((k % 6) < 3) atomicMin(&s_cb[k], v); else atomicMax(&s_cb[k], v);
        }
    }
    __syncthreads();
    if (threadIdx.x < 12) {
        const uint32_t k = threadIdx.x;
        const int ch = nd.child[k / 6];
        const uint32_t v = s_cb[k];
        const bool empty = (k % 6) < 3 ? v == 0xFFFFFFFFu : v == 0u;
        if (!empty) {
            uint32_t* dst = ch >= 0 ? next[ch].cb : clusters[~ch].cb;
            if ((k % 6) < 3) atomicMin(&dst[k % 6], v); else atomicMax(&dst[k % 6], v);
        }
    }
}

// Cluster table in position order: rank r -> (start, count), bounds.
__global__ void k_sah_cluster_table(const SahCluster* __restrict__ clusters, const uint32_t* __restrict__ order,
                                    uint32_t ncl, SegDev* __restrict__ tsegs, uint32_t* __restrict__ tcb) {
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= ncl) return;
    const SahCluster& c = clusters[order[r]];
    tsegs[r] = SegDev{c.start, c.count};
#pragma unroll
    for (int k = 0; k < 6; ++k) tcb[6 * size_t(r) + k] = c.cb[k];
}

__global__ void k_sah_cluster_keys(const SahCluster* __restrict__ clusters, uint32_t ncl, uint32_t* __restrict__ keys,
                                   uint32_t* __restrict__ vals) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ncl) return;
    keys[i] = clusters[i].start;
    vals[i] = i;
}

// Keys cluster << 30 | 30-bit Morton code inside the cluster's centroid bounds.
__global__ void k_sah_codes(const float4* __restrict__ prims, const uint32_t* __restrict__ out_ids, uint32_t n,
                            const SegDev* __restrict__ tsegs, uint32_t ncl, const uint32_t* __restrict__ tcb,
                            unsigned long long* __restrict__ codes, uint32_t* __restrict__ ids) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t r = seg_of(tsegs, ncl, i);
    const uint32_t id = out_ids[i];
    const uint32_t* b = tcb + 6 * size_t(r);
    const float3 lo = mk(fdeord(b[0]), fdeord(b[1]), fdeord(b[2]));
    const float3 hi = mk(fdeord(b[3]), fdeord(b[4]), fdeord(b[5]));
    const float3 ext = sub(hi, lo);
    const float3 c = centroid(prim_box(prims + 3 * size_t(id)));
    const uint32_t qx = uint32_t(quantf(c.x, lo.x, ext.x, 1024.f));
    const uint32_t qy = uint32_t(quantf(c.y, lo.y, ext.y, 1024.f));
    const uint32_t qz = uint32_t(quantf(c.z, lo.z, ext.z, 1024.f));
    codes[i] = ((unsigned long long)r << 30) | ((expand10(qx) << 2) | (expand10(qy) << 1) | expand10(qz));
    ids[i] = id;
}

// One thread per split node: it moves to slot split - 1 (the spare slot of
// the cluster ending at its split); its children become references (split
// child: its slot; cluster of two or more records: the cluster's root slot,
// its first; single record: the leaf) and get their parents.
__global__ void k_sah_stitch(const SahSplit* __restrict__ splits, uint32_t nsplit, float4* __restrict__ nodes,
                             int* __restrict__ parent_leaf, int* __restrict__ parent_int, int* __restrict__ roots) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nsplit) return;
    const SahSplit sp = splits[t];
    const int D = int(sp.split) - 1;
    int ref[2];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        const uint32_t cs = k ? sp.split : sp.start;
        const uint32_t ce = k ? sp.end : sp.split;
        if (sp.child[k] >= 0) {
            ref[k] = int(splits[sp.child[k]].split) - 1;
            parent_int[ref[k]] = D;
        } else if (ce - cs >= 2) {
            ref[k] = int(cs);
            parent_int[cs] = D;
        } else {
            ref[k] = ~int(cs);
            parent_leaf[cs] = D;
        }
    }
    nodes[4 * size_t(D) + 3] = make_float4(__int_as_float(ref[0]), __int_as_float(ref[1]), 0.f, 0.f);
    if (sp.parent < 0) {
        parent_int[D] = -1;
        roots[sp.seg] = D;
    }
}

template <class T>
T* carve(char*& p, size_t count) {
    T* r = reinterpret_cast<T*>(p);
    p += (count * sizeof(T) + 255) & ~size_t(255);
    return r;
}

}  // namespace

void build_sah_topology(Lbvh& L, uint32_t cluster_max, cudaStream_t s) {
    const uint32_t n = L.nprims;
    const uint32_t ns = L.nsegs;
    // segment centroid bounds (already reduced by the caller) to the host
    std::vector<uint32_t> sb(6 * size_t(ns));
    RT_CUDA(cudaMemcpyAsync(sb.data(), L.bounds.p, sb.size() * 4, cudaMemcpyDeviceToHost, s));
    RT_CUDA(cudaStreamSynchronize(s));
    std::vector<SahNode> seed;
    std::vector<SahCluster> seed_cl;
    L.roots.assign(ns, -1);
    for (uint32_t g = 0; g < ns; ++g) {
        const SegDev sg = L.seg_host[g];
        if (sg.prim_count == 0) continue;
        if (sg.prim_count > cluster_max) {
            SahNode nd{};
            nd.start = sg.prim_begin;
            nd.count = sg.prim_count;
            nd.parent = -1;
            nd.seg = g;
            for (int k = 0; k < 6; ++k) nd.cb[k] = sb[6 * g + k];
            seed.push_back(nd);
        } else {
            SahCluster cl{};
            cl.start = sg.prim_begin;
            cl.count = sg.prim_count;
            for (int k = 0; k < 6; ++k) cl.cb[k] = sb[6 * g + k];
            seed_cl.push_back(cl);
            L.roots[g] = int(sg.prim_begin);   // a single cluster: its Karras root (or its only record)
        }
    }
    // scratch: records x2, node lists x2, bins, chunk tables, clusters, splits
    // per level at most n / (cluster_max + 1) nodes are split (disjoint
    // ranges above the cluster size); over all levels there are fewer splits
    // and clusters than records
    const size_t max_nodes = size_t(n) / (cluster_max + 1) + ns + 1;
    const size_t max_chunks = size_t(n) / kSahChunk + max_nodes + 1;
    const size_t max_cl = size_t(n) + 1;
    const size_t max_split = size_t(n) + 1;
    SahRec* rec[2];
    SahNode* nodes[2];
    uint32_t *bins, *chunk_counts, *nch, *chunk0, *chunk_left, *out_ids, *ckeys, *cvals, *tcb;
    SahCluster* clusters;
    SahSplit* splits;
    SegDev* tsegs;
    SahCounters* ctr;
    int* roots_dev;
    auto layout = [&](char* p) {   // carves the scratch; returns its size
        char* const p0 = p;
        rec[0] = carve<SahRec>(p, n);
        rec[1] = carve<SahRec>(p, n);
        nodes[0] = carve<SahNode>(p, max_nodes);
        nodes[1] = carve<SahNode>(p, max_nodes);
        bins = carve<uint32_t>(p, max_nodes * 3 * kSahBins * kBinWords);
        chunk_counts = carve<uint32_t>(p, max_chunks * 3 * kSahBins);
        nch = carve<uint32_t>(p, max_chunks);
        chunk0 = carve<uint32_t>(p, max_chunks);
        chunk_left = carve<uint32_t>(p, max_chunks);
        clusters = carve<SahCluster>(p, max_cl);
        splits = carve<SahSplit>(p, max_split);
        out_ids = carve<uint32_t>(p, n);
        ckeys = carve<uint32_t>(p, max_cl);
        cvals = carve<uint32_t>(p, max_cl);
        tsegs = carve<SegDev>(p, max_cl);
        tcb = carve<uint32_t>(p, max_cl * 6);
        ctr = carve<SahCounters>(p, 1);
        roots_dev = carve<int>(p, ns);
        return size_t(p - p0);
    };
    L.sah_tmp.reserve(layout(reinterpret_cast<char*>(uintptr_t(256))));
    layout(L.sah_tmp.as<char>());

    SahCounters c0{0u, uint32_t(seed_cl.size()), 0u, 0u, 0u};
    RT_CUDA(cudaMemcpyAsync(ctr, &c0, sizeof c0, cudaMemcpyHostToDevice, s));
    if (!seed.empty())
        RT_CUDA(cudaMemcpyAsync(nodes[0], seed.data(), seed.size() * sizeof(SahNode), cudaMemcpyHostToDevice, s));
    if (!seed_cl.empty())
        RT_CUDA(cudaMemcpyAsync(clusters, seed_cl.data(), seed_cl.size() * sizeof(SahCluster), cudaMemcpyHostToDevice,
                                s));
    RT_CUDA(cudaMemsetAsync(roots_dev, 0xFF, ns * 4, s));
    k_sah_records<<<(n + kSahThreads - 1) / kSahThreads, kSahThreads, 0, s>>>(L.prims_flat.as<float4>(), n, rec[0],
                                                                               out_ids);
    RT_CHECK_LAUNCH();
    uint32_t nact = uint32_t(seed.size());
    int cur = 0, level = 0;
    SahCounters hc{};
    for (; nact > 0; ++level) {
        RT_REQUIRE(nact <= max_nodes, "internal: SAH level overflow");
        k_sah_nchunks<<<(nact + kSahThreads - 1) / kSahThreads, kSahThreads, 0, s>>>(nodes[cur], nact, nch);
        RT_CHECK_LAUNCH();
        scan_exclusive_u32(nch, chunk0, nact, L.sort_tmp, s);
        const uint32_t prep_blocks = std::min<uint32_t>(
            4096u, uint32_t((size_t(nact) * 3 * kSahBins * kBinWords + kSahThreads - 1) / kSahThreads));
        k_sah_prepare<<<std::max(prep_blocks, (nact + kSahThreads - 1) / kSahThreads), kSahThreads, 0, s>>>(
            nodes[cur], nact, chunk0, ctr, bins);
        RT_CHECK_LAUNCH();
        RT_CUDA(cudaMemcpyAsync(&hc, ctr, sizeof hc, cudaMemcpyDeviceToHost, s));
        RT_CUDA(cudaStreamSynchronize(s));
        const uint32_t nchunks = hc.nchunks;
        RT_REQUIRE(nchunks <= max_chunks, "internal: SAH chunk overflow");
        k_sah_bin<<<nchunks, kSahThreads, 0, s>>>(rec[cur], nodes[cur], nact, bins, chunk_counts);
        RT_CHECK_LAUNCH();
        k_sah_split<<<(nact * 32 + 127) / 128, 128, 0, s>>>(nodes[cur], nact, bins, chunk_counts, chunk_left,
                                                            nodes[cur ^ 1], clusters, splits, ctr, cluster_max,
                                                            level >= kSahMaxLevels ? 1 : 0);
        RT_CHECK_LAUNCH();
        k_sah_partition<<<nchunks, kSahThreads, 0, s>>>(rec[cur], rec[cur ^ 1], nodes[cur], nact, chunk_left,
                                                        nodes[cur ^ 1], clusters, out_ids, ctr);
        RT_CHECK_LAUNCH();
        RT_CUDA(cudaMemcpyAsync(&hc, ctr, sizeof hc, cudaMemcpyDeviceToHost, s));
        RT_CUDA(cudaStreamSynchronize(s));
        if (hc.err) throw Error(RT_ERR_INTERNAL, "SAH build: partition and binning disagree");
        nact = hc.nnext;
        cur ^= 1;
    }
    RT_CUDA(cudaMemcpyAsync(&hc, ctr, sizeof hc, cudaMemcpyDeviceToHost, s));
    RT_CUDA(cudaStreamSynchronize(s));
    const uint32_t ncl = hc.ncl, nsplit = hc.nsplit;
    RT_REQUIRE(ncl <= max_cl && nsplit <= max_split, "internal: SAH cluster overflow");
    // clusters in position order
    k_sah_cluster_keys<<<(ncl + kSahThreads - 1) / kSahThreads, kSahThreads, 0, s>>>(clusters, ncl, ckeys, cvals);
    RT_CHECK_LAUNCH();
    int pos_bits = 1;
    while ((uint64_t(1) << pos_bits) < n) ++pos_bits;
    radix_sort_pairs_u32(ckeys, cvals, ncl, pos_bits, L.sort_tmp, s);
    k_sah_cluster_table<<<(ncl + kSahThreads - 1) / kSahThreads, kSahThreads, 0, s>>>(clusters, cvals, ncl, tsegs,
                                                                                       tcb);
    RT_CHECK_LAUNCH();
    // cluster-local Morton keys, sorted; Karras per cluster; splits stitched on top
    L.codes.reserve(size_t(n) * 8);
    L.ids.reserve(size_t(n) * 4);
    unsigned long long* codes = L.codes.as<unsigned long long>();
    uint32_t* ids = L.ids.as<uint32_t>();
    k_sah_codes<<<(n + kSahThreads - 1) / kSahThreads, kSahThreads, 0, s>>>(L.prims_flat.as<float4>(), out_ids, n,
                                                                             tsegs, ncl, tcb, codes, ids);
    RT_CHECK_LAUNCH();
    int cl_bits = 1;
    while ((uint64_t(1) << cl_bits) < ncl) ++cl_bits;
    radix_sort_pairs_u64(codes, ids, n, 30 + cl_bits, L.sort_tmp, s);
    int* parents = L.parents.as<int>();
    k_karras<unsigned long long><<<(n + kSahThreads - 1) / kSahThreads, kSahThreads, 0, s>>>(
        codes, tsegs, ncl, n, L.nodes.as<float4>(), parents, parents + n);
    RT_CHECK_LAUNCH();
    if (nsplit) {
        k_sah_stitch<<<(nsplit + kSahThreads - 1) / kSahThreads, kSahThreads, 0, s>>>(
            splits, nsplit, L.nodes.as<float4>(), parents, parents + n, roots_dev);
        RT_CHECK_LAUNCH();
        std::vector<int> r(ns);
        RT_CUDA(cudaMemcpyAsync(r.data(), roots_dev, ns * 4, cudaMemcpyDeviceToHost, s));
        RT_CUDA(cudaStreamSynchronize(s));
        for (uint32_t g = 0; g < ns; ++g)
            if (r[g] >= 0) L.roots[g] = r[g];
    }
    L.nclusters = ncl;
    L.sah_levels = uint32_t(level);
}

}  // namespace rt
