// rt_sah.cu -- binned-SAH hierarchy over the flattened world-space records.
//
// Replaces the closed optixAccelBuild of Scene::build (optx/scene.cxx:227-273)
// by a builder whose tree depends on the geometry, not on a space-filling
// curve alone.  Top-down, one level of the tree per pass over the records:
// every node of the level is binned (32 bins per axis over its centroid
// bounds), the split of least surface-area cost is taken (Wald 2007) and the
// node's records are partitioned stably; nodes of at most `cluster_max`
// records become clusters.  Each cluster then gets a Karras 2012 hierarchy
// over 30-bit Morton codes inside its own centroid bounds (keys cluster << 30
// | code), and the split nodes above the clusters are stitched into the spare
// node slot of each cluster: a split whose left part ends at record position
// p lives in slot p - 1, the last slot of the cluster ending there, which that
// cluster's own n - 1 internal nodes leave free.
//
// A level holds big nodes (more than kSahChunk records: binned by many
// blocks, split by one warp, partitioned by many blocks with offsets from a
// scan), block nodes (binned, split and partitioned by one block in one
// launch) and warp nodes (the same by one warp, at most kWarpNode records).  Everything is a function of the records alone (allocation
// order does not reach the result: slots follow from positions), so a rebuild
// gives the same tree.  The host reads the counters once or twice per level;
// no kernel waits on another block.
#include <algorithm>
#include <vector>

#include "rt_lbvh.cuh"

namespace rt {
namespace {

constexpr int kSahBins = 32;
constexpr uint32_t kSahChunk = 2048;   // records per block; larger nodes are big nodes
constexpr int kSahThreads = 256;
constexpr int kSahMaxLevels = 64;      // deeper levels split at the median position
constexpr int kBinWords = 7;           // count, box lo xyz, box hi xyz (orderable u32)
constexpr uint32_t kBinTotal = 3 * kSahBins * kBinWords;

// A record on its way down: box and record id.
struct SahRec {
    float4 lo_id;   // box lo, record id (bits)
    float4 hi;      // box hi
};

constexpr int kBig = 0, kBlock = 1, kWarp = 2, kCluster = 3;
constexpr uint32_t kWarpNode = 256;   // nodes of at most this many records: one warp each

// A node of the current level.
struct SahNode {
    uint32_t start, count;
    int parent;        // split node of the parent, -1 at a segment root
    uint32_t side;     // which child of the parent
    uint32_t seg;      // segment (scene) of the records
    uint32_t cb[6];    // centroid bounds, orderable u32 (lo xyz, hi xyz)
    uint32_t chunk0;   // big nodes: first chunk in the level's chunk table
    int axis;          // chosen split: axis (-1: median position), bin, left count
    int bin;
    uint32_t nleft;
    int child[2];      // index in the next level's list of its kind, or the cluster
    int ckind[2];      // kBig, kBlock, kWarp or kCluster
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
    uint32_t next[2][3];   // node lists by level parity: big, block, warp nodes
    uint32_t ncl, nchunks, err;
};

// Where the children of a level's nodes go.
struct SahOut {
    SahNode* big;
    SahNode* block;
    SahNode* warp;
    SahCluster* clusters;
    SahSplit* splits;
    SahCounters* ctr;
    uint32_t nx;            // parity of the next level
    uint32_t cluster_max;
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

__device__ __forceinline__ void empty_bins(uint32_t* b, uint32_t first, uint32_t step) {
    for (uint32_t w = first; w < kBinTotal; w += step) {
        const uint32_t k = w % kBinWords;
        b[w] = (k >= 1 && k <= 3) ? 0xFFFFFFFFu : 0u;
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

__device__ __forceinline__ float3 rec_centroid(const SahRec& r) {
    return mk(0.5f * (r.lo_id.x + r.hi.x), 0.5f * (r.lo_id.y + r.hi.y), 0.5f * (r.lo_id.z + r.hi.z));
}

// Adds one batch of records (one per lane, `valid`) to shared bins: lanes of
// a warp in one bin reduce first, their leader updates shared memory.  Every
// lane of the warp must call it.
__device__ __forceinline__ void bin_records(uint32_t* sb, const SahRec& r, bool valid, const float lo[3],
                                            const float scale[3], uint32_t lane) {
    const float3 c = rec_centroid(r);
    const float cc[3] = {c.x, c.y, c.z};
    const uint32_t box[6] = {ford(r.lo_id.x), ford(r.lo_id.y), ford(r.lo_id.z), ford(r.hi.x), ford(r.hi.y),
                             ford(r.hi.z)};
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

// chunk0 of every big node from the scanned chunk counts, the total to the
// counters, the nodes' bins emptied.
__global__ void k_sah_prepare(SahNode* __restrict__ nodes, uint32_t nact, const uint32_t* __restrict__ chunk0,
                              SahCounters* __restrict__ ctr, uint32_t* __restrict__ bins) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nact) {
        nodes[i].chunk0 = chunk0[i];
        if (i == nact - 1) ctr->nchunks = chunk0[i] + (nodes[i].count + kSahChunk - 1) / kSahChunk;
    }
    const size_t words = size_t(nact) * kBinTotal;
    for (size_t w = i; w < words; w += size_t(gridDim.x) * blockDim.x) {
        const uint32_t k = uint32_t(w % kBinWords);
        bins[w] = (k >= 1 && k <= 3) ? 0xFFFFFFFFu : 0u;
    }
}

// Big nodes, one block per chunk: the chunk's bins in shared memory, added to
// the node's bins; the chunk's bin counts kept for the partition offsets.
__global__ void __launch_bounds__(kSahThreads)
    k_sah_bin(const SahRec* __restrict__ recs, const SahNode* __restrict__ nodes, uint32_t nact,
              uint32_t* __restrict__ bins, uint32_t* __restrict__ chunk_counts, const SahCounters* ctr) {
    __shared__ uint32_t sb[kBinTotal];
    const uint32_t c = blockIdx.x;
    if (c >= *((volatile uint32_t*)&ctr->nchunks)) return;   // the grid is an upper bound
    const uint32_t ni = node_of_chunk(nodes, nact, c);
    const SahNode& nd = nodes[ni];
    const uint32_t b = nd.start + (c - nd.chunk0) * kSahChunk;
    const uint32_t e = min(b + kSahChunk, nd.start + nd.count);
    empty_bins(sb, threadIdx.x, blockDim.x);
    float lo[3], scale[3];
    sah_frame(nd.cb, lo, scale);
    __syncthreads();
    const uint32_t lane = threadIdx.x & 31u;
    for (uint32_t base = b; base < e; base += blockDim.x) {
        const uint32_t p = base + threadIdx.x;
        const bool valid = p < e;
        SahRec r{};
        if (valid) r = recs[p];
        bin_records(sb, r, valid, lo, scale, lane);
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

// Least-cost split of one node from its bins (3 axes x 32 bins x kBinWords,
// one warp, lane = bin): the border of least surface-area cost over 3 x 31
// borders (ties: the lower axis, then the lower border); axis stays -1 where
// no border separates records.
__device__ __forceinline__ void best_split(const uint32_t* nb, uint32_t lane, int& axis, int& bin, uint32_t& nleft) {
    float best = INFINITY;
    for (int a = 0; a < 3; ++a) {
        const uint32_t* g = nb + (a * kSahBins + lane) * kBinWords;
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

__device__ __forceinline__ int child_kind(uint32_t count, uint32_t cluster_max) {
    return count <= cluster_max ? kCluster : count > kSahChunk ? kBig : count > kWarpNode ? kBlock : kWarp;
}

__device__ __forceinline__ uint32_t* kind_counter(int kind, const SahOut& out) {
    return kind == kCluster ? &out.ctr->ncl : &out.ctr->next[out.nx][kind];
}

// Records split `sid` of node nd (left part nleft records) and its children,
// whose kinds and list indices the caller allocated: nodes of the next level
// or clusters, each with empty centroid bounds; links the split to its
// parent.  Split ids are positions in the level's node order, so they need
// no counter.  One thread.
__device__ void emit_split(SahNode& nd, uint32_t nleft, uint32_t sid, const int kind[2], const uint32_t id[2],
                           const SahOut& out) {
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
        if (kind[k] != kCluster) {
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
            ch.ckind[0] = ch.ckind[1] = kCluster;
            (kind[k] == kBig ? out.big : kind[k] == kBlock ? out.block : out.warp)[id[k]] = ch;
        } else {
            SahCluster cl;
            cl.start = cs;
            cl.count = cn;
            cl.cb[0] = cl.cb[1] = cl.cb[2] = 0xFFFFFFFFu;
            cl.cb[3] = cl.cb[4] = cl.cb[5] = 0u;
            out.clusters[id[k]] = cl;
        }
        nd.child[k] = int(id[k]);
        nd.ckind[k] = kind[k];
    }
    out.splits[sid] = sp;
    if (nd.parent >= 0) out.splits[nd.parent].child[nd.side] = int(sid);
}

// emit_split with the children allocated one by one (one thread).
__device__ void emit_split_alloc(SahNode& nd, uint32_t nleft, uint32_t sid, const SahOut& out) {
    int kind[2];
    uint32_t id[2];
    for (int k = 0; k < 2; ++k) {
        kind[k] = child_kind(k ? nd.count - nleft : nleft, out.cluster_max);
        id[k] = atomicAdd(kind_counter(kind[k], out), 1u);
    }
    emit_split(nd, nleft, sid, kind, id, out);
}

__device__ __forceinline__ uint32_t* child_cb(const SahNode& nd, int k, const SahOut& out) {
    const int id = nd.child[k];
    const int kind = nd.ckind[k];
    return kind == kBig ? out.big[id].cb : kind == kBlock ? out.block[id].cb : kind == kWarp ? out.warp[id].cb
                                                                                           : out.clusters[id].cb;
}

// Big nodes, one warp each: the split (best_split, or the median position
// where no border separates records or the level cap is reached), children
// allocated.
__global__ void k_sah_split(SahNode* __restrict__ nodes, uint32_t nact, const uint32_t* __restrict__ bins,
                            SahOut out, uint32_t sid0, int median_only) {
    const uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t lane = threadIdx.x & 31u;
    if (w >= nact) return;
    SahNode nd = nodes[w];
    int axis = -1, bin = 0;
    uint32_t nleft = nd.count / 2;
    if (!median_only) best_split(bins + size_t(w) * kBinTotal, lane, axis, bin, nleft);
    if (lane == 0) {
        emit_split_alloc(nd, nleft, sid0 + w, out);
        nd.axis = axis;
        nd.bin = bin;
        nd.nleft = nleft;
        nodes[w] = nd;
    }
}

// Left records of every chunk of the big nodes (one thread per chunk); an
// exclusive scan over all chunks minus its value at the node's first chunk
// gives the left records before a chunk inside its node.
__global__ void k_sah_chunk_left(const SahNode* __restrict__ nodes, uint32_t nact, uint32_t bound,
                                 const uint32_t* __restrict__ chunk_counts, uint32_t* __restrict__ chunk_left,
                                 const SahCounters* ctr) {
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= bound) return;
    if (c >= ctr->nchunks) {   // past the level's chunks: zero, so the scan can run over the bound
        chunk_left[c] = 0;
        return;
    }
    const SahNode& nd = nodes[node_of_chunk(nodes, nact, c)];
    uint32_t l = 0;
    if (nd.axis >= 0) {
        const uint32_t* cc = chunk_counts + size_t(c) * 3 * kSahBins + nd.axis * kSahBins;
        for (int k = 0; k < nd.bin; ++k) l += cc[k];
    } else {
        const uint32_t first = (c - nd.chunk0) * kSahChunk;
        const uint32_t len = min(kSahChunk, nd.count - first);
        l = nd.nleft > first ? min(nd.nleft - first, len) : 0u;
    }
    chunk_left[c] = l;
}

// Stable partition of records [b, e) of node nd (a chunk, or a whole
// block node) into its children: block-wide ranks from warp ballots;
// `left_base` left records of the node precede b.  Records go to `out_rec`
// (child node) or, as ids, to out_ids (cluster); the children's centroid
// bounds are reduced into s_cb (12 orderable u32, lo xyz hi xyz per child).
__device__ __forceinline__ void partition_records(const SahRec* __restrict__ recs, SahRec* __restrict__ out_rec,
                                                  uint32_t* __restrict__ out_ids, const SahNode& nd, uint32_t b,
                                                  uint32_t e, uint32_t left_base, const float lo[3],
                                                  const float scale[3], uint32_t* s_warp, uint32_t* s_cb,
                                                  SahCounters* ctr) {
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t before = b - nd.start;   // records of the node before b
    const int axis = nd.axis;
    const uint32_t bin = uint32_t(nd.bin), nleft = nd.nleft;
    uint32_t acc[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) acc[k] = (k % 6) < 3 ? 0xFFFFFFFFu : 0u;
    uint32_t run = 0;   // left records of [b, e) in earlier rounds
    for (uint32_t base = b; base < e; base += blockDim.x) {
        const uint32_t p = base + threadIdx.x;
        const bool valid = p < e;
        SahRec r{};
        if (valid) r = recs[p];
        const float3 c3 = rec_centroid(r);
        const float cc[3] = {c3.x, c3.y, c3.z};
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
            const uint32_t lbefore = run + woff + __popc(ballot & ((1u << lane) - 1u));   // lefts before p in [b, e)
            const uint32_t dest = left ? nd.start + left_base + lbefore
                                       : nd.start + nleft + (before - left_base) + (p - b - lbefore);
            const int kind = nd.ckind[left ? 0 : 1];
            // binning and partition bin identically, so dest stays inside the
            // child; the check only guards the writes
            const uint32_t cb = left ? nd.start : nd.start + nleft;
            const uint32_t ce = left ? nd.start + nleft : nd.start + nd.count;
            if (dest < cb || dest >= ce) atomicOr(&ctr->err, 1u);
            else if (kind != kCluster) out_rec[dest] = r;
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
}

// Big nodes, one block per chunk: partition with offsets from the scan;
// children's centroid bounds by global atomics (many chunks per node).
__global__ void __launch_bounds__(kSahThreads)
    k_sah_partition(const SahRec* __restrict__ recs, SahRec* __restrict__ out_rec, const SahNode* __restrict__ nodes,
                    uint32_t nact, const uint32_t* __restrict__ chunk_scan, uint32_t* __restrict__ out_ids, SahOut out) {
    __shared__ uint32_t s_warp[kSahThreads / 32];
    __shared__ uint32_t s_cb[12];
    const uint32_t c = blockIdx.x;
    if (c >= *((volatile uint32_t*)&out.ctr->nchunks)) return;   // the grid is an upper bound
    const uint32_t ni = node_of_chunk(nodes, nact, c);
    const SahNode& nd = nodes[ni];
    const uint32_t b = nd.start + (c - nd.chunk0) * kSahChunk;
    const uint32_t e = min(b + kSahChunk, nd.start + nd.count);
    float lo[3], scale[3];
    sah_frame(nd.cb, lo, scale);
    if (threadIdx.x < 12) s_cb[threadIdx.x] = (threadIdx.x % 6) < 3 ? 0xFFFFFFFFu : 0u;
    __syncthreads();
    partition_records(recs, out_rec, out_ids, nd, b, e, chunk_scan[c] - chunk_scan[nd.chunk0], lo, scale, s_warp,
                      s_cb, out.ctr);
    __syncthreads();
    if (threadIdx.x < 12) {
        const uint32_t k = threadIdx.x;
        const uint32_t v = s_cb[k];
        if ((k % 6) < 3 ? v != 0xFFFFFFFFu : v != 0u) {
            uint32_t* dst = child_cb(nd, int(k / 6), out);
            if ((k % 6) < 3) atomicMin(&dst[k % 6], v); else atomicMax(&dst[k % 6], v);
        }
    }
}

// Block nodes (kWarpNode < records <= kSahChunk), one block each: bins in
// shared memory, the split by warp 0, the partition; the children's centroid
// bounds are final when the block ends (no other block touches them).
__global__ void __launch_bounds__(kSahThreads)
    k_sah_node(const SahRec* __restrict__ recs, SahRec* __restrict__ out_rec, const SahNode* __restrict__ nodes,
               uint32_t* __restrict__ out_ids, SahOut out, uint32_t sid0, int median_only) {
    __shared__ uint32_t sb[kBinTotal];
    __shared__ uint32_t s_warp[kSahThreads / 32];
    __shared__ uint32_t s_cb[12];
    __shared__ SahNode s_nd;
    SahNode nd = nodes[blockIdx.x];
    const uint32_t b = nd.start, e = nd.start + nd.count;
    const uint32_t lane = threadIdx.x & 31u;
    float lo[3], scale[3];
    sah_frame(nd.cb, lo, scale);
    if (!median_only) {
        empty_bins(sb, threadIdx.x, blockDim.x);
        __syncthreads();
        for (uint32_t base = b; base < e; base += blockDim.x) {
            const uint32_t p = base + threadIdx.x;
            const bool valid = p < e;
            SahRec r{};
            if (valid) r = recs[p];
            bin_records(sb, r, valid, lo, scale, lane);
        }
        __syncthreads();
    }
    if (threadIdx.x < 32) {
        int axis = -1, bin = 0;
        uint32_t nleft = nd.count / 2;
        if (!median_only) best_split(sb, lane, axis, bin, nleft);
        if (lane == 0) {
            emit_split_alloc(nd, nleft, sid0 + blockIdx.x, out);
            nd.axis = axis;
            nd.bin = bin;
            nd.nleft = nleft;
            s_nd = nd;
        }
    }
    if (threadIdx.x < 12) s_cb[threadIdx.x] = (threadIdx.x % 6) < 3 ? 0xFFFFFFFFu : 0u;
    __syncthreads();
    nd = s_nd;
    partition_records(recs, out_rec, out_ids, nd, b, e, 0u, lo, scale, s_warp, s_cb, out.ctr);
    __syncthreads();
    if (threadIdx.x < 12) {
        const uint32_t k = threadIdx.x;
        child_cb(nd, int(k / 6), out)[k % 6] = s_cb[k];
    }
}

// Warp nodes (cluster_max < records <= kWarpNode), one warp each: the same
// steps as a block node with warp-private bins and warp ballots.
__global__ void __launch_bounds__(kSahThreads)
    k_sah_warp(const SahRec* __restrict__ recs, SahRec* __restrict__ out_rec, const SahNode* __restrict__ nodes,
               uint32_t nw, uint32_t* __restrict__ out_ids, SahOut out, uint32_t sid0, int median_only) {
    __shared__ uint32_t sbins[kSahThreads / 32][kBinTotal];
    __shared__ uint32_t s_cnt[4], s_base[4];   // the block's children per kind, and their first index
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const uint32_t w = blockIdx.x * (kSahThreads / 32) + warp;
    const bool live = w < nw;   // whole warps; every warp reaches the barriers
    if (threadIdx.x < 4) s_cnt[threadIdx.x] = 0;
    uint32_t* sb = sbins[warp];
    SahNode nd = nodes[live ? w : 0];
    const uint32_t b = nd.start, e = live ? nd.start + nd.count : nd.start;
    float lo[3], scale[3];
    sah_frame(nd.cb, lo, scale);
    int axis = -1, bin = 0;
    uint32_t nleft = nd.count / 2;
    if (live && !median_only) {
        empty_bins(sb, lane, 32);
        __syncwarp();
        for (uint32_t base = b; base < e; base += 32) {
            const uint32_t p = base + lane;
            const bool valid = p < e;
            SahRec r{};
            if (valid) r = recs[p];
            bin_records(sb, r, valid, lo, scale, lane);
        }
        __syncwarp();
        best_split(sb, lane, axis, bin, nleft);
    }
    // children: counted per block, one global atomic per kind and block
    int kind[2] = {kCluster, kCluster};
    uint32_t local[2] = {0u, 0u};
    __syncthreads();   // s_cnt is cleared
    if (live && lane == 0) {
        for (int k = 0; k < 2; ++k) {
            kind[k] = child_kind(k ? nd.count - nleft : nleft, out.cluster_max);
            local[k] = atomicAdd(&s_cnt[kind[k]], 1u);
        }
    }
    __syncthreads();
    if (threadIdx.x < 4 && s_cnt[threadIdx.x]) s_base[threadIdx.x] = atomicAdd(kind_counter(threadIdx.x, out), s_cnt[threadIdx.x]);
    __syncthreads();
    if (!live) return;
    if (lane == 0) {
        const uint32_t id[2] = {s_base[kind[0]] + local[0], s_base[kind[1]] + local[1]};
        emit_split(nd, nleft, sid0 + w, kind, id, out);
    }
    nd.child[0] = __shfl_sync(0xFFFFFFFFu, nd.child[0], 0);
    nd.child[1] = __shfl_sync(0xFFFFFFFFu, nd.child[1], 0);
    nd.ckind[0] = __shfl_sync(0xFFFFFFFFu, nd.ckind[0], 0);
    nd.ckind[1] = __shfl_sync(0xFFFFFFFFu, nd.ckind[1], 0);
    uint32_t acc[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) acc[k] = (k % 6) < 3 ? 0xFFFFFFFFu : 0u;
    uint32_t run = 0;
    for (uint32_t base = b; base < e; base += 32) {
        const uint32_t p = base + lane;
        const bool valid = p < e;
        SahRec r{};
        if (valid) r = recs[p];
        const float3 c3 = rec_centroid(r);
        const float cc[3] = {c3.x, c3.y, c3.z};
        bool left = false;
        if (valid) left = axis >= 0 ? sah_bin(cc[axis], lo[axis], scale[axis]) < uint32_t(bin) : (p - b) < nleft;
        const uint32_t ballot = __ballot_sync(0xFFFFFFFFu, left);
        if (valid) {
            const uint32_t lb = run + __popc(ballot & ((1u << lane) - 1u));
            const uint32_t dest = left ? b + lb : b + nleft + (p - b - lb);
            const int kind = nd.ckind[left ? 0 : 1];
            const uint32_t cb = left ? b : b + nleft;
            const uint32_t ce = left ? b + nleft : e;
            if (dest < cb || dest >= ce) atomicOr(&out.ctr->err, 1u);
            else if (kind != kCluster) out_rec[dest] = r;
            else out_ids[dest] = __float_as_uint(r.lo_id.w);
            const int o = left ? 0 : 6;
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                const uint32_t v = ford(cc[a]);
                acc[o + a] = min(acc[o + a], v);
                acc[o + 3 + a] = max(acc[o + 3 + a], v);
            }
        }
        run += __popc(ballot);
    }
#pragma unroll
    for (int k = 0; k < 12; ++k) {
        const uint32_t v = (k % 6) < 3 ? __reduce_min_sync(0xFFFFFFFFu, acc[k]) : __reduce_max_sync(0xFFFFFFFFu, acc[k]);
        if (lane == uint32_t(k)) child_cb(nd, k / 6, out)[k % 6] = v;
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

// Records of every cluster in (code, position) order: a stable insertion sort
// per cluster of at most kSahLocalSort records, one thread each.  Cluster
// ranks rise with position, so this is the order a stable radix sort of the
// full keys (rank << 30 | code) gives, without its passes over all records
// (C1: 8 M keys of 49 bits, 7 passes).
constexpr uint32_t kSahLocalSort = 32;
__global__ void k_sah_sort_clusters(const SegDev* __restrict__ tsegs, uint32_t ncl, unsigned long long* codes,
                                    uint32_t* ids) {
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= ncl) return;
    const SegDev sg = tsegs[r];
    unsigned long long* c = codes + sg.prim_begin;
    uint32_t* d = ids + sg.prim_begin;
    for (uint32_t i = 1; i < sg.prim_count; ++i) {
        const unsigned long long key = c[i];
        const uint32_t val = d[i];
        uint32_t j = i;
        while (j > 0 && c[j - 1] > key) {
            c[j] = c[j - 1];
            d[j] = d[j - 1];
            --j;
        }
        c[j] = key;
        d[j] = val;
    }
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

// Side streams of the level loop.  A level's big, block and warp nodes cover
// disjoint record ranges and share only atomic counters (children and clusters
// are allocated by atomics; where they land does not reach the tree), so the
// block-node and warp-node kernels run beside the big nodes' chain of small
// kernels (C1: 17.7 -> 16.4 ms per build, the same tree).  One set per host
// thread, made on the thread's current device.
struct SahStreams {
    int dev = -1;
    cudaStream_t side[2] = {nullptr, nullptr};
    cudaEvent_t fork = nullptr, join[2] = {nullptr, nullptr};
    void release() noexcept {
        for (int k = 0; k < 2; ++k) {
            if (side[k]) cudaStreamDestroy(side[k]);
            if (join[k]) cudaEventDestroy(join[k]);
            side[k] = nullptr;
            join[k] = nullptr;
        }
        if (fork) cudaEventDestroy(fork);
        fork = nullptr;
        dev = -1;
    }
    void ensure() {
        int d = 0;
        RT_CUDA(cudaGetDevice(&d));
        if (d == dev) return;
        release();
        for (int k = 0; k < 2; ++k) {
            RT_CUDA(cudaStreamCreateWithFlags(&side[k], cudaStreamNonBlocking));
            RT_CUDA(cudaEventCreateWithFlags(&join[k], cudaEventDisableTiming));
        }
        RT_CUDA(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
        dev = d;
    }
    ~SahStreams() { release(); }
};

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
    std::vector<SahNode> seed_big, seed_block, seed_warp;
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
            nd.ckind[0] = nd.ckind[1] = kCluster;
            (sg.prim_count > kSahChunk ? seed_big : sg.prim_count > kWarpNode ? seed_block : seed_warp).push_back(nd);
        } else {
            SahCluster cl{};
            cl.start = sg.prim_begin;
            cl.count = sg.prim_count;
            for (int k = 0; k < 6; ++k) cl.cb[k] = sb[6 * g + k];
            seed_cl.push_back(cl);
            L.roots[g] = int(sg.prim_begin);   // a single cluster: its Karras root (or its only record)
        }
    }
    // scratch: records x2, big, block and warp node lists x2, bins, chunk
    // tables, clusters, splits.  A level holds at most n / (cluster_max + 1)
    // nodes (disjoint ranges above the cluster size) and n / kSahChunk big
    // ones; over all levels there are fewer splits and clusters than records.
    const size_t max_nodes = size_t(n) / (cluster_max + 1) + ns + 1;
    const size_t max_big = size_t(n) / kSahChunk + ns + 1;
    const size_t max_chunks = size_t(n) / kSahChunk + max_big + 1;
    const size_t max_cl = size_t(n) + 1;
    const size_t max_split = size_t(n) + 1;
    SahRec* rec[2];
    SahNode *big[2], *block[2], *warp[2];
    uint32_t *bins, *chunk_counts, *nch, *chunk0, *chunk_left, *chunk_scan, *out_ids, *ckeys, *cvals, *tcb;
    SahCluster* clusters;
    SahSplit* splits;
    SegDev* tsegs;
    SahCounters* ctr;
    int* roots_dev;
    auto layout = [&](char* p) {   // carves the scratch; returns its size
        char* const p0 = p;
        rec[0] = carve<SahRec>(p, n);
        rec[1] = carve<SahRec>(p, n);
        big[0] = carve<SahNode>(p, max_big);
        big[1] = carve<SahNode>(p, max_big);
        block[0] = carve<SahNode>(p, max_nodes);
        block[1] = carve<SahNode>(p, max_nodes);
        warp[0] = carve<SahNode>(p, max_nodes);
        warp[1] = carve<SahNode>(p, max_nodes);
        bins = carve<uint32_t>(p, max_big * kBinTotal);
        chunk_counts = carve<uint32_t>(p, max_chunks * 3 * kSahBins);
        nch = carve<uint32_t>(p, max_chunks);
        chunk0 = carve<uint32_t>(p, max_chunks);
        chunk_left = carve<uint32_t>(p, max_chunks);
        chunk_scan = carve<uint32_t>(p, max_chunks);
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
    // one scratch per host thread, shared by all builds (builds return only
    // when their kernels are done)
    static thread_local DevBuf scratch;
    scratch.reserve(layout(reinterpret_cast<char*>(uintptr_t(256))));
    layout(scratch.as<char>());
    static thread_local SahStreams ss;
    ss.ensure();
    // a build that stopped with an error between a fork and its join may have
    // left kernels on the side streams; they finish before the scratch is reused
    for (int k = 0; k < 2; ++k) RT_CUDA(cudaStreamSynchronize(ss.side[k]));

    SahCounters c0{};
    c0.next[0][kBig] = uint32_t(seed_big.size());
    c0.next[0][kBlock] = uint32_t(seed_block.size());
    c0.next[0][kWarp] = uint32_t(seed_warp.size());
    c0.ncl = uint32_t(seed_cl.size());
    RT_CUDA(cudaMemcpyAsync(ctr, &c0, sizeof c0, cudaMemcpyHostToDevice, s));
    if (!seed_big.empty())
        RT_CUDA(cudaMemcpyAsync(big[0], seed_big.data(), seed_big.size() * sizeof(SahNode), cudaMemcpyHostToDevice, s));
    if (!seed_block.empty())
        RT_CUDA(cudaMemcpyAsync(block[0], seed_block.data(), seed_block.size() * sizeof(SahNode),
                                cudaMemcpyHostToDevice, s));
    if (!seed_warp.empty())
        RT_CUDA(cudaMemcpyAsync(warp[0], seed_warp.data(), seed_warp.size() * sizeof(SahNode), cudaMemcpyHostToDevice,
                                s));
    if (!seed_cl.empty())
        RT_CUDA(cudaMemcpyAsync(clusters, seed_cl.data(), seed_cl.size() * sizeof(SahCluster), cudaMemcpyHostToDevice,
                                s));
    RT_CUDA(cudaMemsetAsync(roots_dev, 0xFF, ns * 4, s));
    k_sah_records<<<(n + kSahThreads - 1) / kSahThreads, kSahThreads, 0, s>>>(L.prims_flat.as<float4>(), n, rec[0],
                                                                               out_ids);
    RT_CHECK_LAUNCH();
    uint32_t nb = c0.next[0][kBig], nbl = c0.next[0][kBlock], nw = c0.next[0][kWarp];
    uint32_t nsplit = 0;   // one split per node of every level, ids in level order
    int cur = 0, level = 0;
    SahCounters hc{};
    for (; nb + nbl + nw > 0; ++level) {
        RT_REQUIRE(nb <= max_big && nbl <= max_nodes && nw <= max_nodes, "internal: SAH level overflow");
        const uint32_t nx = uint32_t(cur ^ 1);
        RT_CUDA(cudaMemsetAsync(ctr->next[nx], 0, sizeof(ctr->next[nx]), s));
        const SahOut out{big[nx], block[nx], warp[nx], clusters, splits, ctr, nx, cluster_max};
        const int median_only = level >= kSahMaxLevels ? 1 : 0;
        // block and warp nodes on the side streams when another kind shares the level
        const bool fork = int(nb != 0) + int(nbl != 0) + int(nw != 0) >= 2;
        cudaStream_t s_block = s, s_warp = s;
        if (fork) {
            RT_CUDA(cudaEventRecord(ss.fork, s));   // after the counters are cleared
            if (nbl) {
                RT_CUDA(cudaStreamWaitEvent(ss.side[0], ss.fork, 0));
                s_block = ss.side[0];
            }
            if (nw) {
                RT_CUDA(cudaStreamWaitEvent(ss.side[1], ss.fork, 0));
                s_warp = ss.side[1];
            }
        }
        if (nbl) {
            k_sah_node<<<nbl, kSahThreads, 0, s_block>>>(rec[cur], rec[nx], block[cur], out_ids, out, nsplit + nb,
                                                         median_only);
            RT_CHECK_LAUNCH();
        }
        if (nw) {
            const uint32_t wpb = kSahThreads / 32;
            k_sah_warp<<<(nw + wpb - 1) / wpb, kSahThreads, 0, s_warp>>>(rec[cur], rec[nx], warp[cur], nw, out_ids,
                                                                         out, nsplit + nb + nbl, median_only);
            RT_CHECK_LAUNCH();
        }
        if (nb) {
            SahNode* nodes = big[cur];
            k_sah_nchunks<<<(nb + kSahThreads - 1) / kSahThreads, kSahThreads, 0, s>>>(nodes, nb, nch);
            RT_CHECK_LAUNCH();
            scan_exclusive_u32(nch, chunk0, nb, L.sort_tmp, s);
            const uint32_t prep_blocks =
                std::min<uint32_t>(4096u, uint32_t((size_t(nb) * kBinTotal + kSahThreads - 1) / kSahThreads));
            k_sah_prepare<<<std::max(prep_blocks, (nb + kSahThreads - 1) / kSahThreads), kSahThreads, 0, s>>>(
                nodes, nb, chunk0, ctr, bins);
            RT_CHECK_LAUNCH();
            // chunks of the level: at most one per kSahChunk records plus one per node
            // (the device holds the exact count; surplus blocks return at once)
            const uint32_t bound = n / kSahChunk + nb + 1;
            k_sah_bin<<<bound, kSahThreads, 0, s>>>(rec[cur], nodes, nb, bins, chunk_counts, ctr);
            RT_CHECK_LAUNCH();
            k_sah_split<<<(nb * 32 + 127) / 128, 128, 0, s>>>(nodes, nb, bins, out, nsplit, median_only);
            RT_CHECK_LAUNCH();
            k_sah_chunk_left<<<(bound + kSahThreads - 1) / kSahThreads, kSahThreads, 0, s>>>(nodes, nb, bound,
                                                                                           chunk_counts, chunk_left, ctr);
            RT_CHECK_LAUNCH();
            scan_exclusive_u32(chunk_left, chunk_scan, bound, L.sort_tmp, s);
            k_sah_partition<<<bound, kSahThreads, 0, s>>>(rec[cur], rec[nx], nodes, nb, chunk_scan, out_ids, out);
            RT_CHECK_LAUNCH();
        }
        if (fork) {   // the level's kernels are done before its counters are read
            for (int k = 0; k < 2; ++k) {
                if (k == 0 ? !nbl : !nw) continue;
                RT_CUDA(cudaEventRecord(ss.join[k], ss.side[k]));
                RT_CUDA(cudaStreamWaitEvent(s, ss.join[k], 0));
            }
        }
        RT_CUDA(cudaMemcpyAsync(&hc, ctr, sizeof hc, cudaMemcpyDeviceToHost, s));
        RT_CUDA(cudaStreamSynchronize(s));
        if (hc.err) throw Error(RT_ERR_INTERNAL, "SAH build: partition and binning disagree");
        nsplit += nb + nbl + nw;
        nb = hc.next[nx][kBig];
        nbl = hc.next[nx][kBlock];
        nw = hc.next[nx][kWarp];
        cur ^= 1;
    }
    if (level == 0) {   // no node above the cluster size: the seed clusters only
        RT_CUDA(cudaMemcpyAsync(&hc, ctr, sizeof hc, cudaMemcpyDeviceToHost, s));
        RT_CUDA(cudaStreamSynchronize(s));
    }
    const uint32_t ncl = hc.ncl;
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
    if (cluster_max <= kSahLocalSort) {
        k_sah_sort_clusters<<<(ncl + kSahThreads - 1) / kSahThreads, kSahThreads, 0, s>>>(tsegs, ncl, codes, ids);
        RT_CHECK_LAUNCH();
    } else {
        int cl_bits = 1;
        while ((uint64_t(1) << cl_bits) < ncl) ++cl_bits;
        radix_sort_pairs_u64(codes, ids, n, 30 + cl_bits, L.sort_tmp, s);
    }
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
    RT_CUDA(cudaStreamSynchronize(s));   // the scratch is free for the next build
}

}  // namespace rt
