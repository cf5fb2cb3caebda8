// rt_scene.h -- library-side scene, geometry and batch objects.
#pragma once

#include <cstdint>
#include <vector>

#include "rt_device.cuh"
#include "rt_internal.h"

namespace rt {

struct MeshDev {
    DevBuf v;          // float3 vertices
    DevBuf i;          // uint3 triangles
    uint32_t nv = 0, ni = 0;
};

struct ThingHost {
    rt_optics optics{};
    int mesh = -1;          // -1: analytic sphere
    float T[12] = {};       // 3x4 row-major object-to-world transform
    float3 center{};        // analytic sphere centre
    float radius = 0.f;     // analytic sphere radius
};

// Segment of an LBVH: its primitives are [prim_begin, prim_begin +
// prim_count) in leaf order and its internal nodes occupy node slots
// [prim_begin, prim_begin + prim_count - 1); the root is node prim_begin.
struct SegDev {
    uint32_t prim_begin, prim_count;
};

// One LBVH over 48-B primitive records, possibly segmented (one independent
// hierarchy per segment, all built in one pass).
struct Lbvh {
    DevBuf segs;            // SegDev[n_segs]
    DevBuf prim_seg;        // segment of each record (record-id order), n_segs > 1 only
    DevBuf prims_flat;      // 3 float4 per record, record-id order
    DevBuf prims;           // 3 float4 per record, leaf order
    DevBuf prims_e;         // the same for traversal: triangles as (A, B - A, C - A)
    DevBuf nodes;           // 4 float4 per node slot (one slot per record)
    DevBuf codes;           // sorted Morton codes (u32 or u64)
    DevBuf ids;             // sorted record ids
    DevBuf parents;         // leaf parents [n] then node parents [n]
    DevBuf flags;           // refit arrival counters [n]
    DevBuf bounds;          // centroid bounds per segment, 6 orderable u32 each
    DevBuf sort_tmp, seg_tmp;
    // things-grouped hierarchy: per-thing centroid bounds, thing codes and order,
    // per-thing record ranges, per-scene thing ranges, thing -> scene, scratch
    DevBuf tbounds, tcodes, tids, tsegs, scene_things, tseg, ttmp;
    uint32_t nprims = 0, nsegs = 0, nthings = 0;
    uint32_t nclusters = 0, sah_levels = 0;   // binned-SAH hierarchies
    int morton_bits = 60;
    int grouped = 0;
    int sah = 0;
    std::vector<SegDev> seg_host;
    std::vector<int> roots;   // per segment, grouped and binned-SAH hierarchies
    size_t device_bytes() const;
    int root(uint32_t seg) const {
        if (grouped || sah) return roots[seg];
        return seg_host[seg].prim_count ? int(seg_host[seg].prim_begin) : -1;
    }
};

struct Scene;

// Device arrays of one or more scenes built together.  The top level holds,
// per scene segment, one record per analytic sphere, one instance record per
// instanced mesh thing and the world-space triangles of flattened mesh things;
// the bottom level holds, per instanced mesh, its object-space triangles.  The
// flat layout (every mesh flattened, no bottom level) is the same structure
// with no instances.
struct Geometry {
    DevBuf things_dev;      // ThingDev[n_things]
    DevBuf desc;            // FlatDesc[n_things]
    DevBuf inst;            // InstDev[n_things]
    DevBuf misc;            // small device scratch (error words)
    Lbvh top, blas;

    uint32_t nprims = 0;    // global primitives (what the scene renders)
    uint32_t nthings = 0, nsegs = 0, ninstances = 0;
    int morton_bits = 60;
    int layout = RT_LAYOUT_FLAT;      // resolved layout of the last build
    int layout_req = RT_LAYOUT_AUTO;  // layout requested at the last build
    std::vector<FlatDesc> desc_host;
    std::vector<uint32_t> thing_begin;   // first global thing of each segment
    std::vector<uint64_t> optics_seen;   // optics version of each segment's scene at the last upload
    std::vector<ThingDev> things_host;   // staging copy of things_dev
    std::vector<int> inst_class;         // per thing: 1 instanced, 0 not (for refit consistency)
    float build_ms = 0.f, refit_ms = 0.f;

    size_t device_bytes() const;
    int root(uint32_t seg) const { return top.root(seg); }
    GeoView view() const;
};

// (Re)builds `g` from the things of `scenes` (one segment each): the bottom
// level over the instanced meshes (one segment each, object space), then the
// top level (one segment per scene); each level is flattened to records, its
// per-segment centroid bounds reduced, Morton codes sorted by (segment, code),
// a Karras hierarchy emitted per segment and refit bottom-up.  Synchronous on
// `s`.
void build_geometry(Geometry& g, const std::vector<Scene*>& scenes, int morton_bits, int layout, cudaStream_t s);

// Binned-SAH topology of an LBVH whose records are in prims_flat and whose
// segment centroid bounds are in `bounds` (rt_sah.cu): leaf order (codes,
// ids), node children, parents and per-segment roots; the refit follows.
constexpr uint32_t kSahClusterMax = 16;
void build_sah_topology(Lbvh& L, uint32_t cluster_max, cudaStream_t s);
// Re-flattens the top level with the scenes' current transforms and refits it
// (a full build when a thing changed between instanced and flattened).
void refit_geometry(Geometry& g, const std::vector<Scene*>& scenes, cudaStream_t s);
// Re-uploads the per-thing optics of `g` when any scene's optics changed
// since they were last uploaded (optics need no refit).
void sync_optics(Geometry& g, const std::vector<Scene*>& scenes, cudaStream_t s);
// Writes the albedos of all things of `g` from a device array (3 floats per
// thing, in thing order) on stream `s`; the scenes' host-side optics are not
// changed, and a later host-side optics change re-uploads every thing's optics.
void set_albedos_device(Geometry& g, const std::vector<Scene*>& scenes, const float* albedo, cudaStream_t s);

struct Scene {
    int layout = RT_LAYOUT_AUTO;  // requested layout of the next build
    std::vector<MeshDev> meshes;
    std::vector<ThingHost> things;
    Geometry geo;
    bool built = false;
    bool topology_dirty = true;   // things added since the last build
    bool xf_dirty = false;        // transforms changed since the last build/update
    uint64_t optics_version = 0;  // bumped by every optics change
    size_t device_bytes() const;
};

Scene* scene_from(rt_scene h);

// One render job: a scene segment of a geometry, its camera, launch
// parameters and output frame.
struct Job {
    uint32_t seg;
    rt_camera cam;
    rt_launch_params params;
    rt_frame frame;
};

// Pixel sums kept across launches (rt_accum): 3 x u64 colour + u32 rays per
// pixel, and the samples per pixel they hold.
struct AccumState {
    uint32_t W = 0, H = 0;
    unsigned long long first = 0;     // sample index of the first sample the sums hold
    unsigned long long samples = 0;   // the sums hold samples [first, first + samples)
    unsigned long long rays = 0;      // sum of the per-pixel ray counts
    DevBuf sums;
};

// Device camera of a host camera; launch-parameter validation (rt_render.cu).
CamDev cam_dev(const rt_camera& c);
void check_params(const rt_launch_params* p);

// Renders all jobs over `g` in one wavefront (rt_render.cu).
// With `accum` (one job only): samples [accum->samples, + spp) of every pixel
// are added to its sums and the frame is their mean over all samples so far.
void render_jobs(const Geometry& g, const std::vector<Job>& jobs, cudaStream_t s, rt_launch_stats* stats,
                 AccumState* accum = nullptr);

// One adjoint job: the rendered image of a job, dL/d(clamped image) and the
// output gradients (device pointers; a NULL output is skipped).
struct AdjointJob {
    uint32_t seg;
    rt_camera cam;
    rt_launch_params params;
    const rt_float3* image;
    const rt_float3* grad_image;
    double* grad_albedo;   // [n_things x 3]
    double* grad_fuzz;     // [n_things]
    double* grad_sky;      // [6]: ambient rgb, white rgb
};

// Device buffers and job tables of adjoint launches (a batch keeps its own,
// so that a launch captured into a CUDA graph owns what it points at).
struct AdjointWorkspace;
AdjointWorkspace* adjoint_workspace_new();
void adjoint_workspace_free(AdjointWorkspace* ws);

// Replays the paths of all jobs and writes their gradients (rt_adjoint.cu),
// with workspace `ws` (NULL: the calling thread's); inside a stream capture
// the error word is ORed into `sticky` instead of being read back.
void adjoint_jobs(const Geometry& g, const std::vector<AdjointJob>& jobs, cudaStream_t s,
                  AdjointWorkspace* ws = nullptr, uint32_t* sticky = nullptr);

}  // namespace rt
