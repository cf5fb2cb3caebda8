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

// Flattening descriptor of one thing (device copy in Geometry::desc).
struct FlatDesc {
    const float3* v;
    const uint3* idx;
    uint32_t prim_offset;   // global first primitive
    uint32_t nprims;
    int analytic;
    uint32_t seg;           // segment (scene) of the thing
    float T[12];
    float4 sphere;          // centre, radius
};

// Segment (one scene) of a geometry: its primitives are [prim_begin,
// prim_begin + prim_count) in leaf order and its internal nodes occupy node
// slots [prim_begin, prim_begin + prim_count - 1); the root is node prim_begin.
struct SegDev {
    uint32_t prim_begin, prim_count;
};

struct Scene;

// Device arrays of one or more scenes built together: primitive records in
// leaf order, LBVH nodes, per-thing optics.  A single scene is a geometry of
// one segment; a batch concatenates many scenes into segments and builds all
// their hierarchies in one segmented pass.
struct Geometry {
    DevBuf things_dev;      // ThingDev[n_things]
    DevBuf desc;            // FlatDesc[n_things]
    DevBuf segs;            // SegDev[n_segs]
    DevBuf prim_seg;        // segment of each primitive (primitive-id order)
    DevBuf prims_flat;      // 3 float4 per primitive, primitive-id order
    DevBuf prims;           // 3 float4 per primitive, LBVH leaf order
    DevBuf nodes;           // 4 float4 per node slot (one slot per primitive)
    DevBuf codes;           // sorted Morton codes (u32 or u64)
    DevBuf ids;             // sorted primitive ids
    DevBuf parents;         // leaf parents [n] then node parents [n]
    DevBuf flags;           // refit arrival counters [n]
    DevBuf bounds;          // centroid bounds per segment, 6 orderable u32 each
    DevBuf sort_tmp, seg_tmp;
    DevBuf misc;            // small device scratch (error words)

    uint32_t nprims = 0, nthings = 0, nsegs = 0;
    int morton_bits = 60;
    std::vector<SegDev> seg_host;
    std::vector<uint32_t> thing_begin;   // first global thing of each segment
    std::vector<uint64_t> optics_seen;   // optics version of each segment's scene at the last upload
    std::vector<ThingDev> things_host;   // staging copy of things_dev
    float build_ms = 0.f, refit_ms = 0.f;

    size_t device_bytes() const;
    int root(uint32_t seg) const { return seg_host[seg].prim_count ? int(seg_host[seg].prim_begin) : -1; }
};

// (Re)builds `g` from the things of `scenes` (one segment each): flattening,
// per-segment centroid bounds, Morton codes, sort by (segment, code), Karras
// hierarchy per segment, bottom-up refit.  Synchronous on `s`.
void build_geometry(Geometry& g, const std::vector<Scene*>& scenes, int morton_bits, cudaStream_t s);
// Re-flattens with the scenes' current transforms/optics and refits.
void refit_geometry(Geometry& g, const std::vector<Scene*>& scenes, cudaStream_t s);
// Re-uploads the per-thing optics of `g` when any scene's optics changed
// since they were last uploaded (optics need no refit).
void sync_optics(Geometry& g, const std::vector<Scene*>& scenes, cudaStream_t s);

struct Scene {
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

// Device camera of a host camera; launch-parameter validation (rt_render.cu).
CamDev cam_dev(const rt_camera& c);
void check_params(const rt_launch_params* p);

// Renders all jobs over `g` in one wavefront (rt_render.cu).
void render_jobs(const Geometry& g, const std::vector<Job>& jobs, cudaStream_t s, rt_launch_stats* stats);

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

// Replays the paths of all jobs and writes their gradients (rt_adjoint.cu).
void adjoint_jobs(const Geometry& g, const std::vector<AdjointJob>& jobs, cudaStream_t s);

}  // namespace rt
