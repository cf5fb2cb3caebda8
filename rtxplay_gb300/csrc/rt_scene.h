// rt_scene.h -- library-side scene object behind the rt_scene handle.
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

// Flattening descriptor of one thing (device copy in Scene::desc).
struct FlatDesc {
    const float3* v;
    const uint3* idx;
    uint32_t prim_offset;
    uint32_t nprims;
    int analytic;
    int pad;
    float T[12];
    float4 sphere;          // centre, radius
};

struct Scene {
    std::vector<MeshDev> meshes;
    std::vector<ThingHost> things;

    // device side, valid after build
    DevBuf things_dev;      // ThingDev[n_things]
    DevBuf desc;            // FlatDesc[n_things]
    DevBuf prims_flat;      // 3 float4 per primitive, primitive-id order
    DevBuf prims;           // 3 float4 per primitive, LBVH leaf order
    DevBuf nodes;           // 4 float4 per internal node (>= 1 node)
    DevBuf codes;           // sorted Morton codes (u32 or u64)
    DevBuf ids;             // sorted primitive ids
    DevBuf parents;         // leaf parents [n] then internal parents [n-1]
    DevBuf flags;           // refit arrival counters [n-1]
    DevBuf bounds;          // centroid bounds as 6 orderable u32
    DevBuf sort_tmp;
    DevBuf misc;            // small device scratch (error words, counters)

    uint32_t nprims = 0;
    int morton_bits = 60;
    bool built = false;
    bool topology_dirty = true;   // things added or removed since the last build
    bool xf_dirty = false;        // transforms/optics changed since the last build/update
    float build_ms = 0.f, refit_ms = 0.f;

    size_t device_bytes() const;
};

Scene* scene_from(rt_scene h);

}  // namespace rt
