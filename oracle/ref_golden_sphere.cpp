// Golden-vector generator for the subdivided-tetrahedron tessellator.
//
// Test infrastructure only: linked by oracle/ref_build.sh with the reference's
// own optx/sphere.cxx (Sphere::tetrahedron/pumpup/reduce, optx/sphere.cxx:28-106)
// and dumps Sphere(radius, ndiv).mesh() as raw bits, so tessellation parity is
// checked bit for bit rather than through the %f text of the reference's
// -DMAIN tool (optx/sphere.cxx:108-140).
//
// Usage: ref_golden_sphere <radius> <ndiv> <out.bin>
// File layout (little endian): u32 nv, u32 ni, nv*3 f32 vertices, ni*3 u32 indices.

#include <cstdio>
#include <cstdlib>
#include <tuple>

#include "sphere.h"

int main(int argc, char** argv) {
    if (argc != 4) {
        fprintf(stderr, "usage: %s <radius> <ndiv> <out.bin>\n", argv[0]);
        return 1;
    }
    const float radius = strtof(argv[1], nullptr);
    const unsigned ndiv = static_cast<unsigned>(strtoul(argv[2], nullptr, 10));
    Sphere sphere(radius, ndiv);
    float3* vces;
    unsigned nv;
    uint3* ices;
    unsigned ni;
    std::tie(vces, nv, ices, ni) = sphere.mesh();
    FILE* f = fopen(argv[3], "wb");
    if (!f) return 2;
    fwrite(&nv, 4, 1, f);
    fwrite(&ni, 4, 1, f);
    fwrite(vces, sizeof(float3), nv, f);
    fwrite(ices, sizeof(uint3), ni, f);
    fclose(f);
    return 0;
}
