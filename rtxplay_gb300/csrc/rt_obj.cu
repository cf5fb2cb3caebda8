// rt_obj.cu -- Wavefront OBJ input (host code).
//
// Replaces class Object (optx/object.cxx:23-106), which reads a file with the
// unpinned third-party tinyobjloader and turns every shape into one mesh.
// This is an own parser of the subset the reference uses: `v x y z` vertex
// records and `f` face records (each face vertex `i`, `i/t`, `i//n` or
// `i/t/n`, negative indices relative to the vertices read so far); `o` and `g`
// records start a new shape; everything else (normals, texture coordinates,
// materials, smoothing groups, comments) is ignored.  A face with more than
// three vertices is split into a fan (v0, vi, vi+1), as the reference's
// loader triangulates polygons before its triangle check.  Coordinates are
// parsed as double and rounded to float, as tinyobjloader does.
//
// Per shape the mesh holds the vertices its faces reference, numbered in
// order of first reference, and the faces renumbered accordingly; for a
// one-shape file whose vertices are listed in order of first reference (the
// files optx/sphere.cxx writes) this is exactly the reference's mesh.
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

#include "rt_internal.h"

namespace rt {
namespace {

struct ObjShape {
    std::vector<rt_float3> v;
    std::vector<rt_uint3> i;
};

// One face vertex token: the vertex index before the first '/'.
long face_index(const char* tok, size_t nverts, const std::string& where) {
    char* end = nullptr;
    errno = 0;
    const long x = std::strtol(tok, &end, 10);
    RT_REQUIRE(end != tok && errno == 0 && (*end == '\0' || *end == '/'), where + ": bad face index '" + tok + "'");
    long idx;
    if (x > 0) idx = x - 1;
    else if (x < 0) idx = long(nverts) + x;
    else throw Error(RT_ERR_INVALID_ARG, where + ": face index 0");
    RT_REQUIRE(idx >= 0 && size_t(idx) < nverts, where + ": face index out of range");
    return idx;
}

std::vector<ObjShape> parse_obj(const char* path) {
    RT_REQUIRE(path != nullptr, "path is NULL");
    FILE* f = std::fopen(path, "r");
    RT_REQUIRE(f != nullptr, std::string("cannot open ") + path);
    std::vector<rt_float3> verts;
    std::vector<ObjShape> shapes;
    ObjShape cur;
    std::unordered_map<long, uint32_t> local;   // file vertex -> shape vertex
    auto flush = [&]() {
        if (!cur.i.empty()) shapes.push_back(std::move(cur));
        cur = ObjShape();
        local.clear();
    };
    std::string line;
    char buf[4096];
    size_t lineno = 0;
    try {
        while (std::fgets(buf, sizeof(buf), f)) {
            line.assign(buf);
            while (!line.empty() && line.back() != '\n' && !std::feof(f) && std::fgets(buf, sizeof(buf), f))
                line.append(buf);   // a line longer than the buffer
            ++lineno;
            const std::string where = std::string(path) + ":" + std::to_string(lineno);
            std::vector<char> tmp(line.begin(), line.end());
            tmp.push_back('\0');
            char* save = nullptr;
            const char* tag = strtok_r(tmp.data(), " \t\r\n", &save);
            if (!tag || tag[0] == '#') continue;
            if (std::strcmp(tag, "v") == 0) {
                double c[3];
                for (int k = 0; k < 3; ++k) {
                    const char* tok = strtok_r(nullptr, " \t\r\n", &save);
                    RT_REQUIRE(tok != nullptr, where + ": vertex needs three coordinates");
                    char* end = nullptr;
                    c[k] = std::strtod(tok, &end);
                    RT_REQUIRE(end != tok && *end == '\0', where + ": bad coordinate '" + tok + "'");
                }
                verts.push_back(rt_float3{float(c[0]), float(c[1]), float(c[2])});
            } else if (std::strcmp(tag, "o") == 0 || std::strcmp(tag, "g") == 0) {
                flush();
            } else if (std::strcmp(tag, "f") == 0) {
                std::vector<uint32_t> fv;
                for (const char* tok = strtok_r(nullptr, " \t\r\n", &save); tok;
                     tok = strtok_r(nullptr, " \t\r\n", &save)) {
                    const long idx = face_index(tok, verts.size(), where);
                    auto it = local.find(idx);
                    uint32_t li;
                    if (it == local.end()) {
                        li = uint32_t(cur.v.size());
                        local.emplace(idx, li);
                        cur.v.push_back(verts[size_t(idx)]);
                    } else {
                        li = it->second;
                    }
                    fv.push_back(li);
                }
                RT_REQUIRE(fv.size() >= 3, where + ": a face needs at least three vertices");
                for (size_t k = 1; k + 1 < fv.size(); ++k) cur.i.push_back(rt_uint3{fv[0], fv[k], fv[k + 1]});
            }
        }
    } catch (...) {
        std::fclose(f);
        throw;
    }
    std::fclose(f);
    flush();
    return shapes;
}

}  // namespace
}  // namespace rt

using namespace rt;

extern "C" {

rt_status rt_obj_parse(const char* path, unsigned int shape, rt_float3* vces, unsigned int* nv, rt_uint3* ices,
                       unsigned int* ni, unsigned int* nshapes) {
    return guarded([&] {
        const std::vector<ObjShape> shapes = parse_obj(path);
        if (nshapes) *nshapes = unsigned(shapes.size());
        if (!nv && !ni && !vces && !ices) return;
        RT_REQUIRE(shape < shapes.size(), "shape index out of range");
        const ObjShape& s = shapes[shape];
        // an array to fill comes with its capacity in *nv / *ni; the file is
        // read again on every call, so check what it holds now against it
        RT_REQUIRE(!vces || nv, "vces needs nv (its capacity on input)");
        RT_REQUIRE(!ices || ni, "ices needs ni (its capacity on input)");
        RT_REQUIRE(!vces || s.v.size() <= *nv, "shape has more vertices than vces holds (*nv)");
        RT_REQUIRE(!ices || s.i.size() <= *ni, "shape has more triangles than ices holds (*ni)");
        if (vces) std::memcpy(vces, s.v.data(), s.v.size() * sizeof(rt_float3));
        if (ices) std::memcpy(ices, s.i.data(), s.i.size() * sizeof(rt_uint3));
        if (nv) *nv = unsigned(s.v.size());
        if (ni) *ni = unsigned(s.i.size());
    });
}

rt_status rt_scene_add_obj(rt_scene scene, const char* path, unsigned int* mesh_ids, unsigned int cap,
                           unsigned int* n_meshes) {
    return guarded([&] {
        const std::vector<ObjShape> shapes = parse_obj(path);
        RT_REQUIRE(!shapes.empty(), std::string(path) + ": no triangle faces");
        RT_REQUIRE(mesh_ids == nullptr || cap >= shapes.size(), "mesh_ids holds fewer entries than the file's shapes");
        if (n_meshes) *n_meshes = 0;
        for (size_t k = 0; k < shapes.size(); ++k) {
            unsigned int id = 0;
            const rt_status st = rt_scene_add_mesh(scene, shapes[k].v.data(), unsigned(shapes[k].v.size()),
                                                   shapes[k].i.data(), unsigned(shapes[k].i.size()), &id);
            // on a failure the meshes added so far stay in the scene and are reported
            if (st != RT_OK) throw Error(st, rt_last_error_string());
            if (mesh_ids) mesh_ids[k] = id;
            if (n_meshes) *n_meshes = unsigned(k + 1);
        }
    });
}

}  // extern "C"
