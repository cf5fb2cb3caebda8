// rt_recipe.cu -- the RTOW final-scene recipe (host code).
//
// RTWO::load (optx/rtwo.cxx:137-244) and rtow's scene() (rtow.cxx:51-80):
// ground sphere, a (2H)x(2H) grid of small spheres with random centre and
// material, three big spheres.  Two random streams:
//   RT_RECIPE_GLIBC   glibc rand() (TYPE_3 additive feedback generator,
//                     restated here) in double precision as rtow.cxx, with
//                     the argument order g++ uses for the reference's
//                     V(rnd(), rnd(), rnd()) and P(a+.9*rnd(), .2, b+.9*rnd())
//                     (last argument drawn first) -- seed 1 reproduces the
//                     reference's 487-sphere scene exactly;
//   RT_RECIPE_COUNTER the same recipe in binary32 with a Philox stream.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "rt_device.cuh"
#include "rt_internal.h"

namespace rt {
namespace {

// glibc random_r TYPE_3: r[i] = r[i-3] + r[i-31] (mod 2^32), output r >> 1,
// seeded by the Park-Miller LCG (Schrage's method) and 310 discarded draws.
struct GlibcRand {
    int32_t st[31];
    int fi = 3, ri = 0;
    explicit GlibcRand(uint32_t seed) {
        if (seed == 0) seed = 1;
        st[0] = int32_t(seed);
        for (int i = 1; i < 31; ++i) {
            const int32_t hi = st[i - 1] / 127773, lo = st[i - 1] % 127773;
            int32_t word = 16807 * lo - 2836 * hi;
            if (word < 0) word += 2147483647;
            st[i] = word;
        }
        for (int i = 0; i < 310; ++i) next();
    }
    uint32_t next() {
        st[fi] = int32_t(uint32_t(st[fi]) + uint32_t(st[ri]));
        const uint32_t r = uint32_t(st[fi]) >> 1;
        if (++fi >= 31) fi = 0;
        if (++ri >= 31) ri = 0;
        return r;
    }
};

void philox_host(const uint32_t in[4], uint32_t k0, uint32_t k1, uint32_t out[4]) {
    uint32_t c0 = in[0], c1 = in[1], c2 = in[2], c3 = in[3];
    for (int r = 0; r < 10; ++r) {
        const uint64_t p0 = uint64_t(0xD2511F53u) * c0, p1 = uint64_t(0xCD9E8D57u) * c2;
        const uint32_t h0 = uint32_t(p0 >> 32), l0 = uint32_t(p0), h1 = uint32_t(p1 >> 32), l1 = uint32_t(p1);
        c0 = h1 ^ c1 ^ k0;
        c1 = l1;
        c2 = h0 ^ c3 ^ k1;
        c3 = l0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

struct Sph {
    float c[3];
    float r;
    int type;
    float albedo[3];
    float fuzz, index;
};

std::vector<Sph> recipe(int kind, uint32_t seed, int H) {
    std::vector<Sph> out;
    auto put = [&](double cx, double cy, double cz, double r, int type, double ar, double ag, double ab, double fz,
                   double ix) {
        out.push_back(Sph{{float(cx), float(cy), float(cz)}, float(r), type, {float(ar), float(ag), float(ab)},
                          float(fz), float(ix)});
    };
    put(0, -1000, 0, 1000, RT_OPTICS_DIFFUSE, .5, .5, .5, 0, 0);
    if (kind == RT_RECIPE_GLIBC) {
        GlibcRand g(seed);
        auto rnd = [&]() { return double(g.next()) / (2147483647.0 + 1.0); };
        auto rndr = [&](double lo, double hi) { return lo + rnd() * (hi - lo); };
        for (int a = -H; a < H; ++a) {
            for (int b = -H; b < H; ++b) {
                const double select = rnd();
                const double rz = rnd();   // P(a+.9*rnd(), .2, b+.9*rnd()): z drawn first
                const double rx = rnd();
                const double cx = a + .9 * rx, cy = .2, cz = b + .9 * rz;
                const double dx = cx - 4, dy = cy - .2, dz = cz;
                if (std::sqrt(dx * dx + dy * dy + dz * dz) > .9) {
                    if (select < .8) {
                        double f1[3], f2[3];
                        for (int i = 2; i >= 0; --i) f1[i] = rnd();
                        for (int i = 2; i >= 0; --i) f2[i] = rnd();
                        put(cx, cy, cz, .2, RT_OPTICS_DIFFUSE, f1[0] * f2[0], f1[1] * f2[1], f1[2] * f2[2], 0, 0);
                    } else if (select < .95) {
                        double al[3];
                        for (int i = 2; i >= 0; --i) al[i] = rndr(.5, 1.);
                        const double fz = rndr(0, .5);
                        put(cx, cy, cz, .2, RT_OPTICS_REFLECT, al[0], al[1], al[2], fz, 0);
                    } else {
                        put(cx, cy, cz, .2, RT_OPTICS_REFRACT, 0, 0, 0, 0, 1.5);
                    }
                }
            }
        }
    } else {
        uint32_t k = 0, buf[4] = {0, 0, 0, 0};
        auto rnd = [&]() {
            if ((k & 3u) == 0) {
                const uint32_t ctr[4] = {k >> 2, 0u, 0u, 0x5343454Eu};
                philox_host(ctr, seed, 0u, buf);
            }
            return u01(buf[(k++) & 3u]);
        };
        auto rndr = [&](float lo, float hi) { return lo + rnd() * (hi - lo); };
        for (int a = -H; a < H; ++a) {
            for (int b = -H; b < H; ++b) {
                const float select = rnd();
                const float rx = rnd();
                const float rz = rnd();
                const float3 c = mk(float(a) + .9f * rx, .2f, float(b) + .9f * rz);
                if (len(sub(c, mk(4.f, .2f, 0.f))) > .9f) {
                    if (select < .8f) {
                        float f1[3], f2[3];
                        for (int i = 0; i < 3; ++i) f1[i] = rnd();
                        for (int i = 0; i < 3; ++i) f2[i] = rnd();
                        put(c.x, c.y, c.z, .2f, RT_OPTICS_DIFFUSE, f1[0] * f2[0], f1[1] * f2[1], f1[2] * f2[2], 0, 0);
                    } else if (select < .95f) {
                        float al[3];
                        for (int i = 0; i < 3; ++i) al[i] = rndr(.5f, 1.f);
                        const float fz = rndr(0.f, .5f);
                        put(c.x, c.y, c.z, .2f, RT_OPTICS_REFLECT, al[0], al[1], al[2], fz, 0);
                    } else {
                        put(c.x, c.y, c.z, .2f, RT_OPTICS_REFRACT, 0, 0, 0, 0, 1.5f);
                    }
                }
            }
        }
    }
    put(0, 1, 0, 1, RT_OPTICS_REFRACT, 0, 0, 0, 0, 1.5);
    put(-4, 1, 0, 1, RT_OPTICS_DIFFUSE, .4, .2, .1, 0, 0);
    put(4, 1, 0, 1, RT_OPTICS_REFLECT, .7, .6, .5, 0, 0);
    return out;
}

}  // namespace
}  // namespace rt

using namespace rt;

extern "C" {

rt_status rt_rtow_spheres(int rng_kind, unsigned int seed, int half_extent, unsigned int cap, rt_float3* centers,
                          float* radii, rt_optics* optics, unsigned int* count) {
    return guarded([&] {
        RT_REQUIRE(rng_kind == RT_RECIPE_GLIBC || rng_kind == RT_RECIPE_COUNTER, "unknown rng_kind");
        RT_REQUIRE(half_extent >= 0 && half_extent <= 1000, "half_extent must be 0..1000");
        RT_REQUIRE(count != nullptr, "count is NULL");
        const std::vector<Sph> s = recipe(rng_kind, seed, half_extent);
        *count = unsigned(s.size());
        if (!centers && !radii && !optics) return;
        RT_REQUIRE(cap >= s.size(), "cap is smaller than the sphere count");
        for (size_t i = 0; i < s.size(); ++i) {
            if (centers) centers[i] = rt_float3{s[i].c[0], s[i].c[1], s[i].c[2]};
            if (radii) radii[i] = s[i].r;
            if (optics) {
                optics[i].type = s[i].type;
                optics[i].albedo = rt_float3{s[i].albedo[0], s[i].albedo[1], s[i].albedo[2]};
                optics[i].fuzz = s[i].fuzz;
                optics[i].index = s[i].index;
            }
        }
    });
}

rt_status rt_scene_load_rtow(rt_scene scene, int rng_kind, unsigned int seed, int half_extent, int ndiv,
                             unsigned int* n_things) {
    return guarded([&] {
        RT_REQUIRE(rng_kind == RT_RECIPE_GLIBC || rng_kind == RT_RECIPE_COUNTER, "unknown rng_kind");
        RT_REQUIRE(half_extent >= 0 && half_extent <= 1000, "half_extent must be 0..1000");
        RT_REQUIRE(ndiv >= -1 && ndiv <= 10, "ndiv must be -1 (analytic) or 0..10");
        const std::vector<Sph> s = recipe(rng_kind, seed, half_extent);
        unsigned mesh = 0, id = 0;
        if (ndiv >= 0) {
            const rt_status st = rt_scene_add_sphere_mesh(scene, 1.f, unsigned(ndiv), &mesh);
            if (st != RT_OK) throw Error(st, rt_last_error_string());
        }
        for (const Sph& p : s) {
            rt_optics o;
            o.type = p.type;
            o.albedo = rt_float3{p.albedo[0], p.albedo[1], p.albedo[2]};
            o.fuzz = p.fuzz;
            o.index = p.index;
            rt_status st;
            if (ndiv < 0) {
                st = rt_scene_add_analytic_sphere(scene, rt_float3{p.c[0], p.c[1], p.c[2]}, p.r, &o, &id);
            } else {
                // optx/rtwo.cxx:157-162: uniform scale by the radius, translation to the centre
                const float T[12] = {p.r, 0, 0, p.c[0], 0, p.r, 0, p.c[1], 0, 0, p.r, p.c[2]};
                st = rt_scene_add_thing(scene, &o, mesh, T, &id);
            }
            if (st != RT_OK) throw Error(st, rt_last_error_string());
        }
        if (n_things) *n_things = unsigned(s.size());
    });
}

}  // extern "C"
