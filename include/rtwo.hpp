// rtwo.hpp -- C++ facade over rt_api.h with the reference's class names.
//
// Mirrors optx/scene.h:19-63 (Scene), optx/thing.h:17-52 (Thing, Optics),
// optx/camera.h:28-94 (Camera), optx/launcher.h:17-31 (Launcher) and
// optx/sphere.h:18-38 (Sphere).  Failing calls throw std::runtime_error with
// the library's message, as the reference's CUDA_CHECK/OPTX_CHECK do
// (optx/util_cpu.h:18-53); Scene::set/get return false for a bad id
// (optx/scene.cxx:198-225).  Header-only; link with -lrtxplay_gb300.
#pragma once

#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

#include "rt_api.h"

namespace rtwo {

inline void check(rt_status s, const char* what) {
    if (s != RT_OK) throw std::runtime_error(std::string(what) + ": " + rt_last_error_string());
}

// optx/thing.h:17-52
struct Optics {
    enum { TYPE_DIFFUSE = RT_OPTICS_DIFFUSE, TYPE_REFLECT = RT_OPTICS_REFLECT, TYPE_REFRACT = RT_OPTICS_REFRACT };
    int type = TYPE_DIFFUSE;
    rt_float3 albedo{0.f, 0.f, 0.f};
    float fuzz = 0.f;
    float index = 0.f;
    rt_optics abi() const { return rt_optics{type, albedo, fuzz, index}; }
};

struct Thing {
    Optics optics;
};

// (vertices, #vertices, triangles, #triangles), as optx/sphere.h:18
using Mesh = std::tuple<const rt_float3*, unsigned int, const rt_uint3*, unsigned int>;

// Sphere(radius, ndiv) of optx/sphere.cxx:17-106, tessellated on the GPU.
class Sphere {
public:
    explicit Sphere(float radius = 1.f, unsigned int ndiv = 6) {
        rt_scene tmp = nullptr;
        check(rt_scene_create(&tmp), "rt_scene_create");
        unsigned int id = 0, nv = 0, ni = 0;
        try {
            check(rt_scene_add_sphere_mesh(tmp, radius, ndiv, &id), "rt_scene_add_sphere_mesh");
            check(rt_scene_get_mesh(tmp, id, nullptr, &nv, nullptr, &ni), "rt_scene_get_mesh");
            vces_.resize(nv);
            ices_.resize(ni);
            check(rt_scene_get_mesh(tmp, id, vces_.data(), &nv, ices_.data(), &ni), "rt_scene_get_mesh");
        } catch (...) {
            rt_scene_destroy(tmp);
            throw;
        }
        rt_scene_destroy(tmp);
    }
    Mesh mesh() const {
        return Mesh(vces_.data(), unsigned(vces_.size()), ices_.data(), unsigned(ices_.size()));
    }

private:
    std::vector<rt_float3> vces_;
    std::vector<rt_uint3> ices_;
};

// optx/camera.h:28-94
class Camera {
public:
    void set(rt_float3 eye, rt_float3 pat, rt_float3 vup, float fov, float aspratio, float aperture, float fostance) {
        check(rt_camera_set(&c_, eye, pat, vup, fov, aspratio, aperture, fostance), "rt_camera_set");
    }
    rt_float3 eye() const { return c_.eye; }
    void eye(rt_float3 v) { set(v, c_.pat, c_.vup, c_.fov, c_.aspratio, c_.aperture, c_.fostance); }
    rt_float3 pat() const { return c_.pat; }
    void pat(rt_float3 v) { set(c_.eye, v, c_.vup, c_.fov, c_.aspratio, c_.aperture, c_.fostance); }
    rt_float3 vup() const { return c_.vup; }
    void vup(rt_float3 v) { set(c_.eye, c_.pat, v, c_.fov, c_.aspratio, c_.aperture, c_.fostance); }
    float fov() const { return c_.fov; }
    void fov(float v) { set(c_.eye, c_.pat, c_.vup, v, c_.aspratio, c_.aperture, c_.fostance); }
    void aspratio(float v) { set(c_.eye, c_.pat, c_.vup, c_.fov, v, c_.aperture, c_.fostance); }
    float aperture() const { return c_.aperture; }
    void aperture(float v) { set(c_.eye, c_.pat, c_.vup, c_.fov, c_.aspratio, v, c_.fostance); }
    float fostance() const { return c_.fostance; }
    void fostance(float v) { set(c_.eye, c_.pat, c_.vup, c_.fov, c_.aspratio, c_.aperture, v); }
    const rt_camera* abi() const { return &c_; }

private:
    rt_camera c_{};
};

// optx/scene.h:19-63 -- load() is the scene recipe of a subclass (RTWO::load).
class Scene {
public:
    Scene() { check(rt_scene_create(&h_), "rt_scene_create"); }
    // ~Scene keeps the hierarchy arrays for the next scene this thread builds
    // (rt_scene_destroy); free_spare_arrays() frees them
    virtual ~Scene() { rt_scene_destroy(h_); }
    static void free_spare_arrays() { check(rt_scene_destroy(nullptr), "rt_scene_destroy"); }
    Scene(const Scene&) = delete;
    Scene& operator=(const Scene&) = delete;

    virtual unsigned int load() = 0;

    // Scene::add(Object&): a mesh ("GAS"); returns its id
    unsigned int add(const Mesh& m) {
        unsigned int id = 0;
        check(rt_scene_add_mesh(h_, std::get<0>(m), std::get<1>(m), std::get<2>(m), std::get<3>(m), &id),
              "rt_scene_add_mesh");
        return id;
    }
    unsigned int add_sphere_mesh(float radius, unsigned int ndiv) {
        unsigned int id = 0;
        check(rt_scene_add_sphere_mesh(h_, radius, ndiv, &id), "rt_scene_add_sphere_mesh");
        return id;
    }
    // Scene::add(Thing&, gas): an instance with the identity transform
    unsigned int add(const Thing& thing, unsigned int mesh) {
        static const float identity[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};
        const rt_optics o = thing.optics.abi();
        unsigned int id = 0;
        check(rt_scene_add_thing(h_, &o, mesh, identity, &id), "rt_scene_add_thing");
        return id;
    }
    bool set(unsigned int thing, const float* transform) {
        return rt_scene_set_transform(h_, thing, transform) == RT_OK;
    }
    bool get(unsigned int thing, float* transform) { return rt_scene_get_transform(h_, thing, transform) == RT_OK; }
    void build(unsigned int morton_bits = 60, void* stream = nullptr) {
        check(rt_scene_build(h_, morton_bits, stream), "rt_scene_build");
    }
    void update(void* stream = nullptr) { check(rt_scene_update(h_, stream), "rt_scene_update"); }
    rt_scene handle() const { return h_; }

private:
    rt_scene h_ = nullptr;
};

// optx/launcher.h:17-31: owns the image buffers; ignite is synchronous.
class Launcher {
public:
    Launcher(unsigned int w, unsigned int h) : w_(w), h_(h) { check(rt_launcher_create(&l_, w, h), "rt_launcher_create"); }
    ~Launcher() { rt_launcher_destroy(l_); }
    Launcher(const Launcher&) = delete;
    Launcher& operator=(const Launcher&) = delete;
    void resize(unsigned int w, unsigned int h) {
        check(rt_launcher_resize(l_, w, h), "rt_launcher_resize");
        w_ = w;
        h_ = h;
    }
    rt_launch_stats ignite(const Scene& scene, const Camera& cam, const rt_launch_params& p, void* stream = nullptr,
                           bool once = false, unsigned int pick_x = 0, unsigned int pick_y = 0) {
        rt_launch_stats st{};
        check(rt_launcher_ignite(l_, scene.handle(), cam.abi(), &p, stream, once ? 1 : 0, pick_x, pick_y, &st),
              "rt_launcher_ignite");
        return st;
    }
    // Progressive form of ignite (no reference counterpart): the next p.spp
    // samples go into `acc`, the launcher's buffers get the mean over all of
    // its samples (image through pp_sRGB as ignite does).
    rt_launch_stats ignite(const Scene& scene, const Camera& cam, const rt_launch_params& p, rt_accum acc,
                           void* stream = nullptr) {
        rt_frame f{};
        rt_uchar4* image = nullptr;
        check(rt_launcher_frame(l_, &f, &image, nullptr), "rt_launcher_frame");
        rt_launch_stats st{};
        check(rt_launch_accum(scene.handle(), cam.abi(), &p, acc, &f, stream, &st), "rt_launch_accum");
        check(rt_postproc_srgb(f.rawRGB, image, int(w_), int(h_), stream), "rt_postproc_srgb");
        return st;
    }
    void download(rt_float3* raw, unsigned int* rpp, rt_float3* normals, rt_float3* albedos, rt_uchar4* image,
                  unsigned int* pick_id) {
        check(rt_launcher_download(l_, raw, rpp, normals, albedos, image, pick_id), "rt_launcher_download");
    }
    unsigned int width() const { return w_; }
    unsigned int height() const { return h_; }

private:
    rt_launcher l_ = nullptr;
    unsigned int w_, h_;
};

// rt_accum: exact pixel sums kept across launches, saved to and restored from
// host bytes (checkpoint and resume).
class Accum {
public:
    Accum(unsigned int w, unsigned int h) { check(rt_accum_create(&a_, w, h), "rt_accum_create"); }
    ~Accum() { rt_accum_destroy(a_); }
    Accum(const Accum&) = delete;
    Accum& operator=(const Accum&) = delete;
    rt_accum handle() const { return a_; }
    unsigned long long samples() const {
        unsigned long long n = 0;
        check(rt_accum_samples(a_, &n), "rt_accum_samples");
        return n;
    }
    std::vector<unsigned char> save() const {
        size_t n = 0;
        check(rt_accum_state_size(a_, &n), "rt_accum_state_size");
        std::vector<unsigned char> b(n);
        check(rt_accum_save(a_, b.data(), n, nullptr), "rt_accum_save");
        return b;
    }
    void load(const std::vector<unsigned char>& b) { check(rt_accum_load(a_, b.data(), b.size(), nullptr), "rt_accum_load"); }

private:
    rt_accum a_ = nullptr;
};

}  // namespace rtwo
