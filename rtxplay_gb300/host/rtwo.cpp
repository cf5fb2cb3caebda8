// rtwo -- batch launcher of the GB300 path tracer with the reference's options.
//
// Options and outputs follow optx/args.cxx:19-151 and optx/rtwo.cxx:78-666:
//   -g, --geometry <w>x<h>|<name>   image size (default 1280x720; names as the
//                                   resolution table of optx/args.h:20-42)
//   -a, --aspect-ratio <w>:<h>      height from width and ratio
//   -s, --samples-per-pixel <n>     default 50
//   -d, --trace-depth <n>           rays per path, default and maximum 50
//   -A, --print-aov RPP             rays per pixel as PGM (P2) after the image
//   -G, --print-guides              normals and albedos as PPM (with -D)
//   -S, --print-statistics          "pixel, rays, milliseconds, fps" on stderr
//   -D, --apply-denoiser <type>     accepted; the OptiX AI denoiser is not part
//                                   of this renderer, so only the guides are kept
//   -q, --quiet / --silent          no image output
//   -v, --verbose; -t, --trace-sm   accepted (the interactive UI is not built)
//   -h, --help / --usage
// Additions of this renderer:
//   --scene rtwo|tess|analytic      rtwo: mesh levels 3/6/8/9 as RTWO::load
//                                   (optx/rtwo.cxx:138-243, default); tess: every
//                                   sphere at --level; analytic: exact spheres
//   --level <n>                     tessellation level for --scene tess (6)
//   --seed <n>                      counter-RNG seed (4711)
//   --scene-seed <n>                glibc rand() seed of the scene recipe (1)
//   --morton 30|60                  LBVH key width (60)
//   --resume <file>                 continue a render from a checkpoint: -s more
//                                   samples on top of the saved ones
//   --checkpoint <file>             save the pixel sums after rendering (the
//                                   image is the mean over all samples so far)
//   --print-args                    print the parsed options as JSON and exit
// The image goes to stdout as PPM (P3), rows bottom-up (optx/rtwo.cxx:622-666).
#include <getopt.h>

#include <chrono>
#include <cstdio>
#include <fstream>
#include <iterator>
#include <memory>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include "rtwo.hpp"

namespace {

const std::map<std::string, std::pair<int, int>>& resolutions() {
    static const std::map<std::string, std::pair<int, int>> m = {
        {"CGA", {320, 200}},     {"HVGA", {480, 320}},    {"VGA", {640, 480}},     {"WVGA", {800, 480}},
        {"SVGA", {800, 600}},    {"XGA", {1024, 768}},    {"HD", {1280, 720}},     {"SXGA", {1280, 1024}},
        {"UXGA", {1600, 1200}},  {"FULLHD", {1920, 1080}}, {"2K", {2048, 1080}},   {"QXGA", {2048, 1536}},
        {"UWHD", {2560, 1080}},  {"WQHD", {2560, 1440}},  {"WQXGA", {2560, 1600}}, {"UWQHD", {3440, 1440}},
        {"UHD-1", {3840, 2160}}, {"4K", {4096, 2160}},    {"5K-UW", {5120, 2160}}, {"5K", {5120, 2880}},
        {"UHD-2", {7680, 4320}}};
    return m;
}

struct Options {
    int w = -1, h = -1, spp = -1, depth = -1;
    std::string denoiser = "none";
    bool verbose = false, help = false, quiet = false, trace = false, guides = false, stats = false, rpp = false;
    std::string scene = "rtwo";
    int level = 6;
    unsigned seed = 4711, scene_seed = 1, morton = 60;
    std::string resume, checkpoint;
    bool print_args = false;
};

void usage() {
    std::cerr << "Usage: rtwo [OPTION...]\n"
                 "  Renders the final image of Ray Tracing in One Weekend on one GB300 and\n"
                 "  writes it (PPM) to stdout.\n\n"
                 "  -g, --geometry <w>x<h>|<name>  -a, --aspect-ratio <w>:<h>\n"
                 "  -s, --samples-per-pixel <n>    -d, --trace-depth <n>\n"
                 "  -A, --print-aov RPP            -G, --print-guides\n"
                 "  -S, --print-statistics         -D, --apply-denoiser <type>\n"
                 "  -q, --quiet, --silent          -v, --verbose   -t, --trace-sm   -h, --help, --usage\n"
                 "  --scene rtwo|tess|analytic     --level <n>     --seed <n>\n"
                 "  --scene-seed <n>               --morton 30|60  --print-args\n"
                 "  --resume <file>                --checkpoint <file>\n";
}

Options parse(int argc, char** argv) {
    Options o;
    int v = 0, t = 0, q = 0, h = 0, G = 0, S = 0, pa = 0;
    const struct option lopts[] = {{"geometry", required_argument, nullptr, 'g'},
                                   {"aspect-ratio", required_argument, nullptr, 'a'},
                                   {"samples-per-pixel", required_argument, nullptr, 's'},
                                   {"trace-depth", required_argument, nullptr, 'd'},
                                   {"verbose", no_argument, &v, 1},
                                   {"trace-sm", no_argument, &t, 1},
                                   {"quiet", no_argument, &q, 1},
                                   {"silent", no_argument, &q, 1},
                                   {"help", no_argument, &h, 1},
                                   {"usage", no_argument, &h, 1},
                                   {"print-aov", required_argument, nullptr, 'A'},
                                   {"print-guides", no_argument, &G, 1},
                                   {"print-statistics", no_argument, &S, 1},
                                   {"apply-denoiser", required_argument, nullptr, 'D'},
                                   {"scene", required_argument, nullptr, 1001},
                                   {"level", required_argument, nullptr, 1002},
                                   {"seed", required_argument, nullptr, 1003},
                                   {"scene-seed", required_argument, nullptr, 1004},
                                   {"morton", required_argument, nullptr, 1005},
                                   {"resume", required_argument, nullptr, 1006},
                                   {"checkpoint", required_argument, nullptr, 1007},
                                   {"print-args", no_argument, &pa, 1},
                                   {nullptr, 0, nullptr, 0}};
    int c;
    while ((c = getopt_long(argc, argv, "g:a:s:d:vtqhA:GSD:", lopts, nullptr)) != -1) {
        switch (c) {
            case 'g': {
                auto it = resolutions().find(optarg);
                if (it != resolutions().end()) {
                    o.w = it->second.first;
                    o.h = it->second.second;
                } else if (std::sscanf(optarg, "%dx%d", &o.w, &o.h) != 2 || o.w < 1 || o.h < 1) {
                    o.w = o.h = -1;
                }
                break;
            }
            case 'a': {
                float aw = 0, ah = 0;
                if (std::sscanf(optarg, "%f:%f", &aw, &ah) == 2 && o.w > 0 && aw > 0 && ah > 0)
                    o.h = int(float(o.w) * ah / aw + .5f);
                break;
            }
            case 's': o.spp = std::abs(std::atoi(optarg)); break;
            case 'd': o.depth = std::abs(std::atoi(optarg)); break;
            case 'v': v = 1; break;
            case 't': t = 1; break;
            case 'q': q = 1; break;
            case 'h': h = 1; break;
            case 'G': G = 1; break;
            case 'S': S = 1; break;
            case 'A': {
                std::string list = optarg;
                size_t pos = 0;
                while (pos <= list.size()) {
                    const size_t e = list.find(',', pos);
                    const std::string item = list.substr(pos, e == std::string::npos ? std::string::npos : e - pos);
                    if (item == "RPP") o.rpp = true;
                    else std::cerr << "rtwo: unknown argument for option A ignored -- " << item << "\n";
                    if (e == std::string::npos) break;
                    pos = e + 1;
                }
                break;
            }
            case 'D': {
                const std::string d = optarg;
                if (d == "SMP" || d == "NRM" || d == "ALB" || d == "NAA" || d == "AOV") o.denoiser = d;
                else std::cerr << "rtwo: unknown argument for option D ignored -- " << d << "\n";
                break;
            }
            case 1001: o.scene = optarg; break;
            case 1002: o.level = std::atoi(optarg); break;
            case 1003: o.seed = unsigned(std::strtoul(optarg, nullptr, 10)); break;
            case 1004: o.scene_seed = unsigned(std::strtoul(optarg, nullptr, 10)); break;
            case 1005: o.morton = unsigned(std::strtoul(optarg, nullptr, 10)); break;
            case 1006: o.resume = optarg; break;
            case 1007: o.checkpoint = optarg; break;
            case 0: break;   // long flag stored through its pointer
            default: throw std::invalid_argument("try 'rtwo --help' for more information.");
        }
    }
    o.verbose = v; o.trace = t; o.quiet = q; o.help = h; o.guides = G; o.stats = S; o.print_args = pa;
    if (o.scene != "rtwo" && o.scene != "tess" && o.scene != "analytic")
        throw std::invalid_argument("--scene must be rtwo, tess or analytic");
    return o;
}

// RTWO::load (optx/rtwo.cxx:137-244): the final scene; ground at level 9,
// small diffuse/metal spheres at 6, small glass at 3, big glass 8, big
// diffuse 6, big metal 3 (scene "rtwo"), or one level for all ("tess").
class RTWO : public rtwo::Scene {
public:
    RTWO(const Options& o) : o_(o) {}
    unsigned int load() override {
        unsigned int n = 0;
        if (o_.scene == "analytic") {
            rtwo::check(rt_scene_load_rtow(handle(), RT_RECIPE_GLIBC, o_.scene_seed, 11, -1, &n), "load");
            return n;
        }
        if (o_.scene == "tess") {
            rtwo::check(rt_scene_load_rtow(handle(), RT_RECIPE_GLIBC, o_.scene_seed, 11, o_.level, &n), "load");
            return n;
        }
        rtwo::check(rt_rtow_spheres(RT_RECIPE_GLIBC, o_.scene_seed, 11, 0, nullptr, nullptr, nullptr, &n), "recipe");
        std::vector<rt_float3> c(n);
        std::vector<float> r(n);
        std::vector<rt_optics> opt(n);
        rtwo::check(rt_rtow_spheres(RT_RECIPE_GLIBC, o_.scene_seed, 11, n, c.data(), r.data(), opt.data(), &n),
                    "recipe");
        const unsigned int gas_3 = add_sphere_mesh(1.f, 3), gas_6 = add_sphere_mesh(1.f, 6),
                           gas_8 = add_sphere_mesh(1.f, 8), gas_9 = add_sphere_mesh(1.f, 9);
        for (unsigned int i = 0; i < n; ++i) {
            unsigned int gas;
            if (i == 0) gas = gas_9;                                   // ground
            else if (i == n - 3) gas = gas_8;                          // big glass
            else if (i == n - 2) gas = gas_6;                          // big diffuse
            else if (i == n - 1) gas = gas_3;                          // big metal
            else gas = opt[i].type == RT_OPTICS_REFRACT ? gas_3 : gas_6;
            rtwo::Thing thing;
            thing.optics.type = opt[i].type;
            thing.optics.albedo = opt[i].albedo;
            thing.optics.fuzz = opt[i].fuzz;
            thing.optics.index = opt[i].index;
            const unsigned int id = add(thing, gas);
            const float T[12] = {r[i], 0, 0, c[i].x, 0, r[i], 0, c[i].y, 0, 0, r[i], c[i].z};
            set(id, T);
        }
        return n;
    }

private:
    const Options& o_;
};

template <class T, class F>
void pnm(const char* magic, unsigned w, unsigned h, int maxval, const std::vector<T>& img, F fmt) {
    std::printf("%s\n%u %u\n%d\n", magic, w, h, maxval);
    for (int y = int(h) - 1; y >= 0; --y)
        for (unsigned x = 0; x < w; ++x) fmt(img[size_t(w) * y + x]);
    std::printf("\n");
}

int clampbyte(float x) { return int((x < 0.f ? 0.f : (x > 1.f ? 1.f : x)) * 255); }

std::vector<unsigned char> read_file(const std::string& path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw std::runtime_error("cannot read " + path);
    return std::vector<unsigned char>(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
}

void write_file(const std::string& path, const std::vector<unsigned char>& b) {
    std::ofstream f(path, std::ios::binary);
    f.write(reinterpret_cast<const char*>(b.data()), std::streamsize(b.size()));
    if (!f) throw std::runtime_error("cannot write " + path);
}

}  // namespace

int main(int argc, char** argv) {
    Options o;
    try {
        o = parse(argc, argv);
    } catch (const std::exception& e) {
        std::cerr << "rtwo: " << e.what() << "\n";
        return 1;
    }
    if (o.help) {
        usage();
        return 0;
    }
    const unsigned w = o.w > 0 ? unsigned(o.w) : 1280u;
    const unsigned h = o.h > 0 ? unsigned(o.h) : 720u;
    const unsigned spp = o.spp >= 0 ? unsigned(o.spp) : 50u;
    unsigned depth = o.depth >= 0 ? unsigned(o.depth) : 50u;
    if (depth > 50) depth = 50;   // MAX_DEPTH of the iterative launcher (optx/rtwo.cxx:92-98)
    if (o.print_args) {
        std::printf("{\"w\": %u, \"h\": %u, \"spp\": %u, \"depth\": %u, \"quiet\": %d, \"stats\": %d, \"rpp\": %d, "
                    "\"guides\": %d, \"denoiser\": \"%s\", \"scene\": \"%s\", \"level\": %d, \"seed\": %u, "
                    "\"scene_seed\": %u, \"morton\": %u, \"verbose\": %d, \"trace\": %d, \"resume\": \"%s\", "
                    "\"checkpoint\": \"%s\"}\n",
                    w, h, spp, depth, int(o.quiet), int(o.stats), int(o.rpp), int(o.guides), o.denoiser.c_str(),
                    o.scene.c_str(), o.level, o.seed, o.scene_seed, o.morton, int(o.verbose), int(o.trace),
                    o.resume.c_str(), o.checkpoint.c_str());
        return 0;
    }
    try {
        if (spp < 1 || depth < 1) throw std::invalid_argument("samples per pixel and trace depth must be >= 1");
        rtwo::Camera camera;
        camera.set({13.f, 2.f, 3.f}, {0.f, 0.f, 0.f}, {0.f, 1.f, 0.f}, 20.f, float(w) / float(h), .1f, 10.f);
        RTWO scene(o);
        scene.load();
        scene.build(o.morton);
        const bool denoise = o.denoiser != "none";
        if (denoise)
            std::cerr << "rtwo: the OptiX AI denoiser is not part of this renderer; -D " << o.denoiser
                      << " keeps the guide layers only\n";
        rt_launch_params p{};
        p.image_w = w;
        p.image_h = h;
        p.spp = spp;
        p.depth = depth;
        p.seed = o.seed;
        p.flags = denoise ? RT_FLAG_GUIDES : 0u;
        p.ambient = rt_float3{.5f, .7f, 1.f};   // miss SBT record, optx/rtwo.cxx:110-111
        p.white = rt_float3{1.f, 1.f, 1.f};
        rtwo::Launcher launcher(w, h);
        std::unique_ptr<rtwo::Accum> acc;   // progressive render: resumed and/or checkpointed
        if (!o.resume.empty() || !o.checkpoint.empty()) {
            if (denoise) throw std::invalid_argument("--resume/--checkpoint do not keep guide layers (-D)");
            acc.reset(new rtwo::Accum(w, h));
            if (!o.resume.empty()) acc->load(read_file(o.resume));
        }
        const auto t0 = std::chrono::high_resolution_clock::now();
        const rt_launch_stats st = acc ? launcher.ignite(scene, camera, p, acc->handle()) : launcher.ignite(scene, camera, p);
        const auto t1 = std::chrono::high_resolution_clock::now();
        if (acc && !o.checkpoint.empty()) write_file(o.checkpoint, acc->save());
        const size_t n = size_t(w) * h;
        std::vector<rt_uchar4> image(n);
        std::vector<unsigned int> rpp(n);
        std::vector<rt_float3> normals(denoise ? n : 0), albedos(denoise ? n : 0);
        launcher.download(nullptr, rpp.data(), denoise ? normals.data() : nullptr,
                          denoise ? albedos.data() : nullptr, image.data(), nullptr);
        if (!o.quiet && denoise && o.guides) {
            auto f3 = [](const rt_float3& c) { std::printf("%d %d %d\n", clampbyte(c.x), clampbyte(c.y), clampbyte(c.z)); };
            pnm("P3", w, h, 255, normals, f3);
            pnm("P3", w, h, 255, albedos, f3);
        }
        if (!o.quiet)
            pnm("P3", w, h, 255, image, [](const rt_uchar4& c) { std::printf("%d %d %d\n", c.x, c.y, c.z); });
        if (!o.quiet && o.rpp) pnm("P2", w, h, 65535, rpp, [](unsigned v) { std::printf("%u\n", v); });
        if (o.stats) {
            const long long dt = std::chrono::duration_cast<std::chrono::milliseconds>(t1 - t0).count();
            unsigned long long rays = 0;
            for (unsigned v : rpp) rays += v;
            std::fprintf(stderr, "%9u %12llu %4lld (pixel, rays, milliseconds) %6.2f fps\n", unsigned(n), rays, dt,
                         dt > 0 ? 1000.f / float(dt) : 0.f);
            if (o.verbose)
                std::fprintf(stderr, "waves %u, kernel launches %u, wave capacity %u\n", st.waves, st.kernel_launches,
                             st.wave_capacity);
        }
    } catch (const std::exception& e) {
        std::cerr << "exception: " << e.what() << "\n";
        return 1;
    }
    return 0;
}
