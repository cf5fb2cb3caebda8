// Golden-vector generator for the RTOW final-scene recipe.
//
// Test infrastructure only: compiled by oracle/ref_build.sh against the
// reference's own, unmodified rtow.cxx (rtow.cxx:51-80, scene()) so that the
// sphere list it prints is exactly what the reference builds with glibc
// rand().  Output: one line per sphere, in insertion order:
//   <type> <cx> <cy> <cz> <radius> <ar> <ag> <ab> <fuzz> <index>
// type 0 = Diffuse, 1 = Reflect, 2 = Refract; values printed with %.17g
// (the reference computes them in double precision).
//
// Usage: ref_golden_scene [seed]   (no seed: glibc's default state, i.e. seed 1)

// Standard headers first, so the access-control override below only applies
// to the reference's own classes.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <limits>
#include <memory>
#include <string>
#include <vector>

#define private public
#define protected public
#define main rtow_reference_main
#include "rtow.cxx"
#undef main
#undef private
#undef protected

int main(int argc, char** argv) {
    if (argc > 1) srand(static_cast<unsigned>(strtoul(argv[1], nullptr, 10)));
    Things things = ::scene();
    for (const auto& thing : things.things_) {
        auto sphere = std::dynamic_pointer_cast<Sphere>(thing);
        if (!sphere) return 2;
        int type = -1;
        double a[3] = {0, 0, 0}, fuzz = 0, index = 0;
        if (auto d = std::dynamic_pointer_cast<Diffuse>(sphere->optics_)) {
            type = 0;
            a[0] = d->albedo_.x(); a[1] = d->albedo_.y(); a[2] = d->albedo_.z();
        } else if (auto r = std::dynamic_pointer_cast<Reflect>(sphere->optics_)) {
            type = 1;
            a[0] = r->albedo_.x(); a[1] = r->albedo_.y(); a[2] = r->albedo_.z();
            fuzz = r->fuzz_;
        } else if (auto g = std::dynamic_pointer_cast<Refract>(sphere->optics_)) {
            type = 2;
            index = g->index_;
        } else {
            return 3;
        }
        printf("%d %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g\n", type,
               sphere->center_.x(), sphere->center_.y(), sphere->center_.z(), sphere->radius_,
               a[0], a[1], a[2], fuzz, index);
    }
    return 0;
}
