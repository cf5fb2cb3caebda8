/* CPU oracle for the GB300 path tracer -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain C++ restatement of the reference's render path, used by tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg, to check the product against.
 * Nothing in the product library links, loads or calls this code.
 *
 * Parity pins: the tessellator and the scene recipe are checked bit for bit
 * (resp. to double rounding) against golden vectors produced by the
 * reference's own optx/sphere.cxx and rtow.cxx (tests/golden/make_golden.py);
 * the counter RNG against the Philox4x32-10 known-answer vectors of Salmon et
 * al. (SC'11).  The reference's GPU path (OptiX traversal) is closed and
 * cannot run here, so first-hit/image parity is defined against this oracle.
 *
 * Every routine states the reference file:line it follows.  All float
 * arithmetic is plain IEEE single precision, compiled without FMA contraction
 * (-ffp-contract=off), in the same operation order as the CUDA kernels.
 */
#ifndef RT_ORACLE_H
#define RT_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- random numbers ---------------------------------------------------- */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
float orc_u01(uint32_t x);
/* glibc random(3) TYPE_3 restatement; out[i] = i-th rand() after srand(seed). */
void orc_glibc_rand(uint32_t seed, int n, int32_t* out);

/* ---- scene recipe (rtow.cxx:51-80, optx/rtwo.cxx:147-243) -------------- */
/* rng_kind 0: glibc rand() stream (reference compatible, float arithmetic as
 * in optx/rtwo.cxx); 1: counter-RNG stream.  half_extent 11 gives the final
 * scene's a,b in [-11,11).  Returns the sphere count (<= cap) or -1. */
int orc_scene_rtow(int rng_kind, uint32_t seed, int half_extent, int cap, float* centers,
                   float* radii, int* types, float* albedos, float* fuzz, float* index);

/* ---- tessellation (optx/sphere.cxx:28-106) ------------------------------ */
/* Sphere(radius, ndiv).mesh(): writes the unique vertices (3 floats each, in
 * first-seen order) and 3 indices per triangle; returns the vertex count.
 * Size vces for 3*nv floats and ices for 3*ni from orc_tessellate_counts. */
void orc_tessellate_counts(unsigned ndiv, unsigned* nv, unsigned* ni);
int orc_tessellate(float radius, unsigned ndiv, float* vces, unsigned* ices);

/* ---- camera (optx/camera.h:30-48) -------------------------------------- */
/* out[18] = u, v, w, hvec, wvec, dvec */
void orc_camera_set(const float eye[3], const float pat[3], const float vup[3], float fov,
                    float aspratio, float aperture, float fostance, float out[18]);

/* ---- LBVH twin ---------------------------------------------------------- */
void orc_morton30(const float* centroids, unsigned n, const float lo[3], const float hi[3],
                  uint32_t* codes);
/* 60-bit codes: 20 bits per axis, same quantisation rule at 2^20 cells. */
void orc_morton60(const float* centroids, unsigned n, const float lo[3], const float hi[3],
                  uint64_t* codes);
void orc_stable_sort_pairs(uint32_t* keys, uint32_t* vals, unsigned n);
void orc_stable_sort_pairs64(uint64_t* keys, uint32_t* vals, unsigned n);
/* Karras 2012 hierarchy over n sorted codes (30- or 60-bit codes held in 64
 * bits): left/right[n-1]; child >= 0 is an internal node, child < 0 is leaf ~child. */
void orc_karras(const uint64_t* sorted_codes, unsigned n, int32_t* left, int32_t* right);

/* ---- world -------------------------------------------------------------- */
typedef struct orc_world orc_world;
orc_world* orc_world_new(void);
void orc_world_free(orc_world* w);
int orc_world_add_mesh(orc_world* w, const float* vces, unsigned nv, const unsigned* ices,
                       unsigned ni);
int orc_world_add_thing(orc_world* w, int type, const float albedo[3], float fuzz, float index,
                        int mesh, const float transform[12]);
int orc_world_add_sphere(orc_world* w, int type, const float albedo[3], float fuzz, float index,
                         const float center[3], float radius);
int orc_world_set_transform(orc_world* w, int thing, const float transform[12]);
/* Flattens things into world-space primitives and builds the LBVH twin with
 * 30- or 60-bit Morton codes. */
int orc_world_build(orc_world* w, int morton_bits);
/* The same world with things-grouped keys: things ranked by a 60-bit code of
 * their centroid-bounds centre, key = rank << 30 | 30-bit code inside the
 * thing's centroid bounds (the product's RT_LAYOUT_GROUPED). */
int orc_world_build_grouped(orc_world* w);
/* The same world under the binned-SAH hierarchy of the product's
 * RT_LAYOUT_SAH (binned surface-area splits down to clusters of at most
 * cluster_max records, a Karras hierarchy per cluster over local 30-bit
 * codes, split nodes stitched into the clusters' spare slots). */
int orc_world_build_sah(orc_world* w, unsigned cluster_max);
unsigned orc_world_nprims(const orc_world* w);
/* Copies out the LBVH: codes[n] (sorted), ids[n] (sorted prim ids), left/right[n-1],
 * boxes[(n-1)*12] (child0 lo,hi then child1 lo,hi per internal node), scene
 * centroid bounds lo/hi[3]. Any pointer may be NULL. */
void orc_world_lbvh(const orc_world* w, uint64_t* codes, uint32_t* ids, int32_t* left,
                    int32_t* right, float* boxes, float* clo, float* chi);
/* World-space triangles (9 floats each) in prim-id order; n = nprims. */
void orc_world_triangles(const orc_world* w, float* tris);

typedef struct {
    float eye[3];
    float u[3], v[3], w[3], hvec[3], wvec[3], dvec[3];
    float aperture;
    int rtow_pixels;   /* 1: rtow's pixel mapping over w - 1, h - 1 (rtow.cxx:112-113) */
} orc_camera;

/* Primary-ray closest hit for sample `sample` of every pixel (x,y) of a w*h
 * image (pixel index w*y+x); prim/thing = -1 on a miss.  use_bvh 0 = brute
 * force over all primitives. t64 (may be NULL) = FP64 distance to the same
 * primitive along the same (FP32) ray, NaN on a miss. */
void orc_first_hit(const orc_world* wd, const orc_camera* cam, unsigned w, unsigned h,
                   uint32_t seed, uint32_t scene, uint32_t sample, int use_bvh, int32_t* prim,
                   int32_t* thing, float* t, float* u, float* v, double* t64, int nthreads);

/* Closest hit of n arbitrary rays (o, d: 3 floats each): mode 0 brute force
 * over all primitives, 1 the hierarchy, 2 brute force over the primitives
 * whose own box passes the slab test.  prim = -1 (t = 0) on a miss. */
void orc_closest(const orc_world* wd, unsigned n, const float* o, const float* d, int mode, int32_t* prim,
                 float* t, int nthreads);

/* Renders the listed pixels (pixels == NULL: all w*h, in index order).
 * Outputs are indexed by list position.  Returns total rays cast. */
uint64_t orc_render(const orc_world* wd, const orc_camera* cam, unsigned w, unsigned h,
                    unsigned spp, unsigned depth, uint32_t seed, uint32_t scene,
                    const float ambient[3], const float white[3], const uint32_t* pixels,
                    unsigned npixels, float* rawRGB, uint32_t* rpp, float* normals,
                    float* albedos, int nthreads);

/* ---- adjoint ------------------------------------------------------------ */
unsigned orc_world_nthings(const orc_world* w);
int orc_world_set_optics(orc_world* w, int thing, int type, const float albedo[3], float fuzz, float index);
void orc_world_get_optics(const orc_world* w, int* types, float* albedos, float* fuzz, float* index);
/* Per-path check of the fuzz derivative (tangent vs central difference of the
 * same path, paths whose hit sequence changes are skipped): out[4] =
 * compared, skipped, max relative error, sum |fd|, paths off by more than 5%,
 * sum of the tangent derivatives, sum of the differences. */
void orc_fuzz_path_check(orc_world* wd, const orc_camera* cam, unsigned w, unsigned h, unsigned spp,
                         unsigned depth, uint32_t seed, int thing, float step, const float ambient[3],
                         const float white[3], double* out);  /* out[7] */
/* Image-level central difference of metal `thing`'s fuzz with visibility
 * held fixed: every sky-ending path that reflects off `thing` is replayed in
 * double precision along its recorded primitives and branches with fuzz
 * f0 and f0 +- step;
 * delta_plus/minus (w*h*3) receive the change of every pixel's mean.  out[4]
 * = paths replayed, degenerate replays left out, paths whose plain re-render
 * changes its hit sequence, and (image and grad_image given, else 0) the
 * adjoint's fuzz gradient over the replayed paths on their replayed
 * trajectories. */
void orc_fuzz_held_delta(const orc_world* wd, const orc_camera* cam, unsigned w, unsigned h, unsigned spp,
                         unsigned depth, uint32_t seed, uint32_t scene, int thing, double step,
                         const float ambient[3], const float white[3], const float* image,
                         const float* grad_image, double* delta_plus, double* delta_minus, double* out,
                         int nthreads);
/* FP64 gradients of a scalar loss of the rendered image, given dL/dI
 * (grad_image, w*h*3, with image = the clamped render): per thing
 * grad_albedo[3*n], grad_fuzz[n]; grad_sky[6] = d/d ambient xyz, d/d white xyz.
 * Every path is replayed as rendered, visibility held fixed. */
void orc_adjoint(const orc_world* wd, const orc_camera* cam, unsigned w, unsigned h, unsigned spp,
                 unsigned depth, uint32_t seed, uint32_t scene, const float ambient[3],
                 const float white[3], const float* image, const float* grad_image,
                 double* grad_albedo, double* grad_fuzz, double* grad_sky, int nthreads);

/* ---- post-processing (optx/postproc.cu:2-47, rtow.cxx:6-21) ------------- */
void orc_pp_srgb(const float* src, uint8_t* dst, int w, int h);
void orc_pp_none(const float* src, uint8_t* dst, int w, int h);
void orc_pp_gamma2(const float* src, uint8_t* dst, int w, int h);

#ifdef __cplusplus
}
#endif
#endif /* RT_ORACLE_H */
