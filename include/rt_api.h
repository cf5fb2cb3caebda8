/* rt_api.h -- C ABI of the GB300 path tracer (librtxplay_gb300.so).
 *
 * Drop-in boundary for the render path behind RTXplay's Scene / Thing /
 * Optics / Camera / Launcher classes and the rtwo launcher (reference project
 * otabuzzman/RTXplay, directory optx/).  Every function is extern "C", takes
 * plain pointers and sizes, returns an rt_status and never throws.  Device
 * buffers named in rt_frame are caller-owned device pointers; everything
 * behind an opaque handle is library-owned.  A failing call leaves a message
 * for rt_last_error_string() in the calling thread.
 *
 * Streams are passed as `void*` holding a cudaStream_t (NULL = legacy default
 * stream).  All launches on a stream are asynchronous unless stated.
 */
#ifndef RT_API_H
#define RT_API_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ status */
typedef enum {
    RT_OK = 0,
    RT_ERR_INVALID_ARG = 1,   /* bad handle, id, size or flag; Scene::set/get's `false` (optx/scene.cxx:198-225) */
    RT_ERR_CUDA = 2,          /* a CUDA runtime call failed; CUDA_CHECK's throw (optx/util_cpu.h:18-28) */
    RT_ERR_OUT_OF_MEMORY = 3,
    RT_ERR_NOT_BUILT = 4,     /* render or update before rt_scene_build */
    RT_ERR_LIMIT = 5,         /* an internal iteration limit was reached (device error word set) */
    RT_ERR_INTERNAL = 6
} rt_status;

/* Message of the last failing call in this thread ("" if none). */
const char* rt_last_error_string(void);
/* Library version string, e.g. "rtxplay_gb300 0.1 sm_103a". */
const char* rt_version(void);

/* Fault injection on the host (tests): the n-th device allocation from now
 * fails as cudaMalloc's out-of-memory would (RT_ERR_OUT_OF_MEMORY from the call
 * that made it); n = 0 switches it off.  Process-wide. */
rt_status rt_debug_fail_alloc(unsigned int n);

/* ------------------------------------------------------------- data types */
typedef struct { float x, y, z; } rt_float3;
typedef struct { unsigned int x, y, z; } rt_uint3;
typedef struct { unsigned char x, y, z, w; } rt_uchar4;

/* Optics: flattened form of the tagged union Optics{type; Diffuse{albedo} /
 * Reflect{albedo,fuzz} / Refract{index}} of optx/thing.h:17-52. */
typedef enum { RT_OPTICS_DIFFUSE = 0, RT_OPTICS_REFLECT = 1, RT_OPTICS_REFRACT = 2 } rt_optics_type;
typedef struct {
    int type;          /* rt_optics_type */
    rt_float3 albedo;  /* Diffuse, Reflect */
    float fuzz;        /* Reflect */
    float index;       /* Refract */
} rt_optics;

/* Camera: host-side state of class Camera (optx/camera.h:28-94).  Filled by
 * rt_camera_set; the derived basis and viewport vectors are what the device
 * ray generator (optx/camera.h:67-77) reads. */
typedef struct {
    rt_float3 eye, pat, vup;
    float fov, aspratio, aperture, fostance;
    rt_float3 u, v, w, hvec, wvec, dvec;
} rt_camera;

/* Per-launch parameters: the render fields of LpGeneral (optx/rtwo.h:26-52)
 * plus the counter-RNG seed and the sky colours of __miss__ambient
 * (optx/camera_i.cu:130-139; ambient is the miss SBT record of
 * optx/rtwo.cxx:110-111, white the constant of optx/camera_i.cu:137). */
typedef struct {
    unsigned int image_w, image_h;
    unsigned int spp;        /* samples per pixel, >= 1 */
    unsigned int depth;      /* rays per path, 1..255; a hit on the depth-th ray is black */
    unsigned int seed;       /* counter-RNG key */
    unsigned int flags;      /* RT_FLAG_* */
    rt_float3 ambient;       /* default (0.5, 0.7, 1.0) */
    rt_float3 white;         /* default (1, 1, 1) */
} rt_launch_params;

#define RT_FLAG_GUIDES        0x1u  /* write normals/albedos guide layers */
#define RT_FLAG_STAGE_TIMING  0x2u  /* time the traversal and shading kernels with CUDA events */
#define RT_FLAG_COUNT_VISITS  0x4u  /* count BVH nodes visited and primitives tested (slower) */
#define RT_FLAG_RTOW_PIXELS   0x8u  /* rtow's pixel mapping s = 2(x+r)/(w-1) - 1 (rtow.cxx:112-113) instead of
                                       rtwo's 2(x+r)/w - 1 (optx/camera_i.cu:61); needs w, h >= 2 */

/* Output buffers (device pointers, caller-owned): the image buffers of
 * LpGeneral allocated by Launcher::resize (optx/launcher.cxx:36-47). */
typedef struct {
    rt_float3* rawRGB;      /* w*h, clamped mean colour (required) */
    unsigned int* rpp;      /* w*h, rays per pixel (may be NULL) */
    rt_float3* normals;     /* w*h, guide layer (NULL unless RT_FLAG_GUIDES) */
    rt_float3* albedos;     /* w*h, guide layer (NULL unless RT_FLAG_GUIDES) */
} rt_frame;

/* Statistics of one rt_launch_ex call (host-side after it returns). */
typedef struct {
    unsigned long long rays;          /* sum of rpp over all pixels */
    unsigned long long paths;
    unsigned long long node_visits;   /* RT_FLAG_COUNT_VISITS only */
    unsigned long long prim_tests;    /* RT_FLAG_COUNT_VISITS only */
    unsigned int waves;               /* extend/shade iterations */
    unsigned int kernel_launches;     /* kernels launched by this call */
    float extend_ms;                  /* RT_FLAG_STAGE_TIMING only: sum over traversal launches */
    float shade_ms;                   /* RT_FLAG_STAGE_TIMING only */
    unsigned int extend_launches;
    unsigned int wave_capacity;       /* rays per wave queue */
} rt_launch_stats;

/* --------------------------------------------------------------- camera */
/* Camera::set (optx/camera.h:30-48): basis w = unit(eye-pat), u, v and the
 * focus-plane vectors, computed on the host in binary32 (tanf only here). */
rt_status rt_camera_set(rt_camera* cam, rt_float3 eye, rt_float3 pat, rt_float3 vup, float fov,
                        float aspratio, float aperture, float fostance);

/* ---------------------------------------------------------------- scene */
typedef struct rt_scene_s* rt_scene;

/* Scene::Scene / ~Scene (optx/scene.cxx:38-45; optx/scene.h:19-63).
 * rt_scene_destroy waits for the device (as freeing device memory does) and
 * keeps the scene's hierarchy arrays for the next scene this host thread
 * builds on the same device, instead of freeing and allocating them again
 * (that scene takes them if they hold at most about twice its records, else
 * they are freed); rt_scene_destroy(NULL) frees the arrays so kept. */
rt_status rt_scene_create(rt_scene* out);
rt_status rt_scene_destroy(rt_scene scene);

/* Scene::add(Object&) (optx/scene.cxx:47-167): copies one indexed triangle
 * mesh to the device and returns its mesh id ("GAS id"). */
rt_status rt_scene_add_mesh(rt_scene scene, const rt_float3* vces, unsigned int nv,
                            const rt_uint3* ices, unsigned int ni, unsigned int* mesh_id);

/* Object(file) + Scene::add per mesh (optx/object.cxx:23-106,
 * optx/rtwo.cxx:138-145): reads a Wavefront OBJ file on the host; every shape
 * (`o`/`g` group with faces) becomes one mesh of the scene.  Only `v` and `f`
 * records are used (face vertices `i`, `i/t`, `i//n`, `i/t/n`, negative
 * indices relative); faces of more than three vertices are split into fans.
 * A shape's mesh holds the vertices its faces reference in order of first
 * reference.  mesh_ids (cap entries, may be NULL) receives the new mesh ids,
 * n_meshes their count.  RT_ERR_INVALID_ARG for unreadable files, malformed
 * records and out-of-range indices (with file:line in the message); nothing
 * is added then.  If adding a later shape's mesh fails (out of memory), the
 * meshes added before it stay in the scene: mesh_ids and n_meshes report
 * them, and the call returns the failure. */
rt_status rt_scene_add_obj(rt_scene scene, const char* path, unsigned int* mesh_ids, unsigned int cap,
                           unsigned int* n_meshes);
/* The same parser alone (host memory, no device use): the number of shapes,
 * and for shape `shape` its vertex and triangle counts and arrays (any
 * pointer may be NULL; with all four NULL only nshapes is filled).  To fill
 * vces (ices), pass its capacity in entries in *nv (*ni); the call fails with
 * RT_ERR_INVALID_ARG, writing nothing, when the shape does not fit (the file
 * is read again on every call).  On return *nv and *ni hold the counts. */
rt_status rt_obj_parse(const char* path, unsigned int shape, rt_float3* vces, unsigned int* nv,
                       rt_uint3* ices, unsigned int* ni, unsigned int* nshapes);

/* Sphere(radius, ndiv) (optx/sphere.cxx:17-106) + Scene::add: tessellates a
 * regular tetrahedron ndiv times on the GPU (4*4^ndiv triangles, vertices
 * deduplicated in first-seen order) and adds the mesh.  ndiv <= 10. */
rt_status rt_scene_add_sphere_mesh(rt_scene scene, float radius, unsigned int ndiv,
                                   unsigned int* mesh_id);

/* Copies a mesh back to the host (Sphere::mesh(), optx/sphere.cxx:21-26).
 * Pass NULL buffers to query the counts only. */
rt_status rt_scene_get_mesh(rt_scene scene, unsigned int mesh_id, rt_float3* vces,
                            unsigned int* nv, rt_uint3* ices, unsigned int* ni);

/* Scene::add(Thing&, gas) + Scene::set (optx/scene.cxx:169-215): an instance
 * of mesh_id with its optics and 3x4 row-major object-to-world transform. */
rt_status rt_scene_add_thing(rt_scene scene, const rt_optics* optics, unsigned int mesh_id,
                             const float transform[12], unsigned int* thing_id);
/* n rt_scene_add_thing calls in one (the loop of RTWO::load,
 * optx/rtwo.cxx:137-244, for callers behind a foreign-function boundary):
 * optics[k], mesh_ids[k] and transforms[12k..12k+11] make thing
 * first_id + k.  All n are checked before any is added. */
rt_status rt_scene_add_things(rt_scene scene, unsigned int n, const rt_optics* optics,
                              const unsigned int* mesh_ids, const float* transforms, unsigned int* first_id);

/* An analytic sphere thing (rtow's Sphere, sphere.h:9-48). */
rt_status rt_scene_add_analytic_sphere(rt_scene scene, rt_float3 center, float radius,
                                       const rt_optics* optics, unsigned int* thing_id);

/* RTWO::load (optx/rtwo.cxx:137-244) / rtow's scene() (rtow.cxx:51-80): the
 * final scene -- ground sphere (r 1000), a grid a,b in [-H,H) of r 0.2
 * spheres with random centre and material, three r 1 spheres.  rng_kind
 * RT_RECIPE_GLIBC reproduces the reference's scene for glibc rand() seeded
 * `seed` (seed 1: 487 spheres); RT_RECIPE_COUNTER draws from a Philox stream.
 * rt_rtow_spheres only lists the spheres (host code, no GPU needed; pass
 * NULL arrays to query the count).  rt_scene_load_rtow adds them as analytic
 * spheres (ndiv = -1) or as instances of one tessellated unit sphere mesh
 * (ndiv >= 0) scaled by the radius and translated to the centre. */
#define RT_RECIPE_GLIBC 0
#define RT_RECIPE_COUNTER 1
rt_status rt_rtow_spheres(int rng_kind, unsigned int seed, int half_extent, unsigned int cap,
                          rt_float3* centers, float* radii, rt_optics* optics, unsigned int* count);
rt_status rt_scene_load_rtow(rt_scene scene, int rng_kind, unsigned int seed, int half_extent,
                             int ndiv, unsigned int* n_things);

/* Scene::set / Scene::get (optx/scene.cxx:198-225); RT_ERR_INVALID_ARG for a
 * bad thing id (the reference returns false).  set takes effect on the next
 * rt_scene_update or rt_scene_build. */
rt_status rt_scene_set_transform(rt_scene scene, unsigned int thing_id, const float transform[12]);
rt_status rt_scene_get_transform(rt_scene scene, unsigned int thing_id, float transform[12]);
/* Replaces a thing's optics (the reference fixes them in the shader binding
 * table, optx/rtwo.cxx:418-447).  Takes effect at the next launch of any
 * geometry holding the scene (its own, or a built batch); no refit. */
rt_status rt_scene_set_optics(rt_scene scene, unsigned int thing_id, const rt_optics* optics);

/* Acceleration-structure layout of the next build.
 *   FLAT: every thing flattened to world-space primitives under one LBVH
 *     over plain Morton codes of the primitive centroids.
 *   GROUPED: the same flat world-space LBVH, but its keys
 *     order the things first (a 60-bit code of each thing's centre, ranked)
 *     and a thing's primitives after (a 30-bit code inside the thing's
 *     bounds), so the hierarchy has the shape of a two-level one -- the
 *     reference's GAS-per-mesh / IAS-over-things split (optx/rtwo.cxx:138-244)
 *     -- at the cost of a flat traversal step.
 *   INSTANCED: the reference's two-level layout itself: one object-space
 *     hierarchy per mesh, a top-level one over instance records, analytic
 *     spheres and the triangles of things that cannot be instanced
 *     (non-diagonal transforms, meshes under 16 triangles), both levels built
 *     like SAH below; memory-lean, more work per step.
 *   SAH (AUTO, the default): the flat world-space hierarchy built top-down
 *     by binned surface-area-heuristic splits (32 bins per axis) down to
 *     clusters of at most 16 primitives, each cluster an LBVH over 30-bit
 *     Morton codes inside its own bounds; fewest node visits per ray (C1: 37
 *     against 46 grouped, 58 flat), build about 4x the LBVH's.
 * Hits, ids and images do not depend on the layout (tested bit for bit). */
typedef enum {
    RT_LAYOUT_AUTO = 0,
    RT_LAYOUT_FLAT = 1,
    RT_LAYOUT_INSTANCED = 2,
    RT_LAYOUT_GROUPED = 3,
    RT_LAYOUT_SAH = 4
} rt_layout;
rt_status rt_scene_set_layout(rt_scene scene, int layout);

/* Scene::build (optx/scene.cxx:227-273, optixAccelBuild): builds the scene's
 * LBVHs in the chosen layout (Morton codes, radix sort, Karras hierarchy,
 * atomic bottom-up refit).  morton_bits 30 or 60 (0 = 60).  Returns after the
 * build has finished on `stream`. */
rt_status rt_scene_build(rt_scene scene, unsigned int morton_bits, void* stream);

/* Scene::update (optx/scene.cxx:275-294, IAS refit): re-flattens the top
 * level with the new transforms and refits its boxes, keeping the topology
 * (object-space bottom levels are untouched); a thing whose transform turned
 * from diagonal to general (or back) triggers a full build instead. */
rt_status rt_scene_update(rt_scene scene, void* stream);

typedef struct {
    unsigned int n_meshes, n_things, n_prims, morton_bits;
    unsigned long long device_bytes;
    float build_ms;   /* last rt_scene_build, CUDA events */
    float refit_ms;   /* last rt_scene_update */
    unsigned int layout;          /* resolved layout: FLAT, GROUPED, SAH or INSTANCED */
    unsigned int n_instances;     /* instanced things */
    unsigned int n_top_records;   /* top-level LBVH leaves */
    unsigned int n_bottom_records;/* bottom-level triangles (all instanced meshes) */
} rt_scene_info;
rt_status rt_scene_info_get(rt_scene scene, rt_scene_info* info);

/* LBVH snapshot for parity tests (the top level; with RT_LAYOUT_FLAT the
 * whole scene): sorted Morton codes (as 64-bit), sorted record ids, Karras
 * children (child >= 0 internal node, < 0 leaf ~child) and per internal node
 * the two child boxes (12 floats: lo0 hi0 lo1 hi1).  Host buffers sized n,
 * n, n-1, n-1, 12*(n-1) with n = n_top_records; any may be NULL. */
rt_status rt_scene_get_lbvh(rt_scene scene, unsigned long long* codes, unsigned int* ids,
                            int* left, int* right, float* boxes);

/* ------------------------------------------------------ progressive render */
/* Progressive rendering with checkpoint and resume (no reference counterpart:
 * every Launcher::ignite renders all spp afresh, optx/camera_i.cu:58).  An
 * accumulator keeps the exact fixed-point pixel sums (colour and rays) of the
 * samples rendered so far, their count and the index of the first.  Sample k of a pixel draws from
 * its own counter-RNG stream, so rendering samples [0, a), then [a, b), ...
 * with one seed gives the sums, and so the image and rays per pixel, of one
 * launch of b samples bit for bit. */
typedef struct rt_accum_s* rt_accum;
rt_status rt_accum_create(rt_accum* out, unsigned int w, unsigned int h);
rt_status rt_accum_destroy(rt_accum acc);
/* Back to zero samples (also the way out of a failed rt_launch_accum). */
rt_status rt_accum_reset(rt_accum acc, void* stream);
rt_status rt_accum_samples(rt_accum acc, unsigned long long* samples);
/* Renders the next params->spp samples of every pixel (sample indices from the
 * accumulator's count on) into the accumulator and writes frame->rawRGB and
 * frame->rpp as the mean, and the sum of rays, over all its samples
 * (stats->rays counts this launch's rays only).
 * params->image_w/h must be the accumulator's size; RT_FLAG_GUIDES is not
 * supported; RT_ERR_LIMIT once samples x depth would reach 2^32.
 * Synchronous like rt_launch. */
rt_status rt_launch_accum(rt_scene scene, const rt_camera* cam, const rt_launch_params* params, rt_accum acc,
                          const rt_frame* frame, void* stream, rt_launch_stats* stats);
/* Checkpoint and resume: the accumulator's state as host bytes (a header with
 * size and sample count, then the sums), and back into an accumulator of the
 * same image size; a render resumed from it continues bit for bit. */
rt_status rt_accum_state_size(rt_accum acc, size_t* bytes);
rt_status rt_accum_save(rt_accum acc, void* host, size_t bytes, void* stream);
rt_status rt_accum_load(rt_accum acc, const void* host, size_t bytes, void* stream);

/* Sample ranges split across processes or GPUs (the one collective of the
 * multi-GPU form of the single optixLaunch at optx/launcher.cxx:60-69: a sum
 * of the accumulation buffers).  Each rank sets its accumulator's first
 * sample index before rendering (rt_accum_set_first_sample, on an empty
 * accumulator: rt_accum_reset clears it to 0) and renders its range;
 * rt_accum_device_sums gives the device arrays of the exact sums (three
 * int64 colour channels in units of 2^-32, and the uint32 rays per pixel,
 * w*h each) for a sum-reduction across the ranks; rt_accum_set_range then
 * declares the samples the reduced sums hold, [first, first + samples), and
 * their total rays, and rt_accum_resolve writes frame->rawRGB (the clamped
 * mean) and frame->rpp from the sums, stream-ordered.  Ranks that tile
 * [0, n) this way give the image and rays per pixel of one n-sample launch
 * bit for bit. */
rt_status rt_accum_set_first_sample(rt_accum acc, unsigned long long first);
rt_status rt_accum_device_sums(rt_accum acc, unsigned long long** red, unsigned long long** green,
                               unsigned long long** blue, unsigned int** rays);
rt_status rt_accum_set_range(rt_accum acc, unsigned long long first, unsigned long long samples,
                             unsigned long long rays);
rt_status rt_accum_resolve(rt_accum acc, const rt_frame* frame, void* stream);

/* -------------------------------------------------------------- tuning */
/* Launch shape of the wavefront (no reference counterpart; OptiX chooses its
 * own): the wave-queue size and the kernels' block shapes.  Process-wide,
 * read by every later launch (rt_launch*, rt_batch_launch, the launcher);
 * the image does not depend on it (tested bit for bit).  A zero field means
 * the built-in default.  rtxplay_gb300/tune.py searches it per workload and
 * keeps the results in a JSON cache. */
typedef struct {
    unsigned int wave_log2;            /* rays per wave queue = 2^wave_log2, 16..26 (default 26, or RTX_WAVE) */
    unsigned int shade_block;          /* threads per shading block: 128, 256, 512 or 1024 (default 512) */
    unsigned int extend_blocks_per_sm; /* persistent traversal blocks per SM, 1..32, capped at what fits
                                          (default: what fits) */
    unsigned int refill_below;         /* a traversal warp takes new rays when at most this many of its
                                          lanes are busy, 1..31 (default 12) */
    unsigned int steps_per_check;      /* traversal steps between those checks, 1..64 (default 16) */
} rt_tuning;

/* Sets the tuning (NULL: all defaults); RT_ERR_INVALID_ARG for a field out
 * of range.  rt_tuning_get returns the tuning in effect, defaults filled in. */
rt_status rt_tuning_set(const rt_tuning* tuning);
rt_status rt_tuning_get(rt_tuning* tuning);

/* -------------------------------------------------------------- render */
/* Launcher::ignite + __raygen__camera / __closesthit__* / __miss__ambient
 * (optx/launcher.cxx:49-77, optx/camera_i.cu:24-141, optx/optics_i.cu:23-288):
 * renders w*h pixels x spp samples with the wavefront path tracer into the
 * caller's device buffers.  Asynchronous on `stream` except for its
 * host-side wave loop. */
rt_status rt_launch(rt_scene scene, const rt_camera* cam, const rt_launch_params* params,
                    const rt_frame* frame, void* stream);
/* Same, filling `stats` (synchronises `stream` before returning). */
rt_status rt_launch_ex(rt_scene scene, const rt_camera* cam, const rt_launch_params* params,
                       const rt_frame* frame, void* stream, rt_launch_stats* stats);

/* Primary-ray closest hit of sample `sample` for every pixel (parity and
 * picking): prim id (global, -1 on a miss), thing id, binary32 distance t
 * and barycentrics u, v of the selection, and t64, the distance to the
 * selected primitive re-evaluated in double precision (NaN on a miss).
 * Device buffers of w*h entries each; any but prim may be NULL. */
rt_status rt_first_hit(rt_scene scene, const rt_camera* cam, const rt_launch_params* params,
                       unsigned int sample, int* prim, int* thing, float* t, float* u, float* v,
                       double* t64, void* stream);

/* Picker: the 1x1 launch of SimpleSM::eaEdtSed (optx/simplesm.cxx:1014-1034,
 * optx/optics_i.cu:25-29): thing id under pixel (x, y), or 0xFFFFFFFF on a
 * miss.  Synchronous. */
rt_status rt_pick(rt_scene scene, const rt_camera* cam, const rt_launch_params* params,
                  unsigned int x, unsigned int y, unsigned int* thing_id, void* stream);

/* ----------------------------------------------------------------- batch */
/* Many independent scenes in one launch (no counterpart in the reference,
 * whose Launcher renders one scene per optixLaunch): every scene keeps its
 * own camera, size, spp, depth, seed and output frame; rt_batch_build builds
 * all their LBVHs in one segmented pass (one Morton sort by (scene, code), a
 * Karras hierarchy per segment, one refit); rt_batch_launch renders all of
 * them with one wavefront whose wave loop runs as a CUDA graph.  Each scene's
 * image equals the one rt_launch renders for it alone.  The scenes must stay
 * alive and unchanged until the batch is destroyed or rebuilt. */
typedef struct rt_batch_s* rt_batch;
rt_status rt_batch_create(rt_batch* out);
rt_status rt_batch_destroy(rt_batch b);
rt_status rt_batch_add(rt_batch b, rt_scene scene, const rt_camera* cam,
                       const rt_launch_params* params, const rt_frame* frame, unsigned int* index);
rt_status rt_batch_set_layout(rt_batch b, int layout);
rt_status rt_batch_build(rt_batch b, unsigned int morton_bits, void* stream);
rt_status rt_batch_launch(rt_batch b, void* stream, rt_launch_stats* stats);
rt_status rt_batch_info(rt_batch b, unsigned int* n_scenes, unsigned int* n_prims, float* build_ms,
                        unsigned long long* device_bytes);

/* Batched adjoint: registers scene `index`'s loss gradient and outputs
 * (device pointers, NULL outputs skipped), then rt_batch_adjoint replays
 * the paths of every registered scene in one launch; the image each scene's
 * gradient is taken at is its frame's rawRGB (the last rt_batch_launch). */
rt_status rt_batch_set_adjoint(rt_batch b, unsigned int index, const rt_float3* grad_image,
                               double* grad_albedo, double* grad_fuzz, double* grad_sky);
rt_status rt_batch_adjoint(rt_batch b, void* stream);

/* One optimisation iteration as one CUDA graph (no reference counterpart):
 * rt_batch_set_albedos, rt_batch_launch, rt_batch_adjoint, rt_l2_loss_grad
 * and rt_adam_step_device may be called on a stream that is being captured
 * (cudaStreamBeginCapture, or a framework's graph capture), after the same
 * calls ran once outside the capture (which sizes the batch's buffers and
 * uploads its job tables and optics).  Inside a capture they enqueue
 * stream-ordered work only: the wave loop becomes a conditional WHILE node
 * of the captured graph, no stats are returned (stats must be NULL), and an
 * error of a captured launch (stack overflow, wave bound) is not returned by
 * the call but kept in the batch's error word.  rt_batch_status synchronises
 * `stream`, returns that error (RT_ERR_LIMIT / RT_ERR_INTERNAL) or RT_OK, and
 * clears the word.  The graph stays valid while the batch and the buffers
 * it was captured with live and the batch is not rebuilt; host-side optics
 * changes (rt_scene_set_optics) need a launch outside the capture. */
rt_status rt_batch_status(rt_batch b, void* stream);

/* Device-side albedos (no reference counterpart): every thing's albedo from
 * a device array of 3 floats per thing (a batch: all scenes' things in the
 * order they were added), on `stream`, without a refit and without touching
 * the host-side optics; a later rt_scene_set_optics of the scene re-uploads
 * every thing's host-side optics. */
rt_status rt_scene_set_albedos(rt_scene scene, const float* albedo, void* stream);
rt_status rt_batch_set_albedos(rt_batch b, const float* albedo, void* stream);

/* Inverse-rendering helpers (device pointers, asynchronous on `stream`):
 * rt_l2_loss_grad writes grad = 2 (clamp(image, 0, 1) - target) for n pixels
 * and adds sum (clamp(image) - target)^2 to *loss (a device double; NULL:
 * not computed).  rt_adam_step is Adam (Kingma and Ba 2015) on n float
 * parameters with a double gradient: m = b1 m + (1 - b1) g, v = b2 v +
 * (1 - b2) g^2, theta -= lr (m / (1 - b1^step)) / (sqrt(v / (1 - b2^step)) +
 * eps), then theta is clamped to [lo, hi]; step counts from 1. */
rt_status rt_l2_loss_grad(const rt_float3* image, const rt_float3* target, rt_float3* grad_image,
                          unsigned int n, double* loss, void* stream);
rt_status rt_adam_step(float* theta, const double* grad, float* m, float* v, unsigned int n, float lr,
                       float beta1, float beta2, float eps, unsigned int step, float lo, float hi,
                       void* stream);
/* The same step with its counter on the device: the step taken is
 * t = *step + 1 (bias corrections from it), after which *step = t.  An
 * iteration captured into a CUDA graph advances with every replay. */
rt_status rt_adam_step_device(float* theta, const double* grad, float* m, float* v, unsigned int n, float lr,
                              float beta1, float beta2, float eps, unsigned int* step, float lo, float hi,
                              void* stream);

/* ------------------------------------------------------------- adjoint */
/* Gradients of an image loss (no counterpart in the reference): given the
 * rendered image `image` of this scene, camera and params (rawRGB of a
 * previous rt_launch) and grad_image = dL/d(clamp(image, 0, 1)), replays
 * every path from its random stream (path replay backpropagation, visibility
 * held fixed) and writes dL/d albedo (n_things x 3, glass entries 0),
 * dL/d fuzz (n_things, non-metal entries 0) and dL/d sky (6: ambient rgb,
 * then the white of the sky gradient).  All pointers are device pointers;
 * outputs are overwritten, any may be NULL.  depth <= 16.  Synchronises
 * `stream` before returning (it reads an error word). */
rt_status rt_adjoint_launch(rt_scene scene, const rt_camera* cam, const rt_launch_params* params,
                            const rt_float3* image, const rt_float3* grad_image, double* grad_albedo,
                            double* grad_fuzz, double* grad_sky, void* stream);

/* ---------------------------------------------------------- post-process */
/* pp_sRGB / pp_none (optx/postproc.cu:49-61; declared at optx/rtwo.cxx:53-54):
 * float3 -> uchar4 through the sRGB curve, or x255 truncation.  Same
 * arguments as the reference plus a stream; device pointers. */
rt_status rt_postproc_srgb(const rt_float3* src, rt_uchar4* dst, int w, int h, void* stream);
rt_status rt_postproc_none(const rt_float3* src, rt_uchar4* dst, int w, int h, void* stream);
/* rtow's gamma-2 writer (rtow.cxx:6-21): int(256*clamp(sqrt(x), 0, .999)). */
rt_status rt_postproc_gamma2(const rt_float3* src, rt_uchar4* dst, int w, int h, void* stream);

/* ------------------------------------------------------------- launcher */
/* class Launcher (optx/launcher.h:17-31, optx/launcher.cxx:24-85): owns the
 * device image buffers of LpGeneral (rawRGB, rpp, normals, albedos, image,
 * pick id) and renders synchronously into them. */
typedef struct rt_launcher_s* rt_launcher;
rt_status rt_launcher_create(rt_launcher* out, unsigned int w, unsigned int h);
rt_status rt_launcher_destroy(rt_launcher l);
rt_status rt_launcher_resize(rt_launcher l, unsigned int w, unsigned int h);
/* Launcher::ignite(stream, once): once != 0 is the 1x1 picker launch at
 * (pick_x, pick_y); otherwise a full render followed by pp_sRGB into the
 * launcher's uchar4 image.  Synchronous, like the reference. */
rt_status rt_launcher_ignite(rt_launcher l, rt_scene scene, const rt_camera* cam,
                             const rt_launch_params* params, void* stream, int once,
                             unsigned int pick_x, unsigned int pick_y, rt_launch_stats* stats);
/* Device pointers of the launcher's buffers (valid until resize/destroy). */
rt_status rt_launcher_frame(rt_launcher l, rt_frame* frame, rt_uchar4** image,
                            unsigned int** pick_id);
/* Copies the launcher's buffers to host memory (any pointer may be NULL):
 * the device-to-host reads of imgtopnm and -S (optx/rtwo.cxx:61-74,578-591). */
rt_status rt_launcher_download(rt_launcher l, rt_float3* rawRGB, unsigned int* rpp,
                               rt_float3* normals, rt_float3* albedos, rt_uchar4* image,
                               unsigned int* pick_id);

/* -------------------------------------------------- device-side helpers */
/* Stable LSD radix sort of (key, value) pairs on the device, in place, with
 * the LBVH builder's kernels (parity hook: bit-exact against a CPU stable
 * sort).  key_bits <= 32 sorts 32-bit keys, otherwise 64-bit keys. */
rt_status rt_radix_sort_pairs(void* keys, unsigned int* vals, unsigned int n,
                              unsigned int key_bits, void* stream);

/* Measurement helper (no reference counterpart): the copy bandwidth, in GB/s
 * of bytes read plus written, of two device buffers of `bytes` each, copied
 * `reps` times inside one launch with loads and stores that bypass L1; with
 * 2 x bytes well inside L2 (e.g. 2 x 16 MiB) this is the L2 bandwidth the
 * traversal's L2 traffic is reported against.  Allocates its buffers;
 * synchronous. */
rt_status rt_measure_copy_bandwidth(size_t bytes, unsigned int reps, double* gbs, void* stream);

/* No counterpart in the reference.  The same stable pair sort for callers
 * that may not allocate device memory while they run (an engine that hands
 * out all device memory from its own pool, or a per-frame loop where a
 * cudaMalloc would synchronise the device): it allocates nothing and sorts
 * out of a fixed 3.1 MiB scratch array that every GPU loading the library
 * holds until the process exits.  n is limited to 262,144 pairs; larger n
 * returns RT_ERR_INVALID_ARG.  Stream-ordered, does not synchronise.  The
 * first call on a device looks up the scratch's device address; make it
 * before any stream capture.  All calls share the scratch, so calls that can
 * overlap on the GPU (other streams, other host threads) race. */
rt_status rt_radix_sort_pairs_noalloc(void* keys, unsigned int* vals, unsigned int n,
                                      unsigned int key_bits, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* RT_API_H */
