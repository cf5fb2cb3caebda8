"""ctypes wrapper of the CPU oracle (``oracle/_build/liboracle.so``).

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()`` and
bench.py's CPU-baseline leg, to check the product against.  The product package
(``rtxplay_gb300``) never imports this module.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
_u64p = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")

OPT_DIFFUSE, OPT_REFLECT, OPT_REFRACT = 0, 1, 2


def build():
    """Compiles liboracle.so with the committed Makefile (a few seconds)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)


class _Camera(ctypes.Structure):
    _fields_ = [("eye", ctypes.c_float * 3), ("u", ctypes.c_float * 3), ("v", ctypes.c_float * 3),
                ("w", ctypes.c_float * 3), ("hvec", ctypes.c_float * 3),
                ("wvec", ctypes.c_float * 3), ("dvec", ctypes.c_float * 3),
                ("aperture", ctypes.c_float), ("rtow_pixels", ctypes.c_int)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        L.orc_philox4x32_10.argtypes = [_u32p, _u32p, _u32p]
        L.orc_u01.argtypes = [ctypes.c_uint32]
        L.orc_u01.restype = ctypes.c_float
        L.orc_glibc_rand.argtypes = [ctypes.c_uint32, ctypes.c_int, _i32p]
        L.orc_scene_rtow.argtypes = [ctypes.c_int, ctypes.c_uint32, ctypes.c_int, ctypes.c_int,
                                     _f32p, _f32p, _i32p, _f32p, _f32p, _f32p]
        L.orc_scene_rtow.restype = ctypes.c_int
        L.orc_tessellate_counts.argtypes = [ctypes.c_uint, ctypes.POINTER(ctypes.c_uint),
                                            ctypes.POINTER(ctypes.c_uint)]
        L.orc_tessellate.argtypes = [ctypes.c_float, ctypes.c_uint, _f32p, _u32p]
        L.orc_tessellate.restype = ctypes.c_int
        L.orc_camera_set.argtypes = [_f32p, _f32p, _f32p, ctypes.c_float, ctypes.c_float,
                                     ctypes.c_float, ctypes.c_float, _f32p]
        L.orc_morton30.argtypes = [_f32p, ctypes.c_uint, _f32p, _f32p, _u32p]
        L.orc_morton60.argtypes = [_f32p, ctypes.c_uint, _f32p, _f32p, _u64p]
        L.orc_stable_sort_pairs.argtypes = [_u32p, _u32p, ctypes.c_uint]
        L.orc_stable_sort_pairs64.argtypes = [_u64p, _u32p, ctypes.c_uint]
        L.orc_karras.argtypes = [_u64p, ctypes.c_uint, _i32p, _i32p]
        L.orc_world_new.restype = ctypes.c_void_p
        L.orc_world_free.argtypes = [ctypes.c_void_p]
        L.orc_world_add_mesh.argtypes = [ctypes.c_void_p, _f32p, ctypes.c_uint, _u32p, ctypes.c_uint]
        L.orc_world_add_mesh.restype = ctypes.c_int
        L.orc_world_add_thing.argtypes = [ctypes.c_void_p, ctypes.c_int, _f32p, ctypes.c_float,
                                          ctypes.c_float, ctypes.c_int, _f32p]
        L.orc_world_add_thing.restype = ctypes.c_int
        L.orc_world_add_sphere.argtypes = [ctypes.c_void_p, ctypes.c_int, _f32p, ctypes.c_float,
                                           ctypes.c_float, _f32p, ctypes.c_float]
        L.orc_world_add_sphere.restype = ctypes.c_int
        L.orc_world_set_transform.argtypes = [ctypes.c_void_p, ctypes.c_int, _f32p]
        L.orc_world_set_transform.restype = ctypes.c_int
        L.orc_world_build.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.orc_world_build.restype = ctypes.c_int
        L.orc_world_build_grouped.argtypes = [ctypes.c_void_p]
        L.orc_world_build_grouped.restype = ctypes.c_int
        L.orc_world_build_sah.argtypes = [ctypes.c_void_p, ctypes.c_uint]
        L.orc_world_build_sah.restype = ctypes.c_int
        L.orc_world_nprims.argtypes = [ctypes.c_void_p]
        L.orc_world_nprims.restype = ctypes.c_uint
        L.orc_world_lbvh.argtypes = [ctypes.c_void_p] + [ctypes.c_void_p] * 7
        L.orc_world_triangles.argtypes = [ctypes.c_void_p, _f32p]
        L.orc_closest.argtypes = [ctypes.c_void_p, ctypes.c_uint, _f32p, _f32p, ctypes.c_int, _i32p, _f32p,
                                  ctypes.c_int]
        L.orc_first_hit.argtypes = [ctypes.c_void_p, ctypes.POINTER(_Camera), ctypes.c_uint,
                                    ctypes.c_uint, ctypes.c_uint32, ctypes.c_uint32,
                                    ctypes.c_uint32, ctypes.c_int, _i32p, _i32p, _f32p, _f32p,
                                    _f32p, ctypes.c_void_p, ctypes.c_int]
        L.orc_render.argtypes = [ctypes.c_void_p, ctypes.POINTER(_Camera), ctypes.c_uint,
                                 ctypes.c_uint, ctypes.c_uint, ctypes.c_uint, ctypes.c_uint32,
                                 ctypes.c_uint32, _f32p, _f32p, ctypes.c_void_p, ctypes.c_uint,
                                 _f32p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                 ctypes.c_int]
        L.orc_render.restype = ctypes.c_uint64
        L.orc_world_nthings.argtypes = [ctypes.c_void_p]
        L.orc_world_nthings.restype = ctypes.c_uint
        L.orc_world_set_optics.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, _f32p, ctypes.c_float,
                                           ctypes.c_float]
        L.orc_world_set_optics.restype = ctypes.c_int
        L.orc_world_get_optics.argtypes = [ctypes.c_void_p, _i32p, _f32p, _f32p, _f32p]
        L.orc_adjoint.argtypes = [ctypes.c_void_p, ctypes.POINTER(_Camera), ctypes.c_uint, ctypes.c_uint,
                                  ctypes.c_uint, ctypes.c_uint, ctypes.c_uint32, ctypes.c_uint32, _f32p, _f32p,
                                  _f32p, _f32p, _f64p, _f64p, _f64p, ctypes.c_int]
        L.orc_fuzz_path_check.argtypes = [ctypes.c_void_p, ctypes.POINTER(_Camera), ctypes.c_uint, ctypes.c_uint,
                                          ctypes.c_uint, ctypes.c_uint, ctypes.c_uint32, ctypes.c_int,
                                          ctypes.c_float, _f32p, _f32p, _f64p]
        L.orc_fuzz_held_delta.argtypes = [ctypes.c_void_p, ctypes.POINTER(_Camera), ctypes.c_uint, ctypes.c_uint,
                                          ctypes.c_uint, ctypes.c_uint, ctypes.c_uint32, ctypes.c_uint32,
                                          ctypes.c_int, ctypes.c_double, _f32p, _f32p, ctypes.c_void_p,
                                          ctypes.c_void_p, _f64p, _f64p, _f64p, ctypes.c_int]
        for name in ("orc_pp_srgb", "orc_pp_none", "orc_pp_gamma2"):
            getattr(L, name).argtypes = [_f32p, _u8p, ctypes.c_int, ctypes.c_int]
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def philox(ctr, key):
    out = np.zeros(4, np.uint32)
    lib().orc_philox4x32_10(np.asarray(ctr, np.uint32), np.asarray(key, np.uint32), out)
    return out


def glibc_rand(seed, n):
    out = np.zeros(n, np.int32)
    lib().orc_glibc_rand(seed, n, out)
    return out


def scene_rtow(rng_kind=0, seed=1, half_extent=11):
    cap = 4 * half_extent * half_extent + 8
    c = np.zeros((cap, 3), np.float32)
    r = np.zeros(cap, np.float32)
    t = np.zeros(cap, np.int32)
    a = np.zeros((cap, 3), np.float32)
    f = np.zeros(cap, np.float32)
    ix = np.zeros(cap, np.float32)
    n = lib().orc_scene_rtow(rng_kind, seed, half_extent, cap, c, r, t, a, f, ix)
    assert n >= 0
    return dict(centers=c[:n], radii=r[:n], types=t[:n], albedos=a[:n], fuzz=f[:n], index=ix[:n])


def tessellate(radius, ndiv):
    nv, ni = ctypes.c_uint(), ctypes.c_uint()
    lib().orc_tessellate_counts(ndiv, ctypes.byref(nv), ctypes.byref(ni))
    v = np.zeros((ni.value * 3, 3), np.float32)   # room for every vertex instance
    i = np.zeros((ni.value, 3), np.uint32)
    n = lib().orc_tessellate(radius, ndiv, v, i)
    return v[:n].copy(), i


def camera_set(eye, pat, vup, fov, aspratio, aperture, fostance):
    out = np.zeros(18, np.float32)
    lib().orc_camera_set(np.asarray(eye, np.float32), np.asarray(pat, np.float32),
                         np.asarray(vup, np.float32), fov, aspratio, aperture, fostance, out)
    cam = _Camera()
    cam.eye[:] = list(np.asarray(eye, np.float32))
    for k, name in enumerate(("u", "v", "w", "hvec", "wvec", "dvec")):
        getattr(cam, name)[:] = list(out[3 * k:3 * k + 3])
    cam.aperture = aperture
    return cam


def rtow_camera(w, h):
    """The final-scene camera of optx/rtwo.cxx:100-108."""
    return camera_set((13, 2, 3), (0, 0, 0), (0, 1, 0), 20.0, np.float32(w) / np.float32(h),
                      0.1, 10.0)


def morton30(centroids, lo, hi):
    c = np.ascontiguousarray(centroids, np.float32)
    out = np.zeros(len(c), np.uint32)
    lib().orc_morton30(c, len(c), np.asarray(lo, np.float32), np.asarray(hi, np.float32), out)
    return out


def morton60(centroids, lo, hi):
    c = np.ascontiguousarray(centroids, np.float32)
    out = np.zeros(len(c), np.uint64)
    lib().orc_morton60(c, len(c), np.asarray(lo, np.float32), np.asarray(hi, np.float32), out)
    return out


def stable_sort_pairs(keys, vals):
    if np.asarray(keys).dtype == np.uint64:
        k = np.array(keys, np.uint64)
        v = np.array(vals, np.uint32)
        lib().orc_stable_sort_pairs64(k, v, len(k))
        return k, v
    k = np.array(keys, np.uint32)
    v = np.array(vals, np.uint32)
    lib().orc_stable_sort_pairs(k, v, len(k))
    return k, v


def karras(sorted_codes):
    c = np.ascontiguousarray(sorted_codes, np.uint64)
    n = len(c)
    left = np.zeros(max(n - 1, 0), np.int32)
    right = np.zeros(max(n - 1, 0), np.int32)
    lib().orc_karras(c, n, left, right)
    return left, right


class World:
    """Oracle twin of a scene: things over meshes or analytic spheres."""

    def __init__(self):
        self._w = lib().orc_world_new()

    def __del__(self):
        if getattr(self, "_w", None) and _lib is not None:
            _lib.orc_world_free(self._w)
            self._w = None

    def add_mesh(self, vces, ices):
        v = np.ascontiguousarray(vces, np.float32)
        i = np.ascontiguousarray(ices, np.uint32)
        m = lib().orc_world_add_mesh(self._w, v, len(v), i, len(i))
        assert m >= 0
        return m

    def add_thing(self, otype, albedo, fuzz, index, mesh, transform):
        return lib().orc_world_add_thing(self._w, otype, np.asarray(albedo, np.float32), fuzz,
                                         index, mesh, np.asarray(transform, np.float32))

    def add_sphere(self, otype, albedo, fuzz, index, center, radius):
        return lib().orc_world_add_sphere(self._w, otype, np.asarray(albedo, np.float32), fuzz,
                                          index, np.asarray(center, np.float32), radius)

    def set_transform(self, thing, transform):
        return lib().orc_world_set_transform(self._w, thing, np.asarray(transform, np.float32))

    def build(self, morton_bits=60, grouped=False, sah_cluster=0):
        """Flat LBVH (30/60-bit Morton), things-grouped keys, or (sah_cluster > 0)
        the binned-SAH hierarchy with clusters of at most sah_cluster records."""
        if sah_cluster:
            assert lib().orc_world_build_sah(self._w, sah_cluster) == 0
        elif grouped:
            assert lib().orc_world_build_grouped(self._w) == 0
        else:
            assert lib().orc_world_build(self._w, morton_bits) == 0

    @property
    def nprims(self):
        return lib().orc_world_nprims(self._w)

    def lbvh(self):
        n = self.nprims
        codes = np.zeros(n, np.uint64)
        ids = np.zeros(n, np.uint32)
        left = np.zeros(max(n - 1, 0), np.int32)
        right = np.zeros(max(n - 1, 0), np.int32)
        boxes = np.zeros((max(n - 1, 0), 12), np.float32)
        clo = np.zeros(3, np.float32)
        chi = np.zeros(3, np.float32)
        lib().orc_world_lbvh(self._w, _ptr(codes), _ptr(ids), _ptr(left), _ptr(right),
                             _ptr(boxes), _ptr(clo), _ptr(chi))
        return dict(codes=codes, ids=ids, left=left, right=right, boxes=boxes, clo=clo, chi=chi)

    def triangles(self):
        t = np.zeros((self.nprims, 9), np.float32)
        lib().orc_world_triangles(self._w, t)
        return t

    def closest(self, o, d, mode, nthreads=0):
        """Closest hits of rays o + t d (n x 3 arrays): mode "brute" (all
        primitives), "bvh" (the hierarchy) or "boxed" (brute force over the
        primitives whose own box passes the slab test).  Returns (prim, t),
        prim -1 on a miss."""
        o = np.ascontiguousarray(o, np.float32)
        d = np.ascontiguousarray(d, np.float32)
        n = len(o)
        prim = np.zeros(n, np.int32)
        t = np.zeros(n, np.float32)
        lib().orc_closest(self._w, n, o, d, {"brute": 0, "bvh": 1, "boxed": 2}[mode], prim, t, nthreads)
        return prim, t

    def first_hit(self, cam, w, h, seed, scene=0, sample=0, use_bvh=True, fp64=False,
                  nthreads=0):
        n = w * h
        prim = np.zeros(n, np.int32)
        thing = np.zeros(n, np.int32)
        t = np.zeros(n, np.float32)
        u = np.zeros(n, np.float32)
        v = np.zeros(n, np.float32)
        t64 = np.zeros(n, np.float64) if fp64 else None
        lib().orc_first_hit(self._w, ctypes.byref(cam), w, h, seed, scene, sample,
                            1 if use_bvh else 0, prim, thing, t, u, v, _ptr(t64), nthreads)
        out = dict(prim=prim, thing=thing, t=t, u=u, v=v)
        if fp64:
            out["t64"] = t64
        return out

    @property
    def nthings(self):
        return lib().orc_world_nthings(self._w)

    def optics(self):
        n = self.nthings
        t = np.zeros(n, np.int32)
        a = np.zeros((n, 3), np.float32)
        f = np.zeros(n, np.float32)
        ix = np.zeros(n, np.float32)
        lib().orc_world_get_optics(self._w, t, a, f, ix)
        return dict(types=t, albedos=a, fuzz=f, index=ix)

    def fuzz_path_check(self, cam, w, h, spp, depth, seed, thing, step=1e-3, ambient=(0.5, 0.7, 1.0),
                        white=(1.0, 1.0, 1.0)):
        out = np.zeros(7, np.float64)
        lib().orc_fuzz_path_check(self._w, ctypes.byref(cam), w, h, spp, depth, seed, thing, step,
                                  np.asarray(ambient, np.float32), np.asarray(white, np.float32), out)
        return dict(compared=int(out[0]), skipped=int(out[1]), max_rel=out[2], sum_abs_fd=out[3],
                    outliers=int(out[4]), sum_adj=out[5], sum_fd=out[6])

    def fuzz_held_delta(self, cam, w, h, spp, depth, seed, thing, step=1e-6, ambient=(0.5, 0.7, 1.0),
                        white=(1.0, 1.0, 1.0), image=None, grad_image=None, scene=0, nthreads=0):
        """Per-pixel change of the image (w*h, 3; doubles) when metal `thing`'s
        fuzz moves by +step and -step with every path's visibility held fixed
        (double-precision replay), counts (replayed, degenerate, paths a plain
        re-render sees jump) and, given image and grad_image, the adjoint's
        fuzz gradient over the replayed paths on their replayed trajectories."""
        dp = np.zeros((w * h, 3), np.float64)
        dm = np.zeros((w * h, 3), np.float64)
        out = np.zeros(4, np.float64)
        im = None if image is None else np.ascontiguousarray(image, np.float32).reshape(-1)
        gi = None if grad_image is None else np.ascontiguousarray(grad_image, np.float32).reshape(-1)
        lib().orc_fuzz_held_delta(self._w, ctypes.byref(cam), w, h, spp, depth, seed, scene, thing, step,
                                  np.asarray(ambient, np.float32), np.asarray(white, np.float32),
                                  _ptr(im), _ptr(gi), dp, dm, out, nthreads)
        return dict(plus=dp, minus=dm, replayed=int(out[0]), degenerate=int(out[1]), changed=int(out[2]),
                    adjoint=float(out[3]))

    def set_optics(self, thing, otype, albedo, fuzz, index):
        assert lib().orc_world_set_optics(self._w, thing, otype, np.asarray(albedo, np.float32), fuzz,
                                          index) == 0

    def adjoint(self, cam, w, h, spp, depth, seed, image, grad_image, scene=0, ambient=(0.5, 0.7, 1.0),
                white=(1.0, 1.0, 1.0), nthreads=0):
        n = self.nthings
        ga = np.zeros((n, 3), np.float64)
        gf = np.zeros(n, np.float64)
        gs = np.zeros(6, np.float64)
        lib().orc_adjoint(self._w, ctypes.byref(cam), w, h, spp, depth, seed, scene,
                          np.asarray(ambient, np.float32), np.asarray(white, np.float32),
                          np.ascontiguousarray(image, np.float32).reshape(-1),
                          np.ascontiguousarray(grad_image, np.float32).reshape(-1), ga, gf, gs, nthreads)
        return dict(albedo=ga, fuzz=gf, sky=gs)

    def render(self, cam, w, h, spp, depth, seed, scene=0, ambient=(0.5, 0.7, 1.0),
               white=(1.0, 1.0, 1.0), pixels=None, guides=True, nthreads=0):
        px = None if pixels is None else np.ascontiguousarray(pixels, np.uint32)
        n = w * h if px is None else len(px)
        raw = np.zeros((n, 3), np.float32)
        rpp = np.zeros(n, np.uint32)
        nrm = np.zeros((n, 3), np.float32) if guides else None
        alb = np.zeros((n, 3), np.float32) if guides else None
        rays = lib().orc_render(self._w, ctypes.byref(cam), w, h, spp, depth, seed, scene,
                                np.asarray(ambient, np.float32), np.asarray(white, np.float32),
                                _ptr(px), 0 if px is None else len(px), raw, _ptr(rpp),
                                _ptr(nrm), _ptr(alb), nthreads)
        return dict(rawRGB=raw, rpp=rpp, normals=nrm, albedos=alb, rays=int(rays))


def pp(kind, raw, w, h):
    src = np.ascontiguousarray(raw, np.float32).reshape(-1)
    dst = np.zeros(w * h * 4, np.uint8)
    getattr(lib(), f"orc_pp_{kind}")(src, dst, w, h)
    return dst.reshape(h * w, 4)


def rtow_world(level=None, rng_kind=0, seed=1, half_extent=11, morton_bits=60, grouped=False, sah_cluster=0):
    """The final scene as analytic spheres (level None) or as spheres
    tessellated at `level` and instanced by their 3x4 transform."""
    sc = scene_rtow(rng_kind, seed, half_extent)
    w = World()
    mesh = None
    if level is not None:
        v, i = tessellate(1.0, level)
        mesh = w.add_mesh(v, i)
    for c, r, t, a, f, ix in zip(sc["centers"], sc["radii"], sc["types"], sc["albedos"],
                                 sc["fuzz"], sc["index"]):
        if mesh is None:
            w.add_sphere(int(t), a, float(f), float(ix), c, float(r))
        else:
            T = np.array([r, 0, 0, c[0], 0, r, 0, c[1], 0, 0, r, c[2]], np.float32)
            w.add_thing(int(t), a, float(f), float(ix), mesh, T)
    w.build(morton_bits, grouped, sah_cluster)
    return w, sc
