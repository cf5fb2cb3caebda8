"""rtxplay_gb300 -- GB300-native path tracer behind RTXplay's render API.

The product is the native library ``_build/librtxplay_gb300.so`` (CUDA
kernels for sm_103a + the C ABI declared in ``include/rt_api.h``).  This module
binds that ABI with ctypes; it never falls back to Python or CPU code.  If the
library is missing, :func:`lib` raises -- build it with
``python -c "import __graft_entry__ as g; g.build()"``.
"""
import ctypes
import os

import numpy as np

from . import _build

# RTX_LIB: another build of the same library (the bounds-checked variant of
# _build.build_checked()); never a non-native fallback
LIB_PATH = os.environ.get("RTX_LIB") or _build.LIB

RT_OK = 0
RT_ERR_INVALID_ARG = 1
RT_ERR_CUDA = 2
RT_ERR_OUT_OF_MEMORY = 3
RT_ERR_NOT_BUILT = 4
RT_ERR_LIMIT = 5
RT_ERR_INTERNAL = 6

RT_OPTICS_DIFFUSE, RT_OPTICS_REFLECT, RT_OPTICS_REFRACT = 0, 1, 2
RT_FLAG_GUIDES, RT_FLAG_STAGE_TIMING, RT_FLAG_COUNT_VISITS, RT_FLAG_RTOW_PIXELS = 0x1, 0x2, 0x4, 0x8
RT_RECIPE_GLIBC, RT_RECIPE_COUNTER = 0, 1
RT_LAYOUT_AUTO, RT_LAYOUT_FLAT, RT_LAYOUT_INSTANCED, RT_LAYOUT_GROUPED, RT_LAYOUT_SAH = 0, 1, 2, 3, 4


class RTError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"rt status {status}: {msg}")
        self.status = status


class float3(ctypes.Structure):
    _fields_ = [("x", ctypes.c_float), ("y", ctypes.c_float), ("z", ctypes.c_float)]


class uint3(ctypes.Structure):
    _fields_ = [("x", ctypes.c_uint), ("y", ctypes.c_uint), ("z", ctypes.c_uint)]


class Optics(ctypes.Structure):
    """rt_optics: flattened Optics union (optx/thing.h:17-52)."""
    _fields_ = [("type", ctypes.c_int), ("albedo", float3), ("fuzz", ctypes.c_float),
                ("index", ctypes.c_float)]


class Camera(ctypes.Structure):
    """rt_camera: class Camera state (optx/camera.h:28-94)."""
    _fields_ = [("eye", float3), ("pat", float3), ("vup", float3), ("fov", ctypes.c_float),
                ("aspratio", ctypes.c_float), ("aperture", ctypes.c_float),
                ("fostance", ctypes.c_float), ("u", float3), ("v", float3), ("w", float3),
                ("hvec", float3), ("wvec", float3), ("dvec", float3)]


class LaunchParams(ctypes.Structure):
    _fields_ = [("image_w", ctypes.c_uint), ("image_h", ctypes.c_uint), ("spp", ctypes.c_uint),
                ("depth", ctypes.c_uint), ("seed", ctypes.c_uint), ("flags", ctypes.c_uint),
                ("ambient", float3), ("white", float3)]


class Frame(ctypes.Structure):
    _fields_ = [("rawRGB", ctypes.c_void_p), ("rpp", ctypes.c_void_p),
                ("normals", ctypes.c_void_p), ("albedos", ctypes.c_void_p)]


class LaunchStats(ctypes.Structure):
    _fields_ = [("rays", ctypes.c_ulonglong), ("paths", ctypes.c_ulonglong),
                ("node_visits", ctypes.c_ulonglong), ("prim_tests", ctypes.c_ulonglong),
                ("waves", ctypes.c_uint), ("kernel_launches", ctypes.c_uint),
                ("extend_ms", ctypes.c_float), ("shade_ms", ctypes.c_float),
                ("extend_launches", ctypes.c_uint), ("wave_capacity", ctypes.c_uint)]


class SceneInfo(ctypes.Structure):
    _fields_ = [("n_meshes", ctypes.c_uint), ("n_things", ctypes.c_uint), ("n_prims", ctypes.c_uint),
                ("morton_bits", ctypes.c_uint), ("device_bytes", ctypes.c_ulonglong),
                ("build_ms", ctypes.c_float), ("refit_ms", ctypes.c_float), ("layout", ctypes.c_uint),
                ("n_instances", ctypes.c_uint), ("n_top_records", ctypes.c_uint), ("n_bottom_records", ctypes.c_uint)]


class Tuning(ctypes.Structure):
    _fields_ = [("wave_log2", ctypes.c_uint), ("shade_block", ctypes.c_uint), ("extend_blocks_per_sm", ctypes.c_uint),
                ("refill_below", ctypes.c_uint), ("steps_per_check", ctypes.c_uint)]


TUNING_FIELDS = tuple(f[0] for f in Tuning._fields_)

_P = ctypes.c_void_p
_U = ctypes.c_uint
_I = ctypes.c_int
_F = ctypes.c_float
_PU = ctypes.POINTER(ctypes.c_uint)

# name -> argtypes (every function returns rt_status)
SIGNATURES = {
    "rt_camera_set": [ctypes.POINTER(Camera), float3, float3, float3, _F, _F, _F, _F],
    "rt_scene_create": [ctypes.POINTER(_P)],
    "rt_scene_destroy": [_P],
    "rt_scene_add_mesh": [_P, _P, _U, _P, _U, _PU],
    "rt_scene_add_sphere_mesh": [_P, _F, _U, _PU],
    "rt_scene_add_obj": [_P, ctypes.c_char_p, _PU, _U, _PU],
    "rt_obj_parse": [ctypes.c_char_p, _U, _P, _PU, _P, _PU, _PU],
    "rt_scene_get_mesh": [_P, _U, _P, _PU, _P, _PU],
    "rt_scene_add_thing": [_P, ctypes.POINTER(Optics), _U, _P, _PU],
    "rt_scene_add_things": [_P, _U, _P, _P, _P, _PU],
    "rt_scene_add_analytic_sphere": [_P, float3, _F, ctypes.POINTER(Optics), _PU],
    "rt_rtow_spheres": [_I, _U, _I, _U, _P, _P, _P, _PU],
    "rt_scene_load_rtow": [_P, _I, _U, _I, _I, _PU],
    "rt_scene_set_transform": [_P, _U, _P],
    "rt_scene_get_transform": [_P, _U, _P],
    "rt_scene_set_optics": [_P, _U, ctypes.POINTER(Optics)],
    "rt_scene_set_layout": [_P, _I],
    "rt_scene_build": [_P, _U, _P],
    "rt_scene_update": [_P, _P],
    "rt_scene_info_get": [_P, ctypes.POINTER(SceneInfo)],
    "rt_scene_get_lbvh": [_P, _P, _P, _P, _P, _P],
    "rt_launch": [_P, ctypes.POINTER(Camera), ctypes.POINTER(LaunchParams), ctypes.POINTER(Frame), _P],
    "rt_launch_ex": [_P, ctypes.POINTER(Camera), ctypes.POINTER(LaunchParams), ctypes.POINTER(Frame), _P,
                     ctypes.POINTER(LaunchStats)],
    "rt_first_hit": [_P, ctypes.POINTER(Camera), ctypes.POINTER(LaunchParams), _U, _P, _P, _P, _P, _P, _P, _P],
    "rt_pick": [_P, ctypes.POINTER(Camera), ctypes.POINTER(LaunchParams), _U, _U, _PU, _P],
    "rt_postproc_srgb": [_P, _P, _I, _I, _P],
    "rt_postproc_none": [_P, _P, _I, _I, _P],
    "rt_postproc_gamma2": [_P, _P, _I, _I, _P],
    "rt_launcher_create": [ctypes.POINTER(_P), _U, _U],
    "rt_launcher_destroy": [_P],
    "rt_launcher_resize": [_P, _U, _U],
    "rt_launcher_ignite": [_P, _P, ctypes.POINTER(Camera), ctypes.POINTER(LaunchParams), _P, _I, _U, _U,
                           ctypes.POINTER(LaunchStats)],
    "rt_launcher_frame": [_P, ctypes.POINTER(Frame), ctypes.POINTER(_P), ctypes.POINTER(_P)],
    "rt_launcher_download": [_P, _P, _P, _P, _P, _P, _P],
    "rt_radix_sort_pairs": [_P, _P, _U, _U, _P],
    "rt_radix_sort_pairs_noalloc": [_P, _P, _U, _U, _P],
    "rt_batch_create": [ctypes.POINTER(_P)],
    "rt_batch_destroy": [_P],
    "rt_batch_add": [_P, _P, ctypes.POINTER(Camera), ctypes.POINTER(LaunchParams), ctypes.POINTER(Frame), _PU],
    "rt_batch_set_layout": [_P, _I],
    "rt_batch_build": [_P, _U, _P],
    "rt_batch_launch": [_P, _P, ctypes.POINTER(LaunchStats)],
    "rt_batch_info": [_P, _PU, _PU, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_ulonglong)],
    "rt_batch_set_adjoint": [_P, _U, _P, _P, _P, _P],
    "rt_batch_adjoint": [_P, _P],
    "rt_adjoint_launch": [_P, ctypes.POINTER(Camera), ctypes.POINTER(LaunchParams), _P, _P, _P, _P, _P, _P],
    "rt_scene_set_albedos": [_P, _P, _P],
    "rt_batch_set_albedos": [_P, _P, _P],
    "rt_l2_loss_grad": [_P, _P, _P, _U, _P, _P],
    "rt_adam_step": [_P, _P, _P, _P, _U, _F, _F, _F, _F, _U, _F, _F, _P],
    "rt_adam_step_device": [_P, _P, _P, _P, _U, _F, _F, _F, _F, _P, _F, _F, _P],
    "rt_accum_create": [ctypes.POINTER(_P), _U, _U],
    "rt_accum_destroy": [_P],
    "rt_accum_reset": [_P, _P],
    "rt_accum_samples": [_P, ctypes.POINTER(ctypes.c_ulonglong)],
    "rt_launch_accum": [_P, ctypes.POINTER(Camera), ctypes.POINTER(LaunchParams), _P, ctypes.POINTER(Frame), _P,
                        ctypes.POINTER(LaunchStats)],
    "rt_accum_state_size": [_P, ctypes.POINTER(ctypes.c_size_t)],
    "rt_accum_save": [_P, _P, ctypes.c_size_t, _P],
    "rt_accum_load": [_P, _P, ctypes.c_size_t, _P],
    "rt_measure_copy_bandwidth": [ctypes.c_size_t, _U, ctypes.POINTER(ctypes.c_double), _P],
    "rt_accum_set_first_sample": [_P, ctypes.c_ulonglong],
    "rt_batch_status": [_P, _P],
    "rt_accum_device_sums": [_P, ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_void_p),
                             ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_void_p)],
    "rt_accum_set_range": [_P, ctypes.c_ulonglong, ctypes.c_ulonglong, ctypes.c_ulonglong],
    "rt_accum_resolve": [_P, _P, _P],
    "rt_tuning_set": [ctypes.POINTER(Tuning)],
    "rt_debug_fail_alloc": [_U],
    "rt_tuning_get": [ctypes.POINTER(Tuning)],
}

_lib = None


def lib():
    """Loads librtxplay_gb300.so; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build it with __graft_entry__.build()")
        L = ctypes.CDLL(LIB_PATH)
        for name, args in SIGNATURES.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = ctypes.c_int
        L.rt_last_error_string.restype = ctypes.c_char_p
        L.rt_last_error_string.argtypes = []
        L.rt_version.restype = ctypes.c_char_p
        L.rt_version.argtypes = []
        _lib = L
    return _lib


def check(status):
    if status != RT_OK:
        raise RTError(status, lib().rt_last_error_string().decode())
    return status


def f3(v):
    return float3(float(v[0]), float(v[1]), float(v[2]))


def _ptr(a):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


def camera_set(eye, pat, vup, fov, aspratio, aperture, fostance):
    cam = Camera()
    check(lib().rt_camera_set(ctypes.byref(cam), f3(eye), f3(pat), f3(vup), fov, aspratio, aperture,
                              fostance))
    return cam


def rtow_camera(w, h):
    """The final-scene camera of optx/rtwo.cxx:100-108 (aspect = w/h in binary32)."""
    return camera_set((13, 2, 3), (0, 0, 0), (0, 1, 0), 20.0,
                      float(np.float32(w) / np.float32(h)), 0.1, 10.0)


def launch_params(w, h, spp, depth=50, seed=4711, flags=0, ambient=(0.5, 0.7, 1.0),
                  white=(1.0, 1.0, 1.0)):
    return LaunchParams(w, h, spp, depth, seed, flags, f3(ambient), f3(white))


def optics(otype, albedo=(0, 0, 0), fuzz=0.0, index=0.0):
    return Optics(int(otype), f3(albedo), float(fuzz), float(index))


def obj_parse(path):
    """Host-side OBJ parse: a list of (vertices [n, 3] float32, triangles [m, 3] uint32) per shape."""
    n = ctypes.c_uint()
    check(lib().rt_obj_parse(path.encode(), 0, None, None, None, None, ctypes.byref(n)))
    out = []
    for k in range(n.value):
        nv, ni = ctypes.c_uint(), ctypes.c_uint()
        check(lib().rt_obj_parse(path.encode(), k, None, ctypes.byref(nv), None, ctypes.byref(ni), None))
        v = np.zeros((nv.value, 3), np.float32)
        i = np.zeros((ni.value, 3), np.uint32)
        check(lib().rt_obj_parse(path.encode(), k, _ptr(v), ctypes.byref(nv), _ptr(i), ctypes.byref(ni), None))
        out.append((v, i))
    return out


def rtow_spheres(rng_kind=RT_RECIPE_GLIBC, seed=1, half_extent=11):
    """The final-scene sphere list (host code, no GPU needed)."""
    n = ctypes.c_uint()
    check(lib().rt_rtow_spheres(rng_kind, seed, half_extent, 0, None, None, None, ctypes.byref(n)))
    c = np.zeros((n.value, 3), np.float32)
    r = np.zeros(n.value, np.float32)
    o = (Optics * n.value)()
    check(lib().rt_rtow_spheres(rng_kind, seed, half_extent, n.value, _ptr(c), _ptr(r),
                                ctypes.cast(o, ctypes.c_void_p), ctypes.byref(n)))
    types = np.array([x.type for x in o], np.int32)
    alb = np.array([[x.albedo.x, x.albedo.y, x.albedo.z] for x in o], np.float32).reshape(-1, 3)
    fuzz = np.array([x.fuzz for x in o], np.float32)
    index = np.array([x.index for x in o], np.float32)
    return dict(centers=c, radii=r, types=types, albedos=alb, fuzz=fuzz, index=index)


def free_spare_scene_arrays():
    """Frees the hierarchy arrays a destroyed scene left for the next scene
    this thread builds (rt_scene_destroy(NULL))."""
    check(lib().rt_scene_destroy(None))


class Scene:
    """Owns an rt_scene handle (the reference's class Scene, optx/scene.h:19-63)."""

    def __init__(self):
        self.h = ctypes.c_void_p()
        check(lib().rt_scene_create(ctypes.byref(self.h)))

    def close(self):
        if self.h:
            lib().rt_scene_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_mesh(self, vces, ices):
        v = np.ascontiguousarray(vces, np.float32)
        i = np.ascontiguousarray(ices, np.uint32)
        mid = ctypes.c_uint()
        check(lib().rt_scene_add_mesh(self.h, _ptr(v), len(v), _ptr(i), len(i), ctypes.byref(mid)))
        return mid.value

    def add_obj(self, path):
        """Object(file): every shape of a Wavefront OBJ file as a mesh; returns the mesh ids."""
        n = ctypes.c_uint()
        check(lib().rt_obj_parse(path.encode(), 0, None, None, None, None, ctypes.byref(n)))
        ids = (ctypes.c_uint * max(1, n.value))()
        got = ctypes.c_uint()
        check(lib().rt_scene_add_obj(self.h, path.encode(), ids, n.value, ctypes.byref(got)))
        return [ids[k] for k in range(got.value)]

    def add_sphere_mesh(self, radius, ndiv):
        mid = ctypes.c_uint()
        check(lib().rt_scene_add_sphere_mesh(self.h, radius, ndiv, ctypes.byref(mid)))
        return mid.value

    def get_mesh(self, mesh_id):
        nv, ni = ctypes.c_uint(), ctypes.c_uint()
        check(lib().rt_scene_get_mesh(self.h, mesh_id, None, ctypes.byref(nv), None, ctypes.byref(ni)))
        v = np.zeros((nv.value, 3), np.float32)
        i = np.zeros((ni.value, 3), np.uint32)
        check(lib().rt_scene_get_mesh(self.h, mesh_id, _ptr(v), ctypes.byref(nv), _ptr(i), ctypes.byref(ni)))
        return v, i

    def add_thing(self, opt, mesh_id, transform):
        t = np.ascontiguousarray(transform, np.float32)
        tid = ctypes.c_uint()
        check(lib().rt_scene_add_thing(self.h, ctypes.byref(opt), mesh_id, _ptr(t), ctypes.byref(tid)))
        return tid.value

    def add_things(self, optics, mesh_ids, transforms):
        """rt_scene_add_things: optics a sequence of Optics (or an Optics array), mesh_ids n ints,
        transforms n x 12 floats; returns the new thing ids."""
        n = len(mesh_ids)
        opt = optics if isinstance(optics, ctypes.Array) else (Optics * max(1, n))(*optics)
        ids = np.ascontiguousarray(mesh_ids, np.uint32)
        T = np.ascontiguousarray(transforms, np.float32).reshape(n, 12) if n else np.zeros((1, 12), np.float32)
        if len(opt) < n or ids.shape != (n,):
            raise ValueError("optics, mesh_ids and transforms need n entries each")
        first = ctypes.c_uint()
        check(lib().rt_scene_add_things(self.h, n, ctypes.cast(opt, ctypes.c_void_p), _ptr(ids), _ptr(T),
                                        ctypes.byref(first)))
        return list(range(first.value, first.value + n))

    def add_analytic_sphere(self, center, radius, opt):
        tid = ctypes.c_uint()
        check(lib().rt_scene_add_analytic_sphere(self.h, f3(center), radius, ctypes.byref(opt),
                                                 ctypes.byref(tid)))
        return tid.value

    def load_rtow(self, rng_kind=RT_RECIPE_GLIBC, seed=1, half_extent=11, ndiv=6):
        n = ctypes.c_uint()
        check(lib().rt_scene_load_rtow(self.h, rng_kind, seed, half_extent, ndiv, ctypes.byref(n)))
        return n.value

    def set_transform(self, thing, transform):
        t = np.ascontiguousarray(transform, np.float32)
        return lib().rt_scene_set_transform(self.h, thing, _ptr(t))

    def get_transform(self, thing):
        t = np.zeros(12, np.float32)
        st = lib().rt_scene_get_transform(self.h, thing, _ptr(t))
        return st, t

    def set_optics(self, thing, opt):
        return lib().rt_scene_set_optics(self.h, thing, ctypes.byref(opt))

    def set_layout(self, layout):
        check(lib().rt_scene_set_layout(self.h, layout))

    def build(self, morton_bits=60, stream=None, layout=None):
        if layout is not None:
            self.set_layout(layout)
        check(lib().rt_scene_build(self.h, morton_bits, stream))

    def set_albedos(self, albedo, stream=None):
        """rt_scene_set_albedos from a device pointer (3 floats per thing)."""
        check(lib().rt_scene_set_albedos(self.h, albedo, stream))

    def adjoint(self, cam, params, image, grad_image, grad_albedo, grad_fuzz, grad_sky, stream=None):
        """rt_adjoint_launch; every buffer argument is a device pointer (int) or None."""
        check(lib().rt_adjoint_launch(self.h, ctypes.byref(cam), ctypes.byref(params), image, grad_image,
                                      grad_albedo, grad_fuzz, grad_sky, stream))

    def update(self, stream=None):
        check(lib().rt_scene_update(self.h, stream))

    def info(self):
        inf = SceneInfo()
        check(lib().rt_scene_info_get(self.h, ctypes.byref(inf)))
        return inf

    def lbvh(self):
        """Top-level LBVH snapshot (the whole scene with RT_LAYOUT_FLAT)."""
        n = self.info().n_top_records
        codes = np.zeros(n, np.uint64)
        ids = np.zeros(n, np.uint32)
        left = np.zeros(max(n - 1, 0), np.int32)
        right = np.zeros(max(n - 1, 0), np.int32)
        boxes = np.zeros((max(n - 1, 0), 12), np.float32)
        check(lib().rt_scene_get_lbvh(self.h, _ptr(codes), _ptr(ids), _ptr(left), _ptr(right), _ptr(boxes)))
        return dict(codes=codes, ids=ids, left=left, right=right, boxes=boxes)


class Launcher:
    """Owns an rt_launcher (class Launcher, optx/launcher.h:17-31): device image buffers."""

    def __init__(self, w, h):
        self.h = ctypes.c_void_p()
        self.w, self.hgt = w, h
        check(lib().rt_launcher_create(ctypes.byref(self.h), w, h))

    def close(self):
        if self.h:
            lib().rt_launcher_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def ignite(self, scene, cam, params, once=False, pick=(0, 0), stream=None):
        stats = LaunchStats()
        check(lib().rt_launcher_ignite(self.h, scene.h, ctypes.byref(cam), ctypes.byref(params), stream,
                                       1 if once else 0, pick[0], pick[1], ctypes.byref(stats)))
        return stats

    def download(self, guides=False):
        n = self.w * self.hgt
        raw = np.zeros((n, 3), np.float32)
        rpp = np.zeros(n, np.uint32)
        img = np.zeros((n, 4), np.uint8)
        pick = np.zeros(1, np.uint32)
        nrm = np.zeros((n, 3), np.float32) if guides else None
        alb = np.zeros((n, 3), np.float32) if guides else None
        check(lib().rt_launcher_download(self.h, _ptr(raw), _ptr(rpp), _ptr(nrm), _ptr(alb), _ptr(img),
                                         _ptr(pick)))
        return dict(rawRGB=raw, rpp=rpp, image=img, pick_id=int(pick[0]), normals=nrm, albedos=alb)

    def frame(self):
        f = Frame()
        img = ctypes.c_void_p()
        pick = ctypes.c_void_p()
        check(lib().rt_launcher_frame(self.h, ctypes.byref(f), ctypes.byref(img), ctypes.byref(pick)))
        return f, img, pick


class Batch:
    """Owns an rt_batch: many scenes built and rendered together.  Device
    output buffers are allocated here (cudaMalloc through the library is not
    exposed, so torch tensors hold them) and kept alive with the batch."""

    def __init__(self):
        self.h = ctypes.c_void_p()
        check(lib().rt_batch_create(ctypes.byref(self.h)))
        self._keep = []

    def close(self):
        if self.h:
            lib().rt_batch_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add(self, scene, cam, params, frame):
        idx = ctypes.c_uint()
        check(lib().rt_batch_add(self.h, scene.h, ctypes.byref(cam), ctypes.byref(params), ctypes.byref(frame),
                                 ctypes.byref(idx)))
        self._keep.append((scene, cam, params, frame))
        return idx.value

    def build(self, morton_bits=60, stream=None, layout=None):
        if layout is not None:
            check(lib().rt_batch_set_layout(self.h, layout))
        check(lib().rt_batch_build(self.h, morton_bits, stream))

    def launch(self, stream=None, stats=True):
        """rt_batch_launch; stats=False passes no stats (required inside a stream capture)."""
        if not stats:
            check(lib().rt_batch_launch(self.h, stream, None))
            return None
        st = LaunchStats()
        check(lib().rt_batch_launch(self.h, stream, ctypes.byref(st)))
        return st

    def set_adjoint(self, index, grad_image, grad_albedo, grad_fuzz, grad_sky):
        """rt_batch_set_adjoint; device pointers (int) or None."""
        check(lib().rt_batch_set_adjoint(self.h, index, grad_image, grad_albedo, grad_fuzz, grad_sky))

    def adjoint(self, stream=None):
        check(lib().rt_batch_adjoint(self.h, stream))

    def status(self, stream=None):
        """rt_batch_status: raises the error of a launch captured into a graph, if any."""
        check(lib().rt_batch_status(self.h, stream))

    def set_albedos(self, albedo, stream=None):
        """rt_batch_set_albedos from a device pointer (3 floats per thing, scenes in order)."""
        check(lib().rt_batch_set_albedos(self.h, albedo, stream))

    def info(self):
        n, p = ctypes.c_uint(), ctypes.c_uint()
        ms = ctypes.c_float()
        b = ctypes.c_ulonglong()
        check(lib().rt_batch_info(self.h, ctypes.byref(n), ctypes.byref(p), ctypes.byref(ms), ctypes.byref(b)))
        return dict(n_scenes=n.value, n_prims=p.value, build_ms=ms.value, device_bytes=b.value)


def l2_loss_grad(image, target, grad_image, n, loss=None, stream=None):
    """rt_l2_loss_grad on device pointers (loss: device double pointer or None)."""
    check(lib().rt_l2_loss_grad(image, target, grad_image, n, loss, stream))


def adam_step(theta, grad, m, v, n, step, lr=1e-2, beta1=0.9, beta2=0.999, eps=1e-8, lo=0.0, hi=1.0, stream=None):
    """rt_adam_step on device pointers."""
    check(lib().rt_adam_step(theta, grad, m, v, n, lr, beta1, beta2, eps, step, lo, hi, stream))


def adam_step_device(theta, grad, m, v, n, step_ptr, lr=1e-2, beta1=0.9, beta2=0.999, eps=1e-8, lo=0.0, hi=1.0,
                     stream=None):
    """rt_adam_step_device: the step counter is a device uint32 (advanced by the call)."""
    check(lib().rt_adam_step_device(theta, grad, m, v, n, lr, beta1, beta2, eps, step_ptr, lo, hi, stream))


class Accum:
    """rt_accum: progressive rendering with checkpoint and resume."""

    def __init__(self, w, h):
        self.h = ctypes.c_void_p()
        self.w, self.hgt = w, h
        check(lib().rt_accum_create(ctypes.byref(self.h), w, h))

    def close(self):
        if self.h:
            lib().rt_accum_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def samples(self):
        n = ctypes.c_ulonglong()
        check(lib().rt_accum_samples(self.h, ctypes.byref(n)))
        return n.value

    def reset(self, stream=None):
        check(lib().rt_accum_reset(self.h, stream))

    def set_first_sample(self, first):
        check(lib().rt_accum_set_first_sample(self.h, first))

    def device_sums(self):
        """Device addresses of the red, green, blue (int64) and rays (uint32) sums, w*h each."""
        ptrs = [ctypes.c_void_p() for _ in range(4)]
        check(lib().rt_accum_device_sums(self.h, *[ctypes.byref(p) for p in ptrs]))
        return [p.value for p in ptrs]

    def set_range(self, first, samples, rays):
        check(lib().rt_accum_set_range(self.h, first, samples, rays))

    def resolve(self, frame, stream=None):
        check(lib().rt_accum_resolve(self.h, ctypes.byref(frame), stream))

    def launch(self, scene, cam, params, frame, stream=None):
        """rt_launch_accum into a Frame of device pointers; returns LaunchStats."""
        st = LaunchStats()
        check(lib().rt_launch_accum(scene.h, ctypes.byref(cam), ctypes.byref(params), self.h, ctypes.byref(frame),
                                    stream, ctypes.byref(st)))
        return st

    def save(self, stream=None):
        """The checkpoint as bytes."""
        n = ctypes.c_size_t()
        check(lib().rt_accum_state_size(self.h, ctypes.byref(n)))
        buf = ctypes.create_string_buffer(n.value)
        check(lib().rt_accum_save(self.h, buf, n.value, stream))
        return buf.raw

    def load(self, state, stream=None):
        buf = ctypes.create_string_buffer(bytes(state), len(state))
        check(lib().rt_accum_load(self.h, buf, len(state), stream))


def tuning_set(tuning=None):
    """rt_tuning_set from a dict of rt_tuning fields (missing or 0: default; None: all defaults)."""
    if tuning is None:
        check(lib().rt_tuning_set(None))
        return
    unknown = set(tuning) - set(TUNING_FIELDS)
    if unknown:
        raise ValueError(f"unknown tuning fields {sorted(unknown)}")
    t = Tuning(**{k: int(v) for k, v in tuning.items()})
    check(lib().rt_tuning_set(ctypes.byref(t)))


def tuning_get():
    """The tuning in effect (rt_tuning_get) as a dict."""
    t = Tuning()
    check(lib().rt_tuning_get(ctypes.byref(t)))
    return {k: getattr(t, k) for k in TUNING_FIELDS}


def render(scene, cam, params, guides=False):
    """Synchronous render through a Launcher; returns host arrays and stats."""
    L = Launcher(params.image_w, params.image_h)
    try:
        stats = L.ignite(scene, cam, params)
        out = L.download(guides=guides)
    finally:
        L.close()
    out["stats"] = stats
    return out


def rtow_scene(level=6, rng_kind=RT_RECIPE_GLIBC, seed=1, half_extent=11, morton_bits=60, layout=RT_LAYOUT_AUTO):
    """The final scene, tessellated at `level` (None: analytic spheres), built."""
    sc = Scene()
    sc.load_rtow(rng_kind, seed, half_extent, -1 if level is None else level)
    sc.build(morton_bits, layout=layout)
    return sc


def version():
    return lib().rt_version().decode()
