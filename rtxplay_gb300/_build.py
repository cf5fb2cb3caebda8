"""Build recipe of the native library (nvcc, sm_103a only).

``build_library()`` compiles every ``csrc/*.cu`` translation unit in parallel
and links ``rtxplay_gb300/_build/librtxplay_gb300.so``; ``build_rtwo()`` builds
the ``rtwo`` command-line launcher against it; ``build_checked()`` builds the
bounds-checked debug variant (``-DRT_CHECKS``) into ``_build/checked/``, which
a process loads instead by setting ``RTX_LIB`` to its path.  Arithmetic-sensitive flags:
``--fmad=false`` (no silent multiply-add contraction on the device),
``-prec-div/-prec-sqrt=true`` (IEEE division and square root) and
``-ffp-contract=off`` for host code, so device kernels, the host camera
set-up and any binary32 CPU restatement agree bit for bit.
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "librtxplay_gb300.so")
RTWO = os.path.join(OUT, "rtwo")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17", "--fmad=false", "-prec-div=true", "-prec-sqrt=true",
    "-Xcompiler", "-fPIC,-ffp-contract=off,-O2", "-Xptxas", "-O3",
    "-I", os.path.join(ROOT, "include"),
]


def nvcc():
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    path = os.path.join(cuda, "bin", "nvcc")
    return path if os.path.exists(path) else (shutil.which("nvcc") or "nvcc")


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _headers():
    return sorted(glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh"))
                  + glob.glob(os.path.join(ROOT, "include", "*.h")))


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src, extra, out=OUT):
    obj = os.path.join(out, os.path.basename(src)[:-3] + ".o")
    if _stale(obj, [src, __file__] + _headers()):
        cmd = [nvcc()] + NVCC_FLAGS + extra + ["-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def build_library(extra=(), verbose=False, jobs=None, out=OUT):
    """Compiles and links librtxplay_gb300.so into `out` (incremental); returns its path."""
    os.makedirs(out, exist_ok=True)
    lib = os.path.join(out, os.path.basename(LIB))
    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, list(extra), out), srcs))
    if _stale(lib, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", lib] + objs + ["-lcudart_static", "-lrt", "-ldl", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose:
        print("built", lib)
    return lib


CHECKED = os.path.join(OUT, "checked")


def build_checked(verbose=False):
    """The bounds-checked debug variant (-DRT_CHECKS); returns its path."""
    return build_library(extra=("-DRT_CHECKS",), verbose=verbose, out=CHECKED)


def build_rtwo():
    """Builds the rtwo launcher (C++ host code over the C ABI)."""
    src = os.path.join(HERE, "host", "rtwo.cpp")
    hdrs = [os.path.join(ROOT, "include", "rtwo.hpp"), os.path.join(ROOT, "include", "rt_api.h")]
    if not os.path.exists(src):
        return None
    if _stale(RTWO, [src, LIB] + hdrs):
        cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
        cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"),
               "-I", os.path.join(HERE, "host"), "-I", os.path.join(cuda, "include"),
               src, "-o", RTWO, "-L", OUT, "-lrtxplay_gb300", "-Wl,-rpath,$ORIGIN",
               "-L", os.path.join(cuda, "lib64"), "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"rtwo build failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return RTWO


if __name__ == "__main__":
    build_library(verbose=True)
    build_rtwo()
