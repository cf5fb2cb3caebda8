"""Generates the committed golden fixtures from the reference's own code.

Test infrastructure only.  Run in a checkout that has the reference sources
(``oracle/ref_build.sh`` compiles them into ``oracle/_ref/``):

    bash oracle/ref_build.sh && python tests/golden/make_golden.py

Fixtures written next to this script:

* ``rtow_scene_seed{1,7}.txt`` -- the sphere list built by the reference's
  ``scene()`` (rtow.cxx:51-80) with glibc ``rand()`` seeded 1 (glibc's default)
  and 7; one line per sphere: type cx cy cz r ar ag ab fuzz index.
* ``sphere_r1_n{0..4}.bin`` -- ``Sphere(1.f, n).mesh()`` (optx/sphere.cxx:17-106)
  as raw bits: u32 nv, u32 ni, nv*3 f32, ni*3 u32.
* ``sphere_hashes.json`` -- sha256 of the vertex and index bytes and the counts
  of ``Sphere(r, n).mesh()`` for larger levels, where the raw mesh is too big
  to commit.
* ``glibc_rand.json`` -- the first 64 outputs of glibc ``rand()`` for a few
  seeds (pins the scene recipe's random stream independently of the host libc).
"""
import ctypes
import hashlib
import json
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF_BIN = os.path.join(ROOT, "oracle", "_ref")


def _run(args, **kw):
    return subprocess.run(args, check=True, **kw)


def main():
    scene_tool = os.path.join(REF_BIN, "ref_golden_scene")
    sphere_tool = os.path.join(REF_BIN, "ref_golden_sphere")
    if not (os.path.exists(scene_tool) and os.path.exists(sphere_tool)):
        sys.exit("run oracle/ref_build.sh first (needs the reference sources)")

    for seed in (1, 7):
        out = _run([scene_tool, str(seed)], capture_output=True, text=True).stdout
        with open(os.path.join(HERE, f"rtow_scene_seed{seed}.txt"), "w") as f:
            f.write(out)

    tmp = os.path.join(REF_BIN, "mesh.bin")
    for n in range(5):
        _run([sphere_tool, "1.0", str(n), os.path.join(HERE, f"sphere_r1_n{n}.bin")])

    hashes = {}
    for radius, levels in (("1.0", range(9)), ("0.2", (3, 6)), ("1000.0", (6,))):
        for n in levels:
            _run([sphere_tool, radius, str(n), tmp])
            with open(tmp, "rb") as f:
                data = f.read()
            nv, ni = int.from_bytes(data[0:4], "little"), int.from_bytes(data[4:8], "little")
            vbytes = data[8:8 + 12 * nv]
            ibytes = data[8 + 12 * nv:8 + 12 * nv + 12 * ni]
            hashes[f"r{radius}_n{n}"] = {
                "radius": float(radius), "ndiv": n, "nv": nv, "ni": ni,
                "vces_sha256": hashlib.sha256(vbytes).hexdigest(),
                "ices_sha256": hashlib.sha256(ibytes).hexdigest(),
            }
    os.remove(tmp)
    with open(os.path.join(HERE, "sphere_hashes.json"), "w") as f:
        json.dump(hashes, f, indent=1, sort_keys=True)

    libc = ctypes.CDLL("libc.so.6")
    seq = {}
    for seed in (1, 7, 42, 4711):
        libc.srand(seed)
        seq[str(seed)] = [libc.rand() for _ in range(64)]
    with open(os.path.join(HERE, "glibc_rand.json"), "w") as f:
        json.dump(seq, f)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
