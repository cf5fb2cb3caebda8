#!/usr/bin/env bash
# Builds the reference's own CPU code, where it lies, into oracle/_ref/.
#
# Test infrastructure only (golden vectors and the unmodified rtow baseline):
#   oracle/_ref/rtow               unmodified rtow.cxx (FP64 CPU renderer)
#   oracle/_ref/ref_golden_scene   rtow.cxx scene() + a dump driver
#   oracle/_ref/ref_golden_sphere  optx/sphere.cxx + a dump driver
# Needs the reference checkout: RTX_REFERENCE, else the checkout location of
# the build container (this recipe is the one place that names it); exits 0
# without doing anything when it is absent (as on the GPU machines), because
# nothing at run time depends on it.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${RTX_REFERENCE:-/root/reference}"
OUT="$HERE/_ref"
if [ ! -f "$REF/rtow.cxx" ]; then
    echo "ref_build: no reference checkout at $REF, skipped"
    exit 0
fi
CUDA_INC="${CUDA_HOME:-/usr/local/cuda}/include"
mkdir -p "$OUT"
CXX="${CXX:-g++}"
# The reference's CPU code is compiled as its own Makefile does for rtow
# (plain -O3), without FMA contraction so results do not depend on the host ISA.
"$CXX" -O3 -ffp-contract=off -o "$OUT/rtow" "$REF/rtow.cxx" &
"$CXX" -O2 -ffp-contract=off -I"$REF" -o "$OUT/ref_golden_scene" "$HERE/ref_golden_scene.cpp" &
"$CXX" -O2 -ffp-contract=off -I"$REF/optx" -I"$CUDA_INC" -o "$OUT/ref_golden_sphere" \
    "$HERE/ref_golden_sphere.cpp" "$REF/optx/sphere.cxx" &
wait
echo "ref_build: built $OUT"
