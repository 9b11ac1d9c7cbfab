#!/bin/sh
# Builds oracle/_ref/libref_bbvh.so from the reference's own CPU ray tracer sources, unmodified,
# and oracle/_ref/libref_sampling.so from its camera, ray and material sources and its sampling /
# shading headers,
# where they lie under the reference checkout named by $GRT_REFERENCE_DIR (oracle/build.py sets
# it). Used only to pin the oracle restatement and to generate golden fixtures; prints a notice
# and exits 0 when the variable is unset or the checkout is absent (for example on the GPU machine).
# -ffp-contract=off keeps every product unfused so the results do not depend on the host ISA.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${GRT_REFERENCE_DIR:-}
OUT="$HERE/_ref"
if [ -z "$REF" ] || [ ! -f "$REF/rt/cpu/bvh2.cpp" ]; then
    echo "build_ref: reference sources not found at $REF; skipping oracle/_ref"
    exit 0
fi
mkdir -p "$OUT"
CXX=${CXX:-g++}
FLAGS="-std=c++17 -O2 -fPIC -fopenmp -ffp-contract=off -DNDEBUG -w -I$HERE/shim -I$REF -I$REF/libgi"
$CXX $FLAGS -shared -o "$OUT/libref_bbvh.so" \
    "$HERE/ref_harness.cpp" "$REF/rt/cpu/bvh2.cpp" "$REF/libgi/timer.cpp" "$REF/libgi/rt.cpp"
$CXX $FLAGS -shared -o "$OUT/libref_sampling.so" "$HERE/ref_sampling.cpp" "$HERE/ref_material.cpp" \
    "$REF/libgi/camera.cpp" "$REF/libgi/rt.cpp"
echo "build_ref: built $OUT/libref_bbvh.so and $OUT/libref_sampling.so"
