#!/bin/sh
# Compile the reference's own CPU octree and flat-model loader
# (src/qubatron/octree.c, src/qubatron/model.c, the four mt_* files they
# link against, and the quaternion helpers src/mt_math/mt_quat.c) from the read-only reference tree into
# oracle/_ref/libqbref.so, together with oracle/ref_shim.c. Nothing from the
# reference is copied into this repository; only the built library lands in
# oracle/_ref (git-ignored). Usage: build_ref.sh REFERENCE_ROOT
# (or QB_REFERENCE_ROOT in the environment).
set -e
REF=${1:-$QB_REFERENCE_ROOT}
if [ -z "$REF" ]; then
    echo "build_ref: give the reference checkout (argument or QB_REFERENCE_ROOT)" >&2
    exit 2
fi
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
if [ ! -f "$REF/src/qubatron/octree.c" ]; then
    echo "build_ref: reference sources not found under $REF" >&2
    exit 2
fi
mkdir -p "$OUT"
CC=${CC:-gcc}
FLAGS="-std=gnu99 -O2 -fPIC -ffp-contract=off -w -I$HERE/ref_stub -I$REF/src/mt_core -I$REF/src/mt_math -I$REF/src/qubatron"
for f in qubatron/octree.c qubatron/model.c mt_core/mt_memory.c mt_core/mt_log.c mt_math/mt_vector_3d.c mt_math/mt_vector_4d.c mt_math/mt_quat.c; do
    $CC $FLAGS -c "$REF/src/$f" -o "$OUT/$(basename "$f" .c).o"
done
$CC $FLAGS -c "$HERE/ref_shim.c" -o "$OUT/ref_shim.o"
$CC -shared -o "$OUT/libqbref.so" "$OUT"/octree.o "$OUT"/model.o "$OUT"/mt_memory.o "$OUT"/mt_log.o "$OUT"/mt_vector_3d.o "$OUT"/mt_vector_4d.o "$OUT"/mt_quat.o "$OUT"/ref_shim.o -lm
rm -f "$OUT"/*.o
echo "build_ref: $OUT/libqbref.so"
