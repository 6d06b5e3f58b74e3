#!/bin/sh
# Builds the reference's own C++ and its shader (read in place from the reference
# checkout, never copied into this repository) into oracle/_ref/ for golden-vector
# generation and oracle pinning.  Test infrastructure only; x86 or Arm, g++ only.
# The checkout's src/ directory: $VRT_REFERENCE_SRC, else reference/src in the directory
# that holds this repository.  Exits 3 (nothing built) when neither exists.
#   oracle/_ref/librefworld.so   src/level.cpp + src/render.cpp + ref_world_stub.cpp
#   oracle/_ref/librefshader.so  src/fshader.glsl via glsl_to_cpp.sed + refshader_harness.cpp
# The reference's own build uses g++ -O2 (compile.bat:3); -ffp-contract=off keeps float
# expressions unfused on CPUs with FMA.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${VRT_REFERENCE_SRC:-$HERE/../../../reference/src}
OUT=$HERE/../_ref
if [ ! -f "$REF/fshader.glsl" ]; then echo "reference sources not found at $REF" >&2; exit 3; fi
mkdir -p "$OUT"
sed -f "$HERE/glsl_to_cpp.sed" "$REF/fshader.glsl" > "$OUT/fshader_glm.inc"
g++ -std=c++17 -O2 -ffp-contract=off -fPIC -shared -w -I"$REF" -I"$OUT" \
    "$HERE/refshader_harness.cpp" -o "$OUT/librefshader.so"
g++ -std=c++17 -O2 -ffp-contract=off -fPIC -shared -w -fopenmp -fno-toplevel-reorder \
    -DGLEW_STATIC -DGLEW_NO_GLU -I"$REF" \
    "$REF/level.cpp" "$REF/render.cpp" "$HERE/ref_world_stub.cpp" -o "$OUT/librefworld.so" -lpthread
echo "built $OUT/librefworld.so $OUT/librefshader.so"
