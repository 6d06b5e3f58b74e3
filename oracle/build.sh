#!/bin/sh
# Builds the CPU oracle (test infrastructure only) next to this script:
#   libvrt_oracle.so       -O2 -ffp-contract=off   parity build
#   libvrt_oracle_fast.so  -O3 -ffp-contract=off   timed CPU baseline (same results)
# IEEE binary32 without contraction on x86 and Arm; OpenMP over image rows.
# Both also carry the library's host-only scene helpers (csrc/host.cpp: uniform defaults,
# camera matrix; csrc/terrain.cpp: the seeded terrain), which need no CUDA, so the CPU
# baseline builds its inputs without loading the CUDA library.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
CSRC="$HERE/../voxel-rt_gb300/csrc"
CXX=${CXX:-g++}
$CXX -std=c++17 -O2 -ffp-contract=off -fno-fast-math -fopenmp -fPIC -shared \
    "$HERE/vrt_oracle.cpp" "$CSRC/host.cpp" "$CSRC/terrain.cpp" -o "$HERE/libvrt_oracle.so" -lpthread
$CXX -std=c++17 -O3 -ffp-contract=off -fno-fast-math -fopenmp -fPIC -shared \
    "$HERE/vrt_oracle.cpp" "$CSRC/host.cpp" "$CSRC/terrain.cpp" -o "$HERE/libvrt_oracle_fast.so" -lpthread
