#!/bin/sh
# Builds the CPU oracle (test infrastructure only) next to this script:
#   libvrt_oracle.so       -O2 -ffp-contract=off   parity build
#   libvrt_oracle_fast.so  -O3 -ffp-contract=off   timed CPU baseline (same results)
# IEEE binary32 without contraction on x86 and Arm; OpenMP over image rows.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
CXX=${CXX:-g++}
$CXX -std=c++17 -O2 -ffp-contract=off -fno-fast-math -fopenmp -fPIC -shared \
    "$HERE/vrt_oracle.cpp" -o "$HERE/libvrt_oracle.so"
$CXX -std=c++17 -O3 -ffp-contract=off -fno-fast-math -fopenmp -fPIC -shared \
    "$HERE/vrt_oracle.cpp" -o "$HERE/libvrt_oracle_fast.so"
