#!/bin/sh
# TEST INFRASTRUCTURE.  Builds the FP64 CPU oracle into oracle/_build/liblsh_oracle.so.
# -ffp-contract=off: no fused multiply-add contraction, so x86 and Arm hosts give
# the same bits.  OpenMP parallelises the race-free colour passes.
set -e
HERE="$(cd "$(dirname "$0")" && pwd)"
mkdir -p "$HERE/_build"
g++ -O2 -std=c++17 -fPIC -shared -fopenmp -ffp-contract=off \
    "$HERE/lsh_oracle.cpp" -o "$HERE/_build/liblsh_oracle.so.tmp"
mv "$HERE/_build/liblsh_oracle.so.tmp" "$HERE/_build/liblsh_oracle.so"
echo "build_oracle: built $HERE/_build/liblsh_oracle.so"
