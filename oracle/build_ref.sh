#!/bin/sh
# TEST INFRASTRUCTURE.  Builds oracle/_ref/liblsh_ref.so: the reference's own
# FP32 kernel sources, compiled where they lie (read-only) as host C++ through
# oracle/ref_shim.h, with oracle/ref_driver.cpp replaying shallowWater()'s
# launch sequence.  Nothing from the reference is copied into this repository;
# the output goes to oracle/_ref/ only (git-ignored).
#
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]
# REFERENCE_ROOT defaults to $LSH_REFERENCE_ROOT, else to the read-only
# checkout this recipe was written against (/root/reference).
# Exits 0 without building when the reference sources are absent.
set -e
REF="${1:-${LSH_REFERENCE_ROOT:-/root/reference}}"
HERE="$(cd "$(dirname "$0")" && pwd)"
if [ ! -f "$REF/src/GPU/Volumen_kernel.cu" ]; then
    echo "build_ref: reference sources not found under $REF; skipping" >&2
    exit 0
fi
CUDA_INC="${CUDA_HOME:-/usr/local/cuda}/include"
mkdir -p "$HERE/_ref"
# the reference as shipped (Coulomb law), and with its Pouliquen law
# (COULOMB undefined before the kernel sources: ref_driver_pouliquen.cpp)
g++ -O2 -std=c++17 -fPIC -shared -ffp-contract=off -w \
    -I"$CUDA_INC" -I"$REF/src/GPU" -I"$HERE" \
    "$HERE/ref_driver.cpp" -o "$HERE/_ref/liblsh_ref.so" &
g++ -O2 -std=c++17 -fPIC -shared -ffp-contract=off -w \
    -I"$CUDA_INC" -I"$REF/src/GPU" -I"$HERE" \
    "$HERE/ref_driver_pouliquen.cpp" -o "$HERE/_ref/liblsh_ref_pouliquen.so" &
wait %1 && wait %2
echo "build_ref: built $HERE/_ref/liblsh_ref.so $HERE/_ref/liblsh_ref_pouliquen.so"
