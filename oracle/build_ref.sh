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
# Also compiles the reference's device code into ref_kernels.cubin (sm_103a,
# through ref_cuda_shim.h) and, wherever that cubin is, the driver that runs
# it on a GPU (liblsh_ref_cuda.so, from ref_cuda_driver.cpp).
# Skips the host builds and the cubin when the reference sources are absent.
set -e
REF="${1:-${LSH_REFERENCE_ROOT:-/root/reference}}"
HERE="$(cd "$(dirname "$0")" && pwd)"
CUDA="${CUDA_HOME:-/usr/local/cuda}"
CUDA_INC="$CUDA/include"
mkdir -p "$HERE/_ref"
if [ -f "$REF/src/GPU/Volumen_kernel.cu" ]; then
    # the reference as shipped (Coulomb law), and with its Pouliquen law
    # (COULOMB undefined before the kernel sources: ref_driver_pouliquen.cpp),
    # compiled as host C++
    g++ -O2 -std=c++17 -fPIC -shared -ffp-contract=off -w \
        -I"$CUDA_INC" -I"$REF/src/GPU" -I"$HERE" \
        "$HERE/ref_driver.cpp" -o "$HERE/_ref/liblsh_ref.so" &
    g++ -O2 -std=c++17 -fPIC -shared -ffp-contract=off -w \
        -I"$CUDA_INC" -I"$REF/src/GPU" -I"$HERE" \
        "$HERE/ref_driver_pouliquen.cpp" -o "$HERE/_ref/liblsh_ref_pouliquen.so" &
    # the reference's device code for sm_103a, with its own default nvcc
    # options (its makefile passes only -arch)
    "$CUDA/bin/nvcc" -cubin -gencode arch=compute_103a,code=sm_103a -w \
        -I"$REF/src/GPU" -I"$HERE" "$HERE/ref_cuda_kernels.cu" -o "$HERE/_ref/ref_kernels.cubin" &
    wait %1 && wait %2 && wait %3
    echo "build_ref: built $HERE/_ref/liblsh_ref.so, liblsh_ref_pouliquen.so, ref_kernels.cubin"
else
    echo "build_ref: reference sources not found under $REF; host builds skipped" >&2
fi
# the driver that runs the cubin on a GPU (this project's code, built
# wherever the cubin is: the reference sources are not needed for it)
if [ -f "$HERE/_ref/ref_kernels.cubin" ] && [ -f "$CUDA_INC/cuda.h" ]; then
    g++ -O2 -std=c++17 -fPIC -shared -I"$CUDA_INC" "$HERE/ref_cuda_driver.cpp" \
        -L"$CUDA/lib64/stubs" -L"$CUDA/lib64" -lcuda -o "$HERE/_ref/liblsh_ref_cuda.so"
    echo "build_ref: built $HERE/_ref/liblsh_ref_cuda.so"
fi
