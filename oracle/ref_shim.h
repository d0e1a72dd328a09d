// ref_shim.h -- TEST INFRASTRUCTURE.  Lets the reference's own CUDA kernel
// sources (src/GPU/Arista_kernel.cu, Volumen_kernel.cu, Matriz.cu,
// Constantes.hxx) compile unmodified as host C++ with g++, so their FP32
// arithmetic can run on the CPU as a pin for the FP64 oracle.
//
// What it supplies, all written for this project:
//   * a `texture<T, dim, mode>` type standing in for the legacy texture
//     reference the reference declares (Constantes.hxx:95-96) -- it just holds
//     a host pointer and the array's width/height;
//   * a tex2D(tex, x, y) macro reading that host array, with a hard bounds
//     check (the reference only ever reads in range; abort otherwise);
//   * host globals threadIdx / blockIdx so a host loop can emulate launches.
// The legacy texture API was removed from CUDA 12+, which is why the
// reference does not compile with nvcc 13 as shipped.
#ifndef LSH_REF_SHIM_H
#define LSH_REF_SHIM_H

#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

template <class T, int D, int M>
struct texture {
    const T* data;
    int width;
    int height;
};

extern uint3 threadIdx;
extern uint3 blockIdx;

template <class T, int D, int M>
static inline T lsh_ref_tex2d(const texture<T, D, M>& t, int x, int y) {
    if (x < 0 || y < 0 || x >= t.width || y >= t.height || t.data == nullptr) {
        fprintf(stderr, "ref shim: texture read out of range (%d, %d) of %dx%d\n", x, y, t.width, t.height);
        abort();
    }
    return t.data[(size_t)y * t.width + x];
}

#define tex2D(tex, x, y) lsh_ref_tex2d((tex), (int)(x), (int)(y))

#endif
