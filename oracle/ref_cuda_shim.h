// ref_cuda_shim.h -- TEST INFRASTRUCTURE.  Lets the reference's own CUDA
// kernel sources (src/GPU/Arista_kernel.cu, Volumen_kernel.cu,
// Reduccion_kernel.cu, Matriz.cu, Constantes.hxx) compile unmodified for
// sm_103a with nvcc 13, so that the reference build can be timed on the same
// GPU as this project.  CUDA 12 removed the legacy texture references the
// reference declares (Constantes.hxx:95-96) and reads with tex2D
// (Arista_kernel.cu:680 ff., Volumen_kernel.cu:203-269); nvcc 13 rejects both.
//
// What it supplies, all written for this project:
//   * `texture<T, dim, mode>` becomes a __device__ variable of a plain struct
//     holding a device pointer and the array's width and height, which the
//     host driver (ref_cuda_driver.cpp) fills through the module's globals;
//   * tex2D(tex, x, y) reads element (x, y) of that array through the
//     read-only data cache (__ldg).  The reference's textures use point
//     sampling with unnormalised coordinates and are only ever read at
//     integer coordinates, so texel (x, y) is the element itself.  A read
//     outside the array is not made: it returns zeros and records the first
//     such coordinate in lsh_ref_tex_fault, which the driver checks.
// The CUDA headers are included first, so the two macros below touch only
// the reference's sources.
#ifndef LSH_REF_CUDA_SHIM_H
#define LSH_REF_CUDA_SHIM_H

#include <cuda.h>
#include <cuda_runtime.h>
#include <float.h>
#include <math.h>

template <class T, int D, int M>
struct lsh_ref_texture {
    const T* data;
    int width;
    int height;
};

// 0 while every texture read stayed inside its array; else 1 + the first
// offending (x, y) packed as x * 65536 + y
__device__ unsigned long long lsh_ref_tex_fault;

template <class T, int D, int M>
__device__ __forceinline__ T lsh_ref_tex2d(const lsh_ref_texture<T, D, M>& t, int x, int y) {
    if (x < 0 || y < 0 || x >= t.width || y >= t.height) {
        atomicCAS(&lsh_ref_tex_fault, 0ull, 1ull + (unsigned long long)(unsigned)x * 65536ull + (unsigned)y);
        T z;
        memset(&z, 0, sizeof(z));
        return z;
    }
    return __ldg(t.data + (size_t)y * t.width + x);
}

#define texture __device__ lsh_ref_texture
#define tex2D(tex, x, y) lsh_ref_tex2d((tex), (int)(x), (int)(y))

#endif
