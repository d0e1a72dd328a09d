// TEST INFRASTRUCTURE: the device side of cmp_cases.h (the integer-pipe
// helpers as the kernels compile them, PTX moves included).  One thread per
// value i checks i alone and every pair (i, j); per-value mismatch counts
// come back in `per` (n entries).
#include <cuda_runtime.h>

#include "cmp_cases.h"

namespace {

__global__ void k_check(const double* v, int n, long long* per) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    long long b = cmpcheck::check_one(v[i]);
    if (v[i] == v[i])
        for (int j = 0; j < n; ++j)
            if (v[j] == v[j]) b += cmpcheck::check_pair(v[i], v[j]);
    per[i] = b;
}

}  // namespace

// Fills per[0..n) with each value's mismatch count; returns 0, or -1 on a
// CUDA error.
extern "C" int cmpc_check_gpu(const double* host_v, int n, long long* host_per) {
    double* v = nullptr;
    long long* per = nullptr;
    int out = -1;
    if (cudaMalloc(&v, sizeof(double) * n) != cudaSuccess) return -1;
    if (cudaMalloc(&per, sizeof(long long) * n) == cudaSuccess &&
        cudaMemcpy(v, host_v, sizeof(double) * n, cudaMemcpyHostToDevice) == cudaSuccess) {
        k_check<<<(n + 127) / 128, 128>>>(v, n, per);
        if (cudaGetLastError() == cudaSuccess &&
            cudaMemcpy(host_per, per, sizeof(long long) * n, cudaMemcpyDeviceToHost) == cudaSuccess)
            out = 0;
    }
    cudaFree(v);
    cudaFree(per);
    return out;
}
