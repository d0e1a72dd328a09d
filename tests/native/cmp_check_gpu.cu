// TEST INFRASTRUCTURE: the device side of cmp_cases.h (the integer-pipe
// helpers as the kernels compile them, PTX moves included).  One thread per
// value i checks i alone and every pair (i, j); the counts are summed.
#include <cuda_runtime.h>

#include "cmp_cases.h"

namespace {

__global__ void k_check(const double* v, int n, unsigned long long* bad) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    long long b = cmpcheck::check_one(v[i]);
    if (v[i] == v[i])
        for (int j = 0; j < n; ++j)
            if (v[j] == v[j]) b += cmpcheck::check_pair(v[i], v[j]);
    if (b) atomicAdd(bad, (unsigned long long)b);
}

}  // namespace

// Returns the mismatch count, or -1 on a CUDA error.
extern "C" long long cmpc_check_gpu(const double* host_v, int n) {
    double* v = nullptr;
    unsigned long long* bad = nullptr;
    long long out = -1;
    if (cudaMalloc(&v, sizeof(double) * n) != cudaSuccess) return -1;
    if (cudaMalloc(&bad, sizeof(unsigned long long)) == cudaSuccess &&
        cudaMemcpy(v, host_v, sizeof(double) * n, cudaMemcpyHostToDevice) == cudaSuccess &&
        cudaMemset(bad, 0, sizeof(unsigned long long)) == cudaSuccess) {
        k_check<<<(n + 127) / 128, 128>>>(v, n, bad);
        unsigned long long h = 0;
        if (cudaGetLastError() == cudaSuccess &&
            cudaMemcpy(&h, bad, sizeof(h), cudaMemcpyDeviceToHost) == cudaSuccess)
            out = (long long)h;
    }
    cudaFree(v);
    cudaFree(bad);
    return out;
}
