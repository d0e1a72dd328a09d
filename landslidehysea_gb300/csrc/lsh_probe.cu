// lsh_probe.cu -- lsh_probe_wait_bound (include/lsh.h): shows on the device
// that the passes' bounded waits give up and report instead of hanging.
//
// One block runs both waits the library uses between passes -- the
// overlapped step's dep_begin (lsh_kernels.cuh) and the work queue's
// queue_wait (lsh_queue.cuh) -- on completion counters that nothing
// increments.  Each gives up after its bound (about 2 s of %globaltimer) and
// records it: dep_begin in the time record's error word, queue_wait in its
// abort flag.  The kernel then returns, and the context stays usable.

#include <cuda_runtime.h>

#include <string>

#include "../../include/lsh.h"
#include "lsh_kernels.cuh"
#include "lsh_queue.cuh"
#include "lsh_setup.h"

namespace {

// out[0]: the time record's timeout bit after dep_begin; out[1]: queue_wait
// gave up; out[2]: the abort flag it left.
__global__ void k_wait_probe(Dep d, TimeRec* tm, const unsigned* qctr, int* qabort, int* out) {
    dep_begin(d, tm, 0, 0);
    if (threadIdx.x == 0) {
        unsigned long long start = 0;
        const bool gave_up = queue_wait(qctr, 0, 0, 1u, qabort, start);
        out[0] = (tm->err >> LSH_ERR_TIMEOUT) & 1;
        out[1] = gave_up ? 1 : 0;
        out[2] = *qabort;
    }
}

int probe_fail(cudaError_t e, const char* what) {
    lsh::set_last_error(std::string(what) + ": " + cudaGetErrorString(e));
    (void)cudaGetLastError();
    return LSH_ERR_CUDA;
}

}  // namespace

extern "C" int lsh_probe_wait_bound(int device, int* status_out, double* ms_out) {
    if (!status_out) return LSH_ERR_INVALID;
    if (lsh_check_device() != 0) return LSH_ERR_NO_DEVICE;
    if (device >= 0) {
        cudaError_t e = cudaSetDevice(device);
        if (e != cudaSuccess) return probe_fail(e, "cudaSetDevice");
    }
    // scratch: the time record, two counters, the abort flag, three results
    void* mem = nullptr;
    cudaError_t e = cudaMalloc(&mem, 256);
    if (e != cudaSuccess) return probe_fail(e, "cudaMalloc");
    e = cudaMemset(mem, 0, 256);
    auto* tm = static_cast<TimeRec*>(mem);
    unsigned* ctr = reinterpret_cast<unsigned*>(static_cast<char*>(mem) + 128);
    int* qabort = reinterpret_cast<int*>(ctr + 2);
    int* out = qabort + 1;
    Dep d;
    d.wait = ctr;  // ctr[0] stays 0: the wait for 1 never ends by itself
    d.target = 1;
    d.kind = kDepCell;
    d.ntiles = 1;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    if (e == cudaSuccess) e = cudaEventRecord(e0);
    if (e == cudaSuccess) {
        k_wait_probe<<<1, 32>>>(d, tm, ctr + 1, qabort, out);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaEventRecord(e1);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    int res[3] = {0, 0, 0};
    if (e == cudaSuccess) e = cudaMemcpy(res, out, sizeof(res), cudaMemcpyDeviceToHost);
    // the device still answers after the waits gave up
    if (e == cudaSuccess) e = cudaMemset(mem, 0, 256);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(mem);
    if (e != cudaSuccess) return probe_fail(e, "lsh_probe_wait_bound");
    if (ms_out) *ms_out = ms;
    *status_out = (res[0] && res[1] && res[2]) ? LSH_ERR_TIMEOUT : LSH_OK;
    return LSH_OK;
}
