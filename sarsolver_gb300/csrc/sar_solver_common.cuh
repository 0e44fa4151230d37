// sar_solver_common.cuh -- pieces shared by the iterative solvers on the plan's operator pair
// (sar_cgls.cu, sar_pdhg.cu): FP64 squared-norm reduction, grid sizing, device scope and status
// helpers.  Each including unit gets its own internal copy.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>

#include "../../include/sargpu.h"
#include "sar_kernels.cuh"

namespace {

constexpr int kThreads = 256;

// ||v||^2 accumulated in FP64 into *out (zeroed by the caller).
__global__ void norm2_kernel(const float2* __restrict__ v, size_t n, double* __restrict__ out) {
    __shared__ double part[kThreads / 32];
    double acc = 0.0;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float2 a = __ldg(v + i);
        acc += (double)fmaf(a.x, a.x, a.y * a.y);
    }
    for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        acc = threadIdx.x < kThreads / 32 ? part[threadIdx.x] : 0.0;
        for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (threadIdx.x == 0) atomicAdd(out, acc);
    }
}

unsigned grid_for(size_t n, int sms) {
    const size_t want = (n + kThreads - 1) / kThreads;
    const size_t cap = (size_t)(sms > 0 ? sms : 152) * 8;
    return (unsigned)std::max<size_t>(1, std::min(want, cap));
}

// Makes the plan's device current for the call and restores the caller's on exit.
struct DeviceScope {
    int prev = -1, target = -1;
    cudaError_t status = cudaSuccess;
    explicit DeviceScope(int dev) : target(dev) {
        status = cudaGetDevice(&prev);
        if (status == cudaSuccess && dev != prev) status = cudaSetDevice(dev);
    }
    ~DeviceScope() {
        if (prev >= 0 && target != prev) cudaSetDevice(prev);
    }
};

int cuda_status(cudaError_t e, const char* what) {
    char buf[256];
    snprintf(buf, sizeof buf, "%s: %s", what, cudaGetErrorString(e));
    sar::sar_internal_set_error(buf);
    return e == cudaErrorMemoryAllocation ? SAR_ERR_OUT_OF_MEMORY : SAR_ERR_CUDA;
}

int arg_error(const char* msg) {
    sar::sar_internal_set_error(msg);
    return SAR_ERR_INVALID_ARGUMENT;
}

#define CG_CUDA(call, what)                                  \
    do {                                                     \
        cudaError_t _e = (call);                             \
        if (_e != cudaSuccess) return cuda_status(_e, what); \
    } while (0)

#define CG_CALL(call)            \
    do {                         \
        int _rc = (call);        \
        if (_rc) return _rc;     \
    } while (0)

}  // namespace
