// sar_cgls.cu -- CGLS on the normal equations A^H A x = A^H y with the plan's operator pair
// (sar_cgls, include/sargpu.h).
//
// Replaces the CIL CGLS the reference's tests run on its operator (tests/test_cil.py:18-22): the
// iteration is the standard CGLS recurrence,
//   r = y - A x0,  s = A^H r,  p = s,  gamma = ||s||^2
//   repeat:  q = A p;  alpha = gamma / ||q||^2;  x += alpha p;  r -= alpha q
//            s = A^H r;  gamma' = ||s||^2;  stop if sqrt(gamma') <= tol * ||A^H y||
//            p = s + (gamma' / gamma) p;  gamma = gamma'
// and the stopping rule is the normal-equations residual ||A^H (y - A x)|| / ||A^H y|| (CGLS's own
// ||s||), since with noisy data ||y - A x|| / ||y|| stalls at the noise level.
//
// Vector work (the K5 kernels below) is fused so that each iteration reads every vector once per
// update: one kernel updates x and r together, one updates p, and squared norms are reduced in
// FP64.  Scalars stay on the device (alpha and beta are formed by the kernels from the reduced
// norms); the host reads two doubles per iteration to decide whether to stop.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <vector>

#include "../../include/sargpu.h"
#include "sar_kernels.cuh"
#include "sar_solver_common.cuh"

namespace {

// x += alpha p over P entries and r -= alpha q over NS entries, alpha = sc[ig] / sc[iq]
// (0 when the denominator is not positive: the caller then stops).
__global__ void update_xr_kernel(float2* __restrict__ x, const float2* __restrict__ p, size_t P,
                                 float2* __restrict__ r, const float2* __restrict__ q, size_t NS,
                                 const double* __restrict__ sc, int ig, int iq) {
    const double den = sc[iq];
    const float alpha = den > 0.0 ? (float)(sc[ig] / den) : 0.f;
    const size_t total = P + NS;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        if (i < P) {
            float2 a = x[i];
            const float2 b = __ldg(p + i);
            a.x = fmaf(alpha, b.x, a.x);
            a.y = fmaf(alpha, b.y, a.y);
            x[i] = a;
        } else {
            const size_t j = i - P;
            float2 a = r[j];
            const float2 b = __ldg(q + j);
            a.x = fmaf(-alpha, b.x, a.x);
            a.y = fmaf(-alpha, b.y, a.y);
            r[j] = a;
        }
    }
}

// p = s + beta p, beta = sc[inew] / sc[iold].
__global__ void update_p_kernel(float2* __restrict__ p, const float2* __restrict__ s, size_t P,
                                const double* __restrict__ sc, int inew, int iold) {
    const double den = sc[iold];
    const float beta = den > 0.0 ? (float)(sc[inew] / den) : 0.f;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < P; i += (size_t)gridDim.x * blockDim.x) {
        float2 a = p[i];
        const float2 b = __ldg(s + i);
        a.x = fmaf(beta, a.x, b.x);
        a.y = fmaf(beta, a.y, b.y);
        p[i] = a;
    }
}

// Re<a, b> = sum Re(conj(a) b) accumulated in FP64 into *out (zeroed by the caller).
__global__ void dot_re_kernel(const float2* __restrict__ a, const float2* __restrict__ b, size_t n,
                              double* __restrict__ out) {
    __shared__ double part[kThreads / 32];
    double acc = 0.0;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float2 u = __ldg(a + i), v = __ldg(b + i);
        acc += (double)fmaf(u.x, v.x, u.y * v.y);
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

// Scaled start: c = sc[inum] / sc[iden]; x = c x over P entries, r = y - c r over NS entries
// (x holds the direction z and r holds A z on entry).
__global__ void scale_start_kernel(float2* __restrict__ x, size_t P, float2* __restrict__ r,
                                   const float2* __restrict__ y, size_t NS, const double* __restrict__ sc, int inum,
                                   int iden) {
    const double den = sc[iden];
    const float c = den > 0.0 ? (float)(sc[inum] / den) : 0.f;
    const size_t total = P + NS;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        if (i < P) {
            const float2 a = x[i];
            x[i] = make_float2(c * a.x, c * a.y);
        } else {
            const size_t j = i - P;
            const float2 a = r[j], b = __ldg(y + j);
            r[j] = make_float2(fmaf(-c, a.x, b.x), fmaf(-c, a.y, b.y));
        }
    }
}

// r = y - r (r holds A x0 on entry).
__global__ void residual_kernel(float2* __restrict__ r, const float2* __restrict__ y, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float2 a = r[i], b = __ldg(y + i);
        r[i] = make_float2(b.x - a.x, b.y - a.y);
    }
}

struct Work {
    float2 *r = nullptr, *q = nullptr, *s = nullptr, *p = nullptr;
    double* sc = nullptr;
    cudaStream_t st = nullptr;
    ~Work() {
        for (void* b : {(void*)r, (void*)q, (void*)s, (void*)p, (void*)sc})
            if (b) cudaFreeAsync(b, st);
    }
};

}  // namespace

// Scalar slots on the device: 0 and 1 hold gamma of alternate iterations, 2 holds ||A p||^2,
// 3 holds ||A^H y||^2, 4 and 5 hold <z, A^H y> and ||A z||^2 of a scaled start.
extern "C" int sar_cgls_ex(sar_plan* plan, const void* y_dev, void* x_dev, int start, const void* ahy_dev,
                           int max_iterations, double tolerance, double* history, sar_cgls_result* result,
                           void* stream) {
    if (!plan || !y_dev || !x_dev || !result) return arg_error("null argument");
    if (max_iterations < 0 || !(tolerance >= 0.0)) return arg_error("max_iterations >= 0 and tolerance >= 0 required");
    if (start != SAR_CGLS_START_GIVEN && start != SAR_CGLS_START_ZERO && start != SAR_CGLS_START_SCALED)
        return arg_error("unknown CGLS start mode");
    sar_plan_info info;
    CG_CALL(sar_plan_get_info(plan, &info));
    const size_t P = info.num_scatterers, NS = info.num_slow_times * info.num_fast_times;
    cudaStream_t st = (cudaStream_t)stream;
    DeviceScope scope(info.device);
    if (scope.status != cudaSuccess) return cuda_status(scope.status, "select device");
    int sms = 0;
    CG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, info.device), "device attribute");
    *result = sar_cgls_result{};

    Work w;
    w.st = st;
    CG_CUDA(cudaMallocAsync((void**)&w.r, sizeof(float2) * NS, st), "CGLS work r");
    CG_CUDA(cudaMallocAsync((void**)&w.q, sizeof(float2) * NS, st), "CGLS work q");
    CG_CUDA(cudaMallocAsync((void**)&w.s, sizeof(float2) * P, st), "CGLS work s");
    CG_CUDA(cudaMallocAsync((void**)&w.p, sizeof(float2) * P, st), "CGLS work p");
    CG_CUDA(cudaMallocAsync((void**)&w.sc, sizeof(double) * 6, st), "CGLS scalars");
    CG_CUDA(cudaMemsetAsync(w.sc, 0, sizeof(double) * 6, st), "clear scalars");
    float2* x = (float2*)x_dev;
    const float2* y = (const float2*)y_dev;

    // ||A^H y|| (the residual's denominator), then the initial r = y - A x0 and s = A^H r.
    if (ahy_dev)
        CG_CUDA(cudaMemcpyAsync(w.s, ahy_dev, sizeof(float2) * P, cudaMemcpyDeviceToDevice, st), "A^H y");
    else
        CG_CALL(sar_adjoint(plan, y, w.s, st));
    norm2_kernel<<<grid_for(P, sms), kThreads, 0, st>>>(w.s, P, w.sc + 3);
    if (start == SAR_CGLS_START_ZERO) {
        CG_CUDA(cudaMemsetAsync(x, 0, sizeof(float2) * P, st), "zero x");
        CG_CUDA(cudaMemcpyAsync(w.r, y, sizeof(float2) * NS, cudaMemcpyDeviceToDevice, st), "r = y");
    } else if (start == SAR_CGLS_START_SCALED) {
        // x0 = c z with c = Re<z, A^H y> / ||A z||^2, the minimiser of ||y - c A z||.
        CG_CALL(sar_forward(plan, x, w.r, st));
        dot_re_kernel<<<grid_for(P, sms), kThreads, 0, st>>>(x, w.s, P, w.sc + 4);
        norm2_kernel<<<grid_for(NS, sms), kThreads, 0, st>>>(w.r, NS, w.sc + 5);
        scale_start_kernel<<<grid_for(P + NS, sms), kThreads, 0, st>>>(x, P, w.r, y, NS, w.sc, 4, 5);
        CG_CALL(sar_adjoint(plan, w.r, w.s, st));
    } else {
        CG_CALL(sar_forward(plan, x, w.r, st));
        residual_kernel<<<grid_for(NS, sms), kThreads, 0, st>>>(w.r, y, NS);
        CG_CALL(sar_adjoint(plan, w.r, w.s, st));
    }
    norm2_kernel<<<grid_for(P, sms), kThreads, 0, st>>>(w.s, P, w.sc + 0);
    CG_CUDA(cudaMemcpyAsync(w.p, w.s, sizeof(float2) * P, cudaMemcpyDeviceToDevice, st), "p = s");
    CG_CUDA(cudaGetLastError(), "CGLS set-up kernels");

    double host_sc[6];
    CG_CUDA(cudaMemcpyAsync(host_sc, w.sc, sizeof host_sc, cudaMemcpyDeviceToHost, st), "read scalars");
    CG_CUDA(cudaStreamSynchronize(st), "CGLS set-up");
    const double norm_ahy = std::sqrt(host_sc[3]);
    result->norm_ahy = norm_ahy;
    if (!std::isfinite(host_sc[0]) || !std::isfinite(host_sc[3]))
        return arg_error("CGLS: non-finite value in the data or the start (A^H y or A^H (y - A x0))");
    double res = norm_ahy > 0.0 ? std::sqrt(host_sc[0]) / norm_ahy : 0.0;
    if (history) history[0] = res;
    result->residual = res;
    if (res <= tolerance || host_sc[0] == 0.0) {
        result->converged = 1;
        return SAR_OK;
    }
    int cur = 0;
    for (int it = 1; it <= max_iterations; ++it) {
        const int nxt = cur ^ 1;
        CG_CALL(sar_forward(plan, w.p, w.q, st));
        CG_CUDA(cudaMemsetAsync(w.sc + 2, 0, sizeof(double), st), "clear |q|^2");
        norm2_kernel<<<grid_for(NS, sms), kThreads, 0, st>>>(w.q, NS, w.sc + 2);
        update_xr_kernel<<<grid_for(P + NS, sms), kThreads, 0, st>>>(x, w.p, P, w.r, w.q, NS, w.sc, cur, 2);
        CG_CALL(sar_adjoint(plan, w.r, w.s, st));
        CG_CUDA(cudaMemsetAsync(w.sc + nxt, 0, sizeof(double), st), "clear gamma");
        norm2_kernel<<<grid_for(P, sms), kThreads, 0, st>>>(w.s, P, w.sc + nxt);
        CG_CUDA(cudaGetLastError(), "CGLS kernels");
        CG_CUDA(cudaMemcpyAsync(host_sc, w.sc, sizeof(double) * 3, cudaMemcpyDeviceToHost, st), "read scalars");
        CG_CUDA(cudaStreamSynchronize(st), "CGLS iteration");
        result->iterations = it;
        if (!std::isfinite(host_sc[2]) || !std::isfinite(host_sc[nxt]))
            return arg_error("CGLS: non-finite value during the iteration");
        if (!(host_sc[2] > 0.0)) {   // A p = 0 with gamma > 0: no progress possible
            result->breakdown = 1;
            return SAR_OK;
        }
        res = std::sqrt(host_sc[nxt]) / norm_ahy;
        if (history) history[it] = res;
        result->residual = res;
        if (res <= tolerance) {
            result->converged = 1;
            return SAR_OK;
        }
        update_p_kernel<<<grid_for(P, sms), kThreads, 0, st>>>(w.p, w.s, P, w.sc, nxt, cur);
        cur = nxt;
    }
    CG_CUDA(cudaGetLastError(), "CGLS kernels");
    return SAR_OK;
}

extern "C" int sar_cgls(sar_plan* plan, const void* y_dev, void* x_dev, int zero_start, int max_iterations,
                        double tolerance, double* history, sar_cgls_result* result, void* stream) {
    return sar_cgls_ex(plan, y_dev, x_dev, zero_start ? SAR_CGLS_START_ZERO : SAR_CGLS_START_GIVEN, nullptr,
                       max_iterations, tolerance, history, result, stream);
}
