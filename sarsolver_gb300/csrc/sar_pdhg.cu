// sar_pdhg.cu -- primal-dual hybrid gradient (Chambolle-Pock) on the plan's operator pair
// (sar_pdhg, include/sargpu.h).
//
// Replaces the CIL PDHG the reference's tests run on its operator (tests/test_cil.py:25-37):
//   min_x  f(A x) + g(x),   f(u) = ||u - b||^2 (CIL's L2NormSquared(b)),
//                           g = 0 (CIL's ZeroFunction) or g(x) = lambda ||x||_1 (complex modulus)
// with the iteration in CIL's order, starting from xbar = x0 and the dual variable y = 0:
//   y    <- prox_{sigma f*}(y + sigma A xbar) = (y + sigma (A xbar - b)) / (1 + sigma / 2)
//   x'   <- prox_{tau g}(x - tau A^H y)       (g = 0: identity; L1: soft threshold of the modulus
//                                             at tau lambda)
//   xbar <- x' + theta (x' - x),   x <- x'
// Step sizes: given, or from a power-method estimate of ||A||: sigma = tau = 1 / ||A|| when
// neither is given (CIL's default), the missing one from sigma tau ||A||^2 = 1 when one is.
//
// Each iteration is one forward projection, one backprojection and two fused vector kernels (the
// dual update, which also reduces ||A xbar - b||^2 in FP64 for the history, and the primal update
// of x and xbar together).  Nothing is read back inside the loop.
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "../../include/sargpu.h"
#include "sar_kernels.cuh"
#include "sar_solver_common.cuh"

namespace {

// Block-reduce a per-thread FP64 partial into *out (kThreads threads).
__device__ __forceinline__ void block_add(double acc, double* out) {
    __shared__ double part[kThreads / 32];
    for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        acc = threadIdx.x < kThreads / 32 ? part[threadIdx.x] : 0.0;
        for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (threadIdx.x == 0) atomicAdd(out, acc);
    }
}

// y = (y + sigma (q - b)) / (1 + sigma / 2) with q = A xbar; *res += ||q - b||^2.
__global__ void pdhg_dual_kernel(float2* __restrict__ y, const float2* __restrict__ q, const float2* __restrict__ b,
                                 size_t n, float sigma, float inv_den, double* __restrict__ res) {
    double acc = 0.0;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float2 qv = __ldg(q + i), bv = __ldg(b + i);
        const float2 d = make_float2(qv.x - bv.x, qv.y - bv.y);
        acc += (double)fmaf(d.x, d.x, d.y * d.y);
        float2 yv = y[i];
        yv.x = fmaf(sigma, d.x, yv.x) * inv_den;
        yv.y = fmaf(sigma, d.y, yv.y) * inv_den;
        y[i] = yv;
    }
    block_add(acc, res);
}

// z = x - tau s;  x' = z (thr = 0) or max(|z| - thr, 0) z / |z|;  xbar = x' + theta (x' - x);  x = x'.
__global__ void pdhg_primal_kernel(float2* __restrict__ x, float2* __restrict__ xbar, const float2* __restrict__ s,
                                   size_t n, float tau, float thr, float theta) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float2 xo = x[i], sv = __ldg(s + i);
        float2 z = make_float2(fmaf(-tau, sv.x, xo.x), fmaf(-tau, sv.y, xo.y));
        if (thr > 0.f) {
            const float m = sqrtf(fmaf(z.x, z.x, z.y * z.y));
            const float k = m > thr ? (m - thr) / m : 0.f;
            z.x *= k;
            z.y *= k;
        }
        x[i] = z;
        xbar[i] = make_float2(fmaf(theta, z.x - xo.x, z.x), fmaf(theta, z.y - xo.y, z.y));
    }
}

// Deterministic start of the power method: unit-modulus entries of pseudo-random phase.
__global__ void power_start_kernel(float2* __restrict__ v, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        uint32_t h = (uint32_t)i * 2654435761u + 0x9e3779b9u;
        h ^= h >> 16;
        h *= 0x85ebca6bu;
        h ^= h >> 13;
        const float ph = (float)(h >> 8) * (6.2831853f / 16777216.0f);
        float sn, cs;
        sincosf(ph, &sn, &cs);
        v[i] = make_float2(cs, sn);
    }
}

// v *= 1 / sqrt(*n2) (left unchanged when the norm is zero).
__global__ void normalise_kernel(float2* __restrict__ v, size_t n, const double* __restrict__ n2) {
    const double s2 = *n2;
    const float k = s2 > 0.0 ? (float)(1.0 / std::sqrt(s2)) : 1.f;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        float2 a = v[i];
        a.x *= k;
        a.y *= k;
        v[i] = a;
    }
}

struct PdWork {
    float2 *y = nullptr, *q = nullptr, *s = nullptr, *xbar = nullptr;
    double* sc = nullptr;
    cudaStream_t st = nullptr;
    ~PdWork() {
        for (void* b : {(void*)y, (void*)q, (void*)s, (void*)xbar, (void*)sc})
            if (b) cudaFreeAsync(b, st);
    }
};

}  // namespace

// Power-method estimate of ||A||: v <- A^H A v / ||A^H A v||; the estimate is ||A v|| with
// ||v|| = 1 (the Rayleigh quotient, a lower bound that rises to ||A||).  Work vectors: v, s [P],
// q [NS]; sc has two free slots.
static int estimate_norm(sar_plan* plan, size_t P, size_t NS, int iterations, float2* v, float2* q, float2* s,
                         double* sc, int sms, cudaStream_t st, double* norm_out) {
    power_start_kernel<<<grid_for(P, sms), kThreads, 0, st>>>(v, P);
    CG_CUDA(cudaMemsetAsync(sc, 0, sizeof(double), st), "clear norm");
    norm2_kernel<<<grid_for(P, sms), kThreads, 0, st>>>(v, P, sc);
    normalise_kernel<<<grid_for(P, sms), kThreads, 0, st>>>(v, P, sc);
    double aq = 0.0;
    for (int it = 0; it < iterations; ++it) {
        CG_CALL(sar_forward(plan, v, q, st));
        CG_CUDA(cudaMemsetAsync(sc, 0, 2 * sizeof(double), st), "clear norms");
        norm2_kernel<<<grid_for(NS, sms), kThreads, 0, st>>>(q, NS, sc);
        CG_CALL(sar_adjoint(plan, q, s, st));
        norm2_kernel<<<grid_for(P, sms), kThreads, 0, st>>>(s, P, sc + 1);
        CG_CUDA(cudaMemcpyAsync(v, s, sizeof(float2) * P, cudaMemcpyDeviceToDevice, st), "v = A^H A v");
        normalise_kernel<<<grid_for(P, sms), kThreads, 0, st>>>(v, P, sc + 1);
    }
    CG_CUDA(cudaGetLastError(), "power method kernels");
    CG_CUDA(cudaMemcpyAsync(&aq, sc, sizeof(double), cudaMemcpyDeviceToHost, st), "read norm");
    CG_CUDA(cudaStreamSynchronize(st), "power method");
    if (!std::isfinite(aq)) return arg_error("PDHG: non-finite operator norm estimate");
    *norm_out = std::sqrt(aq);
    return SAR_OK;
}

// Scalar slots: [0, 1] power method, [2 + k] ||A xbar_k - b||^2 of iteration k.
extern "C" int sar_pdhg(sar_plan* plan, const void* b_dev, void* x_dev, int zero_start, int iterations, double sigma,
                        double tau, double theta, double l1_weight, int norm_iterations, double* residual_history,
                        sar_pdhg_result* result, void* stream) {
    if (!plan || !b_dev || !x_dev || !result) return arg_error("null argument");
    if (iterations < 0 || norm_iterations < 0) return arg_error("iterations >= 0 and norm_iterations >= 0 required");
    if (!(sigma >= 0.0) || !(tau >= 0.0) || !std::isfinite(sigma) || !std::isfinite(tau))
        return arg_error("sigma and tau must be finite and >= 0 (0: from the operator norm)");
    if (!std::isfinite(theta) || !(l1_weight >= 0.0) || !std::isfinite(l1_weight))
        return arg_error("theta must be finite and l1_weight finite and >= 0");
    if ((sigma == 0.0 || tau == 0.0) && norm_iterations == 0)
        return arg_error("PDHG: step sizes need either both sigma and tau or norm_iterations > 0");
    sar_plan_info info;
    CG_CALL(sar_plan_get_info(plan, &info));
    const size_t P = info.num_scatterers, NS = info.num_slow_times * info.num_fast_times;
    cudaStream_t st = (cudaStream_t)stream;
    DeviceScope scope(info.device);
    if (scope.status != cudaSuccess) return cuda_status(scope.status, "select device");
    int sms = 0;
    CG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, info.device), "device attribute");
    *result = sar_pdhg_result{};

    PdWork w;
    w.st = st;
    CG_CUDA(cudaMallocAsync((void**)&w.y, sizeof(float2) * NS, st), "PDHG dual variable");
    CG_CUDA(cudaMallocAsync((void**)&w.q, sizeof(float2) * NS, st), "PDHG A xbar");
    CG_CUDA(cudaMallocAsync((void**)&w.s, sizeof(float2) * P, st), "PDHG A^H y");
    CG_CUDA(cudaMallocAsync((void**)&w.xbar, sizeof(float2) * P, st), "PDHG xbar");
    CG_CUDA(cudaMallocAsync((void**)&w.sc, sizeof(double) * (2 + (size_t)iterations), st), "PDHG scalars");
    CG_CUDA(cudaMemsetAsync(w.sc, 0, sizeof(double) * (2 + (size_t)iterations), st), "clear scalars");
    float2* x = (float2*)x_dev;
    const float2* b = (const float2*)b_dev;

    if (sigma == 0.0 || tau == 0.0) {
        double nrm = 0.0;
        CG_CALL(estimate_norm(plan, P, NS, norm_iterations, w.xbar, w.q, w.s, w.sc, sms, st, &nrm));
        result->operator_norm = nrm;
        if (!(nrm > 0.0)) return arg_error("PDHG: the operator is zero (no step size from its norm)");
        if (sigma == 0.0 && tau == 0.0) {
            sigma = tau = 1.0 / nrm;
        } else if (sigma == 0.0) {
            sigma = 1.0 / (tau * nrm * nrm);
        } else {
            tau = 1.0 / (sigma * nrm * nrm);
        }
        CG_CUDA(cudaMemsetAsync(w.sc, 0, 2 * sizeof(double), st), "clear scalars");
    }
    result->sigma = sigma;
    result->tau = tau;
    result->theta = theta;

    if (zero_start) CG_CUDA(cudaMemsetAsync(x, 0, sizeof(float2) * P, st), "zero x");
    CG_CUDA(cudaMemcpyAsync(w.xbar, x, sizeof(float2) * P, cudaMemcpyDeviceToDevice, st), "xbar = x0");
    CG_CUDA(cudaMemsetAsync(w.y, 0, sizeof(float2) * NS, st), "y = 0");
    const float fs = (float)sigma, ft = (float)tau, fth = (float)theta;
    const float inv_den = (float)(1.0 / (1.0 + 0.5 * sigma));
    const float thr = (float)(tau * l1_weight);
    for (int it = 0; it < iterations; ++it) {
        CG_CALL(sar_forward(plan, w.xbar, w.q, st));
        pdhg_dual_kernel<<<grid_for(NS, sms), kThreads, 0, st>>>(w.y, w.q, b, NS, fs, inv_den, w.sc + 2 + it);
        CG_CALL(sar_adjoint(plan, w.y, w.s, st));
        pdhg_primal_kernel<<<grid_for(P, sms), kThreads, 0, st>>>(x, w.xbar, w.s, P, ft, thr, fth);
        CG_CUDA(cudaGetLastError(), "PDHG kernels");
    }
    std::vector<double> hist((size_t)iterations);
    if (iterations)
        CG_CUDA(cudaMemcpyAsync(hist.data(), w.sc + 2, sizeof(double) * iterations, cudaMemcpyDeviceToHost, st),
                "read residuals");
    CG_CUDA(cudaStreamSynchronize(st), "PDHG");
    for (int it = 0; it < iterations; ++it) {
        if (!std::isfinite(hist[it])) return arg_error("PDHG: non-finite value during the iteration");
        if (residual_history) residual_history[it] = std::sqrt(hist[it]);
    }
    result->iterations = iterations;
    return SAR_OK;
}
