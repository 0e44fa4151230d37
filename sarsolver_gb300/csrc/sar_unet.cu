// sar_unet.cu -- the learned warm start's network: a 4-level U-Net in bf16 with FP32
// accumulation, trained and run by hand-written kernels (sar_unet_*, sar_conv2d_*, include/sargpu.h).
//
// Network (base width c, a multiple of 32; levels L0..L3 at H, H/2, H/4, H/8):
//   L0  enc0: conv3x3 32->c, conv3x3 c->c                 (input: re, im scaled, padded to 32 ch)
//   L1  enc1: avgpool, conv3x3 c->2c, conv3x3 2c->2c
//   L2  enc2: avgpool, conv3x3 2c->4c, conv3x3 4c->4c
//   L3  bottleneck: avgpool, conv3x3 4c->8c, conv3x3 8c->8c
//   L2  dec2: nearest 2x upsample, concat enc2, conv3x3 12c->4c, conv3x3 4c->4c
//   L1  dec1: upsample, concat enc1, conv3x3 6c->2c, conv3x3 2c->2c
//   L0  dec0: upsample, concat enc0, conv3x3 3c->c, conv3x3 c->c
//   out: conv1x1 c->32 of which channels 0, 1 are the output (re, im), FP32, no activation.
// ReLU after every 3x3 convolution.  Activations NHWC bf16; parameters FP32 (master copy, Adam
// moments, gradients) with bf16 copies of each filter in forward [Cout][tap][Cin] and
// backward-data [Cin][flipped tap][Cout] order.  All convolutions run on the tensor cores
// (unet_tc.cuh); pooling, upsampling, masks, bias gradients and Adam are small elementwise kernels.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/sargpu.h"
#include "sar_kernels.cuh"
#include "unet_tc.cuh"

using bf16 = __nv_bfloat16;

namespace {

// ------------------------------------------------------------------ errors
int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    sar::sar_internal_set_error(buf);
    return code;
}
int cuda_fail(cudaError_t e, const char* what) {
    return fail(e == cudaErrorMemoryAllocation ? SAR_ERR_OUT_OF_MEMORY : SAR_ERR_CUDA, "%s: %s", what,
                cudaGetErrorString(e));
}
#define U_CUDA(call, what)                                  \
    do {                                                    \
        cudaError_t _e = (call);                            \
        if (_e != cudaSuccess) return cuda_fail(_e, what);  \
    } while (0)
#define U_CALL(call)          \
    do {                      \
        int _rc = (call);     \
        if (_rc) return _rc;  \
    } while (0)

// ------------------------------------------------------------------ tensor maps
PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
std::once_flag g_encode_once;

int encoder(PFN_cuTensorMapEncodeTiled_v12000* fn) {
    std::call_once(g_encode_once, [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_encode = (PFN_cuTensorMapEncodeTiled_v12000)f;
    });
    if (!g_encode) return fail(SAR_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
    *fn = g_encode;
    return SAR_OK;
}

CUtensorMapSwizzle swizzle_of(int row_bytes) {
    return row_bytes == 128 ? CU_TENSOR_MAP_SWIZZLE_128B : row_bytes == 64 ? CU_TENSOR_MAP_SWIZZLE_64B
                                                                           : CU_TENSOR_MAP_SWIZZLE_32B;
}

// NHWC bf16 activation [images][H][W][C] as a 4-D map (C, W, H, images), box (cb, bw, bh, 1).
int map_nhwc(CUtensorMap* m, const void* base, int C, int W, int H, int images, int cb, int bw, int bh) {
    PFN_cuTensorMapEncodeTiled_v12000 enc;
    U_CALL(encoder(&enc));
    if (((uintptr_t)base & 15) || (C * 2) % 16) return fail(SAR_ERR_INVALID_ARGUMENT, "activation not 16-byte aligned");
    cuuint64_t dims[4] = {(cuuint64_t)C, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)images};
    cuuint64_t strides[3] = {(cuuint64_t)C * 2, (cuuint64_t)W * C * 2, (cuuint64_t)H * W * C * 2};
    cuuint32_t box[4] = {(cuuint32_t)cb, (cuuint32_t)bw, (cuuint32_t)bh, 1};
    cuuint32_t es[4] = {1, 1, 1, 1};
    CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void*>(base), dims, strides, box, es,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle_of(cb * 2), CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(SAR_ERR_CUDA, "tensor map (activation, C=%d W=%d H=%d): error %d", C, W, H, (int)r);
    return SAR_OK;
}

// Row-major bf16 matrix [rows][cols] as a 2-D map (cols, rows), box (bc, br).
int map_matrix(CUtensorMap* m, const void* base, int cols, int rows, int bc, int br) {
    PFN_cuTensorMapEncodeTiled_v12000 enc;
    U_CALL(encoder(&enc));
    if (((uintptr_t)base & 15) || (cols * 2) % 16) return fail(SAR_ERR_INVALID_ARGUMENT, "matrix not 16-byte aligned");
    cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)cols * 2};
    cuuint32_t box[2] = {(cuuint32_t)bc, (cuuint32_t)br};
    cuuint32_t es[2] = {1, 1};
    CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, es,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle_of(bc * 2), CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(SAR_ERR_CUDA, "tensor map (matrix %dx%d): error %d", rows, cols, (int)r);
    return SAR_OK;
}

int device_sms() {
    int dev = 0, sms = 152;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms;
}

constexpr int kSmemBudget = 200 * 1024;

// ------------------------------------------------------------------ conv launchers
struct Src {
    const bf16* p = nullptr;
    int C = 0;
};
struct Dst {
    bf16* p = nullptr;
    int C = 0;
    const bf16* mask = nullptr;
    int accumulate = 0;
};

int pixel_box(int W, int H, int* bw, int* bh) {
    *bw = std::min(W, 128);
    *bh = 128 / *bw;
    if (*bw * *bh != 128 || W % *bw || H % *bh)
        return fail(SAR_ERR_NOT_SUPPORTED, "image %dx%d: W must be a power of two >= 16 and H a multiple of 128/min(W,128)", W, H);
    return SAR_OK;
}

// y = conv(x0 ++ x1) with weights wk [Nout][taps * (C0 + C1)] (bf16), epilogue per ConvArgs.
int conv_forward(Src s0, Src s1, int images, int H, int W, int taps, const bf16* wk, int Nout, const float* bias,
                 int relu, Dst d0, Dst d1, float* out_f32, int f32_keep, unsigned* flags, cudaStream_t st) {
    using namespace unet;
    const int nsrc = s1.p ? 2 : 1;
    const int Ctot = s0.C + (nsrc > 1 ? s1.C : 0);
    if (s0.C % 32 || (nsrc > 1 && s1.C % 32) || Nout % 32 || Nout <= 0)
        return fail(SAR_ERR_NOT_SUPPORTED, "conv: channel counts must be multiples of 32");
    if (!(taps == 1 || taps == 9)) return fail(SAR_ERR_INVALID_ARGUMENT, "conv: taps must be 1 or 9");
    const bool bk64 = s0.C % 64 == 0 && (nsrc == 1 || s1.C % 64 == 0);
    const int BK = bk64 ? 64 : 32;
    int bw, bh;
    U_CALL(pixel_box(W, H, &bw, &bh));
    int BN = Nout;
    while (BN > 256) {
        if (BN % 2 || (BN / 2) % 32) return fail(SAR_ERR_NOT_SUPPORTED, "conv: output channels %d cannot be tiled", Nout);
        BN /= 2;
    }
    if (!out_f32 && d0.C + (d1.p ? d1.C : 0) != Nout) return fail(SAR_ERR_INVALID_ARGUMENT, "conv: output split != Nout");
    ConvMaps maps;
    memset(&maps, 0, sizeof maps);
    U_CALL(map_nhwc(&maps.src[0], s0.p, s0.C, W, H, images, BK, bw, bh));
    if (nsrc > 1) U_CALL(map_nhwc(&maps.src[1], s1.p, s1.C, W, H, images, BK, bw, bh));
    U_CALL(map_matrix(&maps.wts, wk, taps * Ctot, Nout, BK, BN));
    ConvArgs a;
    memset(&a, 0, sizeof a);
    a.nsrc = nsrc;
    a.C0 = s0.C;
    a.C1 = nsrc > 1 ? s1.C : 0;
    a.Ctot = Ctot;
    a.taps = taps;
    a.W = W;
    a.H = H;
    a.BW = bw;
    a.BH = bh;
    a.tiles_x = W / bw;
    a.tiles_y = H / bh;
    a.BN = BN;
    a.Nout = Nout;
    const int stage = (128 + BN) * BK * 2;
    a.stages = std::max(2, std::min(8, (kSmemBudget - 2048) / stage));
    a.bias = bias;
    a.relu = relu;
    a.out[0] = d0.p;
    a.out[1] = d1.p;
    a.outc[0] = d0.C;
    a.outc[1] = d1.C;
    a.mask[0] = d0.mask;
    a.mask[1] = d1.mask;
    a.accumulate[0] = d0.accumulate;
    a.accumulate[1] = d1.accumulate;
    a.out_f32 = out_f32;
    a.f32_keep = f32_keep;
    a.flags = flags;
    size_t smem = 1024 + (size_t)a.stages * stage + (2 * a.stages + 4) * 8 + 16;
    // Persistent grid: as many CTAs as fit on the SMs, by shared memory and by TMEM (two
    // accumulators each).  When TMEM is the tighter limit the shared-memory request is raised so
    // that no more CTAs than that share an SM (a CTA beyond it would wait in tcgen05.alloc).
    a.images = images;
    const int items = images * a.tiles_x * a.tiles_y * (Nout / BN);
    const size_t sm_smem = 227u * 1024u;
    const int by_smem = std::max(1, (int)(sm_smem / smem));
    const int by_tmem = std::max(1, (int)(512u / (2u * tmem_cols(BN))));
    const int per_sm = std::max(1, std::min(by_smem, by_tmem));
    if (by_tmem < by_smem) smem = std::max(smem, sm_smem / (size_t)(per_sm + 1) + 1024);
    dim3 grid((unsigned)std::min(items, device_sms() * per_sm));
    if (bk64) {
        U_CUDA(cudaFuncSetAttribute(conv_fwd_kernel<64>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem), "smem attr");
        conv_fwd_kernel<64><<<grid, kThreads, smem, st>>>(maps, a);
    } else {
        U_CUDA(cudaFuncSetAttribute(conv_fwd_kernel<32>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem), "smem attr");
        conv_fwd_kernel<32><<<grid, kThreads, smem, st>>>(maps, a);
    }
    U_CUDA(cudaGetLastError(), "conv forward launch");
    return SAR_OK;
}

// dw[Cout][taps * Ctot] += sum_pixels dz[p][co] * (x0 ++ x1)[p + tap][ci]  (FP32 accumulate).
int conv_wgrad(Src s0, Src s1, const bf16* dz, int Cout, int images, int H, int W, int taps, float* dw,
               unsigned* flags, cudaStream_t st) {
    using namespace unet;
    const int nsrc = s1.p ? 2 : 1;
    const int Ctot = s0.C + (nsrc > 1 ? s1.C : 0);
    if (s0.C % 32 || (nsrc > 1 && s1.C % 32) || Cout % 32) return fail(SAR_ERR_NOT_SUPPORTED, "wgrad: channels must be multiples of 32");
    const bool ci64 = s0.C % 64 == 0 && (nsrc == 1 || s1.C % 64 == 0);
    const bool co64 = Cout % 64 == 0;
    const int CIB = ci64 ? 64 : 32, COB = co64 ? 64 : 32;
    int bw, bh;
    U_CALL(pixel_box(W, H, &bw, &bh));
    const int BN = std::min(Cout, 128);
    if (Cout % BN) return fail(SAR_ERR_NOT_SUPPORTED, "wgrad: output channels %d cannot be tiled", Cout);
    WgradMaps maps;
    memset(&maps, 0, sizeof maps);
    U_CALL(map_nhwc(&maps.x[0], s0.p, s0.C, W, H, images, CIB, bw, bh));
    if (nsrc > 1) U_CALL(map_nhwc(&maps.x[1], s1.p, s1.C, W, H, images, CIB, bw, bh));
    U_CALL(map_nhwc(&maps.dz, dz, Cout, W, H, images, COB, bw, bh));
    WgradArgs a;
    memset(&a, 0, sizeof a);
    a.nsrc = nsrc;
    a.C0 = s0.C;
    a.C1 = nsrc > 1 ? s1.C : 0;
    a.Ctot = Ctot;
    a.taps = taps;
    a.Cout = Cout;
    a.W = W;
    a.H = H;
    a.BW = bw;
    a.BH = bh;
    a.tiles_x = W / bw;
    a.tiles_y = H / bh;
    a.num_tiles = images * a.tiles_x * a.tiles_y;
    a.BN = BN;
    const int tpg = 128 / CIB;
    const int ngroups = (taps + tpg - 1) / tpg;
    const int mtiles = ngroups * (Ctot / CIB), ntiles = Cout / BN;
    const int want = 3 * device_sms();
    int splits = std::max(1, std::min(a.num_tiles, (want + mtiles * ntiles - 1) / (mtiles * ntiles)));
    a.tiles_per_split = (a.num_tiles + splits - 1) / splits;
    splits = (a.num_tiles + a.tiles_per_split - 1) / a.tiles_per_split;
    const int stage = 128 * 128 * 2 + BN * 128 * 2;
    a.stages = std::max(2, std::min(6, (kSmemBudget - 2048) / stage));
    a.dw = dw;
    a.flags = flags;
    const size_t smem = 1024 + (size_t)a.stages * stage + (2 * a.stages + 2) * 8 + 16;
    dim3 grid((unsigned)splits, (unsigned)mtiles, (unsigned)ntiles);
#define U_WG(CI, CO)                                                                                                 \
    do {                                                                                                             \
        U_CUDA(cudaFuncSetAttribute(conv_wgrad_kernel<CI, CO>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem), \
               "smem attr");                                                                                         \
        conv_wgrad_kernel<CI, CO><<<grid, kThreads, smem, st>>>(maps, a);                                            \
    } while (0)
    if (ci64 && co64) U_WG(64, 64);
    else if (ci64) U_WG(64, 32);
    else if (co64) U_WG(32, 64);
    else U_WG(32, 32);
#undef U_WG
    U_CUDA(cudaGetLastError(), "wgrad launch");
    return SAR_OK;
}

// ------------------------------------------------------------------ elementwise kernels
__device__ __forceinline__ float bf(bf16 v) { return __bfloat162float(v); }

// complex64 image -> bf16 NHWC [P][32]: channels 0, 1 = scale * (re, im), the rest zero.
__global__ void prep_input_kernel(const float2* __restrict__ z, float scale, bf16* __restrict__ out, size_t P) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < P * 4; i += (size_t)gridDim.x * blockDim.x) {
        const size_t p = i >> 2;
        uint4 pk = make_uint4(0, 0, 0, 0);
        if ((i & 3) == 0) {
            const float2 v = z[p];
            __nv_bfloat162 h = __floats2bfloat162_rn(scale * v.x, scale * v.y);
            pk.x = *reinterpret_cast<uint32_t*>(&h);
        }
        reinterpret_cast<uint4*>(out)[i] = pk;
    }
}

// 2x2 average pool, NHWC: in [n][2h][2w][C] -> out [n][h][w][C].
__global__ void avgpool_kernel(const bf16* __restrict__ in, bf16* __restrict__ out, int images, int H, int W, int C) {
    const int h = H / 2, w = W / 2, cv = C / 2;
    const size_t total = (size_t)images * h * w * cv;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const int c2 = (int)(i % cv);
        size_t r = i / cv;
        const int x = (int)(r % w);
        r /= w;
        const int y = (int)(r % h);
        const size_t n = r / h;
        const __nv_bfloat162* src = reinterpret_cast<const __nv_bfloat162*>(in);
        const size_t b = ((n * H + 2 * y) * W + 2 * x) * cv + c2;
        const float2 a = __bfloat1622float2(src[b]), bb = __bfloat1622float2(src[b + cv]);
        const float2 c = __bfloat1622float2(src[b + (size_t)W * cv]), d = __bfloat1622float2(src[b + (size_t)W * cv + cv]);
        reinterpret_cast<__nv_bfloat162*>(out)[i] =
            __floats2bfloat162_rn(0.25f * (a.x + bb.x + c.x + d.x), 0.25f * (a.y + bb.y + c.y + d.y));
    }
}

// Nearest 2x upsample, NHWC: in [n][h][w][C] -> out [n][2h][2w][C].
__global__ void upsample_kernel(const bf16* __restrict__ in, bf16* __restrict__ out, int images, int h, int w, int C) {
    const int cv = C / 8;   // 16-byte vectors
    const size_t total = (size_t)images * 4 * h * w * cv;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const int c = (int)(i % cv);
        size_t r = i / cv;
        const int X = (int)(r % (2 * w));
        r /= 2 * w;
        const int Y = (int)(r % (2 * h));
        const size_t n = r / (2 * h);
        reinterpret_cast<uint4*>(out)[i] = reinterpret_cast<const uint4*>(in)[((n * h + Y / 2) * w + X / 2) * cv + c];
    }
}

// Backward of the nearest upsample followed by the ReLU mask of its input:
// out[n][y][x][c] = (sum of g over the 2x2 children) * (act[n][y][x][c] > 0).
__global__ void upsample_bwd_mask_kernel(const bf16* __restrict__ g, const bf16* __restrict__ act, bf16* __restrict__ out,
                                         int images, int h, int w, int C) {
    const int cv = C / 2;
    const size_t total = (size_t)images * h * w * cv;
    const __nv_bfloat162* g2 = reinterpret_cast<const __nv_bfloat162*>(g);
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const int c2 = (int)(i % cv);
        size_t r = i / cv;
        const int x = (int)(r % w);
        r /= w;
        const int y = (int)(r % h);
        const size_t n = r / h;
        const size_t W2 = 2 * (size_t)w;
        const size_t b = ((n * 2 * h + 2 * y) * W2 + 2 * x) * cv + c2;
        const float2 a = __bfloat1622float2(g2[b]), bb = __bfloat1622float2(g2[b + cv]);
        const float2 c = __bfloat1622float2(g2[b + W2 * cv]), d = __bfloat1622float2(g2[b + W2 * cv + cv]);
        const float2 m = __bfloat1622float2(reinterpret_cast<const __nv_bfloat162*>(act)[i]);
        const float sx = m.x > 0.f ? a.x + bb.x + c.x + d.x : 0.f;
        const float sy = m.y > 0.f ? a.y + bb.y + c.y + d.y : 0.f;
        reinterpret_cast<__nv_bfloat162*>(out)[i] = __floats2bfloat162_rn(sx, sy);
    }
}

// Gradient of an encoder output that feeds both a skip connection and a 2x2 average pool:
// out = (g_skip + g_pool[parent] / 4) * (act > 0), all [n][H][W][C] except g_pool [n][H/2][W/2][C].
__global__ void pool_bwd_add_mask_kernel(const bf16* __restrict__ gpool, const bf16* __restrict__ gskip,
                                         const bf16* __restrict__ act, bf16* __restrict__ out, int images, int H, int W,
                                         int C) {
    const int cv = C / 2;
    const size_t total = (size_t)images * H * W * cv;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const int c2 = (int)(i % cv);
        size_t r = i / cv;
        const int x = (int)(r % W);
        r /= W;
        const int y = (int)(r % H);
        const size_t n = r / H;
        const float2 gp = __bfloat1622float2(
            reinterpret_cast<const __nv_bfloat162*>(gpool)[((n * (H / 2) + y / 2) * (W / 2) + x / 2) * cv + c2]);
        const float2 gs = __bfloat1622float2(reinterpret_cast<const __nv_bfloat162*>(gskip)[i]);
        const float2 m = __bfloat1622float2(reinterpret_cast<const __nv_bfloat162*>(act)[i]);
        reinterpret_cast<__nv_bfloat162*>(out)[i] =
            __floats2bfloat162_rn(m.x > 0.f ? gs.x + 0.25f * gp.x : 0.f, m.y > 0.f ? gs.y + 0.25f * gp.y : 0.f);
    }
}

// db[c] += sum_p dz[p][c].  256 threads = (256 / C) pixel lanes x C channels (C divides 256),
// grid-stride over pixels with coalesced rows, a shared-memory sum over the pixel lanes and one
// atomic per channel per CTA.
__global__ void bias_grad_kernel(const bf16* __restrict__ dz, size_t P, int C, float* __restrict__ db) {
    __shared__ float part[256];
    const int lanes = blockDim.x / C, c = threadIdx.x % C, pl = threadIdx.x / C;
    float acc = 0.f;
    for (size_t p = (size_t)blockIdx.x * lanes + pl; p < P; p += (size_t)gridDim.x * lanes) acc += bf(dz[p * C + c]);
    part[threadIdx.x] = acc;
    __syncthreads();
    if (threadIdx.x < C) {
        float sum = 0.f;
        for (int l = 0; l < lanes; ++l) sum += part[l * C + threadIdx.x];
        atomicAdd(db + threadIdx.x, sum);
    }
}

// FP32 master -> bf16 forward [Cout][tap][Cin] and backward-data [Cin][8 - tap][Cout] copies.
__global__ void weight_prep_kernel(const float* __restrict__ w, bf16* __restrict__ wf, bf16* __restrict__ wt, int Cout,
                                   int taps, int Cin) {
    const size_t total = (size_t)Cout * taps * Cin;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const int ci = (int)(i % Cin);
        const int tap = (int)((i / Cin) % taps);
        const int co = (int)(i / ((size_t)Cin * taps));
        const bf16 v = __float2bfloat16_rn(w[i]);
        wf[i] = v;
        wt[((size_t)ci * taps + (taps - 1 - tap)) * Cout + co] = v;
    }
}

__global__ void adam_kernel(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                            size_t n, float lr, float b1, float b2, float eps, float bc1, float bc2) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        p[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
    }
}

unsigned ew_grid(size_t n) {
    const size_t want = (n + 255) / 256;
    return (unsigned)std::max<size_t>(1, std::min<size_t>(want, (size_t)device_sms() * 16));
}


// ------------------------------------------------------------------ network
constexpr int kLayers = SAR_UNET_LAYERS;

struct LayerSpec {
    int c0, c1, cout, taps, relu, level;
};

}  // namespace

struct sar_unet {
    int device = 0, c = 32;
    LayerSpec L[kLayers];
    size_t w_off[kLayers], b_off[kLayers], n_params = 0;
    float *params = nullptr, *grads = nullptr, *m = nullptr, *v = nullptr;
    bf16 *wf[kLayers] = {}, *wt[kLayers] = {};
    bf16* wbuf = nullptr;
    unsigned* flags = nullptr;
    // activations and gradients of the current (B, H, W)
    int B = 0, H = 0, W = 0;
    std::vector<void*> bufs;
    bf16 *in0 = nullptr, *a[14] = {}, *p[3] = {}, *u[3] = {};
    bf16 *dz[kLayers] = {}, *du[3] = {}, *de[3] = {}, *dp[3] = {};
    bool have_forward = false;
    std::mutex mu;

    size_t pixels(int level) const { return (size_t)B * (size_t)(H >> level) * (size_t)(W >> level); }

    ~sar_unet() {
        int prev = -1;
        cudaGetDevice(&prev);
        cudaSetDevice(device);
        release_activations();
        for (void* q : {(void*)params, (void*)grads, (void*)m, (void*)v, (void*)wbuf, (void*)flags})
            if (q) cudaFree(q);
        if (prev >= 0) cudaSetDevice(prev);
    }
    void release_activations() {
        for (void* q : bufs) cudaFree(q);
        bufs.clear();
        B = H = W = 0;
        have_forward = false;
    }
    int alloc_bf16(bf16** q, size_t n) {
        void* ptr = nullptr;
        U_CUDA(cudaMalloc(&ptr, std::max<size_t>(n, 8) * sizeof(bf16)), "U-Net activations");
        bufs.push_back(ptr);
        *q = (bf16*)ptr;
        return SAR_OK;
    }
    int ensure_activations(int b, int h, int w) {
        if (b == B && h == H && w == W) return SAR_OK;
        release_activations();
        B = b;
        H = h;
        W = w;
        U_CALL(alloc_bf16(&in0, pixels(0) * 32));
        for (int i = 0; i < 14; ++i) U_CALL(alloc_bf16(&a[i], pixels(L[i].level) * L[i].cout));
        for (int l = 0; l < 3; ++l) {
            U_CALL(alloc_bf16(&p[l], pixels(l + 1) * (c << l)));       // pooled encoder output, level l+1
            U_CALL(alloc_bf16(&u[l], pixels(l) * (c << (l + 1))));     // upsampled decoder input, level l
            U_CALL(alloc_bf16(&du[l], pixels(l) * (c << (l + 1))));
            U_CALL(alloc_bf16(&de[l], pixels(l) * (c << l)));
            U_CALL(alloc_bf16(&dp[l], pixels(l + 1) * (c << l)));
        }
        for (int i = 0; i < kLayers; ++i) U_CALL(alloc_bf16(&dz[i], pixels(L[i].level) * L[i].cout));
        return SAR_OK;
    }
    int refresh_weights(cudaStream_t st) {
        for (int i = 0; i < kLayers; ++i) {
            const int cin = L[i].c0 + L[i].c1;
            const size_t n = (size_t)L[i].cout * L[i].taps * cin;
            weight_prep_kernel<<<ew_grid(n), 256, 0, st>>>(params + w_off[i], wf[i], wt[i], L[i].cout, L[i].taps, cin);
        }
        U_CUDA(cudaGetLastError(), "weight prep");
        return SAR_OK;
    }
    // Sources of layer i's input in concatenation order.
    void inputs(int i, Src* s0, Src* s1) const {
        static const int prev[kLayers] = {-1, 0, -2, 2, -3, 4, -4, 6, -5, 8, -6, 10, -7, 12, 13};
        *s1 = Src{};
        switch (i) {
            case 0: *s0 = Src{in0, 32}; break;
            case 2: *s0 = Src{p[0], c}; break;
            case 4: *s0 = Src{p[1], 2 * c}; break;
            case 6: *s0 = Src{p[2], 4 * c}; break;
            case 8: *s0 = Src{u[2], 8 * c}; *s1 = Src{a[5], 4 * c}; break;
            case 10: *s0 = Src{u[1], 4 * c}; *s1 = Src{a[3], 2 * c}; break;
            case 12: *s0 = Src{u[0], 2 * c}; *s1 = Src{a[1], c}; break;
            default: *s0 = Src{a[prev[i]], L[prev[i]].cout}; break;
        }
    }
};

namespace {

int layer_forward(sar_unet* n, int i, float* out_f32, cudaStream_t st) {
    const LayerSpec& l = n->L[i];
    Src s0, s1;
    n->inputs(i, &s0, &s1);
    const int h = n->H >> l.level, w = n->W >> l.level;
    Dst d0{i < 14 ? n->a[i] : nullptr, l.cout, nullptr, 0};
    return conv_forward(s0, s1, n->B, h, w, l.taps, n->wf[i], l.cout, n->params + n->b_off[i], l.relu, d0, Dst{},
                        i == 14 ? out_f32 : nullptr, 2, n->flags, st);
}

// Weight and bias gradients of layer i from dz[i], then (i > 0) the gradient of its input.
int layer_backward(sar_unet* n, int i, cudaStream_t st) {
    const LayerSpec& l = n->L[i];
    Src s0, s1;
    n->inputs(i, &s0, &s1);
    const int h = n->H >> l.level, w = n->W >> l.level;
    const size_t P = n->pixels(l.level);
    U_CALL(conv_wgrad(s0, s1, n->dz[i], l.cout, n->B, h, w, l.taps, n->grads + n->w_off[i], n->flags, st));
    const size_t lanes = 256 / l.cout;
    bias_grad_kernel<<<(unsigned)std::max<size_t>(1, std::min<size_t>((size_t)device_sms() * 4, P / (lanes * 16))), 256,
                       0, st>>>(n->dz[i], P, l.cout, n->grads + n->b_off[i]);
    U_CUDA(cudaGetLastError(), "bias gradient");
    if (i == 0) return SAR_OK;
    Dst d0, d1;
    switch (i) {
        case 2: d0 = Dst{n->dp[0], l.c0, nullptr, 0}; break;
        case 4: d0 = Dst{n->dp[1], l.c0, nullptr, 0}; break;
        case 6: d0 = Dst{n->dp[2], l.c0, nullptr, 0}; break;
        case 8: d0 = Dst{n->du[2], l.c0, nullptr, 0}; d1 = Dst{n->de[2], l.c1, nullptr, 0}; break;
        case 10: d0 = Dst{n->du[1], l.c0, nullptr, 0}; d1 = Dst{n->de[1], l.c1, nullptr, 0}; break;
        case 12: d0 = Dst{n->du[0], l.c0, nullptr, 0}; d1 = Dst{n->de[0], l.c1, nullptr, 0}; break;
        default: d0 = Dst{n->dz[i - 1], l.c0, s0.p, 0}; break;   // previous layer feeds this one directly
    }
    // Backward data: dX = conv(dz, flipped transposed filter); its input channels are l.cout.
    return conv_forward(Src{n->dz[i], l.cout}, Src{}, n->B, h, w, l.taps, n->wt[i], l.c0 + l.c1, nullptr, 0, d0, d1,
                        nullptr, 0, n->flags, st);
}

int do_forward(sar_unet* n, const float2* in, float scale, float* out, cudaStream_t st) {
    const size_t P0 = n->pixels(0);
    prep_input_kernel<<<ew_grid(P0 * 4), 256, 0, st>>>(in, scale, n->in0, P0);
    U_CUDA(cudaGetLastError(), "input");
    for (int lvl = 0; lvl < 4; ++lvl) {
        const int i0 = 2 * lvl;
        U_CALL(layer_forward(n, i0, nullptr, st));
        U_CALL(layer_forward(n, i0 + 1, nullptr, st));
        if (lvl < 3) {
            const size_t np = n->pixels(lvl + 1) * (size_t)(n->c << lvl) / 2;
            avgpool_kernel<<<ew_grid(np), 256, 0, st>>>(n->a[i0 + 1], n->p[lvl], n->B, n->H >> lvl, n->W >> lvl,
                                                        n->c << lvl);
        }
    }
    for (int lvl = 2; lvl >= 0; --lvl) {
        const int src = lvl == 2 ? 7 : (lvl == 1 ? 9 : 11);   // decoder input from the level below
        const int C = n->L[src].cout;
        const size_t nu = n->pixels(lvl) * (size_t)C / 8;
        upsample_kernel<<<ew_grid(nu), 256, 0, st>>>(n->a[src], n->u[lvl], n->B, n->H >> (lvl + 1), n->W >> (lvl + 1), C);
        const int i0 = lvl == 2 ? 8 : (lvl == 1 ? 10 : 12);
        U_CALL(layer_forward(n, i0, nullptr, st));
        U_CALL(layer_forward(n, i0 + 1, nullptr, st));
    }
    U_CALL(layer_forward(n, 14, out, st));
    U_CUDA(cudaGetLastError(), "U-Net forward");
    return SAR_OK;
}

int do_backward(sar_unet* n, const float2* gout, cudaStream_t st) {
    const size_t P0 = n->pixels(0);
    prep_input_kernel<<<ew_grid(P0 * 4), 256, 0, st>>>(gout, 1.f, n->dz[14], P0);
    U_CALL(layer_backward(n, 14, st));   // -> dz[13]
    U_CALL(layer_backward(n, 13, st));   // -> dz[12]
    // Decoder, top level first: concat conv -> (du, de); du -> gradient of the level below.
    for (int lvl = 0; lvl <= 2; ++lvl) {
        const int cat = 12 - 2 * lvl;          // 12, 10, 8
        if (lvl > 0) U_CALL(layer_backward(n, cat + 1, st));
        U_CALL(layer_backward(n, cat, st));    // -> du[lvl], de[lvl]
        const int below = cat - 1;             // 11, 9, 7: output upsampled into this level
        const int C = n->L[below].cout;
        const size_t nb = n->pixels(lvl + 1) * (size_t)C / 2;
        upsample_bwd_mask_kernel<<<ew_grid(nb), 256, 0, st>>>(n->du[lvl], n->a[below], n->dz[below], n->B,
                                                              n->H >> (lvl + 1), n->W >> (lvl + 1), C);
    }
    U_CALL(layer_backward(n, 7, st));          // bottleneck -> dz[6]
    // Encoder, bottom level first: first conv of level lvl -> dp[lvl-1]; pooled + skip gradients
    // of the encoder output below; then that level's second conv.
    for (int lvl = 3; lvl >= 1; --lvl) {
        const int first = 2 * lvl;             // 6, 4, 2
        U_CALL(layer_backward(n, first, st));  // -> dp[lvl - 1]
        const int enc = first - 1;             // 5, 3, 1
        const int C = n->L[enc].cout;
        const size_t ne = n->pixels(lvl - 1) * (size_t)C / 2;
        pool_bwd_add_mask_kernel<<<ew_grid(ne), 256, 0, st>>>(n->dp[lvl - 1], n->de[lvl - 1], n->a[enc], n->dz[enc], n->B,
                                                              n->H >> (lvl - 1), n->W >> (lvl - 1), C);
        U_CALL(layer_backward(n, enc, st));    // -> dz[enc - 1]
    }
    U_CALL(layer_backward(n, 0, st));
    U_CUDA(cudaGetLastError(), "U-Net backward");
    return SAR_OK;
}

struct DevScope {
    int prev = -1, target;
    cudaError_t status = cudaSuccess;
    explicit DevScope(int d) : target(d) {
        status = cudaGetDevice(&prev);
        if (status == cudaSuccess && prev != d) status = cudaSetDevice(d);
    }
    ~DevScope() {
        if (prev >= 0 && prev != target) cudaSetDevice(prev);
    }
};

}  // namespace

// ------------------------------------------------------------------ C ABI
extern "C" {

int sar_unet_create(int base_channels, int device, sar_unet** out) {
    if (!out) return fail(SAR_ERR_INVALID_ARGUMENT, "null argument");
    *out = nullptr;
    if (base_channels <= 0 || base_channels % 32 || base_channels > 64)
        return fail(SAR_ERR_NOT_SUPPORTED, "base_channels must be 32 or 64");
    if (device < 0 && cudaGetDevice(&device) != cudaSuccess) return fail(SAR_ERR_CUDA, "no current device");
    DevScope scope(device);
    if (scope.status != cudaSuccess) return cuda_fail(scope.status, "select device");
    sar_unet* n = new (std::nothrow) sar_unet();
    if (!n) return fail(SAR_ERR_OUT_OF_MEMORY, "host allocation");
    n->device = device;
    const int c = base_channels;
    n->c = c;
    const LayerSpec spec[kLayers] = {
        {32, 0, c, 9, 1, 0},          {c, 0, c, 9, 1, 0},          {c, 0, 2 * c, 9, 1, 1},
        {2 * c, 0, 2 * c, 9, 1, 1},   {2 * c, 0, 4 * c, 9, 1, 2},  {4 * c, 0, 4 * c, 9, 1, 2},
        {4 * c, 0, 8 * c, 9, 1, 3},   {8 * c, 0, 8 * c, 9, 1, 3},  {8 * c, 4 * c, 4 * c, 9, 1, 2},
        {4 * c, 0, 4 * c, 9, 1, 2},   {4 * c, 2 * c, 2 * c, 9, 1, 1}, {2 * c, 0, 2 * c, 9, 1, 1},
        {2 * c, c, c, 9, 1, 0},       {c, 0, c, 9, 1, 0},          {c, 0, 32, 1, 0, 0}};
    size_t off = 0, woff = 0;
    for (int i = 0; i < kLayers; ++i) {
        n->L[i] = spec[i];
        const size_t nw = (size_t)spec[i].cout * spec[i].taps * (spec[i].c0 + spec[i].c1);
        n->w_off[i] = off;
        off += nw;
        n->b_off[i] = off;
        off += spec[i].cout;
        woff += nw;
    }
    n->n_params = off;
    int rc = SAR_OK;
    auto get = [&](void** q, size_t bytes) {
        if (rc == SAR_OK && cudaMalloc(q, bytes) != cudaSuccess) rc = fail(SAR_ERR_OUT_OF_MEMORY, "U-Net parameters");
    };
    get((void**)&n->params, off * 4);
    get((void**)&n->grads, off * 4);
    get((void**)&n->m, off * 4);
    get((void**)&n->v, off * 4);
    get((void**)&n->wbuf, woff * 2 * sizeof(bf16));
    get((void**)&n->flags, 16);
    if (rc) {
        delete n;
        return rc;
    }
    size_t wo = 0;
    for (int i = 0; i < kLayers; ++i) {
        const size_t nw = (size_t)spec[i].cout * spec[i].taps * (spec[i].c0 + spec[i].c1);
        n->wf[i] = n->wbuf + wo;
        n->wt[i] = n->wbuf + woff + wo;
        wo += nw;
    }
    cudaMemset(n->params, 0, off * 4);
    cudaMemset(n->grads, 0, off * 4);
    cudaMemset(n->m, 0, off * 4);
    cudaMemset(n->v, 0, off * 4);
    cudaMemset(n->wbuf, 0, woff * 2 * sizeof(bf16));
    if (cudaMemset(n->flags, 0, 16) != cudaSuccess) {
        delete n;
        return fail(SAR_ERR_CUDA, "U-Net initialisation");
    }
    *out = n;
    return SAR_OK;
}

int sar_unet_destroy(sar_unet* n) {
    delete n;
    return SAR_OK;
}

int sar_unet_info(const sar_unet* n, size_t* num_params, sar_unet_layer* layers) {
    if (!n) return fail(SAR_ERR_INVALID_ARGUMENT, "null argument");
    if (num_params) *num_params = n->n_params;
    if (layers)
        for (int i = 0; i < kLayers; ++i) {
            layers[i].weight_offset = n->w_off[i];
            layers[i].bias_offset = n->b_off[i];
            layers[i].cin0 = n->L[i].c0;
            layers[i].cin1 = n->L[i].c1;
            layers[i].cout = n->L[i].cout;
            layers[i].taps = n->L[i].taps;
            layers[i].relu = n->L[i].relu;
            layers[i].level = n->L[i].level;
        }
    return SAR_OK;
}

int sar_unet_set_params(sar_unet* n, const float* params_dev, void* stream) {
    if (!n || !params_dev) return fail(SAR_ERR_INVALID_ARGUMENT, "null argument");
    std::lock_guard<std::mutex> lock(n->mu);
    DevScope scope(n->device);
    cudaStream_t st = (cudaStream_t)stream;
    U_CUDA(cudaMemcpyAsync(n->params, params_dev, n->n_params * 4, cudaMemcpyDeviceToDevice, st), "set params");
    U_CUDA(cudaMemsetAsync(n->m, 0, n->n_params * 4, st), "reset moments");
    U_CUDA(cudaMemsetAsync(n->v, 0, n->n_params * 4, st), "reset moments");
    return n->refresh_weights(st);
}

int sar_unet_get_params(const sar_unet* n, float* params_dev, void* stream) {
    if (!n || !params_dev) return fail(SAR_ERR_INVALID_ARGUMENT, "null argument");
    DevScope scope(n->device);
    U_CUDA(cudaMemcpyAsync(params_dev, n->params, n->n_params * 4, cudaMemcpyDeviceToDevice, (cudaStream_t)stream),
           "get params");
    return SAR_OK;
}

int sar_unet_get_grads(const sar_unet* n, float* grads_dev, void* stream) {
    if (!n || !grads_dev) return fail(SAR_ERR_INVALID_ARGUMENT, "null argument");
    DevScope scope(n->device);
    U_CUDA(cudaMemcpyAsync(grads_dev, n->grads, n->n_params * 4, cudaMemcpyDeviceToDevice, (cudaStream_t)stream),
           "get grads");
    return SAR_OK;
}

int sar_unet_zero_grad(sar_unet* n, void* stream) {
    if (!n) return fail(SAR_ERR_INVALID_ARGUMENT, "null argument");
    DevScope scope(n->device);
    U_CUDA(cudaMemsetAsync(n->grads, 0, n->n_params * 4, (cudaStream_t)stream), "zero grads");
    return SAR_OK;
}

int sar_unet_forward(sar_unet* n, const void* in_dev, float in_scale, int batch, int height, int width, void* out_dev,
                     void* stream) {
    if (!n || !in_dev || !out_dev) return fail(SAR_ERR_INVALID_ARGUMENT, "null argument");
    if (batch <= 0 || height <= 0 || width <= 0 || height % 8 || width % 8)
        return fail(SAR_ERR_INVALID_ARGUMENT, "batch, height and width must be positive, height and width multiples of 8");
    if ((width >> 3) < 16 || ((width >> 3) & ((width >> 3) - 1)) || ((height >> 3) % std::max(1, 128 / std::min(width >> 3, 128))))
        return fail(SAR_ERR_NOT_SUPPORTED, "image %dx%d: width/8 must be a power of two >= 16", width, height);
    std::lock_guard<std::mutex> lock(n->mu);
    DevScope scope(n->device);
    if (scope.status != cudaSuccess) return cuda_fail(scope.status, "select device");
    U_CALL(n->ensure_activations(batch, height, width));
    U_CALL(do_forward(n, (const float2*)in_dev, in_scale, (float*)out_dev, (cudaStream_t)stream));
    n->have_forward = true;
    return SAR_OK;
}

int sar_unet_backward(sar_unet* n, const void* grad_out_dev, void* stream) {
    if (!n || !grad_out_dev) return fail(SAR_ERR_INVALID_ARGUMENT, "null argument");
    std::lock_guard<std::mutex> lock(n->mu);
    if (!n->have_forward) return fail(SAR_ERR_INVALID_ARGUMENT, "sar_unet_backward needs a preceding sar_unet_forward");
    DevScope scope(n->device);
    return do_backward(n, (const float2*)grad_out_dev, (cudaStream_t)stream);
}

int sar_unet_adam_step(sar_unet* n, float lr, float beta1, float beta2, float eps, int step, void* stream) {
    if (!n || step < 1) return fail(SAR_ERR_INVALID_ARGUMENT, "null argument or step < 1");
    std::lock_guard<std::mutex> lock(n->mu);
    DevScope scope(n->device);
    cudaStream_t st = (cudaStream_t)stream;
    const float bc1 = 1.f - std::pow(beta1, (float)step), bc2 = 1.f - std::pow(beta2, (float)step);
    adam_kernel<<<ew_grid(n->n_params), 256, 0, st>>>(n->params, n->grads, n->m, n->v, n->n_params, lr, beta1, beta2,
                                                      eps, bc1, bc2);
    U_CUDA(cudaGetLastError(), "adam");
    return n->refresh_weights(st);
}

int sar_unet_flags(sar_unet* n, unsigned* flags) {
    if (!n || !flags) return fail(SAR_ERR_INVALID_ARGUMENT, "null argument");
    DevScope scope(n->device);
    U_CUDA(cudaDeviceSynchronize(), "synchronise");
    U_CUDA(cudaMemcpy(flags, n->flags, sizeof(unsigned), cudaMemcpyDeviceToHost), "read flags");
    U_CUDA(cudaMemset(n->flags, 0, sizeof(unsigned)), "clear flags");
    return SAR_OK;
}

int sar_conv2d_forward_bf16(const void* x0, int c0, const void* x1, int c1, int batch, int height, int width, int taps,
                            const void* w, const float* bias, int cout, int relu, void* y, unsigned* flags_dev,
                            void* stream) {
    if (!x0 || !w || !y || !flags_dev) return fail(SAR_ERR_INVALID_ARGUMENT, "null argument");
    return conv_forward(Src{(const bf16*)x0, c0}, Src{(const bf16*)x1, x1 ? c1 : 0}, batch, height, width, taps,
                        (const bf16*)w, cout, bias, relu, Dst{(bf16*)y, cout, nullptr, 0}, Dst{}, nullptr, 0, flags_dev,
                        (cudaStream_t)stream);
}

int sar_conv2d_wgrad_bf16(const void* x0, int c0, const void* x1, int c1, const void* dz, int cout, int batch, int height,
                          int width, int taps, float* dw, unsigned* flags_dev, void* stream) {
    if (!x0 || !dz || !dw || !flags_dev) return fail(SAR_ERR_INVALID_ARGUMENT, "null argument");
    return conv_wgrad(Src{(const bf16*)x0, c0}, Src{(const bf16*)x1, x1 ? c1 : 0}, (const bf16*)dz, cout, batch, height,
                      width, taps, dw, flags_dev, (cudaStream_t)stream);
}

}  // extern "C"
