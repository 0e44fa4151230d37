// unet_tc.cuh -- tensor-core (tcgen05 + TMA) convolution kernels of the learned warm start.
//
// Activations are NHWC bf16 tensors whose channel counts are multiples of 32.  Two kernels cover
// every convolution of the U-Net, forward and backward:
//
//  * conv_fwd_kernel<BK>: implicit GEMM  D[pixel][n] = sum_{tap, c} X[pixel + tap][c] * Wk[n][tap, c]
//    for 3x3 (pad 1) or 1x1 filters over one or two channel-concatenated sources.  M = 128 pixels
//    of one image (a BW x BH box), N = BN output channels, K stepped in blocks of BK channels of
//    one tap.  Each K block is one 4-D TMA box of the source at (c, x + dx, y + dy, image): the
//    tap shift moves the W/H coordinates, and out-of-image rows and columns arrive as zeros (the
//    padding).  Weights come as 2-D TMA boxes of the [N][taps * C] matrix.  Both operands are
//    K-major with a BK * 2-byte swizzle (128 B for BK = 64, 64 B for BK = 32).  The same kernel
//    runs the backward-data pass with the flipped, transposed filter.  The epilogue adds the
//    bias, applies ReLU or a ReLU-derivative mask, can add into the destination, splits the
//    columns over two destination tensors (the two halves of a concatenated input) and can write
//    FP32 (the network output).
//  * conv_wgrad_kernel<CIB, COB>: weight gradient  dW[co][tap, ci] = sum_pixel dZ[pixel][co] *
//    X[pixel + tap][ci].  M = 128 rows = (128 / CIB) taps x CIB input channels, N = BN output
//    channels, K = pixels.  Both operands are read MN-major straight from the NHWC tensors
//    (channel rows of 128 pixels, 4-D TMA boxes as above), so no transposed copy is made.  The
//    pixel range is split over CTAs and each CTA adds its FP32 partial sums into dW.
//
// Warp roles (192 threads): warp 0 issues TMA loads into a ring of shared-memory stages, warp 1
// owns the TMEM accumulator and issues tcgen05.mma from one lane, warps 2-5 drain TMEM with
// tcgen05.ld (each warp reads the 32 TMEM lanes its warp index selects).  Stages are handed over
// with mbarriers: TMA completes "full[s]", tcgen05.commit arrives on "empty[s]" once the MMAs
// reading stage s are done, and a final commit arrives on "done".  Every wait is bounded; on
// expiry the kernel sets a flag bit, drains what it issued and frees its TMEM.
#pragma once

#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace unet {

constexpr int kThreads = 192;
constexpr unsigned kFlagTimeout = 8u;
constexpr long long kWaitCycles = 4000000000ll;   // ~2 s at 2 GHz

// ------------------------------------------------------------------ PTX wrappers
__device__ __forceinline__ uint32_t su32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void bar_init(uint64_t* b, uint32_t n) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(b)), "r"(n) : "memory");
}
__device__ __forceinline__ void bar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void bar_try_arrive(uint64_t* b) {
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(su32(b)) : "memory");
}
__device__ __forceinline__ void bar_expect_tx(uint64_t* b, uint32_t bytes) {
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(su32(b)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool bar_try(uint64_t* b, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(su32(b)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait on the phase of the given parity (nanosleep back-off between polls).
__device__ __forceinline__ bool bar_wait(uint64_t* b, uint32_t parity, unsigned max_ns) {
    if (bar_try(b, parity)) return true;
    const long long t0 = clock64();
    unsigned ns = 32;
    while (true) {
        __nanosleep(ns);
        if (bar_try(b, parity)) return true;
        if (clock64() - t0 > kWaitCycles) return false;
        ns = min(2 * ns, max_ns);
    }
}

__device__ __forceinline__ void tma_prefetch(const CUtensorMap* m) {
    asm volatile("prefetch.tensormap [%0];" ::"l"(m) : "memory");
}
__device__ __forceinline__ void tma_4d(void* dst, const CUtensorMap* m, int c0, int c1, int c2, int c3, uint64_t* b) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
        "[%6];" ::"r"(su32(dst)),
        "l"(m), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(su32(b))
        : "memory");
}
__device__ __forceinline__ void tma_2d(void* dst, const CUtensorMap* m, int c0, int c1, uint64_t* b) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            su32(dst)),
        "l"(m), "r"(c0), "r"(c1), "r"(su32(b))
        : "memory");
}

__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t cols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(slot)), "r"(cols)
                 : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t cols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(cols) : "memory");
}
__device__ __forceinline__ void tc_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// D[tmem] (+)= A[smem] * B[smem]^T, bf16 inputs, FP32 accumulator (kind::f16).
__device__ __forceinline__ void mma_bf16(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\ttcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(
            d),
        "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}
// Arrive on the mbarrier once all previously issued tcgen05 operations of this thread are done.
__device__ __forceinline__ void mma_commit(uint64_t* b) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(su32(b))
                 : "memory");
}

// 32 consecutive FP32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
        "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
          "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// Shared-memory matrix descriptor (tcgen05): start address, leading / stride byte offsets (both
// >> 4), descriptor version 1, swizzle layout in bits 61-63 (2 = 128 B, 4 = 64 B).
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo, uint32_t layout) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46) | ((uint64_t)layout << 61);
}
__host__ __device__ constexpr uint32_t swizzle_layout(int row_bytes) { return row_bytes == 128 ? 2u : 4u; }

// Instruction descriptor of kind::f16: FP32 accumulator, bf16 A and B, K- or MN-major operands,
// N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N, bool a_mn, bool b_mn) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((a_mn ? 1u : 0u) << 15) | ((b_mn ? 1u : 0u) << 16) |
           ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__host__ __device__ constexpr uint32_t tmem_cols(int n) { return n <= 32 ? 32u : n <= 64 ? 64u : n <= 128 ? 128u : 256u; }

// ------------------------------------------------------------------ forward / backward-data conv
struct ConvMaps {
    CUtensorMap src[2];   // 4-D (C, W, H, images), box (BK, BW, BH, 1)
    CUtensorMap wts;      // 2-D (taps * Ctot, Nout), box (BK, BN)
};

struct ConvArgs {
    int nsrc, C0, C1, Ctot, taps, images;
    int W, H, BW, BH, tiles_x, tiles_y;
    int BN, Nout, stages;
    const float* bias;                 // [Nout] or null
    int relu;
    __nv_bfloat16* out[2];             // columns [0, outc[0]) -> out[0], the rest -> out[1]
    int outc[2];
    const __nv_bfloat16* mask[2];      // zero the value where mask <= 0 (same layout as out)
    int accumulate[2];                 // add into the destination
    float* out_f32;                    // when set: columns [0, f32_keep) as FP32 [pixel][f32_keep]
    int f32_keep;
    unsigned* flags;
};

// Epilogue of one output tile: 32 columns at a time from this warp's TMEM lanes.
template <int BK>
__device__ __forceinline__ void conv_epilogue(const ConvArgs& a, uint32_t tacc, int q, int lane, int img, int x0,
                                              int y0, int n0) {
    const int row = 32 * q + lane;
    const int px = x0 + row % a.BW, py = y0 + row / a.BW;
    const size_t pix = ((size_t)img * a.H + py) * a.W + px;
    for (int c0 = 0; c0 < a.BN; c0 += 32) {
        float v[32];
        tmem_ld32(tacc + ((uint32_t)(32 * q) << 16) + (uint32_t)c0, v);
        const int n = n0 + c0;
        if (a.bias) {
#pragma unroll
            for (int i = 0; i < 32; ++i) v[i] += __ldg(a.bias + n + i);
        }
        if (a.relu) {
#pragma unroll
            for (int i = 0; i < 32; ++i) v[i] = fmaxf(v[i], 0.f);
        }
        if (a.out_f32) {
#pragma unroll
            for (int i = 0; i < 32; ++i)
                if (n + i < a.f32_keep) a.out_f32[pix * a.f32_keep + n + i] = v[i];
            continue;
        }
        const int d = n >= a.outc[0] ? 1 : 0;
        const int ch = d ? n - a.outc[0] : n;
        __nv_bfloat16* dst = a.out[d] + pix * a.outc[d] + ch;
        if (a.mask[d]) {
            const uint4* m4 = reinterpret_cast<const uint4*>(a.mask[d] + pix * a.outc[d] + ch);
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const uint4 mm = m4[j];
                const __nv_bfloat16* mb = reinterpret_cast<const __nv_bfloat16*>(&mm);
#pragma unroll
                for (int i = 0; i < 8; ++i)
                    if (!(__bfloat162float(mb[i]) > 0.f)) v[8 * j + i] = 0.f;
            }
        }
        uint4* d4 = reinterpret_cast<uint4*>(dst);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            if (a.accumulate[d]) {
                const uint4 old = d4[j];
                const __nv_bfloat16* ob = reinterpret_cast<const __nv_bfloat16*>(&old);
#pragma unroll
                for (int i = 0; i < 8; ++i) v[8 * j + i] += __bfloat162float(ob[i]);
            }
            uint4 pk;
            __nv_bfloat162* pb = reinterpret_cast<__nv_bfloat162*>(&pk);
#pragma unroll
            for (int i = 0; i < 4; ++i) pb[i] = __floats2bfloat162_rn(v[8 * j + 2 * i], v[8 * j + 2 * i + 1]);
            d4[j] = pk;
        }
    }
}

// Persistent: CTA c handles work items c, c + gridDim.x, ... (item = M tile x N tile).  The TMA
// ring runs on across items, and two TMEM accumulators alternate so that the epilogue of one
// item overlaps the MMAs of the next ("tfull[b]" committed by the MMA lane when accumulator b
// holds a finished item, "tempty[b]" arrived at by the four epilogue warps once they have read it).
template <int BK>
__global__ void __launch_bounds__(kThreads, 1) conv_fwd_kernel(const __grid_constant__ ConvMaps maps, const ConvArgs a) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    const int a_bytes = 128 * BK * 2, b_bytes = a.BN * BK * 2, stage_bytes = a_bytes + b_bytes;
    uint64_t* full = (uint64_t*)(smem + a.stages * stage_bytes);
    uint64_t* empty = full + a.stages;
    uint64_t* tfull = empty + a.stages;   // [2]
    uint64_t* tempty = tfull + 2;         // [2]
    uint32_t* tslot = (uint32_t*)(tempty + 2);
    __shared__ int timed_out;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int per_img = a.tiles_x * a.tiles_y;
    const int ntn = a.Nout / a.BN;
    const int items = a.images * per_img * ntn;
    const uint32_t ncols = tmem_cols(a.BN);

    if (threadIdx.x == 0) {
        for (int s = 0; s < a.stages; ++s) {
            bar_init(&full[s], 1);
            bar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            bar_init(&tfull[b], 1);
            bar_init(&tempty[b], 4);
        }
        bar_fence_init();
        timed_out = 0;
    }
    if (warp == 1) {
        tmem_alloc(tslot, 2 * ncols);
        tmem_relinquish();
    }
    __syncthreads();
    tc_after();
    const uint32_t tmem = *tslot;
    const int kpt = a.Ctot / BK, nkb = a.taps * kpt;

    if (warp == 0 && lane == 0) {
        tma_prefetch(&maps.src[0]);
        if (a.nsrc > 1) tma_prefetch(&maps.src[1]);
        tma_prefetch(&maps.wts);
        long long g = 0;
        bool stop = false;
        for (int it = blockIdx.x; it < items && !stop; it += gridDim.x) {
            const int mt = it / ntn, n0 = (it % ntn) * a.BN;
            const int img = mt / per_img, rem = mt % per_img;
            const int x0 = (rem % a.tiles_x) * a.BW, y0 = (rem / a.tiles_x) * a.BH;
            for (int kb = 0; kb < nkb; ++kb, ++g) {
                const int s = (int)(g % a.stages);
                const long long round = g / a.stages;
                if (g >= a.stages && !bar_wait(&empty[s], (uint32_t)((round - 1) & 1), 256)) {
                    atomicOr(a.flags, kFlagTimeout);
                    timed_out = 1;
                    stop = true;
                    break;
                }
                const int tap = kb / kpt, c = (kb % kpt) * BK;
                const int src = c >= a.C0 ? 1 : 0, cs = src ? c - a.C0 : c;
                const int dy = a.taps == 9 ? tap / 3 - 1 : 0, dx = a.taps == 9 ? tap % 3 - 1 : 0;
                uint8_t* st = smem + s * stage_bytes;
                bar_expect_tx(&full[s], (uint32_t)stage_bytes);
                tma_4d(st, &maps.src[src], cs, x0 + dx, y0 + dy, img, &full[s]);
                tma_2d(st + a_bytes, &maps.wts, tap * a.Ctot + c, n0, &full[s]);
            }
        }
        // Drain: every issued load has landed before the CTA may exit.
        for (long long k = (g > a.stages ? g - a.stages : 0); k < g; ++k)
            if (!bar_wait(&full[k % a.stages], (uint32_t)((k / a.stages) & 1), 256)) atomicOr(a.flags, kFlagTimeout);
    } else if (warp == 1 && lane == 0) {
        const uint32_t idesc = idesc_bf16(128, a.BN, false, false);
        const uint32_t lay = swizzle_layout(BK * 2), sbo = 8 * BK * 2;
        long long g = 0;
        int i = 0;
        bool stop = false;
        for (int it = blockIdx.x; it < items && !stop; it += gridDim.x, ++i) {
            const int b = i & 1;
            if (i >= 2 && !bar_wait(&tempty[b], (uint32_t)(((i >> 1) - 1) & 1), 256)) {
                atomicOr(a.flags, kFlagTimeout);
                timed_out = 1;
                break;
            }
            tc_after();
            const uint32_t tacc = tmem + (uint32_t)(b * ncols);
            for (int kb = 0; kb < nkb; ++kb, ++g) {
                const int s = (int)(g % a.stages);
                if (!bar_wait(&full[s], (uint32_t)((g / a.stages) & 1), 64)) {
                    atomicOr(a.flags, kFlagTimeout);
                    timed_out = 1;
                    stop = true;
                    break;
                }
                tc_after();
                const uint32_t sa = su32(smem + s * stage_bytes), sb = sa + a_bytes;
#pragma unroll
                for (int k = 0; k < BK / 16; ++k)
                    mma_bf16(tacc, smem_desc(sa + 32 * k, 16, sbo, lay), smem_desc(sb + 32 * k, 16, sbo, lay), idesc,
                             (kb | k) != 0);
                mma_commit(&empty[s]);
            }
            mma_commit(&tfull[b]);   // also on the timeout path, so the epilogue warps are released
        }
    } else if (warp >= 2) {
        const int q = warp & 3;
        int i = 0;
        for (int it = blockIdx.x; it < items; it += gridDim.x, ++i) {
            const int b = i & 1;
            const bool ok = __all_sync(0xffffffffu, bar_wait(&tfull[b], (uint32_t)((i >> 1) & 1), 1024));
            tc_after();
            if (!ok) {
                if (lane == 0) atomicOr(a.flags, kFlagTimeout);
                break;
            }
            if (__shfl_sync(0xffffffffu, timed_out, 0) == 0) {
                const int mt = it / ntn, n0 = (it % ntn) * a.BN;
                const int img = mt / per_img, rem = mt % per_img;
                conv_epilogue<BK>(a, tmem + (uint32_t)(b * ncols), q, lane, img, (rem % a.tiles_x) * a.BW,
                                  (rem / a.tiles_x) * a.BH, n0);
            }
            tc_before();
            __syncwarp();
            if (lane == 0) bar_try_arrive(&tempty[b]);
        }
    }
    __syncthreads();
    if (warp == 1) {
        tc_after();
        tmem_dealloc(tmem, 2 * ncols);
    }
}

// ------------------------------------------------------------------ weight gradient
struct WgradMaps {
    CUtensorMap x[2];   // 4-D (C, W, H, images), box (CIB, BW, BH, 1)
    CUtensorMap dz;     // 4-D (Cout, W, H, images), box (COB, BW, BH, 1)
};

struct WgradArgs {
    int nsrc, C0, C1, Ctot, taps, Cout;
    int W, H, BW, BH, tiles_x, tiles_y;
    int num_tiles, tiles_per_split;
    int BN, stages;
    float* dw;   // FP32 [Cout][taps * Ctot], accumulated
    unsigned* flags;
};

template <int CIB, int COB>
__global__ void __launch_bounds__(kThreads, 1) conv_wgrad_kernel(const __grid_constant__ WgradMaps maps,
                                                                  const WgradArgs a) {
    constexpr int TPG = 128 / CIB;                 // taps per 128-row M tile
    constexpr int A_BOX = 128 * CIB * 2;           // one tap's box: 128 pixel rows of CIB channels
    constexpr int B_BOX = 128 * COB * 2;
    constexpr int A_BYTES = TPG * A_BOX;
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    const int nb = a.BN / COB;
    const int stage_bytes = A_BYTES + nb * B_BOX;
    uint64_t* full = (uint64_t*)(smem + a.stages * stage_bytes);
    uint64_t* empty = full + a.stages;
    uint64_t* done = empty + a.stages;
    uint32_t* tslot = (uint32_t*)(done + 1);
    __shared__ int timed_out;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int ngroups = (a.taps + TPG - 1) / TPG;
    const int tg = blockIdx.y % ngroups, cb = blockIdx.y / ngroups;
    const int cglob = cb * CIB, src = cglob >= a.C0 ? 1 : 0, cs = src ? cglob - a.C0 : cglob;
    const int n0 = blockIdx.z * a.BN;
    const int t_begin = blockIdx.x * a.tiles_per_split;
    const int t_end = min(a.num_tiles, t_begin + a.tiles_per_split);
    const int nkb = max(0, t_end - t_begin);
    const uint32_t ncols = tmem_cols(a.BN);
    const int per_img = a.tiles_x * a.tiles_y;

    if (threadIdx.x == 0) {
        for (int s = 0; s < a.stages; ++s) {
            bar_init(&full[s], 1);
            bar_init(&empty[s], 1);
        }
        bar_init(done, 1);
        bar_fence_init();
        timed_out = 0;
    }
    if (warp == 1) {
        tmem_alloc(tslot, ncols);
        tmem_relinquish();
    }
    __syncthreads();
    tc_after();
    const uint32_t tmem = *tslot;

    if (warp == 0 && lane == 0) {
        tma_prefetch(&maps.x[src]);
        tma_prefetch(&maps.dz);
        int issued = 0;
        for (int kb = 0; kb < nkb; ++kb) {
            const int s = kb % a.stages, round = kb / a.stages;
            if (kb >= a.stages && !bar_wait(&empty[s], (round - 1) & 1, 256)) {
                atomicOr(a.flags, kFlagTimeout);
                timed_out = 1;
                break;
            }
            const int t = t_begin + kb, img = t / per_img, rem = t % per_img;
            const int x0 = (rem % a.tiles_x) * a.BW, y0 = (rem / a.tiles_x) * a.BH;
            uint8_t* st = smem + s * stage_bytes;
            bar_expect_tx(&full[s], (uint32_t)stage_bytes);
#pragma unroll
            for (int j = 0; j < TPG; ++j) {
                const int tap = tg * TPG + j;
                int dx = 0, dy = 0;
                if (tap >= a.taps) {
                    dy = -4 * a.BH - 8 - y0;   // a box wholly above the image: zeros
                } else if (a.taps == 9) {
                    dy = tap / 3 - 1;
                    dx = tap % 3 - 1;
                }
                tma_4d(st + j * A_BOX, &maps.x[src], cs, x0 + dx, y0 + dy, img, &full[s]);
            }
            for (int j = 0; j < nb; ++j) tma_4d(st + A_BYTES + j * B_BOX, &maps.dz, n0 + j * COB, x0, y0, img, &full[s]);
            ++issued;
        }
        for (int kb = max(0, issued - a.stages); kb < issued; ++kb)
            if (!bar_wait(&full[kb % a.stages], (kb / a.stages) & 1, 256)) atomicOr(a.flags, kFlagTimeout);
    } else if (warp == 1 && lane == 0) {
        const uint32_t idesc = idesc_bf16(128, a.BN, true, true);
        const uint32_t la = swizzle_layout(CIB * 2), lb = swizzle_layout(COB * 2);
        const uint32_t atom_a = 8 * CIB * 2, atom_b = 8 * COB * 2;
        for (int kb = 0; kb < nkb; ++kb) {
            const int s = kb % a.stages, round = kb / a.stages;
            if (!bar_wait(&full[s], round & 1, 64)) {
                atomicOr(a.flags, kFlagTimeout);
                timed_out = 1;
                break;
            }
            tc_after();
            const uint32_t sa = su32(smem + s * stage_bytes), sb = sa + A_BYTES;
#pragma unroll
            for (int k = 0; k < 8; ++k)   // 16 pixel rows (two 8-row groups) per MMA
                mma_bf16(tmem, smem_desc(sa + 2 * atom_a * k, A_BOX, atom_a, la),
                         smem_desc(sb + 2 * atom_b * k, B_BOX, atom_b, lb), idesc, (kb | k) != 0);
            mma_commit(&empty[s]);
        }
        mma_commit(done);
    } else if (warp >= 2) {
        const bool ok = __all_sync(0xffffffffu, bar_wait(done, 0, 1024));
        const bool go = ok && nkb > 0 && __shfl_sync(0xffffffffu, timed_out, 0) == 0;
        tc_after();
        if (!ok) {
            if (lane == 0) atomicOr(a.flags, kFlagTimeout);
        } else if (go) {
            const int q = warp & 3, row = 32 * q + lane;
            const int tap = tg * TPG + row / CIB, ci = cglob + row % CIB;
            const size_t ktot = (size_t)a.taps * a.Ctot;
            for (int c0 = 0; c0 < a.BN; c0 += 32) {
                float v[32];
                tmem_ld32(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)c0, v);
                if (tap < a.taps) {
                    float* dst = a.dw + (size_t)(n0 + c0) * ktot + (size_t)tap * a.Ctot + ci;
#pragma unroll
                    for (int i = 0; i < 32; ++i) atomicAdd(dst + (size_t)i * ktot, v[i]);
                }
            }
        }
        tc_before();
    }
    __syncthreads();
    if (warp == 1) {
        tc_after();
        tmem_dealloc(tmem, ncols);
    }
}

}  // namespace unet
