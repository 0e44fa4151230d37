// sar_kernels.cu -- sm_103a kernels of the SAR operator pair.
//
//   K1  upsample_pairs (fused, N = 1024, 2048, 4096) or pack_adjoint / cuFFT / unpack_pairs
//                                      range-profile upsampling (replaces sarsolver_cxx.cpp:331-344)
//   K2  bp_grid_ws_pair / bp_grid / bp_points
//                                      backprojection gather (replaces :345-350)
//   K3  fp_grid_ws / fp_points         forward scatter, the exact transpose of K2 (:284-291)
//   K4  downsample_forward (fused) or pack_forward / cuFFT / extract_forward
//                                      range-profile downsampling around the FFT (:292-307)
//
// Nearest-bin sampling (the reference's rule) on the grid kernels uses split bins and decides
// every bin within 5e-5 of a rounding boundary again in double-float (exact_grid_bin), so the
// bins equal those of FP64 rounding; the per-pixel kernels compute every bin that way.
//
// Layout in HBM: images are complex64 [nz][ny][nx]; phase histories complex64 [S][N] with
// fast time fftshifted (the Python API's convention, forward.py:44); range profiles are kept
// only over the bins the scene can reach, [S][Lg] starting at bin bg0, as float4
// (value at the interpolation midpoint, difference to the next bin) so that one 16-byte
// load gives a linearly interpolated sample.
#include "sar_kernels.cuh"

#include <type_traits>

namespace sar {

#define SAR_TWO_PI 6.28318530717958647692f

__device__ __forceinline__ void raise_flag(unsigned* flags, unsigned bit) {
    if (flags) atomicOr(flags, bit);
}

__device__ __forceinline__ PulseGeom load_pulse(const PulseGeom* p) {
    const float4* v = reinterpret_cast<const float4*>(p);
    const float4 a = __ldg(v), b = __ldg(v + 1), c = __ldg(v + 2), d = __ldg(v + 3);
    PulseGeom g;
    g.atx_hi[0] = a.x; g.atx_hi[1] = a.y; g.atx_hi[2] = a.z; g.atx_lo[0] = a.w;
    g.atx_lo[1] = b.x; g.atx_lo[2] = b.y; g.arx_hi[0] = b.z; g.arx_hi[1] = b.w;
    g.arx_hi[2] = c.x; g.arx_lo[0] = c.y; g.arx_lo[1] = c.z; g.arx_lo[2] = c.w;
    g.rref_hi = d.x; g.rref_lo = d.y; g.monostatic = d.z; g.pad = d.w;
    return g;
}

// ------------------------------------------------------------ tile bookkeeping
// Thread layout of a 32x32 tile CTA: lane = column (i), warp w owns rows 4w .. 4w+3.
// Sub-tile q (16x16) = (column >= 16) + 2 (row >= 16); offsets are relative to the
// sub-tile anchor at (8, 8) inside it.
struct TileThread {
    int q;
    float di, di2, di3;
    float dj[4], dj2[4], dj3[4];
};

__device__ __forceinline__ TileThread tile_thread() {
    TileThread t;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    t.q = (lane >= 16) + 2 * (warp >= 4);
    t.di = (float)(lane - 8 - 16 * (lane >= 16));
    t.di2 = t.di * t.di;
    t.di3 = t.di2 * t.di;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const float d = (float)(4 * warp + r - 8 - 16 * (warp >= 4));
        t.dj[r] = d;
        t.dj2[r] = d * d;
        t.dj3[r] = d * d * d;
    }
    return t;
}

__device__ __forceinline__ df3 subtile_anchor(int ti, int tj, int k, int q, const GridConst& g) {
    return pixel_position(ti * kTile + 8 + 16 * (q & 1) + g.a_off, tj * kTile + 8 + 16 * (q >> 1), k, g);
}

// One (pulse, sub-tile) coefficient set per thread of the first ceil(4 pb / 32) warps.
// Coefficient sets are kSetF4 = 6 float4:
//   [c0 c1 c2 c3][c4 c5 c6 c7][c8 c9 v0 v1][v2 v3 v4 v5][ia ib w6 w7][w8 w9 i0 -]
// (the last two are read only in precise-bin mode).
// The tile's base bin (floor of the mean anchor bin) is agreed across the four lanes of a
// pulse by shuffles, so all sub-tiles of a pulse share it.
__device__ __forceinline__ void coeff_stage(const GridConst& g, const PulseGeom* __restrict__ pulses,
                                            int s0, int npb, int pb, const df3* anchors,
                                            float4* coef, int* base) {
    const int t = threadIdx.x;
    const int nthr = (4 * pb + 31) & ~31;
    if (t >= nthr) return;
    const int pi = t >> 2, q = t & 3;
    const bool valid = (t < 4 * pb) && (pi < npb);
    AnchorExpansion ae = {};
    Coeffs co = {};
    df vb = df_make(0.0f, 0.0f);
    if (valid) {
        const PulseGeom pg = load_pulse(pulses + s0 + pi);
        ae = expand_anchor(anchors[q], pg, g);
        phase_coeffs(ae, g, co.c);
        vb = anchor_bin(ae, g);
    }
    const unsigned all = 0xffffffffu;
    df sum = df_add(vb, df_make(__shfl_xor_sync(all, vb.hi, 1), __shfl_xor_sync(all, vb.lo, 1)));
    sum = df_add(sum, df_make(__shfl_xor_sync(all, sum.hi, 2), __shfl_xor_sync(all, sum.lo, 2)));
    int b = base_bin_of(sum, 4.0f);
    b = __shfl_sync(all, b, (t & 31) & ~3);
    if (valid) {
        bin_coeffs(ae, vb, b, g, co);
        float4* dst = coef + (pi * 4 + q) * kSetF4;
        dst[0] = make_float4(co.c[0], co.c[1], co.c[2], co.c[3]);
        dst[1] = make_float4(co.c[4], co.c[5], co.c[6], co.c[7]);
        dst[2] = make_float4(co.c[8], co.c[9], co.v[0], co.v[1]);
        dst[3] = make_float4(co.v[2], co.v[3], co.v[4], co.v[5]);
        dst[4] = make_float4(co.ia, co.ib, co.w[0], co.w[1]);
        dst[5] = make_float4(co.w[2], co.w[3], co.i0, 0.f);
        if (q == 0) base[pi] = b;
    }
}

struct PixelEval {
    float f;    // phase, cycles in [-0.5, 0.5]
    float sf;   // interpolation coordinate in [-0.5, 0.5] about bin n
    int n;      // bin relative to the tile's base bin
};

// The thread's polynomials in the offset it walks, from a coefficient set: in dj for a fixed di
// (TRANSPOSED false), or in di for a fixed dj (TRANSPOSED true; tt.di then holds the dj offset).
template <bool PRECISE, bool TRANSPOSED = false>
__device__ __forceinline__ ColumnTerms load_column(const float4* cs, const TileThread& tt, float& c9,
                                                   float& w9, float& ib) {
    const float4 A = cs[0], B = cs[1], C = cs[2], D = cs[3];
    Coeffs co;
    if (PRECISE) {
        const float4 E = cs[4], F = cs[5];
        co.ia = E.x;
        co.ib = E.y;
        co.w[0] = E.z;
        co.w[1] = E.w;
        co.w[2] = F.x;
        co.w[3] = F.y;
        co.i0 = F.z;
    } else {
        co.i0 = co.ia = co.ib = 0.f;
        co.w[0] = co.w[1] = co.w[2] = co.w[3] = 0.f;
    }
    co.c[0] = A.x; co.c[1] = A.y; co.c[2] = A.z; co.c[3] = A.w;
    co.c[4] = B.x; co.c[5] = B.y; co.c[6] = B.z; co.c[7] = B.w;
    co.c[8] = C.x; co.c[9] = C.y; co.v[0] = C.z; co.v[1] = C.w;
    co.v[2] = D.x; co.v[3] = D.y; co.v[4] = D.z; co.v[5] = D.w;
    if (TRANSPOSED) {
        ib = co.ia;
        w9 = co.w[0];
        c9 = co.c[6];
        return row_terms<PRECISE>(co, tt.di, tt.di2, tt.di3);
    }
    ib = co.ib;
    w9 = co.w[3];
    c9 = co.c[9];
    return column_terms<PRECISE>(co, tt.di, tt.di2, tt.di3);
}

template <bool PRECISE>
__device__ __forceinline__ PixelEval eval_pixel(const ColumnTerms& ct, float c9, float w9, float ib,
                                                const TileThread& tt, int r) {
    PixelEval e;
    const float ph = pixel_phase(ct, c9, tt.dj[r], tt.dj2[r], tt.dj3[r]);
    e.f = ph - rintf(ph);   // exact: |ph| < 2^22
    const float v = pixel_bin<PRECISE>(ct, w9, tt.dj[r], tt.dj2[r], tt.dj3[r]);
    const BinPos b = bin_position<PRECISE>(v, PRECISE ? fmaf(ib, tt.dj[r], ct.ci) : 0.f);
    e.sf = b.s;
    e.n = b.n;
    return e;
}

// Nearest-bin sampling on the grid paths.  The FP32 bin coordinate s (about the chosen bin, in
// [-0.5, 0.5]) is within ~5e-6 bins of the FP64 position (split bins, sar_geom.cuh); where |s|
// exceeds kNearEdge the bin is decided again from the per-pixel double-float range with the
// unstructured path's exact rule (exact_bin: FP64 rounding of the same value, ties away from
// zero), so the grid kernels pick the bins the per-pixel path picks.  About 1e-4 of the
// pixel·pulses take this branch.
constexpr float kNearEdge = 0.49995f;

// Stored-span index (bins from bg0) of grid pixel (i, j, k) for pulse s under nearest rule `rule`:
// pixel offset from the grid origin in FP64 as the host forms it, then the double-float range and
// rounding of the per-pixel kernels (eval_point).
__device__ __noinline__ int exact_grid_bin(const double* __restrict__ steps, const PulseGeom* __restrict__ pulses,
                                           const float4* __restrict__ alpha2, float sr_hi, float sr_lo, int bg0,
                                           int rule, int i, int j, int k, int s) {
    double q[3];
#pragma unroll
    for (int c = 0; c < 3; ++c)
        q[c] = __dadd_rn(__dadd_rn(__dmul_rn((double)i, steps[c]), __dmul_rn((double)j, steps[3 + c])),
                         __dmul_rn((double)k, steps[6 + c]));
    const double qq = __dadd_rn(__dadd_rn(__dmul_rn(q[0], q[0]), __dmul_rn(q[1], q[1])), __dmul_rn(q[2], q[2]));
    PointGeom pt;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        pt.qh[c] = __double2float_rn(q[c]);
        pt.ql[c] = __double2float_rn(__dsub_rn(q[c], (double)pt.qh[c]));
    }
    pt.qh[3] = __double2float_rn(qq);
    pt.ql[3] = __double2float_rn(__dsub_rn(qq, (double)pt.qh[3]));
    const PulseGeom pg = load_pulse(pulses + s);
    const float4 a2 = __ldg(alpha2 + s);
    df r = point_range(pulse_tx(pg), df_make(a2.x, a2.y), pt);
    if (pg.monostatic != 0.0f)
        r = df_mulf(r, 2.0f);
    else
        r = df_add(r, point_range(pulse_rx(pg), df_make(a2.z, a2.w), pt));
    r = df_sub(r, df_make(pg.rref_hi, pg.rref_lo));
    const df V = df_sub(df_mul(df_make(sr_hi, sr_lo), r), df_make((float)bg0, 0.0f));
    int gi;
    float sf;
    exact_bin(V, bg0, rule, &gi, &sf);
    return gi;
}

// ------------------------------------------------------------------- K2 (grid, wide windows)
// Fallback for tiles whose range window is too wide to stage in shared memory: coefficient sets
// per block of pulses in shared memory, profile pairs read straight from global memory (L2).
size_t bp_grid_smem_bytes(int wwin, int pb, int staged) {
    (void)wwin;
    (void)staged;
    return ((size_t)pb * 4 * kSetF4 + (size_t)((pb + 3) / 4) + 6) * sizeof(float4);
}

template <bool PRECISE, bool NEAREST>
__global__ void __launch_bounds__(kThreads, 2) bp_grid_kernel(const BpGridArgs a) {
    extern __shared__ float4 smem[];
    const int pb = a.pb;
    float4* coef = smem;
    int* base = reinterpret_cast<int*>(coef + pb * 4 * kSetF4);
    df3* anchors = reinterpret_cast<df3*>(base + ((pb + 3) & ~3));

    const GridConst& g = a.g;
    int tile = blockIdx.x;
    const int ti = tile % g.tiles_x;
    tile /= g.tiles_x;
    const int tj = tile % g.tiles_y;
    const int k = tile / g.tiles_y;
    const TileThread tt = tile_thread();
    if (threadIdx.x < 4) anchors[threadIdx.x] = subtile_anchor(ti, tj, k, threadIdx.x, g);

    float acc_re[4] = {0.f, 0.f, 0.f, 0.f}, acc_im[4] = {0.f, 0.f, 0.f, 0.f};
    for (int s0 = 0; s0 < a.S; s0 += pb) {
        const int npb = min(pb, a.S - s0);
        __syncthreads();
        coeff_stage(g, a.pulses, s0, npb, pb, anchors, coef, base);
        __syncthreads();
        float st_re[4] = {0.f, 0.f, 0.f, 0.f}, st_im[4] = {0.f, 0.f, 0.f, 0.f};
        for (int pi = 0; pi < npb; ++pi) {
            float c9, w9, ib;
            const ColumnTerms ct = load_column<PRECISE>(coef + (pi * 4 + tt.q) * kSetF4, tt, c9, w9, ib);
            const float4* gp = a.pairs + (size_t)(s0 + pi) * a.Lg;
            const int bb = base[pi] - a.bg0;
            // bins of the thread's four pixels first, the rare exact re-decisions next, then the four
            // loads: the loads are not held behind the (non-inlined) re-decision call
            PixelEval e4[4];
            int gi4[4];
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                e4[r] = eval_pixel<PRECISE>(ct, c9, w9, ib, tt, r);
                gi4[r] = min(max(bb + e4[r].n, 0), a.Lg - 1);
            }
            if (NEAREST) {
#pragma unroll
                for (int r = 0; r < 4; ++r)
                    if (fabsf(e4[r].sf) > kNearEdge)
                        gi4[r] = min(max(exact_grid_bin(a.steps, a.pulses, a.alpha2, g.s_r.hi, g.s_r.lo, a.bg0,
                                                        BIN_ADJ_NEAREST, ti * kTile + (threadIdx.x & 31),
                                                        tj * kTile + 4 * (threadIdx.x >> 5) + r, k, s0 + pi),
                                         0), a.Lg - 1);
            }
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                const PixelEval e = e4[r];
                const int gi = gi4[r];
                float re, im;
                if (NEAREST && a.values) {   // nearest-bin profiles stored as plain values (float2 rows)
                    const float2 pv = __ldg(reinterpret_cast<const float2*>(a.pairs) + (size_t)(s0 + pi) * a.Lg + gi);
                    re = pv.x;
                    im = pv.y;
                } else {
                    const float4 pv = __ldg(gp + gi);
                    re = fmaf(e.sf, pv.z, pv.x);
                    im = fmaf(e.sf, pv.w, pv.y);
                }
                float sn, cn;
                __sincosf(SAR_TWO_PI * e.f, &sn, &cn);
                // x += value * exp(-2 pi i f)
                st_re[r] = fmaf(re, cn, fmaf(im, sn, st_re[r]));
                st_im[r] = fmaf(im, cn, fmaf(-re, sn, st_im[r]));
            }
        }
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            acc_re[r] += st_re[r];
            acc_im[r] += st_im[r];
        }
    }
    const int i = ti * kTile + (threadIdx.x & 31);
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const int j = tj * kTile + 4 * (threadIdx.x >> 5) + r;
        if (i < g.nx && j < g.ny) {
            const size_t p = ((size_t)k * g.ny + j) * g.nx + i;
            float2 o = make_float2(acc_re[r], acc_im[r]);
            if (a.accumulate) {
                const float2 old = a.x[p];
                o.x += old.x;
                o.y += old.y;
            }
            a.x[p] = o;
        }
    }
}

template <bool PRECISE, bool NEAREST>
static cudaError_t launch_bp_grid_t(const BpGridArgs& a, cudaStream_t st) {
    const size_t smem = bp_grid_smem_bytes(a.wwin, a.pb, 0);
    const unsigned blocks = (unsigned)(a.g.tiles_x * a.g.tiles_y * a.g.nz);
    cudaError_t e = cudaFuncSetAttribute(bp_grid_kernel<PRECISE, NEAREST>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    bp_grid_kernel<PRECISE, NEAREST><<<blocks, kThreads, smem, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_bp_grid(const BpGridArgs& a, cudaStream_t st) {
    if (a.g.shear) return cudaErrorInvalidValue;   // sheared lattices run on the staged gather only
    if (a.nearest) {
        if (!a.g.precise_bins || !a.steps || !a.alpha2) return cudaErrorInvalidValue;
        return launch_bp_grid_t<true, true>(a, st);
    }
    return a.g.precise_bins ? launch_bp_grid_t<true, false>(a, st) : launch_bp_grid_t<false, false>(a, st);
}

// ------------------------------------------- warp-specialised pipelines (K2 gather, K3 scatter)
// Producer warps (8 and 9): for the next stage they compute the (pulse, sub-tile) coefficient
// sets and the tile base bins (the gather also issues, one lane per pulse, a 1-D bulk copy
// (cp.async.bulk) of that pulse's profile window into the stage's shared-memory buffer,
// completing on the buffer's "full" mbarrier).  Consumer warps (0..7) wait on "full", work, and
// arrive on the buffer's "empty" mbarrier, which the producers wait on before reusing the
// buffer.  Every wait is bounded by a clock budget; on expiry the kernel raises
// FLAG_WAIT_TIMEOUT and leaves the loop instead of hanging.
constexpr int kWsConsumers = 256;
constexpr int kWsProducers = 2;   // producer warps; producer w handles pulse passes 8w, 8w + 16, ...
constexpr int kWsThreads = kWsConsumers + 32 * kWsProducers;
constexpr long long kWaitBudgetCycles = kDefaultWaitBudgetCycles;

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(smem_addr(bar))
                 : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(
                     smem_addr(bar)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return done != 0;
}
// Bounded wait for completion of the barrier phase with the given parity.  Between polls the
// warp sleeps with exponential backoff (first_ns doubling up to max_ns), so waiting warps leave
// the issue slots to the gathering warps and poll only a few times per wait; the wait gives up
// after `budget` clock cycles (kWaitBudgetCycles unless the launch sets its own).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, unsigned first_ns, unsigned max_ns,
                                          long long budget = kWaitBudgetCycles) {
    if (mbar_try_wait(bar, parity)) return true;
    const long long t0 = clock64();
    unsigned ns = first_ns;
    while (true) {
        __nanosleep(ns);
        if (mbar_try_wait(bar, parity)) return true;
        if (clock64() - t0 > budget) return false;
        ns = min(2 * ns, max_ns);
    }
}
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
// 1-D bulk copy global -> shared (16-byte aligned addresses, size a multiple of 16).
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}

// Producer: coefficient sets for pulses s0 + pass .. s0 + pass + 7 (lane = 4*pulse + sub-tile).
__device__ __forceinline__ void producer_coeffs(const GridConst& g, const PulseGeom* __restrict__ pulses, int s0,
                                                int npb, int pass, const df3* anchors, float4* coef, int* base,
                                                int lane, int ring_half = 0, unsigned* flags = nullptr) {
    const int pi = pass + (lane >> 2), q = lane & 3;
    const bool valid = pi < npb;
    AnchorExpansion ae = {};
    Coeffs co = {};
    df vb = df_make(0.0f, 0.0f);
    if (valid) {
        const PulseGeom pg = load_pulse(pulses + s0 + pi);
        ae = expand_anchor(anchors[q], pg, g);
        phase_coeffs(ae, g, co.c);
        vb = anchor_bin(ae, g);
    }
    const unsigned all = 0xffffffffu;
    df sum = df_add(vb, df_make(__shfl_xor_sync(all, vb.hi, 1), __shfl_xor_sync(all, vb.lo, 1)));
    sum = df_add(sum, df_make(__shfl_xor_sync(all, sum.hi, 2), __shfl_xor_sync(all, sum.lo, 2)));
    int b = base_bin_of(sum, 4.0f);
    b = __shfl_sync(all, b, lane & ~3);
    if (valid) {
        bin_coeffs(ae, vb, b, g, co);
        if (ring_half > 0) {
            // ring windows: every bin the sub-tile touches (n - 1 .. n + 1 around its position) must
            // lie within ring_half of the base bin, or it would alias another bin's slot
            float lo, hi;
            bin_extent(co, &lo, &hi);
            const float lim = (float)(ring_half - 2);
            if (!(lo >= -lim && hi <= lim)) {
                raise_flag(flags, FLAG_STRIP_WINDOW);
                co = Coeffs{};   // invalid result (flagged), every bin then at the base
            }
        }
        float4* dst = coef + (pi * 4 + q) * kSetF4;
        dst[0] = make_float4(co.c[0], co.c[1], co.c[2], co.c[3]);
        dst[1] = make_float4(co.c[4], co.c[5], co.c[6], co.c[7]);
        dst[2] = make_float4(co.c[8], co.c[9], co.v[0], co.v[1]);
        dst[3] = make_float4(co.v[2], co.v[3], co.v[4], co.v[5]);
        dst[4] = make_float4(co.ia, co.ib, co.w[0], co.w[1]);
        dst[5] = make_float4(co.w[2], co.w[3], co.i0, 0.f);
        if (q == 0) base[pi] = b;
    }
}

// Pair-interleaved coefficient set of one (pulse pair, sub-tile): 2 kSetF4 float4 plus one float4
// of padding, so that consecutive sets start 20 banks apart (48 words would put every second set
// on the same banks and the producers' scalar stores 8-way on four banks; 52 words: 2-way).
constexpr int kPairSetF4 = 2 * kSetF4 + 1;
__host__ __device__ inline size_t pair_coef_f4(int pb) { return (size_t)((pb + 1) / 2) * 4 * kPairSetF4; }

// Staged window per pulse: linear, wwin (value, difference) pairs of 16 bytes; nearest-bin, wwin + 2
// plain 8-byte values starting at an even bin, so that every bulk copy starts on a 16-byte
// boundary (the bin the window is centred on sits one value later when its start is odd).
__host__ __device__ inline int win_elems(int wwin, int values) { return values ? wwin + 2 : wwin; }
__host__ __device__ inline int win_elem_bytes(int values) { return values ? 8 : 16; }

size_t bp_grid_ws_smem_bytes(int wwin, int pb, int values) {
    // windows [2][pb][elems] + coefficient sets [2][pb/2][4] + base bins [2][pb] + 4 mbarriers + 4 anchors
    return (size_t)2 * pb * win_elems(wwin, values) * win_elem_bytes(values) + sizeof(float4) * 2 * pair_coef_f4(pb) +
           sizeof(int) * 2 * pb + 4 * sizeof(uint64_t) + 4 * sizeof(df3);
}

// First stored-span element a nearest-bin window copies for a pulse whose window is centred on
// bin `base`: the window's first bin rounded down to even, kept inside [0, Lg - (wwin + 2)]
// (*clamped when that moved it; Lg is even).
__device__ __forceinline__ long value_window_start(int base, int wwin, int bg0, int Lg, bool* clamped) {
    long g0 = ((long)base - wwin / 2 - bg0) & ~1L;
    const long last = ((long)Lg - (wwin + 2)) & ~1L;
    *clamped = g0 < 0 || g0 > last;
    return g0 < 0 ? 0 : (g0 > last ? last : g0);
}

// ------------------------------------------- K2: two pulses per packed instruction
// The same pipeline with the consumers' arithmetic on FP32 pairs (fma.rn.f32x2 and friends,
// one instruction for two values, each rounded as the scalar operation): the two values are
// the same pixel for two consecutive pulses p (even) and p + 1.  Coefficient sets are stored
// pair-interleaved, kSetF4 * 2 float4 per (pulse pair, sub-tile) (+ one float4 of padding):
//   [c0 c0' c1 c1'] [c2 c2' c3 c3'] [c4 c4' c5 c5'] [c6 c6' c7 c7'] [c8 c8' c9 c9']
//   [v0 v0' v1 v1'] [v2 v2' v3 v3'] [v4 v4' v5 v5']
//   [ia ia' ib ib'] [w0 w0' w1 w1'] [w2 w2' w3 w3'] [i0 i0' - -]  (primed: pulse p + 1; the last
//   four only read with split bins: nearest-bin modes and windows wider than 256 bins)
// so that each half of a 16-byte shared-memory load is one operand pair.  Per pixel the
// polynomials are evaluated in Horner form in the row offset dj (the only per-row constant a
// thread keeps); the thread's phase constant is reduced mod 1 once per pulse pair, so every pixel's
// phase stays below ~5 cycles and goes to __sincosf without a per-pixel reduction (the special-
// function pipe then carries only sine and cosine: two of its operations per pixel-pulse), and
// the complex multiply-accumulate runs on (pulse p, pulse p + 1) accumulator pairs.  A stage with an odd
// number of pulses gets a padding pulse with zero coefficients and a zeroed window.
__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
// 16-byte shared-memory load at a 32-bit shared address.
// volatile: the loads stay after the (volatile) mbarrier wait that publishes the staged windows,
// which a non-volatile statement without a memory clobber could be moved across.
__device__ __forceinline__ float4 lds_f4(uint32_t addr) {
    float4 v;
    asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];" : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "r"(addr));
    return v;
}

__device__ __forceinline__ void producer_coeffs_pair(const GridConst& g, const PulseGeom* __restrict__ pulses, int s0,
                                                     int npb, int pass, const df3* anchors, float4* coef, int* base,
                                                     int lane, int ww, unsigned* flags) {
    const int pi = pass + (lane >> 2), q = lane & 3;
    const bool valid = pi < npb;
    const bool pad = pi == npb && (npb & 1);   // partner of the last pulse of an odd stage
    AnchorExpansion ae = {};
    Coeffs co = {};
    df vb = df_make(0.0f, 0.0f);
    if (valid) {
        const PulseGeom pg = load_pulse(pulses + s0 + pi);
        ae = expand_anchor(anchors[q], pg, g);
        phase_coeffs(ae, g, co.c);
        vb = anchor_bin(ae, g);
    }
    const unsigned all = 0xffffffffu;
    df sum = df_add(vb, df_make(__shfl_xor_sync(all, vb.hi, 1), __shfl_xor_sync(all, vb.lo, 1)));
    sum = df_add(sum, df_make(__shfl_xor_sync(all, sum.hi, 2), __shfl_xor_sync(all, sum.lo, 2)));
    int b = base_bin_of(sum, 4.0f);
    b = __shfl_sync(all, b, lane & ~3);
    if (valid) {
        bin_coeffs(ae, vb, b, g, co);
        // every pixel's bin must fall inside the tile's staged window: index rint(v) + ww / 2 in
        // [0, ww - 1] (an undersized window would otherwise be clamped silently, or read out of it)
        float lo, hi;
        bin_extent(co, &lo, &hi);
        const float half = 0.5f * (float)ww;
        if (!(lo >= -half - 0.49f && hi <= half - 0.51f)) {
            // the result is invalid (flagged); a zero set keeps every consumer index at ww / 2,
            // inside the window, so the lanes-along-x consumers may address without clamping
            raise_flag(flags, FLAG_GATHER_WINDOW);
            co = Coeffs{};
        }
    }
    if (valid || pad) {   // the padding pulse stores zeros (co = {})
        float* dst = reinterpret_cast<float*>(coef + ((pi >> 1) * 4 + q) * kPairSetF4) + (pi & 1);
        const float vals[24] = {co.c[0], co.c[1], co.c[2], co.c[3], co.c[4], co.c[5], co.c[6], co.c[7],
                                co.c[8], co.c[9], co.v[0], co.v[1], co.v[2], co.v[3], co.v[4], co.v[5],
                                co.ia,   co.ib,   co.w[0], co.w[1], co.w[2], co.w[3], co.i0,   0.f};
#pragma unroll
        for (int k = 0; k < 24; ++k) dst[2 * k] = vals[k];
        if (valid && q == 0) base[pi] = b;
    }
}

// LANES_Y = false: lane = column i, warp w owns rows 4w .. 4w + 3 (the thread's column terms
// are polynomials in dj); LANES_Y = true: lane = row j, warp w owns columns 4w .. 4w + 3 (line
// terms in di).  A quarter-warp's eight 16-byte window loads are conflict-free when they fall
// in distinct 16-byte bank groups or on the same bin; lanes along the axis where bins change
// slowly (cross-range) make them land on one or two bins.
// SHEARED: the tiles are those of a sheared lattice (GridConst.shear; linear sampling, lanes
// along its second axis), written through the shear to the image.
template <bool LANES_Y, bool PRECISE, bool NEAREST, bool VALUES = false, bool SHEARED = false>
__global__ void __launch_bounds__(kWsThreads, 2) bp_grid_ws_pair_kernel(const BpGridArgs a) {
    extern __shared__ __align__(16) float4 smem[];
    const int pb = a.pb, ww = a.wwin;
    // VALUES (wide windows): windows of plain values, half the bytes of pairs; nearest-bin sampling
    // reads one value, linear sampling two neighbours.  A window's size in float4 units: ww pairs,
    // or (ww + 2) / 2 for ww + 2 values
    const int wst = VALUES ? win_elems(ww, 1) / 2 : ww;
    float4* win0 = smem;
    float4* coef0 = win0 + 2 * pb * wst;
    int* base0 = reinterpret_cast<int*>(coef0 + 2 * pair_coef_f4(pb));
    uint64_t* bars = reinterpret_cast<uint64_t*>(base0 + 2 * pb);   // full[0..1], empty[2..3]
    df3* anchors = reinterpret_cast<df3*>(bars + 4);

    const GridConst& g = a.g;
    int tile = blockIdx.x / a.parts;
    const int part = blockIdx.x % a.parts;
    const int tj = tile % g.tiles_y;
    tile /= g.tiles_y;
    const int ti = tile % g.tiles_x;
    const int k = tile / g.tiles_x;
    if constexpr (SHEARED) {   // a lattice tile without image pixels leaves before any barrier exists
        int lo, hi;
        lattice_tile_range(g, ti, &lo, &hi);
        if (tj < lo || tj > hi) return;
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x < 4) anchors[threadIdx.x] = subtile_anchor(ti, tj, k, threadIdx.x, g);
    if (threadIdx.x == 0) {
        mbar_init(&bars[0], kWsProducers);
        mbar_init(&bars[1], kWsProducers);
        mbar_init(&bars[2], kWsConsumers / 32);
        mbar_init(&bars[3], kWsConsumers / 32);
        mbar_fence_init();
    }
    __syncthreads();
    // this CTA's share of the pulse stages: global stage st0 + st for local stage st
    const int nst_all = (a.S + pb - 1) / pb;
    const int st0 = part * nst_all / a.parts, nst = (part + 1) * nst_all / a.parts - st0;

    if (warp >= kWsConsumers / 32) {
        // ----------------------------------------------------------- producers
        const int pw = warp - kWsConsumers / 32;
        bool ok = true;
        int issued = 0;
        for (int st = 0; st < nst; ++st) {
            const int b = st & 1;
            if (st >= 2 && !mbar_wait(&bars[2 + b], ((st - 2) >> 1) & 1, 128, 2048, a.wait_budget)) {
                ok = false;
                break;
            }
            if (st == 0 && a.hold_first_stage) {   // nothing computed, copied or arrived for it
                issued = 1;
                continue;
            }
            const int s0 = (st0 + st) * pb, npb = min(pb, a.S - s0);
            float4* coef = coef0 + b * pair_coef_f4(pb);
            int* base = base0 + b * pb;
            float4* win = win0 + (size_t)b * pb * wst;
            int mine = 0;   // pulses of this stage staged by this warp
            for (int pass = 8 * pw; pass < npb; pass += 8 * kWsProducers) {
                producer_coeffs_pair(g, a.pulses, s0, npb, pass, anchors, coef, base, lane, ww, a.flags);
                mine += min(8, npb - pass);
                if ((npb & 1) && npb - pass < 8) {   // this pass holds the padding pulse: zero its window
                    float4* pw_ = win + (size_t)npb * wst;
                    for (int e = lane; e < wst; e += 32) pw_[e] = make_float4(0.f, 0.f, 0.f, 0.f);
                }
            }
            __syncwarp();
            if (lane == 0) mbar_arrive_expect_tx(&bars[b], (uint32_t)(mine * wst * sizeof(float4)));
            for (int pass = 8 * pw; pass < npb; pass += 8 * kWsProducers) {
                const int pi = pass + lane;
                if (lane < 8 && pi < npb) {
                    const void* src;
                    if (VALUES) {
                        bool clamped;
                        const long g0 = value_window_start(base[pi], ww, a.bg0, a.Lg, &clamped);
                        if (clamped) raise_flag(a.flags, FLAG_TILE_WINDOW);
                        src = reinterpret_cast<const float2*>(a.pairs) + (size_t)(s0 + pi) * a.Lg + g0;
                    } else {
                        long gi = (long)base[pi] - ww / 2 - a.bg0;
                        if (gi < 0 || gi > (long)a.Lg - ww) {
                            raise_flag(a.flags, FLAG_TILE_WINDOW);
                            gi = gi < 0 ? 0 : (long)a.Lg - ww;
                        }
                        src = a.pairs + (size_t)(s0 + pi) * a.Lg + gi;
                    }
                    fence_proxy_async_smem();
                    bulk_g2s(win + (size_t)pi * wst, src, (uint32_t)(wst * sizeof(float4)), &bars[b]);
                }
            }
            issued = st + 1;
        }
        // drain: wait (with the full budget) for this warp's own copies of the last two stages, so
        // that no bulk copy into this CTA's shared memory is in flight when it exits
        for (int st = max(0, issued - 2); st < issued; ++st)
            if (!(st == 0 && a.hold_first_stage) && !mbar_wait(&bars[st & 1], (st >> 1) & 1, 128, 2048)) ok = false;
        if (!ok && lane == 0) raise_flag(a.flags, FLAG_WAIT_TIMEOUT);
        return;
    }

    // -------------------------------------------------------------- consumers
    // u: the thread's fixed offset (from the lane), DU[r]: its four offsets along the other axis
    const int q = LANES_Y ? (warp >= 4) + 2 * (lane >= 16) : (lane >= 16) + 2 * (warp >= 4);
    const float u = (float)(lane - 8 - 16 * (lane >= 16));
    const float2 U1 = f2(u, u), U2 = f2(u * u, u * u), U3 = f2(u * u * u, u * u * u);
    float2 DU[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const float d = (float)(4 * warp + r - 8 - 16 * (warp >= 4));
        DU[r] = f2(d, d);
    }
    const float2 SH = f2(SAR_SHIFTER, SAR_SHIFTER), NSH = f2(-SAR_SHIFTER, -SAR_SHIFTER);
    const float2 M1 = f2(-1.f, -1.f), TWO_PI2 = f2(SAR_TWO_PI, SAR_TWO_PI);
    const int idx_bias = ww / 2 - SAR_SHIFTER_BITS;
    const unsigned idx_max = (unsigned)(ww - 1);
    float acc_re[4], acc_im[4];
    float2 acc2_re[4], acc2_im[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) acc2_re[r] = acc2_im[r] = f2(0.f, 0.f);
    bool ok = true;
    for (int st = 0; st < nst; ++st) {
        const int b = st & 1;
        if (!mbar_wait(&bars[b], (st >> 1) & 1, 32, 256, a.wait_budget)) {
            ok = false;
            break;
        }
        const int npp = (min(pb, a.S - (st0 + st) * pb) + 1) >> 1;
        const float4* coef = coef0 + b * pair_coef_f4(pb) + q * kPairSetF4;
        const float4* win = win0 + (size_t)b * pb * wst;
        float2* st_re = acc2_re;
        float2* st_im = acc2_im;
#pragma unroll 1
        for (int pp = 0; pp < npp; ++pp) {
            const float4* cs = coef + pp * (4 * kPairSetF4);
            const float4 A = cs[0], B = cs[1], C = cs[2], D = cs[3], E = cs[4], F = cs[5], G = cs[6], H = cs[7];
            // The thread's terms of both pulses: ph = cph + b1 d + b2 d^2 + c9 d^3 and
            // v = cv + bv1 d + bv2 d^2 in the offset d along the warp's axis (sar_geom.cuh Coeffs:
            // c0..c9 = A.xy A.zw B.xy B.zw C.xy C.zw D.xy D.zw E.xy E.zw, v0..v5 = F.xy .. H.zw).
            float2 cph, b1, b2, c9, cv, bv1, bv2;
            float2 vtop = f2(0.f, 0.f), ci = f2(0.f, 0.f), cid = f2(0.f, 0.f);   // split-bin terms
            if (PRECISE) {
                // v also has the cubic monomials w0 di^3 + w1 di^2 dj + w2 di dj^2 + w3 dj^3 and an
                // exact integer part i0 + ia di + ib dj (I = [ia ib], J = [w0 w1], K = [w2 w3], L = [i0])
                const float4 I = cs[8], J = cs[9], K = cs[10], L = cs[11];
                if (LANES_Y) {   // u = dj, d = di
                    cv = fma2(f2(K.z, K.w), U3, fma2(f2(H.z, H.w), U2, fma2(f2(G.x, G.y), U1, f2(F.x, F.y))));
                    bv1 = fma2(f2(K.x, K.y), U2, fma2(f2(H.x, H.y), U1, f2(F.z, F.w)));
                    bv2 = fma2(f2(J.z, J.w), U1, f2(G.z, G.w));
                    vtop = f2(J.x, J.y);
                    ci = fma2(f2(I.z, I.w), U1, f2(L.x, L.y));
                    cid = f2(I.x, I.y);
                } else {         // u = di, d = dj
                    cv = fma2(f2(J.x, J.y), U3, fma2(f2(G.z, G.w), U2, fma2(f2(F.z, F.w), U1, f2(F.x, F.y))));
                    bv1 = fma2(f2(J.z, J.w), U2, fma2(f2(H.x, H.y), U1, f2(G.x, G.y)));
                    bv2 = fma2(f2(K.x, K.y), U1, f2(H.z, H.w));
                    vtop = f2(K.z, K.w);
                    ci = fma2(f2(I.x, I.y), U1, f2(L.x, L.y));
                    cid = f2(I.z, I.w);
                }
            }
            if (LANES_Y) {   // u = dj, d = di
                cph = fma2(f2(E.z, E.w), U3, fma2(f2(C.z, C.w), U2, fma2(f2(B.x, B.y), U1, f2(A.x, A.y))));
                b1 = fma2(f2(E.x, E.y), U2, fma2(f2(C.x, C.y), U1, f2(A.z, A.w)));
                b2 = fma2(f2(D.z, D.w), U1, f2(B.z, B.w));
                c9 = f2(D.x, D.y);
                if (!PRECISE) {
                    cv = fma2(f2(H.z, H.w), U2, fma2(f2(G.x, G.y), U1, f2(F.x, F.y)));
                    bv1 = fma2(f2(H.x, H.y), U1, f2(F.z, F.w));
                    bv2 = f2(G.z, G.w);
                }
            } else {         // u = di, d = dj (as column_terms, linear bins)
                cph = fma2(f2(D.x, D.y), U3, fma2(f2(B.z, B.w), U2, fma2(f2(A.z, A.w), U1, f2(A.x, A.y))));
                b1 = fma2(f2(D.z, D.w), U2, fma2(f2(C.x, C.y), U1, f2(B.x, B.y)));
                b2 = fma2(f2(E.x, E.y), U1, f2(C.z, C.w));
                c9 = f2(E.z, E.w);
                if (!PRECISE) {
                    cv = fma2(f2(G.z, G.w), U2, fma2(f2(F.z, F.w), U1, f2(F.x, F.y)));
                    bv1 = fma2(f2(H.x, H.y), U1, f2(G.x, G.y));
                    bv2 = f2(H.z, H.w);
                }
            }
            // the thread's phase constant mod 1 (once per pulse pair): its pixels' phases then stay
            // below ~5 cycles, which __sincosf's own argument reduction takes as is
            cph = fma2(f2(rintf(cph.x), rintf(cph.y)), M1, cph);
            const float4* wa = win + (size_t)(2 * pp) * wst;
            const float4* wb = wa + wst;
            // nearest-bin value windows: the pulse's window start within its copy (0 or 1 value; a
            // window clamped at the span's end is flagged, and the offset stays 0 or 1 regardless)
            const float2 *va = nullptr, *vb = nullptr;
            if (VALUES) {   // the copy starts at the window's first bin rounded down to even
                const int* bp = base0 + b * pb + 2 * pp;
                va = reinterpret_cast<const float2*>(wa) + ((bp[0] - ww / 2 - a.bg0) & 1);
                vb = reinterpret_cast<const float2*>(wa + wst) + ((bp[1] - ww / 2 - a.bg0) & 1);
            }
            // lanes along x: window addresses straight from the shifter's bits (index rint(v) +
            // ww / 2 = bits + idx_bias; 32-bit shared addresses, mod 2^32) with no clamp -- the
            // producers' bound on every set keeps the index in [0, ww - 1] (measured 4 % faster
            // there; lanes along y keep the clamped form, which is faster for them)
            const uint32_t wa_s = smem_addr(wa), wb_s = wa_s + 16u * (uint32_t)ww;
            const uint32_t wa_b = wa_s + 16u * (uint32_t)idx_bias, wb_b = wb_s + 16u * (uint32_t)idx_bias;
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                const float2 d = DU[r];
                const float2 ph = fma2(fma2(fma2(c9, d, b2), d, b1), d, cph);
                const float2 v = PRECISE ? fma2(fma2(fma2(vtop, d, bv2), d, bv1), d, cv) : fma2(fma2(bv2, d, bv1), d, cv);
                float2 r1 = add2(v, SH);
                const float2 s = fma2(add2(r1, NSH), M1, v);               // v - rint(v), exact
                if (PRECISE) r1 = add2(r1, fma2(cid, d, ci));              // + the exact integer part
                unsigned ia = 0, ib = 0;
                uint32_t aa = 0, ab = 0;
                if (LANES_Y || VALUES) {
                    ia = min((unsigned)(__float_as_int(r1.x) + idx_bias), idx_max);
                    ib = min((unsigned)(__float_as_int(r1.y) + idx_bias), idx_max);
                } else {
                    aa = wa_b + ((uint32_t)__float_as_int(r1.x) << 4);
                    ab = wb_b + ((uint32_t)__float_as_int(r1.y) << 4);
                }
                if (NEAREST && (fabsf(s.x) > kNearEdge || fabsf(s.y) > kNearEdge)) {
                    // near a rounding boundary: the exact bin, as a window index of the pulse (of the
                    // image pixel, on a sheared lattice)
                    const int py = tj * kTile + (LANES_Y ? lane : 4 * warp + r);
                    const int px = ti * kTile + (LANES_Y ? 4 * warp + r : lane) + (SHEARED ? g.a_off + g.shear * py : 0);
                    const int sp = (st0 + st) * pb + 2 * pp;
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        if (fabsf(h ? s.y : s.x) <= kNearEdge || sp + h >= a.S) continue;
                        // the window's first bin: for value windows (index 0 of va / vb) unclamped -- a
                        // clamped window is flagged, and the index below is clamped into the window
                        // either way; for pair windows where the producer placed it
                        const int g0 = VALUES ? base0[b * pb + 2 * pp + h] - ww / 2 - a.bg0
                                              : min(max(base0[b * pb + 2 * pp + h] - ww / 2 - a.bg0, 0), a.Lg - ww);
                        const int gi = exact_grid_bin(a.steps, a.pulses, a.alpha2, g.s_r.hi, g.s_r.lo, a.bg0,
                                                      BIN_ADJ_NEAREST, px, py, k, sp + h);
                        const unsigned w = min((unsigned)(gi - g0), idx_max);
                        if (LANES_Y || VALUES) {
                            if (h) ib = w; else ia = w;
                        } else {
                            if (h) ab = wb_s + 16u * w; else aa = wa_s + 16u * w;
                        }
                    }
                }
                float2 re, im;
                if (VALUES && NEAREST) {   // the bin's value, no interpolation
                    const float2 pa = va[ia], pq = vb[ib];
                    re = f2(pa.x, pq.x);
                    im = f2(pa.y, pq.y);
                } else if (VALUES) {   // p(n) + (s + 1/2) (p(n + 1) - p(n)), s in [-1/2, 1/2]
                    const float2 pa = va[ia], pq = vb[ib], pa1 = va[ia + 1], pq1 = vb[ib + 1];
                    const float2 t = add2(s, f2(0.5f, 0.5f));
                    re = fma2(t, f2(pa1.x - pa.x, pq1.x - pq.x), f2(pa.x, pq.x));
                    im = fma2(t, f2(pa1.y - pa.y, pq1.y - pq.y), f2(pa.y, pq.y));
                } else {
                    const float4 pa = LANES_Y ? wa[ia] : lds_f4(aa), pq = LANES_Y ? wb[ib] : lds_f4(ab);
                    re = f2(fmaf(s.x, pa.z, pa.x), fmaf(s.y, pq.z, pq.x));
                    im = f2(fmaf(s.x, pa.w, pa.y), fmaf(s.y, pq.w, pq.y));
                }
                const float2 x = mul2(ph, TWO_PI2);   // |ph| < ~5 cycles: no per-pixel reduction
                float2 sn, cn;
                __sincosf(x.x, &sn.x, &cn.x);
                __sincosf(x.y, &sn.y, &cn.y);
                st_re[r] = fma2(re, cn, fma2(im, sn, st_re[r]));
                st_im[r] = fma2(im, cn, fma2(f2(-re.x, -re.y), sn, st_im[r]));
            }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&bars[2 + b]);
    }
    if (!ok) {
        if (lane == 0) raise_flag(a.flags, FLAG_WAIT_TIMEOUT);
        return;
    }
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        acc_re[r] = acc2_re[r].x + acc2_re[r].y;
        acc_im[r] = acc2_im[r].x + acc2_im[r].y;
    }
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        // lattice pixel (a, j) is image pixel (a + a_off + shear j, j)
        const int j = tj * kTile + (LANES_Y ? lane : 4 * warp + r);
        const int i = ti * kTile + (LANES_Y ? 4 * warp + r : lane) + (SHEARED ? g.a_off + g.shear * j : 0);
        if ((SHEARED ? (i >= 0 && i < g.img_nx) : i < g.nx) && j < g.ny) {
            const size_t p = ((size_t)k * g.ny + j) * (SHEARED ? g.img_nx : g.nx) + i;
            if (a.parts > 1) {   // the image was zeroed by the launcher (parts > 1 never accumulates)
                atomicAdd(&a.x[p].x, acc_re[r]);
                atomicAdd(&a.x[p].y, acc_im[r]);
                continue;
            }
            float2 o = make_float2(acc_re[r], acc_im[r]);
            if (a.accumulate) {
                const float2 old = a.x[p];
                o.x += old.x;
                o.y += old.y;
            }
            a.x[p] = o;
        }
    }
}

// CTAs per tile: two CTAs (each over half of the pulse stages) when that fills the last wave of
// the two-CTAs-per-SM grid clearly better (4096 tiles on 152 SMs: 13.5 waves, 96 % of the last
// one idle-free time; 8192 CTAs: 27.0 waves, 99.8 %).  Two partial sums added to a zeroed image
// give the same bits in either order; added onto an image that already holds a sum (accumulate)
// they would be three terms in run-dependent order, so accumulating launches use one CTA per tile.
static int ws_parts(long tiles, int nst, int accumulate) {
    int dev = 0, sms = 0;
    if (accumulate || nst < 4 || cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0)
        return 1;
    const double w1 = (double)tiles / (2.0 * sms), w2 = 2.0 * w1;
    const double e1 = w1 / std::ceil(w1), e2 = w2 / std::ceil(w2);
    return e2 > e1 + 0.02 ? 2 : 1;
}

cudaError_t launch_bp_grid_ws(const BpGridArgs& a_in, cudaStream_t st) {
    if (a_in.pb < 1 || a_in.pb > 32 || a_in.wwin < 4 || (a_in.wwin & 3)) return cudaErrorInvalidValue;
    BpGridArgs a = a_in;
    const long tiles = (long)a.g.tiles_x * a.g.tiles_y * a.g.nz;
    a.parts = ws_parts(a.tiles_valid > 0 ? a.tiles_valid : tiles, (a.S + a.pb - 1) / a.pb, a.accumulate);
    if (a.parts > 1) {
        const cudaError_t z =
            cudaMemsetAsync(a.x, 0, sizeof(float2) * (size_t)a.g.img_nx * a.g.ny * a.g.nz, st);
        if (z != cudaSuccess) return z;
    }
    // value windows copy from even bins of rows of an even length (16-byte aligned)
    if (a.values && ((a.Lg & 1) || a.Lg < a.wwin + 2)) return cudaErrorInvalidValue;
    const size_t smem = bp_grid_ws_smem_bytes(a.wwin, a.pb, a.values);
    const unsigned blocks = (unsigned)(tiles * a.parts);
    cudaError_t e;
    auto go = [&](auto kernel) -> cudaError_t {
        cudaError_t err = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (err != cudaSuccess) return err;
        kernel<<<blocks, kWsThreads, smem, st>>>(a);
        return cudaSuccess;
    };
    if (a.g.shear) {   // sheared lattices: linear sampling, lanes along the lattice's second axis
        if (a.nearest || !a.lanes_y || (a.values && !a.g.precise_bins)) return cudaErrorInvalidValue;
        if (a.values)
            e = go(bp_grid_ws_pair_kernel<true, true, false, true, true>);
        else
            e = a.g.precise_bins ? go(bp_grid_ws_pair_kernel<true, true, false, false, true>)
                                 : go(bp_grid_ws_pair_kernel<true, false, false, false, true>);
    } else if (a.nearest) {
        if (!a.g.precise_bins || !a.steps || !a.alpha2) return cudaErrorInvalidValue;
        if (a.values)
            e = a.lanes_y ? go(bp_grid_ws_pair_kernel<true, true, true, true>)
                          : go(bp_grid_ws_pair_kernel<false, true, true, true>);
        else
            e = a.lanes_y ? go(bp_grid_ws_pair_kernel<true, true, true>) : go(bp_grid_ws_pair_kernel<false, true, true>);
    } else if (a.values) {   // linear sampling from value windows (wide windows: split bins)
        if (!a.g.precise_bins) return cudaErrorInvalidValue;
        e = a.lanes_y ? go(bp_grid_ws_pair_kernel<true, true, false, true>)
                      : go(bp_grid_ws_pair_kernel<false, true, false, true>);
    } else if (a.g.precise_bins) {
        e = a.lanes_y ? go(bp_grid_ws_pair_kernel<true, true, false>) : go(bp_grid_ws_pair_kernel<false, true, false>);
    } else {
        e = a.lanes_y ? go(bp_grid_ws_pair_kernel<true, false, false>)
                      : go(bp_grid_ws_pair_kernel<false, false, false>);
    }
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
}

// ------------------------------------------- K3 (grid, warp-specialised pipeline)
// CTA = (strip segment of tiles along y, block of pbf pulses), 8 gathering warps + 2 producers,
// pipelined per tile with two buffers.  Producers, per tile: load the tile's image values into
// shared memory, compute the coefficient sets of every (pulse, sub-tile) and a per-pulse "fast"
// flag, then arrive on the buffer's "full" mbarrier.  Gathering warp w owns pulses w, w+8, ...:
// for each, lanes run along the tile's x axis and the warp walks the 32 rows; contributions go
// to the pulse's shared-memory window, which only this warp touches.  When the bin rate along x
// is at least 1.05 bins/pixel over the whole tile (checked by the producer from the quadratic
// bin model, with margin for FP32 rounding), the 32 lanes of a row always hit 32 distinct bins,
// so plain read-modify-writes are safe: first to bin n, then to bin n + 1, with __syncwarp in
// between.  Otherwise shared-memory atomics are used.  After the strip the windows are merged
// into the global accumulator with one atomic add per bin.
// Template argument TRANSPOSED: lanes run along y and the warp walks the tile's 32 columns (the
// image tile is staged transposed, rows padded to 33 values), for collections whose range bins
// change fast along y and slowly along x; the producer's tests then take the bin rates along y
// for the lanes and along x for the rows.
constexpr float kFastBinRate = 1.05f;
constexpr int kXtStride = kTile + 1;   // staged image tile: 32 lines of 33 values

__device__ __forceinline__ size_t align_up(size_t n, size_t a) { return (n + a - 1) & ~(a - 1); }

__host__ __device__ inline int window_slots(int ws) { return ws + (ws >> 4) + 1; }

struct FpWsLayout {
    size_t win, coef, xt, base, fast, wst, bars, anchors, total;
};

// wide_x: image values staged as (re, re, im, im) (the linear run-window kernels), else (re, im).
__host__ __device__ inline FpWsLayout fp_ws_layout(int ws, int pbf, int wide_x) {
    FpWsLayout L;
    L.win = 0;
    L.coef = L.win + (size_t)pbf * window_slots(ws) * sizeof(float2);
    L.coef = (L.coef + 15) & ~(size_t)15;
    L.xt = L.coef + (size_t)2 * pbf * 4 * kSetF4 * sizeof(float4);
    L.base = L.xt + (size_t)2 * kTile * kXtStride * (wide_x ? sizeof(float4) : sizeof(float2));
    L.fast = L.base + (size_t)2 * pbf * sizeof(int);
    L.wst = L.fast + (size_t)2 * pbf * sizeof(int);
    L.bars = (L.wst + (size_t)pbf * sizeof(int) + 7) & ~(size_t)7;
    L.anchors = L.bars + 4 * sizeof(uint64_t);
    L.total = L.anchors + (size_t)kWsProducers * 4 * sizeof(df3);
    return L;
}

size_t fp_grid_ws_smem_bytes(int ws, int pbf, int wide_x) { return fp_ws_layout(ws, pbf, wide_x).total; }

// Window slot of bin w: one padding slot every 16 bins, so lanes whose bins differ by a
// multiple of 16 do not share a shared-memory bank pair.
__device__ __forceinline__ int wslot(int w) { return w + (w >> 4); }

template <bool PRECISE>
struct RowEval {
    BinPos bp;
    float cr, ci;
};

template <bool PRECISE>
__device__ __forceinline__ RowEval<PRECISE> scatter_eval(const ColumnTerms& ct, float c9, float w9, float ib, float dj,
                                                         float2 xv) {
    RowEval<PRECISE> e;
    const float dj2 = dj * dj, dj3 = dj2 * dj;
    const float ph = pixel_phase(ct, c9, dj, dj2, dj3);
    const float v = pixel_bin<PRECISE>(ct, w9, dj, dj2, dj3);
    e.bp = bin_position<PRECISE>(v, PRECISE ? fmaf(ib, dj, ct.ci) : 0.f);
    float sn, cn;
    __sincosf(SAR_TWO_PI * ph, &sn, &cn);   // |ph| < ~5 cycles: the caller reduced the constants
    e.cr = fmaf(xv.x, cn, -xv.y * sn);   // x * exp(+2 pi i f)
    e.ci = fmaf(xv.x, sn, xv.y * cn);
    return e;
}

__device__ __forceinline__ void rmw_add(float2* wp, int idx, float w, float cr, float ci) {
    float2* q = wp + wslot(idx);
    float2 u = *q;
    u.x = fmaf(w, cr, u.x);
    u.y = fmaf(w, ci, u.y);
    *q = u;
}

// A staged image value: (re, im), or (re, re, im, im) for the linear run-window kernels.
__device__ __forceinline__ float2 staged_value(const float2 v) { return v; }
__device__ __forceinline__ float2 staged_value(const float4 v) { return make_float2(v.x, v.z); }

// What the nearest-bin scatter needs to decide a bin again exactly (exact_grid_bin): the pixel of
// row 0 / lane 0 of the half tile, the walk direction, both pulses and their window starts.
struct NearCtx {
    const double* steps;
    const PulseGeom* pulses;
    const float4* alpha2;
    float sr_hi, sr_lo;
    int bg0, i0, j0, k, transposed;
    int sp, sq;     // pulse indices
    int wsp, wsq;   // first bin (absolute) of each pulse's window
    int a_off, shear;   // lattice pixel (i, j) is image pixel (i + a_off + shear j, j)
};

// 16 rows of one half tile for the pulse pair (p, q).  MODE 2: bins n, n+1 of different lanes
// disjoint (one phase per row); MODE 1: bins n distinct (two phases); MODE 0: atomics.  Nearest
// bins within 5e-5 of a rounding boundary are decided again exactly; such a bin may equal a
// neighbouring lane's, so those contributions go in with atomics in a phase of their own.
// RING: ring windows (ws a power of two; off_p / off_q are the pulses' absolute base bins and a
// bin's slot is its absolute index mod ws), else strip windows (off = base - window start).
template <bool LINEAR, bool PRECISE, int MODE, bool TWO, typename XT, bool RING = false>
__device__ __forceinline__ void scatter_rows(const ColumnTerms& ctp, float c9p, float w9p, float ibp,
                                             const ColumnTerms& ctq, float c9q, float w9q, float ibq,
                                             const XT* xrow, float2* wp, float2* wq, int off_p, int off_q,
                                             int ws, int lane, const NearCtx& nc) {
    const int mask = ws - 1;
    // the slot after slot i (the second tap of linear sampling)
    auto next = [&](int i) { return RING ? ((i + 1) & mask) : i + 1; };
    // the lane's phase constant and its rate along the rows mod 1 (rows are integer offsets)
    ColumnTerms cp = ctp, cq = ctq;
    cp.cph -= rintf(cp.cph);
    cp.b1 -= rintf(cp.b1);
    cq.cph -= rintf(cq.cph);
    cq.b1 -= rintf(cq.b1);
    unsigned edge = 0;   // nearest bins: bit 2 row + h for the pulse h contribution near a rounding boundary
#pragma unroll 2
    for (int rr = 0; rr < 16; ++rr) {
        const float dj = (float)(rr - 8);
        const float2 xv = staged_value(xrow[rr * kXtStride + lane]);
        const RowEval<PRECISE> ep = scatter_eval<PRECISE>(cp, c9p, w9p, ibp, dj, xv);
        const int ip = RING ? ((ep.bp.n + off_p) & mask) : (int)min((unsigned)(ep.bp.n + off_p), (unsigned)(ws - 2));
        RowEval<PRECISE> eq;
        int iq = 0;
        if (TWO) {
            eq = scatter_eval<PRECISE>(cq, c9q, w9q, ibq, dj, xv);
            iq = RING ? ((eq.bp.n + off_q) & mask) : (int)min((unsigned)(eq.bp.n + off_q), (unsigned)(ws - 2));
        }
        if (LINEAR) {
            const float w0p = 0.5f - ep.bp.s, w1p = 0.5f + ep.bp.s;
            const float w0q = TWO ? 0.5f - eq.bp.s : 0.f, w1q = TWO ? 0.5f + eq.bp.s : 0.f;
            if (MODE == 2) {
                rmw_add(wp, ip, w0p, ep.cr, ep.ci);
                rmw_add(wp, next(ip), w1p, ep.cr, ep.ci);
                if (TWO) {
                    rmw_add(wq, iq, w0q, eq.cr, eq.ci);
                    rmw_add(wq, next(iq), w1q, eq.cr, eq.ci);
                }
                __syncwarp();
            } else if (MODE == 1) {
                rmw_add(wp, ip, w0p, ep.cr, ep.ci);
                if (TWO) rmw_add(wq, iq, w0q, eq.cr, eq.ci);
                __syncwarp();
                rmw_add(wp, next(ip), w1p, ep.cr, ep.ci);
                if (TWO) rmw_add(wq, next(iq), w1q, eq.cr, eq.ci);
                __syncwarp();
            } else {
                float2* a0 = wp + wslot(ip);
                float2* a1 = wp + wslot(next(ip));
                atomicAdd(&a0->x, w0p * ep.cr); atomicAdd(&a0->y, w0p * ep.ci);
                atomicAdd(&a1->x, w1p * ep.cr); atomicAdd(&a1->y, w1p * ep.ci);
                if (TWO) {
                    float2* b0 = wq + wslot(iq);
                    float2* b1 = wq + wslot(next(iq));
                    atomicAdd(&b0->x, w0q * eq.cr); atomicAdd(&b0->y, w0q * eq.ci);
                    atomicAdd(&b1->x, w1q * eq.cr); atomicAdd(&b1->y, w1q * eq.ci);
                }
            }
        } else {
            if (PRECISE)   // decided again after the rows, off the common path
                edge |= ((fabsf(ep.bp.s) > kNearEdge ? 1u : 0u) | (TWO && fabsf(eq.bp.s) > kNearEdge ? 2u : 0u))
                        << (2 * rr);
            if (MODE >= 1) {
                rmw_add(wp, ip, 1.0f, ep.cr, ep.ci);
                if (TWO) rmw_add(wq, iq, 1.0f, eq.cr, eq.ci);
                __syncwarp();
            } else {
                float2* a0 = wp + wslot(ip);
                atomicAdd(&a0->x, ep.cr); atomicAdd(&a0->y, ep.ci);
                if (TWO) {
                    float2* b0 = wq + wslot(iq);
                    atomicAdd(&b0->x, eq.cr); atomicAdd(&b0->y, eq.ci);
                }
            }
        }
    }
    if (!LINEAR && PRECISE && __any_sync(0xffffffffu, edge != 0u)) {
        // Contributions whose FP32 bin position lay within 5e-5 of a rounding boundary: the exact bin
        // from the per-pixel double-float range; where it differs from the FP32 bin (where the rows
        // added it) the contribution moves there, with shared-memory atomics (the lanes' exact bins
        // may coincide).  The row's evaluation is repeated exactly as the rows made it.
        for (unsigned m = edge; m != 0u; m &= m - 1u) {
            const int bit = __ffs(m) - 1, rr = bit >> 1, h = bit & 1;
            const float dj = (float)(rr - 8);
            const float2 xv = staged_value(xrow[rr * kXtStride + lane]);
            const RowEval<PRECISE> e = h ? scatter_eval<PRECISE>(cq, c9q, w9q, ibq, dj, xv)
                                         : scatter_eval<PRECISE>(cp, c9p, w9p, ibp, dj, xv);
            const int off = h ? off_q : off_p;
            const int i32 = RING ? ((e.bp.n + off) & mask) : (int)min((unsigned)(e.bp.n + off), (unsigned)(ws - 2));
            const int pj = nc.j0 + (nc.transposed ? lane : rr);
            const int pi = nc.i0 + (nc.transposed ? rr : lane) + nc.a_off + nc.shear * pj;
            const int bx = exact_grid_bin(nc.steps, nc.pulses, nc.alpha2, nc.sr_hi, nc.sr_lo, nc.bg0, BIN_FWD_NEAREST,
                                          pi, pj, nc.k, h ? nc.sq : nc.sp) + nc.bg0;
            const int ix = RING ? (bx & mask) : min(max(bx - (h ? nc.wsq : nc.wsp), 0), ws - 1);
            if (ix == i32) continue;
            float2* w = h ? wq : wp;
            atomicAdd(&w[wslot(i32)].x, -e.cr);
            atomicAdd(&w[wslot(i32)].y, -e.ci);
            atomicAdd(&w[wslot(ix)].x, e.cr);
            atomicAdd(&w[wslot(ix)].y, e.ci);
        }
        __syncwarp();
    }
}

// MODES 5, 4 and 3 (linear bins): the producer has shown that a sub-tile's bin is monotonic down
// its rows and moves by less than kRunSpan over G = 16 (MODE 5), 8 (MODE 4) or 4 (MODE 3) rows, so in each
// group of G rows a lane's bin takes at most two values n0, n0 + 1 (n0 = the smaller of the bins
// at the group's first and last rows) and its taps lie in n0 .. n0 + 2.  The lane accumulates
// those three bins in registers for both pulses and adds them to the windows once per group, in
// three phases (lanes' bins are distinct at any one row, MODE >= 1), instead of two
// read-modify-writes per contribution.
//
// With u = v + 1/2 the tap position (taps floor(u), floor(u) + 1) and a = u - (n0 + 1) in [-1, 1),
// the three slot weights are the hat functions max(0, -a), 1 - |a| and max(0, a).  The lane keeps
// per pulse the sums C = sum c, D = sum a c and E = sum |a| c, packed over the pulse pair, and
// the slots are (E - D) / 2, C - E and (E + D) / 2: no per-row bin test or weight selection.
constexpr float kRunSpan = 0.98f;

template <bool TWO, int G>
__device__ __forceinline__ void scatter_rows_runs(const ColumnTerms& ctp, float c9p, const ColumnTerms& ctq, float c9q,
                                                  const float4* xrow, float2* wp, float2* wq, int off_p, int off_q,
                                                  int ws, int lane) {
    // the lane's phase constant and its rate along the walked rows mod 1 (rows are integer offsets),
    // so that each row's phase stays below ~5 cycles and goes to __sincosf without reduction; the
    // phase polynomial then in radians (scaled once here, not per row)
    const float2 TWO_PI2 = f2(SAR_TWO_PI, SAR_TWO_PI);
    const float2 cph = mul2(f2(ctp.cph - rintf(ctp.cph), ctq.cph - rintf(ctq.cph)), TWO_PI2);
    const float2 b1 = mul2(f2(ctp.b1 - rintf(ctp.b1), ctq.b1 - rintf(ctq.b1)), TWO_PI2);
    const float2 b2 = mul2(f2(ctp.b2, ctq.b2), TWO_PI2), c9 = mul2(f2(c9p, c9q), TWO_PI2);
    const float2 cv = f2(ctp.cv, ctq.cv), bv1 = f2(ctp.bv1, ctq.bv1), bv2 = f2(ctp.bv2, ctq.bv2);
    const float2 SH = f2(SAR_SHIFTER, SAR_SHIFTER);
    const float2 M1 = f2(-1.f, -1.f);
#pragma unroll
  for (int g0 = 0; g0 < 16; g0 += G) {
    // window slot n0 of each pulse: the smaller bin of the group's first and last rows
    int n0p, n0q;
    {
        const float2 da = f2((float)(g0 - 8), (float)(g0 - 8)), db = f2((float)(g0 + G - 9), (float)(g0 + G - 9));
        const float2 ra = add2(fma2(fma2(bv2, da, bv1), da, cv), SH);
        const float2 rb = add2(fma2(fma2(bv2, db, bv1), db, cv), SH);
        n0p = min(max(min(__float_as_int(ra.x), __float_as_int(rb.x)) - SAR_SHIFTER_BITS + off_p, 0), ws - 3);
        n0q = min(max(min(__float_as_int(ra.y), __float_as_int(rb.y)) - SAR_SHIFTER_BITS + off_q, 0), ws - 3);
    }
    // a = v - (n0 + 1/2): the bin polynomial's constant moved by -(n0 + 1/2) (exact for |n0| < 2^22)
    const float2 cva = add2(cv, f2(-((float)(n0p - off_p) + 0.5f), -((float)(n0q - off_q) + 0.5f)));
    float2 Cr = f2(0.f, 0.f), Ci = f2(0.f, 0.f), Dr = f2(0.f, 0.f), Di = f2(0.f, 0.f);
    float2 Er = f2(0.f, 0.f), Ei = f2(0.f, 0.f);
#pragma unroll 4
    for (int rr = g0; rr < g0 + G; ++rr) {
        const float dj = (float)(rr - 8);
        const float2 d = f2(dj, dj);
        // the pixel value staged as (re, re, im, im): both pulses' products packed
        const float4 X = xrow[rr * kXtStride + lane];
        const float2 XR = f2(X.x, X.y), XI = f2(X.z, X.w);
        const float2 x = fma2(fma2(fma2(c9, d, b2), d, b1), d, cph);
        const float2 av = fma2(fma2(bv2, d, bv1), d, cva);
        const float2 aa = f2(fabsf(av.x), fabsf(av.y));
        float2 sn, cn;
        __sincosf(x.x, &sn.x, &cn.x);
        __sincosf(x.y, &sn.y, &cn.y);
        // c = x exp(+i phase) for both pulses
        const float2 xs = mul2(XI, sn);
        const float2 cr = fma2(XR, cn, f2(-xs.x, -xs.y));
        const float2 ci = fma2(XR, sn, mul2(XI, cn));
        Cr = add2(Cr, cr);
        Ci = add2(Ci, ci);
        Dr = fma2(av, cr, Dr);
        Di = fma2(av, ci, Di);
        Er = fma2(aa, cr, Er);
        Ei = fma2(aa, ci, Ei);
    }
    {
        const float2 s0r = mul2(add2(Er, mul2(Dr, M1)), f2(0.5f, 0.5f)), s0i = mul2(add2(Ei, mul2(Di, M1)), f2(0.5f, 0.5f));
        const float2 s1r = add2(Cr, mul2(Er, M1)), s1i = add2(Ci, mul2(Ei, M1));
        const float2 s2r = mul2(add2(Er, Dr), f2(0.5f, 0.5f)), s2i = mul2(add2(Ei, Di), f2(0.5f, 0.5f));
        rmw_add(wp, n0p, 1.0f, s0r.x, s0i.x);
        if (TWO) rmw_add(wq, n0q, 1.0f, s0r.y, s0i.y);
        __syncwarp();
        rmw_add(wp, n0p + 1, 1.0f, s1r.x, s1i.x);
        if (TWO) rmw_add(wq, n0q + 1, 1.0f, s1r.y, s1i.y);
        __syncwarp();
        rmw_add(wp, n0p + 2, 1.0f, s2r.x, s2i.x);
        if (TWO) rmw_add(wq, n0q + 2, 1.0f, s2r.y, s2i.y);
        __syncwarp();
    }
  }
}

// Mode of a pulse pair that shares one pass over the rows: a mode both pulses' guarantees admit.
// The run modes nest (16-row runs imply 8- and 4-row runs), so two of them take the smaller; any
// other two different modes share only the distinct-bin guarantee (a run mode may rest on MODE 1's
// rather than MODE 2's) or nothing (MODE 0).
__device__ __forceinline__ int pair_mode(int a, int b) {
    if (a == b) return a;
    if (a >= 3 && b >= 3) return min(a, b);
    return min(min(a, b), 1);
}

template <bool LINEAR, bool PRECISE, bool TWO, typename XT, bool RING = false>
__device__ __forceinline__ void scatter_half(int mode, const ColumnTerms& ctp, float c9p, float w9p, float ibp,
                                             const ColumnTerms& ctq, float c9q, float w9q, float ibq,
                                             const XT* xrow, float2* wp, float2* wq, int off_p, int off_q,
                                             int ws, int lane, const NearCtx& nc) {
    if constexpr (LINEAR && !PRECISE && !RING) {
        if (mode == 5) {
            scatter_rows_runs<TWO, 16>(ctp, c9p, ctq, c9q, xrow, wp, wq, off_p, off_q, ws, lane);
            return;
        }
        if (mode == 4) {
            scatter_rows_runs<TWO, 8>(ctp, c9p, ctq, c9q, xrow, wp, wq, off_p, off_q, ws, lane);
            return;
        }
        if (mode == 3) {
            scatter_rows_runs<TWO, 4>(ctp, c9p, ctq, c9q, xrow, wp, wq, off_p, off_q, ws, lane);
            return;
        }
    }
    if (mode >= 2)
        scatter_rows<LINEAR, PRECISE, 2, TWO, XT, RING>(ctp, c9p, w9p, ibp, ctq, c9q, w9q, ibq, xrow, wp, wq, off_p, off_q, ws, lane,
                                              nc);
    else if (mode == 1)
        scatter_rows<LINEAR, PRECISE, 1, TWO, XT, RING>(ctp, c9p, w9p, ibp, ctq, c9q, w9q, ibq, xrow, wp, wq, off_p, off_q, ws, lane,
                                              nc);
    else
        scatter_rows<LINEAR, PRECISE, 0, TWO, XT, RING>(ctp, c9p, w9p, ibp, ctq, c9q, w9q, ibq, xrow, wp, wq, off_p, off_q, ws, lane,
                                              nc);
}

// Adds the window slots of bins [lo, hi] (absolute) of one pulse into its accumulator row and clears
// them (ring windows: the bins a tile step leaves behind, and the last tile's at the end).
__device__ __forceinline__ void ring_flush(float2* wp, int lo, int hi, int mask, const FpGridArgs& a, int s,
                                           int lane) {
    for (int bin = lo + lane; bin <= hi; bin += 32) {
        float2* q = wp + wslot(bin & mask);
        const float2 v = *q;
        if (v.x == 0.f && v.y == 0.f) continue;
        *q = make_float2(0.f, 0.f);
        const long gi = (long)bin - a.bg0;
        if (gi < 0 || gi >= a.Lg) {
            raise_flag(a.flags, FLAG_STRIP_WINDOW);
            continue;
        }
        atomicAdd(a.acc + (size_t)s * a.Lg + gi, v);
    }
}

// RING (split bins only): ring windows instead of strip windows (FpGridArgs.ring_half): a CTA walks
// its whole line of tiles and, between tiles, each warp adds and clears the bins its pulses leave
// behind, so windows no longer bound the length of a strip (1-tile strips at upsample 128 otherwise).
template <bool LINEAR, bool PRECISE, bool TRANSPOSED, bool RING = false>
__global__ void __launch_bounds__(kWsThreads, RING ? 1 : 2) fp_grid_ws_kernel(const FpGridArgs a) {
    extern __shared__ __align__(16) unsigned char fsm[];
    const int pbf = a.pbf, ws = a.ws, wslots = window_slots(ws);
    constexpr bool WIDE_X = LINEAR && !PRECISE;
    using XT = typename std::conditional<WIDE_X, float4, float2>::type;
    const FpWsLayout L = fp_ws_layout(ws, pbf, WIDE_X);
    float2* win = reinterpret_cast<float2*>(fsm + L.win);
    float4* coef0 = reinterpret_cast<float4*>(fsm + L.coef);
    XT* xt0 = reinterpret_cast<XT*>(fsm + L.xt);
    int* base0 = reinterpret_cast<int*>(fsm + L.base);
    int* fast0 = reinterpret_cast<int*>(fsm + L.fast);
    int* wst = reinterpret_cast<int*>(fsm + L.wst);
    uint64_t* bars = reinterpret_cast<uint64_t*>(fsm + L.bars);   // full[0..1], empty[2..3]
    df3* anchors_all = reinterpret_cast<df3*>(fsm + L.anchors);

    const GridConst& g = a.g;
    // Strips are lines of tiles along the walked axis: columns along y, or rows along x when
    // TRANSPOSED (range bins change slowly along them, so their windows stay short).
    const int lines = TRANSPOSED ? g.tiles_y : g.tiles_x, along = TRANSPOSED ? g.tiles_x : g.tiles_y;
    int bidx = blockIdx.x;
    const int seg = bidx % a.segs_per_column;
    bidx /= a.segs_per_column;
    const int line = bidx % lines;
    const int k = bidx / lines;
    const int strip = (k * lines + line) * a.segs_per_column + seg;
    const int s0 = blockIdx.y * pbf;
    const int npb = min(pbf, a.S - s0);
    // the line's tiles (on a sheared lattice only those holding image pixels) and this segment's
    int t_lo = 0, t_hi = along - 1;
    if (!TRANSPOSED) lattice_tile_range(g, line, &t_lo, &t_hi);
    const int t0 = t_lo + seg * a.seg_tiles;
    const int ntile = min(a.seg_tiles, t_hi + 1 - t0);
    if (ntile <= 0) return;   // no tile: the whole CTA leaves before any barrier exists
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    for (int e = threadIdx.x; e < pbf * wslots; e += blockDim.x) win[e] = make_float2(0.f, 0.f);
    for (int e = threadIdx.x; e < npb; e += blockDim.x)
        wst[e] = RING ? 0 : a.strip_start[(size_t)strip * a.strip_stride + s0 + e];
    if (threadIdx.x == 0) {
        mbar_init(&bars[0], kWsProducers);
        mbar_init(&bars[1], kWsProducers);
        mbar_init(&bars[2], kWsConsumers / 32);
        mbar_init(&bars[3], kWsConsumers / 32);
        mbar_fence_init();
    }
    __syncthreads();

    if (warp >= kWsConsumers / 32) {
        // ----------------------------------------------------------- producers
        const int pw = warp - kWsConsumers / 32;
        df3* anchors = anchors_all + 4 * pw;
        for (int t = 0; t < ntile; ++t) {
            const int b = t & 1;
            if (t >= 2 && !mbar_wait(&bars[2 + b], ((t - 2) >> 1) & 1, 128, 2048)) {
                if (lane == 0) raise_flag(a.flags, FLAG_WAIT_TIMEOUT);
                return;   // the gathering warps time out on "full" and leave as well
            }
            const int ti = TRANSPOSED ? t0 + t : line, tj = TRANSPOSED ? line : t0 + t;
            if (lane < 4) anchors[lane] = subtile_anchor(ti, tj, k, lane, g);
            // this warp's half of the tile's image values (rows 16 pw .. 16 pw + 15); lattice pixel
            // (i, j) is image pixel (i + a_off + shear j, j), zero outside the image
            XT* xt = xt0 + b * kTile * kXtStride;
            const int i = ti * kTile + lane;
            for (int r = 16 * pw; r < 16 * pw + 16; ++r) {
                const int j = tj * kTile + r;
                const int ic = i + g.a_off + g.shear * j;
                const float2 xv = (ic >= 0 && ic < g.img_nx && j < g.ny) ? a.x[((size_t)k * g.ny + j) * g.img_nx + ic]
                                                                        : make_float2(0.f, 0.f);
                XT sv;   // (re, im), or (re, re, im, im)
                if constexpr (WIDE_X)
                    sv = make_float4(xv.x, xv.x, xv.y, xv.y);
                else
                    sv = xv;
                xt[TRANSPOSED ? lane * kXtStride + r : r * kXtStride + lane] = sv;   // line = walked offset
            }
            __syncwarp();
            float4* coef = coef0 + b * pbf * 4 * kSetF4;
            int* base = base0 + b * pbf;
            int* fast = fast0 + b * pbf;
            for (int pass = 8 * pw; pass < npb; pass += 8 * kWsProducers) {
                producer_coeffs(g, a.pulses, s0, npb, pass, anchors, coef, base, lane, RING ? a.ring_half : 0, a.flags);
                __syncwarp();
                // Distinct-bin guarantee along x for each pulse of the pass: the smallest
                // |dv/di| over the sub-tile from the quadratic bin model (di, dj in [-8, 7]).
                // The rate must also have one sign in all four sub-tiles, so that bins along a
                // row are monotonic across the sub-tile boundary.
                const int pi = pass + (lane >> 2), q = lane & 3;
                bool ok_q = true, wide_q = true, pos_q = true, runs_q = true, runs8_q = true, runs4_q = true;
                if (pi < npb) {
                    const float4* cs = coef + (pi * 4 + q) * kSetF4;
                    const float4 C = cs[2], D = cs[3], E = cs[4];
                    // bin rates along x: dv/di = v1 (+ ia) + 2 v3 di + v4 dj; along y: dv/dj = v2 (+ ib) +
                    // v4 di + 2 v5 dj, with di, dj in [-8, 7]
                    const float rx = C.w + E.x, ry = D.x + E.y;
                    const float cx = 16.0f * fabsf(D.y) + 8.0f * fabsf(D.z), cy = 8.0f * fabsf(D.z) + 16.0f * fabsf(D.w);
                    const float r1 = TRANSPOSED ? ry : rx;            // along the lanes
                    const float rmin = fabsf(r1) - (TRANSPOSED ? cy : cx);
                    ok_q = rmin >= kFastBinRate;
                    wide_q = rmin >= kFastBinRate + 1.0f;
                    pos_q = r1 > 0.0f;
                    // bin down the 16 walked lines of the sub-tile: monotonic (the rate keeps its
                    // sign) and changing by less than kRunSpan in all
                    const float rw = fabsf(TRANSPOSED ? C.w : D.x), curv = TRANSPOSED ? cx : cy;
                    runs_q = rw > curv && 15.0f * (rw + curv) < kRunSpan;    // 16-line runs
                    runs8_q = rw > curv && 7.0f * (rw + curv) < kRunSpan;    // 8-line runs
                    runs4_q = rw > curv && 3.0f * (rw + curv) < kRunSpan;    // 4-line runs
                }
                const unsigned all4 = __ballot_sync(0xffffffffu, ok_q);
                const unsigned wide4 = __ballot_sync(0xffffffffu, wide_q);
                const unsigned pos4 = __ballot_sync(0xffffffffu, pos_q);
                const unsigned runs4 = __ballot_sync(0xffffffffu, runs_q);
                const unsigned runs8 = __ballot_sync(0xffffffffu, runs8_q);
                const unsigned runs4g = __ballot_sync(0xffffffffu, runs4_q);
                const unsigned grp = lane & ~3;
                const unsigned sgn = (pos4 >> grp) & 0xFu;
                const bool mono = sgn == 0xFu || sgn == 0u;
                if (pi < npb && q == 0) {
                    int m = !mono ? 0 : (((wide4 >> grp) & 0xFu) == 0xFu ? 2 : (((all4 >> grp) & 0xFu) == 0xFu ? 1 : 0));
                    if (LINEAR && !PRECISE && m >= 1) {
                        if (((runs4 >> grp) & 0xFu) == 0xFu)
                            m = 5;
                        else if (((runs8 >> grp) & 0xFu) == 0xFu)
                            m = 4;
                        else if (((runs4g >> grp) & 0xFu) == 0xFu)
                            m = 3;
                    }
                    fast[pi] = m;
                }
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(&bars[b]);
        }
        return;
    }

    // ------------------------------------------------------------------ gathering warps
    const int qx = lane >= 16;
    const float di = (float)(lane - 8 - 16 * qx);
    TileThread tt;
    tt.q = qx;
    tt.di = di;
    tt.di2 = di * di;
    tt.di3 = tt.di2 * di;
    bool ok = true;
    // ring windows: the base bin of each of this warp's pulses (warp + 8 k) at the previous tile
    const int mask = ws - 1, rh = a.ring_half;
    int prev_base[kMaxStagePulses / (kWsConsumers / 32)];
    for (int t = 0; t < ntile; ++t) {
        const int b = t & 1;
        if (ok && !mbar_wait(&bars[b], (t >> 1) & 1, 32, 256)) ok = false;
        if (ok && RING) {
            // bins the step from the previous tile's range [base - rh, base + rh] leaves behind
#pragma unroll
            for (int k = 0; k < kMaxStagePulses / (kWsConsumers / 32); ++k) {
                const int p = warp + k * (kWsConsumers / 32);
                if (p >= npb) break;
                const int nb = base0[b * pbf + p];
                if (t > 0 && nb != prev_base[k]) {
                    const int ob = prev_base[k];
                    if (nb > ob)
                        ring_flush(win + p * wslots, ob - rh, min(ob + rh, nb - rh - 1), mask, a, s0 + p, lane);
                    else
                        ring_flush(win + p * wslots, max(ob - rh, nb + rh + 1), ob + rh, mask, a, s0 + p, lane);
                }
                prev_base[k] = nb;
            }
            __syncwarp();
        }
        if (ok) {
            const float4* coef = coef0 + b * pbf * 4 * kSetF4;
            const XT* xt = xt0 + b * kTile * kXtStride;
            // Pulses are processed in pairs (p, p + 8): both share each image value and give the
            // warp two independent accumulation chains.
            for (int p = warp; p < npb; p += 2 * (kWsConsumers / 32)) {
                const int p2 = p + kWsConsumers / 32;
                const bool two = p2 < npb;
                const int pq = two ? p2 : p;
                float2* wp = win + p * wslots;
                float2* wq = win + pq * wslots;
                const int off_p = base0[b * pbf + p] - wst[p];    // ring: the absolute base bin
                const int off_q = base0[b * pbf + pq] - wst[pq];
                const int mode = two ? pair_mode(fast0[b * pbf + p], fast0[b * pbf + p2]) : fast0[b * pbf + p];
#pragma unroll
                for (int half = 0; half < 2; ++half) {
                    float c9p, w9p, ibp, c9q, w9q, ibq;
                    // sub-tile: lanes >= 16 are its upper half along the lane axis, half along the other
                    const int qs = TRANSPOSED ? half + 2 * qx : qx + 2 * half;
                    const ColumnTerms ctp =
                        load_column<PRECISE, TRANSPOSED>(coef + (p * 4 + qs) * kSetF4, tt, c9p, w9p, ibp);
                    const ColumnTerms ctq =
                        load_column<PRECISE, TRANSPOSED>(coef + (pq * 4 + qs) * kSetF4, tt, c9q, w9q, ibq);
                    const XT* xrow = xt + 16 * half * kXtStride;
                    NearCtx nc;
                    if (!LINEAR) {
                        nc.steps = a.steps;
                        nc.pulses = a.pulses;
                        nc.alpha2 = a.alpha2;
                        nc.sr_hi = g.s_r.hi;
                        nc.sr_lo = g.s_r.lo;
                        nc.bg0 = a.bg0;
                        nc.transposed = TRANSPOSED;
                        nc.i0 = (TRANSPOSED ? t0 + t : line) * kTile + (TRANSPOSED ? 16 * half : 0);
                        nc.j0 = (TRANSPOSED ? line : t0 + t) * kTile + (TRANSPOSED ? 0 : 16 * half);
                        nc.k = k;
                        nc.sp = s0 + p;
                        nc.sq = s0 + pq;
                        nc.wsp = wst[p];
                        nc.wsq = wst[pq];
                        nc.a_off = g.a_off;
                        nc.shear = g.shear;
                    }
                    if (two)
                        scatter_half<LINEAR, PRECISE, true, XT, RING>(mode, ctp, c9p, w9p, ibp, ctq, c9q, w9q, ibq,
                                                                      xrow, wp, wq, off_p, off_q, ws, lane, nc);
                    else
                        scatter_half<LINEAR, PRECISE, false, XT, RING>(mode, ctp, c9p, w9p, ibp, ctq, c9q, w9q, ibq,
                                                                       xrow, wp, wq, off_p, off_q, ws, lane, nc);
                }
            }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&bars[2 + b]);
    }
    if (!ok) {
        if (lane == 0) raise_flag(a.flags, FLAG_WAIT_TIMEOUT);
        return;
    }
    __syncwarp();
    if constexpr (RING) {   // the last tile's ranges
#pragma unroll
        for (int k = 0; k < kMaxStagePulses / (kWsConsumers / 32); ++k) {
            const int p = warp + k * (kWsConsumers / 32);
            if (p >= npb) break;
            ring_flush(win + p * wslots, prev_base[k] - rh, prev_base[k] + rh, mask, a, s0 + p, lane);
        }
    } else {
        // merge this warp's windows into the global accumulator
        for (int p = warp; p < npb; p += kWsConsumers / 32) {
            const float2* wp = win + p * wslots;
            for (int w = lane; w < ws; w += 32) {
                const float2 v = wp[wslot(w)];
                if (v.x == 0.f && v.y == 0.f) continue;
                const long gi = (long)wst[p] + w - a.bg0;
                if (gi < 0 || gi >= a.Lg) {
                    raise_flag(a.flags, FLAG_STRIP_WINDOW);
                    continue;
                }
                float2* dst = a.acc + (size_t)(s0 + p) * a.Lg + gi;
                atomicAdd(dst, v);   // one vector reduction for both components
            }
        }
    }
}

template <bool LINEAR, bool PRECISE, bool TRANSPOSED, bool RING = false>
static cudaError_t launch_fp_grid_ws_t(const FpGridArgs& a, cudaStream_t st) {
    const size_t smem = fp_grid_ws_smem_bytes(a.ws, a.pbf, LINEAR && !PRECISE);
    const int lines = TRANSPOSED ? a.g.tiles_y : a.g.tiles_x;
    const dim3 grid((unsigned)(a.segs_per_column * lines * a.g.nz), (unsigned)((a.S + a.pbf - 1) / a.pbf));
    cudaError_t e = cudaFuncSetAttribute(fp_grid_ws_kernel<LINEAR, PRECISE, TRANSPOSED, RING>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    fp_grid_ws_kernel<LINEAR, PRECISE, TRANSPOSED, RING><<<grid, kWsThreads, smem, st>>>(a);
    return cudaGetLastError();
}

template <bool TRANSPOSED>
static cudaError_t launch_fp_grid_ws_o(const FpGridArgs& a, cudaStream_t st) {
    if (a.ring_half > 0)   // ring windows: split bins only
        return a.linear ? launch_fp_grid_ws_t<true, true, TRANSPOSED, true>(a, st)
                        : launch_fp_grid_ws_t<false, true, TRANSPOSED, true>(a, st);
    if (a.linear)
        return a.g.precise_bins ? launch_fp_grid_ws_t<true, true, TRANSPOSED>(a, st)
                                : launch_fp_grid_ws_t<true, false, TRANSPOSED>(a, st);
    return a.g.precise_bins ? launch_fp_grid_ws_t<false, true, TRANSPOSED>(a, st)
                            : launch_fp_grid_ws_t<false, false, TRANSPOSED>(a, st);
}

cudaError_t launch_fp_grid_ws(const FpGridArgs& a, cudaStream_t st) {
    if (a.pbf < 8 || a.pbf > 32 || (a.pbf & 7) || a.ws < 32 || (a.ws & 31)) return cudaErrorInvalidValue;
    // ring windows: split bins, a power-of-two ring holding a tile's whole range
    if (a.ring_half > 0 && (!a.g.precise_bins || (a.ws & (a.ws - 1)) || 2 * a.ring_half + 1 > a.ws))
        return cudaErrorInvalidValue;
    if (!a.linear && a.g.precise_bins && (!a.steps || !a.alpha2)) return cudaErrorInvalidValue;
    return a.transposed ? launch_fp_grid_ws_o<true>(a, st) : launch_fp_grid_ws_o<false>(a, st);
}

// ------------------------------------------------------- K2 / K3 (points)
constexpr int kPointThreads = 256;
constexpr int kPointPulses = 64;

__device__ __forceinline__ PointGeom load_point(const PointGeom* p) {
    const float4* v = reinterpret_cast<const float4*>(p);
    const float4 h = __ldg(v), l = __ldg(v + 1);
    PointGeom g;
    g.qh[0] = h.x; g.qh[1] = h.y; g.qh[2] = h.z; g.qh[3] = h.w;
    g.ql[0] = l.x; g.ql[1] = l.y; g.ql[2] = l.z; g.ql[3] = l.w;
    return g;
}

struct PointEval {
    float f, sf;
    int gi;
};

__device__ __forceinline__ PointEval eval_point(const PointArgs& a, const PulseGeom& pg, float4 a2,
                                                const PointGeom& pt) {
    df r = point_range(pulse_tx(pg), df_make(a2.x, a2.y), pt);
    if (pg.monostatic != 0.0f)
        r = df_mulf(r, 2.0f);
    else
        r = df_add(r, point_range(pulse_rx(pg), df_make(a2.z, a2.w), pt));
    r = df_sub(r, df_make(pg.rref_hi, pg.rref_lo));
    PointEval e;
    e.f = df_frac(df_mul(a.kappa, r));
    const df V = df_sub(df_mul(a.s_r, r), df_make((float)a.bg0, 0.0f));
    int gi;
    exact_bin(V, a.bg0, a.bin_rule, &gi, &e.sf);
    e.gi = min(max(gi, 0), a.Lg - 2);
    return e;
}

__global__ void __launch_bounds__(kPointThreads) bp_points_kernel(const PointArgs a, const float4* __restrict__ pairs,
                                                                  float2* x, int accumulate) {
    __shared__ PulseGeom sp[kPointPulses];
    __shared__ float4 sa2[kPointPulses];
    const int p = blockIdx.x * kPointThreads + threadIdx.x;
    PointGeom pt = {};
    if (p < a.P) pt = load_point(a.points + p);
    float ar = 0.f, ai = 0.f;
    for (int s0 = 0; s0 < a.S; s0 += kPointPulses) {
        const int n = min(kPointPulses, a.S - s0);
        __syncthreads();
        for (int e = threadIdx.x; e < n; e += kPointThreads) {
            sp[e] = load_pulse(a.pulses + s0 + e);
            sa2[e] = __ldg(a.alpha2 + s0 + e);
        }
        __syncthreads();
        float sr = 0.f, si = 0.f;
        for (int j = 0; j < n; ++j) {
            const PointEval e = eval_point(a, sp[j], sa2[j], pt);
            float re, im;
            if (a.values) {   // nearest-bin profiles stored as plain values (float2 rows)
                const float2 pv = __ldg(reinterpret_cast<const float2*>(pairs) + (size_t)(s0 + j) * a.Lg + e.gi);
                re = pv.x;
                im = pv.y;
            } else {
                const float4 pv = __ldg(pairs + (size_t)(s0 + j) * a.Lg + e.gi);
                re = fmaf(e.sf, pv.z, pv.x);
                im = fmaf(e.sf, pv.w, pv.y);
            }
            float sn, cn;
            __sincosf(SAR_TWO_PI * e.f, &sn, &cn);
            sr = fmaf(re, cn, fmaf(im, sn, sr));
            si = fmaf(im, cn, fmaf(-re, sn, si));
        }
        ar += sr;
        ai += si;
    }
    if (p < a.P) {
        float2 o = make_float2(ar, ai);
        if (accumulate) {
            o.x += x[p].x;
            o.y += x[p].y;
        }
        x[p] = o;
    }
}

template <bool LINEAR>
__global__ void __launch_bounds__(kPointThreads) fp_points_kernel(const PointArgs a, const float2* __restrict__ x,
                                                                  float2* acc) {
    __shared__ PulseGeom sp[kPointPulses];
    __shared__ float4 sa2[kPointPulses];
    const int p = blockIdx.x * kPointThreads + threadIdx.x;
    const int s0 = blockIdx.y * kPointPulses;
    const int n = min(kPointPulses, a.S - s0);
    for (int e = threadIdx.x; e < n; e += kPointThreads) {
        sp[e] = load_pulse(a.pulses + s0 + e);
        sa2[e] = __ldg(a.alpha2 + s0 + e);
    }
    __syncthreads();
    if (p >= a.P) return;
    const PointGeom pt = load_point(a.points + p);
    const float2 xv = x[p];
    for (int j = 0; j < n; ++j) {
        const PointEval e = eval_point(a, sp[j], sa2[j], pt);
        float sn, cn;
        __sincosf(SAR_TWO_PI * e.f, &sn, &cn);
        const float cr = xv.x * cn - xv.y * sn;
        const float ci = fmaf(xv.x, sn, xv.y * cn);
        float2* dst = acc + (size_t)(s0 + j) * a.Lg + e.gi;
        if (LINEAR) {
            const float w0 = 0.5f - e.sf, w1 = 0.5f + e.sf;
            atomicAdd(&dst[0].x, w0 * cr);
            atomicAdd(&dst[0].y, w0 * ci);
            atomicAdd(&dst[1].x, w1 * cr);
            atomicAdd(&dst[1].y, w1 * ci);
        } else {
            atomicAdd(&dst[0].x, cr);
            atomicAdd(&dst[0].y, ci);
        }
    }
}

cudaError_t launch_bp_points(const PointArgs& a, const float4* pairs, float2* x, int accumulate, cudaStream_t st) {
    const unsigned blocks = (unsigned)((a.P + kPointThreads - 1) / kPointThreads);
    bp_points_kernel<<<blocks, kPointThreads, 0, st>>>(a, pairs, x, accumulate);
    return cudaGetLastError();
}

cudaError_t launch_fp_points(const PointArgs& a, const float2* x, float2* acc, cudaStream_t st) {
    const dim3 grid((unsigned)((a.P + kPointThreads - 1) / kPointThreads), (unsigned)((a.S + kPointPulses - 1) / kPointPulses));
    if (a.linear)
        fp_points_kernel<true><<<grid, kPointThreads, 0, st>>>(a, x, acc);
    else
        fp_points_kernel<false><<<grid, kPointThreads, 0, st>>>(a, x, acc);
    return cudaGetLastError();
}

// ------------------------------------------------------------------- K1 / K4
__device__ __forceinline__ long pos_mod(long a, long m) {
    long r = a % m;
    return r < 0 ? r + m : r;
}

// Spectrum rows are complex64 (float2) or, for working lengths with large prime factors
// where the FP32 transform loses accuracy, complex128 (double2).
__device__ __forceinline__ float2 to_f2(float2 v) { return v; }
__device__ __forceinline__ float2 to_f2(double2 v) { return make_float2((float)v.x, (float)v.y); }
template <class T>
__device__ __forceinline__ T make_spec(float x, float y);
template <>
__device__ __forceinline__ float2 make_spec<float2>(float x, float y) { return make_float2(x, y); }
template <>
__device__ __forceinline__ double2 make_spec<double2>(float x, float y) { return make_double2(x, y); }

// spec[row][m] = conj(W[i]) y_fft[i] placed at the zero-padded position of FFT index i
// (sarsolver_cxx.cpp:331-342); y is read from its fftshifted layout.
template <class T>
__global__ void pack_adjoint_kernel(const float2* __restrict__ y, const float2* __restrict__ wave,
                                    T* __restrict__ spec, int N, long M, int first) {
    const long m = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= M) return;
    const long row = blockIdx.y;
    const int half = N / 2;
    int i = -1;
    if (m < half)
        i = (int)m;
    else if (m >= M - half)
        i = (int)(N - M + m);
    else if ((N & 1) && m == half)
        i = half;
    float2 v = make_float2(0.f, 0.f);
    if (i >= 0) {
        const float2 yv = y[(size_t)(first + row) * N + (i + half) % N];
        const float2 w = __ldg(wave + i);
        v = make_float2(w.x * yv.x + w.y * yv.y, w.x * yv.y - w.y * yv.x);
    }
    spec[row * M + m] = make_spec<T>(v.x, v.y);
}

// pairs[s][w] for bin b = bg0 + w by `format` (kProfPairs...): linear, (p(b) + 0.5 d, d) with
// d = p(b+1) - p(b), both scaled by the pulse factor; nearest, (p(b), 0); values, the scaled p(b)
// alone in float2 rows of the same length.  Bins wrap modulo M (sarsolver_cxx.cpp:22-24).
template <class T>
__global__ void unpack_pairs_kernel(const T* __restrict__ spec, const float2* __restrict__ wfac,
                                    float4* __restrict__ pairs, long M, int Lg, long bg0, int first,
                                    int linear) {
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= Lg) return;
    const long row = blockIdx.y;
    const long m0 = pos_mod(bg0 + w, M);
    const long m1 = (m0 + 1 == M) ? 0 : m0 + 1;
    const float2 f = __ldg(wfac + first + row);
    const float2 a = to_f2(spec[row * M + m0]);
    const float2 p0 = make_float2(a.x * f.x - a.y * f.y, a.x * f.y + a.y * f.x);
    if (linear == kProfValues) {
        reinterpret_cast<float2*>(pairs)[(size_t)(first + row) * Lg + w] = p0;
        return;
    }
    if (linear == kProfNearestPairs) {
        pairs[(size_t)(first + row) * Lg + w] = make_float4(p0.x, p0.y, 0.f, 0.f);
        return;
    }
    const float2 b = to_f2(spec[row * M + m1]);
    const float2 p1 = make_float2(b.x * f.x - b.y * f.y, b.x * f.y + b.y * f.x);
    const float dx = p1.x - p0.x, dy = p1.y - p0.y;
    pairs[(size_t)(first + row) * Lg + w] = make_float4(fmaf(0.5f, dx, p0.x), fmaf(0.5f, dy, p0.y), dx, dy);
}

// Stored span from the callback transform's compact output compact[row][w] (w = bin - bg0;
// Lc = min(Lg + 1, M) columns, taken modulo M when the span wraps): pairs as unpack_pairs_kernel,
// or plain profiles when `pairs` is null.
__global__ void unpack_compact_kernel(const float2* __restrict__ compact, int Lc, const float2* __restrict__ wfac,
                                      float4* __restrict__ pairs, float2* __restrict__ prof, long M, int Lg, int first,
                                      int linear) {
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= Lg) return;
    const long row = blockIdx.y;
    const float2* c = compact + (size_t)row * Lc;
    const int w0 = (Lc == M) ? (int)(w % M) : w;
    if (!pairs) {
        prof[(size_t)(first + row) * Lg + w] = c[w0];
        return;
    }
    const int w1 = (Lc == M) ? (int)((w + 1) % M) : w + 1;
    const float2 f = __ldg(wfac + first + row);
    const float2 a = c[w0];
    const float2 p0 = make_float2(a.x * f.x - a.y * f.y, a.x * f.y + a.y * f.x);
    if (linear == kProfValues) {   // float2 rows of values
        reinterpret_cast<float2*>(pairs)[(size_t)(first + row) * Lg + w] = p0;
        return;
    }
    if (linear == kProfNearestPairs) {
        pairs[(size_t)(first + row) * Lg + w] = make_float4(p0.x, p0.y, 0.f, 0.f);
        return;
    }
    const float2 b = c[w1];
    const float2 p1 = make_float2(b.x * f.x - b.y * f.y, b.x * f.y + b.y * f.x);
    const float dx = p1.x - p0.x, dy = p1.y - p0.y;
    pairs[(size_t)(first + row) * Lg + w] = make_float4(fmaf(0.5f, dx, p0.x), fmaf(0.5f, dy, p0.y), dx, dy);
}

cudaError_t launch_unpack_compact(const float2* compact, int Lc, const float2* wfac, float4* pairs, float2* prof,
                                  long M, int Lg, int rows, int first, int linear, cudaStream_t st) {
    const dim3 grid((unsigned)((Lg + 255) / 256), (unsigned)rows);
    unpack_compact_kernel<<<grid, 256, 0, st>>>(compact, Lc, wfac, pairs, prof, M, Lg, first, linear);
    return cudaGetLastError();
}

template <class T>
__global__ void unpack_profiles_kernel(const T* __restrict__ spec, float2* __restrict__ prof, long M, int Lg,
                                       long bg0, int first) {
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= Lg) return;
    const long row = blockIdx.y;
    prof[(size_t)(first + row) * Lg + w] = to_f2(spec[row * M + pos_mod(bg0 + w, M)]);
}

// spec[row][m] = sum of accumulated bins congruent to m modulo M.
template <class T>
__global__ void pack_forward_kernel(const float2* __restrict__ acc, T* __restrict__ spec, long M, int Lg, long bg0,
                                    int first) {
    const long m = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= M) return;
    const long row = blockIdx.y;
    float2 s = make_float2(0.f, 0.f);
    for (long w = pos_mod(m - bg0, M); w < Lg; w += M) {
        const float2 v = acc[(size_t)(first + row) * Lg + w];
        s.x += v.x;
        s.y += v.y;
    }
    spec[row * M + m] = make_spec<T>(s.x, s.y);
}

// y_fft[i] = W[i] K[i] (low half), W[N-1-i] K[M-1-i] (high half), odd middle
// (sarsolver_cxx.cpp:295-307), times the pulse factor, written fftshifted (forward.py:44).
template <class T>
__global__ void extract_forward_kernel(const T* __restrict__ spec, const float2* __restrict__ wave,
                                       const float2* __restrict__ wfac, float2* __restrict__ y, int N, long M,
                                       int first) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const long row = blockIdx.y;
    const int half = N / 2;
    long m;
    if (i < half)
        m = i;
    else if (i >= N - half)
        m = M - N + i;
    else
        m = half;
    const float2 k = to_f2(spec[row * M + m]);
    const float2 w = __ldg(wave + i);
    const float2 f = __ldg(wfac + first + row);
    const float2 a = make_float2(w.x * k.x - w.y * k.y, w.x * k.y + w.y * k.x);
    y[(size_t)(first + row) * N + (i + half) % N] = make_float2(a.x * f.x - a.y * f.y, a.x * f.y + a.y * f.x);
}

// K6: per-pulse phase-error gradient of an image-domain objective.  For the sharpness
// S = sum |I|^4 of I = A_phi^H y (slow-time weights w_s = exp(i phi_s)), dS/dphi_s =
// 4 Im( sum_f conj((A_phi G)_{s,f}) y_{s,f} ) with G = |I|^2 I.  One CTA per pulse row: a
// strided FP32 dot product per thread (a few terms each), then FP64 warp shuffles and a
// shared-memory reduction across warps.
__global__ void phase_grad_kernel(const float2* __restrict__ ag, const float2* __restrict__ y, float* __restrict__ g,
                                  int N, float scale) {
    __shared__ double part[32];
    const size_t row = blockIdx.x;
    const float2* a = ag + row * N;
    const float2* b = y + row * N;
    float acc = 0.f;
    for (int f = threadIdx.x; f < N; f += blockDim.x) {
        const float2 u = __ldg(a + f), v = __ldg(b + f);
        acc = fmaf(u.x, v.y, fmaf(-u.y, v.x, acc));   // Im(conj(u) v)
    }
    double d = acc;
    for (int o = 16; o; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = d;
    __syncthreads();
    if (threadIdx.x < 32) {
        d = threadIdx.x < (blockDim.x >> 5) ? part[threadIdx.x] : 0.0;
        for (int o = 16; o; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
        if (threadIdx.x == 0) g[row] = (float)(scale * d);
    }
}

cudaError_t launch_phase_grad(const float2* ag, const float2* y, float* g, int S, int N, float scale, cudaStream_t st) {
    phase_grad_kernel<<<S, 256, 0, st>>>(ag, y, g, N, scale);
    return cudaGetLastError();
}

// Image sharpness: G = |I|^2 I (optional) and sum |I|^4 accumulated in FP64 (one atomic per CTA;
// the caller zeroes *sum).  Grid-stride over pixel pairs with 16-byte loads; an odd tail pixel
// is taken by thread 0 of CTA 0.
__global__ void sharpness_kernel(const float2* __restrict__ img, float2* __restrict__ G, double* __restrict__ sum,
                                 size_t P) {
    __shared__ double part[32];
    double acc = 0.0;
    const size_t pairs = P >> 1;
    const float4* in4 = reinterpret_cast<const float4*>(img);
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < pairs; i += (size_t)gridDim.x * blockDim.x) {
        const float4 v = __ldg(in4 + i);
        const float m0 = fmaf(v.x, v.x, v.y * v.y), m1 = fmaf(v.z, v.z, v.w * v.w);
        acc += (double)(m0 * m0) + (double)(m1 * m1);
        if (G) reinterpret_cast<float4*>(G)[i] = make_float4(m0 * v.x, m0 * v.y, m1 * v.z, m1 * v.w);
    }
    if ((P & 1) && blockIdx.x == 0 && threadIdx.x == 0) {
        const float2 v = img[P - 1];
        const float m = fmaf(v.x, v.x, v.y * v.y);
        acc += (double)(m * m);
        if (G) G[P - 1] = make_float2(m * v.x, m * v.y);
    }
    for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        acc = threadIdx.x < (blockDim.x >> 5) ? part[threadIdx.x] : 0.0;
        for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (threadIdx.x == 0) atomicAdd(sum, acc);
    }
}

cudaError_t launch_sharpness(const float2* img, float2* G, double* sum, size_t P, int num_sms, cudaStream_t st) {
    const size_t pairs = (P >> 1) ? (P >> 1) : 1;
    size_t blocks = (pairs + 255) / 256;
    const size_t cap = (size_t)(num_sms > 0 ? num_sms : 152) * 8;
    if (blocks > cap) blocks = cap;
    sharpness_kernel<<<(unsigned)blocks, 256, 0, st>>>(img, G, sum, P);
    return cudaGetLastError();
}

__global__ void weights_kernel(const float2* __restrict__ w, float2* wadj, float2* wfwd, int S, int conj_adjoint) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= S) return;
    const float2 v = w[s];
    wfwd[s] = v;
    wadj[s] = conj_adjoint ? make_float2(v.x, -v.y) : v;
}

cudaError_t launch_pack_adjoint(const float2* y, const float2* wave, void* spec, int dbl, int N, long M, int rows,
                                int first, cudaStream_t st) {
    const dim3 grid((unsigned)((M + 255) / 256), (unsigned)rows);
    if (dbl)
        pack_adjoint_kernel<double2><<<grid, 256, 0, st>>>(y, wave, (double2*)spec, N, M, first);
    else
        pack_adjoint_kernel<float2><<<grid, 256, 0, st>>>(y, wave, (float2*)spec, N, M, first);
    return cudaGetLastError();
}

cudaError_t launch_unpack_pairs(const void* spec, int dbl, const float2* wfac, float4* pairs, long M, int Lg,
                                long bg0, int rows, int first, int linear, cudaStream_t st) {
    const dim3 grid((unsigned)((Lg + 255) / 256), (unsigned)rows);
    if (dbl)
        unpack_pairs_kernel<double2><<<grid, 256, 0, st>>>((const double2*)spec, wfac, pairs, M, Lg, bg0, first, linear);
    else
        unpack_pairs_kernel<float2><<<grid, 256, 0, st>>>((const float2*)spec, wfac, pairs, M, Lg, bg0, first, linear);
    return cudaGetLastError();
}

// ------------------------------------------- K1 fused: upsampling FFT straight into pairs
// For N = 512, 1024, 2048, 4096 or 8192 and M = U N (integer U): bin b = U j + r of the inverse length-M transform of the
// zero-padded spectrum (frequencies k in [-N/2, N/2), X_k = conj(W) y at k mod N) is
//   p(U j + r) = sum_k X_k e^{2 pi i k r / M} e^{2 pi i k j / N},
// an N-point inverse DFT of the spectrum twiddled by e^{2 pi i k r / M} (the same holds for any
// integer r, r >= U giving the bins U (j + 1) + r - U).  One CTA of N / 16 threads per pulse row
// computes the U such transforms in shared memory (Stockham: a radix-N/256 first pass on the 16
// values each thread holds, then two radix-16 passes with one 16-point butterfly per thread),
// keeps the bins of the stored span [bg0, bg0 + Lg] (taken modulo M) and writes the (value,
// difference) pairs of unpack_pairs_kernel directly: the row is read once (N values) and only the
// span is written, where the unfused path writes and reads the M-point rows three times.
// Twiddles come from FP64-computed tables e^{2 pi i q / N} and e^{2 pi i q / M}.  A thread holds
// the frequencies k = t + T e (e < 16, minus N for e >= 8), so a transform's e^{2 pi i k r / M}
// factors into e^{2 pi i t r / M} (one table read per thread, t r < M / 8) times
// e^{2 pi i (T e - N [e >= 8]) r / M}, the same for every thread (a small table after the first, read
// as broadcasts): no chained products, so any U keeps FP32 accuracy, and one scattered read per
// thread and transform instead of sixteen.
//
// Staged form (spans whose U residues fit shared memory): the span is gathered residue-major in
// shared memory and written row-contiguously at the end.  Direct form (longer spans, i.e. large
// U): transform q in [0, U) takes r = (bg0 mod U) + q, whose bins are exactly the span's bins
// w = q + U i, and writes them straight to global memory at stride U; linear pairs of the bins of
// transform q - 1 are written once transform q (their right neighbours) is known, from a
// shared-memory copy of the previous transform's span values, and those of the last transform
// from a copy of the first's.
template <int N>
struct UpShape {
    static constexpr int T = N / 16;                // threads per row: one radix-16 butterfly each
    static constexpr int P = N >= 8192 ? 3 : 2;     // radix-16 passes after the first
    static constexpr int R0 = N / (P == 3 ? 4096 : 256);   // radix of the first pass: 2, 4, 8 or 16
    static constexpr int NB = 16 / R0;              // first-pass butterflies per thread
    static_assert(R0 >= 2 && R0 <= 16 && R0 * (P == 3 ? 4096 : 256) == N, "unsupported transform length");
};

__device__ __forceinline__ int up_pad(int x) { return x + (x >> 4); }   // one slot per 16: no bank conflicts
__device__ __forceinline__ float2 cmulf(float2 a, float2 b) {
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ void dft4_inv(float2& x0, float2& x1, float2& x2, float2& x3) {
    const float2 t0 = make_float2(x0.x + x2.x, x0.y + x2.y), t1 = make_float2(x0.x - x2.x, x0.y - x2.y);
    const float2 t2 = make_float2(x1.x + x3.x, x1.y + x3.y);
    const float2 t3 = make_float2(-(x1.y - x3.y), x1.x - x3.x);   // i (x1 - x3)
    x0 = make_float2(t0.x + t2.x, t0.y + t2.y);
    x1 = make_float2(t1.x + t3.x, t1.y + t3.y);
    x2 = make_float2(t0.x - t2.x, t0.y - t2.y);
    x3 = make_float2(t1.x - t3.x, t1.y - t3.y);
}
// v[k] <- sum_n v[n] e^{+2 pi i n k / 16}: n = 4 n1 + n2, k = k1 + 4 k2 (two radix-4 stages).
__device__ __forceinline__ void dft16_inv(float2 (&v)[16]) {
#pragma unroll
    for (int n2 = 0; n2 < 4; ++n2) dft4_inv(v[n2], v[4 + n2], v[8 + n2], v[12 + n2]);   // -> Y[n2][k1] at v[4 k1 + n2]
    const float c1 = 0.92387953251128674f, s1 = 0.38268343236508977f, h = 0.70710678118654752f;
    // W16^(n2 k1) for (n2, k1) in {1,2,3} x {1,2,3}: exponents 1 2 3 / 2 4 6 / 3 6 9
    v[4 + 1] = cmulf(v[4 + 1], make_float2(c1, s1));
    v[8 + 1] = cmulf(v[8 + 1], make_float2(h, h));
    v[12 + 1] = cmulf(v[12 + 1], make_float2(s1, c1));
    v[4 + 2] = cmulf(v[4 + 2], make_float2(h, h));
    v[8 + 2] = make_float2(-v[8 + 2].y, v[8 + 2].x);   // W16^4 = i
    v[12 + 2] = cmulf(v[12 + 2], make_float2(-h, h));
    v[4 + 3] = cmulf(v[4 + 3], make_float2(s1, c1));
    v[8 + 3] = cmulf(v[8 + 3], make_float2(-h, h));
    v[12 + 3] = cmulf(v[12 + 3], make_float2(-c1, -s1));
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) dft4_inv(v[4 * k1], v[4 * k1 + 1], v[4 * k1 + 2], v[4 * k1 + 3]);
    // now v[4 k1 + k2] holds X[k1 + 4 k2]: transpose the 4x4 index to natural order
    float2 t[16];
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1)
#pragma unroll
        for (int k2 = 0; k2 < 4; ++k2) t[k1 + 4 * k2] = v[4 * k1 + k2];
#pragma unroll
    for (int k = 0; k < 16; ++k) v[k] = t[k];
}

// v[k] <- sum_n v[n] e^{+2 pi i n k / 8}: n = 2 n1 + n2, k = k1 + 4 k2 (radix 4, then radix 2).
__device__ __forceinline__ void dft8_inv(float2 (&v)[8]) {
    dft4_inv(v[0], v[2], v[4], v[6]);   // n2 = 0: Y0[k1] at v[2 k1]
    dft4_inv(v[1], v[3], v[5], v[7]);   // n2 = 1: Y1[k1] at v[2 k1 + 1]
    const float h = 0.70710678118654752f;
    v[3] = cmulf(v[3], make_float2(h, h));            // W8^1
    v[5] = make_float2(-v[5].y, v[5].x);              // W8^2 = i
    v[7] = cmulf(v[7], make_float2(-h, h));           // W8^3
    float2 t[8];
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) {
        const float2 a = v[2 * k1], b = v[2 * k1 + 1];
        t[k1] = make_float2(a.x + b.x, a.y + b.y);
        t[k1 + 4] = make_float2(a.x - b.x, a.y - b.y);
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) v[k] = t[k];
}

// First Stockham pass (sub-transform length 1) on the 16 values x[e] = element t + T e a thread
// holds: butterfly j = t + T e1 (e1 < NB) combines elements j + 256 m (m < R0), which are
// x[e1 + NB m], and writes out[j R0 + m].
template <int N>
__device__ __forceinline__ void up_first_pass(const float2 (&x)[16], float2* out, int t) {
    constexpr int T = UpShape<N>::T, R0 = UpShape<N>::R0, NB = UpShape<N>::NB;
#pragma unroll
    for (int e1 = 0; e1 < NB; ++e1) {
        const int j = t + T * e1;
        if constexpr (R0 == 16) {
            float2 v[16];
#pragma unroll
            for (int m = 0; m < 16; ++m) v[m] = x[m];
            dft16_inv(v);
#pragma unroll
            for (int m = 0; m < 16; ++m) out[up_pad(j * 16 + m)] = v[m];
        } else if constexpr (R0 == 8) {
            float2 v[8];
#pragma unroll
            for (int m = 0; m < 8; ++m) v[m] = x[e1 + NB * m];
            dft8_inv(v);
#pragma unroll
            for (int m = 0; m < 8; ++m) out[up_pad(j * 8 + m)] = v[m];
        } else if constexpr (R0 == 4) {
            float2 a = x[e1], b = x[e1 + NB], c = x[e1 + 2 * NB], d = x[e1 + 3 * NB];
            dft4_inv(a, b, c, d);
            out[up_pad(j * 4)] = a;
            out[up_pad(j * 4 + 1)] = b;
            out[up_pad(j * 4 + 2)] = c;
            out[up_pad(j * 4 + 3)] = d;
        } else {
            const float2 a = x[e1], b = x[e1 + NB];
            out[up_pad(j * 2)] = make_float2(a.x + b.x, a.y + b.y);
            out[up_pad(j * 2 + 1)] = make_float2(a.x - b.x, a.y - b.y);
        }
    }
}

// v[r] *= w^r for r = 1..15, the powers built by squaring (at most four chained products).
__device__ __forceinline__ void apply_powers(float2 (&v)[16], float2 w) {
    const float2 w2 = cmulf(w, w), w4 = cmulf(w2, w2), w8 = cmulf(w4, w4);
    const float2 w3 = cmulf(w2, w), w5 = cmulf(w4, w), w6 = cmulf(w4, w2), w7 = cmulf(w4, w3);
    v[1] = cmulf(v[1], w);
    v[2] = cmulf(v[2], w2);
    v[3] = cmulf(v[3], w3);
    v[4] = cmulf(v[4], w4);
    v[5] = cmulf(v[5], w5);
    v[6] = cmulf(v[6], w6);
    v[7] = cmulf(v[7], w7);
    v[8] = cmulf(v[8], w8);
    v[9] = cmulf(v[9], cmulf(w8, w));
    v[10] = cmulf(v[10], cmulf(w8, w2));
    v[11] = cmulf(v[11], cmulf(w8, w3));
    v[12] = cmulf(v[12], cmulf(w8, w4));
    v[13] = cmulf(v[13], cmulf(w8, w5));
    v[14] = cmulf(v[14], cmulf(w8, w6));
    v[15] = cmulf(v[15], cmulf(w8, w7));
}

// e^{2 pi i k r / M} for the 16 frequencies k = t + T e of thread t (signed: minus N for e >= 8),
// 0 <= r < 2U, as the product of e^{2 pi i t r / M} (tw_m[t r]) and the thread-independent factor
// tw_e[16 r + e] = e^{2 pi i (T e - N [e >= 8]) r / M} (stored after the M entries of tw_m).
template <int N>
__device__ __forceinline__ void residue_twiddles(const float2* __restrict__ tw_m, long M, int t, int r,
                                                 float2 (&w)[16]) {
    const float2 a = __ldg(tw_m + t * r);
    const float2* __restrict__ b = tw_m + M + 16 * r;
#pragma unroll
    for (int e = 0; e < 16; ++e) w[e] = cmulf(a, __ldg(b + e));
}

// Radix-16 Stockham pass over N points (sub-transform length ns = N / 256 or N / 16 before it).
template <int N>
__device__ __forceinline__ void up_pass(const float2* in, float2* out, int ns, const float2* __restrict__ tw_n) {
    const int j = threadIdx.x;
    float2 v[16];
#pragma unroll
    for (int r = 0; r < 16; ++r) v[r] = in[up_pad(j + r * (N / 16))];
    const int k = j & (ns - 1);
    apply_powers(v, __ldg(tw_n + k * (N / (ns * 16))));   // e^{2 pi i r k / (16 ns)}
    dft16_inv(v);
    const int base = (j / ns) * ns * 16 + k;
#pragma unroll
    for (int r = 0; r < 16; ++r) out[up_pad(base + r * ns)] = v[r];
}

// The radix-16 passes after the first (from `in`, ping-ponging with `tmp`): returns the buffer that
// holds the transform.  The caller synchronises before; each pass ends with a barrier.
template <int N>
__device__ __forceinline__ float2* up_passes(float2* in, float2* tmp, const float2* __restrict__ tw_n) {
    constexpr int R0 = UpShape<N>::R0;
    up_pass<N>(in, tmp, R0, tw_n);
    __syncthreads();
    up_pass<N>(tmp, in, 16 * R0, tw_n);
    __syncthreads();
    if constexpr (UpShape<N>::P == 3) {
        up_pass<N>(in, tmp, 256 * R0, tw_n);
        __syncthreads();
        return tmp;
    }
    return in;
}

template <int N, bool DIRECT>
__global__ void __launch_bounds__(N / 16, 8192 / N) upsample_pairs_kernel(
    const float2* __restrict__ y, const float2* __restrict__ wave, const float2* __restrict__ wfac,
    const float2* __restrict__ tw_n, const float2* __restrict__ tw_m, float4* __restrict__ pairs, int U, long M,
    int Lg, long bg0, int first, int linear, int C) {
    constexpr int T = UpShape<N>::T;
    extern __shared__ __align__(16) float2 upsm[];
    float2* A = upsm;
    float2* B = upsm + up_pad(N);
    // staged: span bins bg0 .. bg0 + Lg (mod M), residue-major: bin w of residue r = (bg0 + w) mod U
    // at stage[r C + w / U], C = 2 (mod 16) so that both the scatter and the pair reads avoid bank
    // conflicts.  Direct (linear pairs): the previous transform's and the first transform's span
    // values, C each.
    float2* stage = upsm + 2 * up_pad(N);
    float2* prev = stage;
    float2* res0 = stage + C;
    const int t = threadIdx.x;
    const long s = (long)first + blockIdx.x;
    const float2 f = __ldg(wfac + s);
    float4* dst = pairs + s * Lg;                                   // (value, difference) pairs
    float2* vdst = reinterpret_cast<float2*>(pairs) + s * Lg;       // plain values
    // this thread's spectrum values, k' = t + T e (FFT order index = k mod N)
    float2 X[16];
#pragma unroll
    for (int e = 0; e < 16; ++e) {
        const int kp = t + T * e;
        const float2 yv = y[s * N + ((kp + N / 2) & (N - 1))];
        const float2 w = __ldg(wave + kp);
        X[e] = make_float2(w.x * yv.x + w.y * yv.y, w.x * yv.y - w.y * yv.x);
    }
    const int bmod = (int)(((bg0 % U) + U) % U);
    // direct: bin bg0 + q + U i = U (j0 + i) + bmod + q
    const long j0 = (bg0 - bmod) / U;
    for (int q = 0; q < U; ++q) {
        const int r = DIRECT ? bmod + q : q;
        // pass 1 straight from registers: the spectrum times e^{2 pi i k r / M}
        float2 v[16];
        residue_twiddles<N>(tw_m, M, t, r, v);
#pragma unroll
        for (int e = 0; e < 16; ++e) v[e] = cmulf(X[e], v[e]);
        up_first_pass<N>(v, A, t);
        __syncthreads();
        const float2* F = up_passes<N>(A, B, tw_n);   // F[j] = p(U j + r)
        if (DIRECT) {
            // the span's bins w = q + U i, at j = j0 + i (mod N)
            for (int i = t; q + U * i <= Lg; i += T) {
                const int w = q + U * i;
                const float2 a = F[up_pad((int)((j0 + i) & (N - 1)))];   // j mod N (N a power of two)
                const float2 p1 = make_float2(a.x * f.x - a.y * f.y, a.x * f.y + a.y * f.x);
                if (linear == kProfValues) {
                    if (w < Lg) vdst[w] = p1;
                } else if (linear == kProfNearestPairs) {
                    if (w < Lg) dst[w] = make_float4(p1.x, p1.y, 0.f, 0.f);
                } else {
                    if (q == 0) {
                        res0[i] = p1;
                    } else if (w - 1 < Lg) {   // the pair of bin w - 1 (transform q - 1, same i)
                        const float2 p0 = prev[i];
                        const float dx = p1.x - p0.x, dy = p1.y - p0.y;
                        dst[w - 1] = make_float4(fmaf(0.5f, dx, p0.x), fmaf(0.5f, dy, p0.y), dx, dy);
                    }
                    prev[i] = p1;
                }
            }
        } else {
            // keep the span's bins with this residue
            int w0 = r - bmod;
            if (w0 < 0) w0 += U;
            const long jb = (bg0 + w0 - r) / U;   // bin bg0 + w0 + U i = U (jb + i) + r
            for (int i = t; w0 + U * i <= Lg; i += T) stage[r * C + i] = F[up_pad((int)((jb + i) & (N - 1)))];
        }
        __syncthreads();
    }
    if constexpr (DIRECT) {
        // linear pairs of the last transform's bins w = U - 1 + U i: right neighbour U (i + 1), the
        // first transform's value i + 1
        if (linear == kProfLinearPairs)
            for (int i = t; U - 1 + U * i < Lg; i += T) {
                const float2 p0 = prev[i], p1 = res0[i + 1];
                const float dx = p1.x - p0.x, dy = p1.y - p0.y;
                dst[U - 1 + U * i] = make_float4(fmaf(0.5f, dx, p0.x), fmaf(0.5f, dy, p0.y), dx, dy);
            }
        return;
    } else {
    for (int w = t; w < Lg; w += T) {
        const int r0 = (bmod + w) % U, r1 = (bmod + w + 1) % U;
        const float2 a = stage[r0 * C + w / U];
        const float2 p0 = make_float2(a.x * f.x - a.y * f.y, a.x * f.y + a.y * f.x);
        if (linear == kProfValues) {
            vdst[w] = p0;
            continue;
        }
        if (linear == kProfNearestPairs) {
            dst[w] = make_float4(p0.x, p0.y, 0.f, 0.f);
            continue;
        }
        const float2 c = stage[r1 * C + (w + 1) / U];
        const float2 p1 = make_float2(c.x * f.x - c.y * f.y, c.x * f.y + c.y * f.x);
        const float dx = p1.x - p0.x, dy = p1.y - p0.y;
        dst[w] = make_float4(fmaf(0.5f, dx, p0.x), fmaf(0.5f, dy, p0.y), dx, dy);
    }
    }
}

// Staging row length: ceil((Lg + 1) / U) rounded up to 2 (mod 16).
static int up_stage_row(int Lg, int U) {
    const int n = (Lg + 1 + U - 1) / U;
    return ((n + 13) & ~15) + 2;
}

// Fused forward downsampling for N = 512 ... 8192, M = U N: the transpose of the fused upsampling.  With
// the accumulated bins a[b] (b = U j + r, taken modulo M) the forward transform at frequency k in
// [-N/2, N/2) is  K(k) = sum_r e^{-2 pi i k r / M} DFT_N(a_r)[k mod N],  a_r[j] = a[U j + r]; each
// forward DFT is computed as conj(inverse DFT(conj a_r)) with the Stockham passes above, and
// y[(i + N/2) mod N] = W[i] f K(k_i) is written directly (replaces pack_forward + FFT + extract).
// The twiddle e^{2 pi i k r / M} is read from the table at k r mod M; the accumulation runs on
// the conjugate and is conjugated once at the end.
template <int N>
__global__ void __launch_bounds__(N / 16, 8192 / N) downsample_forward_kernel(
    const float2* __restrict__ acc, const float2* __restrict__ wave, const float2* __restrict__ wfac,
    const float2* __restrict__ tw_n, const float2* __restrict__ tw_m, float2* __restrict__ y, int U, long M, int Lg,
    long bg0, int first) {
    constexpr int T = UpShape<N>::T;
    extern __shared__ __align__(16) float2 dnsm[];
    float2* A = dnsm;
    float2* B = dnsm + up_pad(N);
    const int t = threadIdx.x;
    const long s = (long)first + blockIdx.x;
    const float2* arow = acc + s * Lg;
    const int bmod = (int)(((bg0 % U) + U) % U);
    float2 Y[16];   // conj of the output at k = t + T e
#pragma unroll
    for (int e = 0; e < 16; ++e) Y[e] = make_float2(0.f, 0.f);
    for (int r = 0; r < U; ++r) {
        // conj(a_r) into A
        for (int e = t; e < up_pad(N); e += T) A[e] = make_float2(0.f, 0.f);
        __syncthreads();
        int w0 = r - bmod;
        if (w0 < 0) w0 += U;
        for (int w = w0 + U * t; w < Lg; w += U * T) {
            long b = (bg0 + w) % M;
            if (b < 0) b += M;
            const float2 v = __ldg(arow + w);
            A[up_pad((int)(b / U))] = make_float2(v.x, -v.y);
        }
        __syncthreads();
        float2 v[16];
#pragma unroll
        for (int e = 0; e < 16; ++e) v[e] = A[up_pad(t + T * e)];
        up_first_pass<N>(v, B, t);
        __syncthreads();
        const float2* F = up_passes<N>(B, A, tw_n);
        // Y += e^{2 pi i k r / M} F[k]  (conjugate domain)
        float2 w[16];
        residue_twiddles<N>(tw_m, M, t, r, w);
#pragma unroll
        for (int e = 0; e < 16; ++e) {
            const int kp = t + T * e;
            const float2 c = cmulf(w[e], F[up_pad(kp)]);
            Y[e].x += c.x;
            Y[e].y += c.y;
        }
        __syncthreads();
    }
    const float2 f = __ldg(wfac + s);
#pragma unroll
    for (int e = 0; e < 16; ++e) {
        const int i = t + T * e;
        const float2 k = make_float2(Y[e].x, -Y[e].y);
        const float2 w = __ldg(wave + i);
        const float2 a = make_float2(w.x * k.x - w.y * k.y, w.x * k.y + w.y * k.x);
        y[s * N + ((i + N / 2) & (N - 1))] = make_float2(a.x * f.x - a.y * f.y, a.x * f.y + a.y * f.x);
    }
}

static bool fused_fft_length(int N) { return N == 512 || N == 1024 || N == 2048 || N == 4096 || N == 8192; }

// Shared memory a fused transform kernel may take: two CTAs per SM up to N = 4096, one for 8192.
static size_t fused_smem_budget(int N) { return N >= 8192 ? 220 * 1024 : 112 * 1024; }

bool downsample_fused_supported(int N, long M, int Lg) {
    return fused_fft_length(N) && M % N == 0 && M < (1L << 30) && Lg >= 1 && Lg <= M;
}

template <int N>
static cudaError_t launch_down_t(const float2* acc, const float2* wave, const float2* wfac, const float2* tw_n,
                                 const float2* tw_m, float2* y, long M, int Lg, long bg0, int rows, int first,
                                 cudaStream_t st) {
    const size_t smem = sizeof(float2) * 2 * (N + N / 16);
    cudaError_t e = cudaFuncSetAttribute(downsample_forward_kernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    downsample_forward_kernel<N><<<rows, N / 16, smem, st>>>(acc, wave, wfac, tw_n, tw_m, y, (int)(M / N), M, Lg, bg0,
                                                             first);
    return cudaGetLastError();
}

cudaError_t launch_downsample_forward_fused(const float2* acc, const float2* wave, const float2* wfac,
                                            const float2* tw_n, const float2* tw_m, float2* y, int N, long M, int Lg,
                                            long bg0, int rows, int first, cudaStream_t st) {
    if (!downsample_fused_supported(N, M, Lg) || rows < 1) return cudaErrorInvalidValue;
    if (N == 512) return launch_down_t<512>(acc, wave, wfac, tw_n, tw_m, y, M, Lg, bg0, rows, first, st);
    if (N == 1024) return launch_down_t<1024>(acc, wave, wfac, tw_n, tw_m, y, M, Lg, bg0, rows, first, st);
    if (N == 2048) return launch_down_t<2048>(acc, wave, wfac, tw_n, tw_m, y, M, Lg, bg0, rows, first, st);
    if (N == 4096) return launch_down_t<4096>(acc, wave, wfac, tw_n, tw_m, y, M, Lg, bg0, rows, first, st);
    return launch_down_t<8192>(acc, wave, wfac, tw_n, tw_m, y, M, Lg, bg0, rows, first, st);
}

// Shared memory of the staged form (transform buffers and the residue-major span), and of the
// direct form (transform buffers and two rows of span values for linear pairs).
size_t upsample_fused_smem_bytes(int N, int Lg, int U) {
    return sizeof(float2) * ((size_t)2 * (N + N / 16) + (size_t)U * up_stage_row(Lg, U));
}
static size_t upsample_direct_smem_bytes(int N, int Lg, int U) {
    return sizeof(float2) * ((size_t)2 * (N + N / 16) + (size_t)2 * up_stage_row(Lg, U));
}
bool upsample_fused_supported(int N, long M, int Lg) {
    return fused_fft_length(N) && M % N == 0 && M < (1L << 30) && Lg >= 1 && Lg <= M &&
           upsample_direct_smem_bytes(N, Lg, (int)(M / N)) <= fused_smem_budget(N);
}

template <int N>
static cudaError_t launch_up_t(const float2* y, const float2* wave, const float2* wfac, const float2* tw_n,
                               const float2* tw_m, float4* pairs, long M, int Lg, long bg0, int rows, int first,
                               int linear, cudaStream_t st) {
    const int U = (int)(M / N);
    const bool staged = upsample_fused_smem_bytes(N, Lg, U) <= fused_smem_budget(N);
    const size_t smem = staged ? upsample_fused_smem_bytes(N, Lg, U) : upsample_direct_smem_bytes(N, Lg, U);
    auto go = [&](auto kern) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        kern<<<rows, N / 16, smem, st>>>(y, wave, wfac, tw_n, tw_m, pairs, U, M, Lg, bg0, first, linear,
                                         up_stage_row(Lg, U));
        return cudaGetLastError();
    };
    return staged ? go(upsample_pairs_kernel<N, false>) : go(upsample_pairs_kernel<N, true>);
}

cudaError_t launch_upsample_pairs_fused(const float2* y, const float2* wave, const float2* wfac, const float2* tw_n,
                                        const float2* tw_m, float4* pairs, int N, long M, int Lg, long bg0, int rows,
                                        int first, int linear, cudaStream_t st) {
    if (!upsample_fused_supported(N, M, Lg) || rows < 1) return cudaErrorInvalidValue;
    if (N == 512) return launch_up_t<512>(y, wave, wfac, tw_n, tw_m, pairs, M, Lg, bg0, rows, first, linear, st);
    if (N == 1024) return launch_up_t<1024>(y, wave, wfac, tw_n, tw_m, pairs, M, Lg, bg0, rows, first, linear, st);
    if (N == 2048) return launch_up_t<2048>(y, wave, wfac, tw_n, tw_m, pairs, M, Lg, bg0, rows, first, linear, st);
    if (N == 4096) return launch_up_t<4096>(y, wave, wfac, tw_n, tw_m, pairs, M, Lg, bg0, rows, first, linear, st);
    return launch_up_t<8192>(y, wave, wfac, tw_n, tw_m, pairs, M, Lg, bg0, rows, first, linear, st);
}

cudaError_t launch_unpack_profiles(const void* spec, int dbl, float2* prof, long M, int Lg, long bg0, int rows,
                                   int first, cudaStream_t st) {
    const dim3 grid((unsigned)((Lg + 255) / 256), (unsigned)rows);
    if (dbl)
        unpack_profiles_kernel<double2><<<grid, 256, 0, st>>>((const double2*)spec, prof, M, Lg, bg0, first);
    else
        unpack_profiles_kernel<float2><<<grid, 256, 0, st>>>((const float2*)spec, prof, M, Lg, bg0, first);
    return cudaGetLastError();
}

cudaError_t launch_pack_forward(const float2* acc, void* spec, int dbl, long M, int Lg, long bg0, int rows, int first,
                                cudaStream_t st) {
    const dim3 grid((unsigned)((M + 255) / 256), (unsigned)rows);
    if (dbl)
        pack_forward_kernel<double2><<<grid, 256, 0, st>>>(acc, (double2*)spec, M, Lg, bg0, first);
    else
        pack_forward_kernel<float2><<<grid, 256, 0, st>>>(acc, (float2*)spec, M, Lg, bg0, first);
    return cudaGetLastError();
}

cudaError_t launch_extract_forward(const void* spec, int dbl, const float2* wave, const float2* wfac, float2* y,
                                   int N, long M, int rows, int first, cudaStream_t st) {
    const dim3 grid((unsigned)((N + 255) / 256), (unsigned)rows);
    if (dbl)
        extract_forward_kernel<double2><<<grid, 256, 0, st>>>((const double2*)spec, wave, wfac, y, N, M, first);
    else
        extract_forward_kernel<float2><<<grid, 256, 0, st>>>((const float2*)spec, wave, wfac, y, N, M, first);
    return cudaGetLastError();
}

cudaError_t launch_weights(const float2* w, float2* wadj, float2* wfwd, int S, int conj_adjoint, cudaStream_t st) {
    weights_kernel<<<(S + 255) / 256, 256, 0, st>>>(w, wadj, wfwd, S, conj_adjoint);
    return cudaGetLastError();
}

}  // namespace sar
