// The fused positivity-loop passes over a complex64 R^3 volume, templated on the
// FFT plan so the autotuner can pick a plan per pass and size.
//
// Reference path (y-h-Lin/cTDM): the loop of BatchRecon (cTDM/HilbertTransform.cu:
// 1943-2004) calls cuFFT3D (cTDM/FFT.cu:807-838), calculate_n3D (cTDM/
// Recon_kernel.cu:305-342), Modify_F3D (:370-383) and check_F3D (:396-412) as separate
// full-volume passes.  Here one loop body {modify, FFT3, replace, IFFT3, est_n} is
// four line passes over HBM:
//   x pass: IFFT_x, 1/R^3, est_n, modify, FFT_x   (the real-space operators)
//   y pass: FFT_y
//   z pass: FFT_z, replace with the measured data, IFFT_z   (k-space operator)
//   y pass: IFFT_y
// Each size's instantiations live in their own translation unit (k_loop_*.cu).
#pragma once
#include <mutex>

#include "fft_line.cuh"
#include "kernels.cuh"
#include "point_ops.cuh"
#include "tma.cuh"

namespace ctdm {

// Large dynamic shared memory opt-in and the largest carveout, once per kernel and
// device (kernel_configured / mark_kernel_configured keep the set of configured pairs).

template <class K>
static cudaError_t prep_plan_kernel(K kernel, int L, size_t smem)
{
    if (!twiddles(L)) return cudaErrorInitializationError;   // device tables not built on this device
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const void *fn = reinterpret_cast<const void *>(kernel);
    if (kernel_configured(fn, dev)) return cudaSuccess;
    if (smem > 48 * 1024) {
        e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                             (int)cudaSharedmemCarveoutMaxShared);
    if (e == cudaSuccess) mark_kernel_configured(fn, dev);
    return e;
}

// Lines one wave ahead for a z-pass kernel: its resident CTAs on the device x lines per
// CTA (0 when the occupancy query fails), once per kernel and device.  A z-pass CTA
// prefetches into L2 the z lines of the CTA that starts when it ends, so that CTA's
// strided loads (one 8 B x B segment per plane) find L2 instead of HBM: the pass's
// loads all issue at its start, and with 3 or 4 CTAs per SM the transforms otherwise
// leave HBM idle.  At 256^3 the packed z pass went from 77.6 to 69.2 us per launch in
// the headline step (69.0 to 61.5 without Goldstein beside it).
template <class P, class K>
static long zpass_ahead(K kernel, size_t smem)
{
    static long cached[64];
    static bool known[64];
    static std::mutex mu;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 0;
    std::lock_guard<std::mutex> lk(mu);
    if (!known[dev]) {
        int per_sm = 0, sms = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, P::THREADS, smem) != cudaSuccess ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
            cudaGetLastError();
            per_sm = sms = 0;
        }
        cached[dev] = (long)per_sm * sms * P::B;
        known[dev] = true;
    }
    return cached[dev];
}

// One wave ahead: the L z segments of lines [line0 + ahead, + B) into L2.
template <class P>
__device__ __forceinline__ void prefetch_next_wave(const float2 *G, long line0, long ahead)
{
    constexpr int L = P::L;
    const long nl = (long)L * L, ln = line0 + ahead;
    if (ahead <= 0 || ln >= nl) return;
    for (int z = threadIdx.x; z < L; z += P::THREADS) prefetch_l2(&G[ln + (long)z * nl]);
}

// ------------------------------------------------------------ x pass
// Rows are contiguous, so the pass runs under the row mapping: each thread loads
// its first-stage points straight from HBM (unit stride across the warp), the
// inverse transform ends in registers, the point operators run on the registers,
// and the forward transform in the reversed radix order stores straight back.
template <class P, bool FINAL, bool MOM = false>
__global__ void __launch_bounds__(P::THREADS, fftl::plan_min_ctas<P>(4)) xpass_kernel(LoopArgs a,
                                                                                      const float2 *__restrict__ tw)
{
    constexpr int L = P::L;
    extern __shared__ float4 smem4[];
    float2 *buf = reinterpret_cast<float2 *>(smem4);
    const int t = threadIdx.x % P::T, b = threadIdx.x / P::T;
    const long l = (long)blockIdx.x * P::B + b;   // row y + L z (the grid covers the L^2 rows exactly)
    const float2 *src = a.G + l * L;
    if constexpr (MOM && !FINAL) {
        // the previous iterate of this row comes from HBM during the inverse transform
#pragma unroll
        for (int i = 0; i < P::E; i++) prefetch_l2(a.xprev + l * L + fftl::slot_pos<L, P::T, P::RV0>(i, t));
    }
    float2 v[P::E];
#pragma unroll
    for (int i = 0; i < P::E; i++) v[i] = __ldcs(&src[fftl::slot_pos<L, P::T, P::F0>(i, t)]);
    P::template seq_row<true>(buf, v, tw);
    if constexpr (FINAL) {
        // est_n then the octant shift (cuFFT3Dshift, cTDM/FFT.cu:324-350) on the write
        const int y = (int)(l % L), z = (int)(l / L);
        float2 *dst = a.out + (long)L * ((y + L / 2) % L) + (long)L * L * ((z + L / 2) % L);
#pragma unroll
        for (int i = 0; i < P::E; i++) {
            const int p = fftl::slot_pos<L, P::T, P::RV0>(i, t);
            dst[(p + L / 2) % L] = est_n_scaled(v[i], a.s1, a.n_med);
        }
    } else {
#pragma unroll
        for (int i = 0; i < P::E; i++) v[i] = modify_f_scaled(est_n_scaled(v[i], a.s1, a.n_med), a.s2, a.k2);
        if constexpr (MOM) {
            float2 *xp = a.xprev + l * L;
#pragma unroll
            for (int i = 0; i < P::E; i++) {
                const int o = fftl::slot_pos<L, P::T, P::RV0>(i, t);
                const float2 prev = xp[o];
                xp[o] = v[i];
                v[i] = momentum_step(v[i], prev, a.beta);
            }
        }
        P::template seqr_row<false>(buf, v, tw);
        float2 *dst = a.G + l * L;
#pragma unroll
        for (int i = 0; i < P::E; i++) __stcs(&dst[fftl::slot_pos<L, P::T, P::F0>(i, t)], v[i]);
    }
}

// ------------------------------------------------------------ y pass
// Lines (x, z) with B consecutive x per CTA (coalesced B*8-byte segments per row).
template <class P, bool INV>
__global__ void __launch_bounds__(P::THREADS, fftl::plan_min_ctas<P>(5)) ypass_kernel(LoopArgs a,
                                                                                      const float2 *__restrict__ tw)
{
    constexpr int L = P::L;
    extern __shared__ float4 smem4[];
    float2 *buf = reinterpret_cast<float2 *>(smem4);
    // planes in descending z: the x pass runs them ascending, so each pass starts on
    // the planes the previous one wrote last (still in L2)
    const long line0 = (long)(gridDim.x - 1 - blockIdx.x) * P::B;
    const int b = threadIdx.x % P::B, t = threadIdx.x / P::B;
    const long l = line0 + b;
    const long base = (l % L) + (l / L) * (long)L * L;
    float2 v[P::E];
#pragma unroll
    for (int i = 0; i < P::E; i++) v[i] = __ldcs(&a.G[base + (long)fftl::slot_pos<L, P::T, P::F0>(i, t) * L]);
    P::template seq<INV, false, false>(buf, v, tw);
#pragma unroll
    for (int i = 0; i < P::E; i++) __stcs(&a.G[base + (long)fftl::slot_pos<L, P::T, P::RV0>(i, t) * L], v[i]);
}

// ------------------------------------------------------------ z pass
// check_F3D (cTDM/Recon_kernel.cu:396-412): F <- F2 where F2.re != 0 and F2.im != 0
// (mode 0, the reference predicate) or where the voxel was hit (mode 1).
//
// When the plan's F2 tile (B columns x R planes, and the hit-mask tile in mode 1)
// fits beside the transform buffer, it is staged into shared memory by TMA bulk
// tensor loads issued before the forward transform, so the measured data arrive
// while the transform runs instead of as a second dependent round trip to HBM.
template <class P>
constexpr bool zpass_tma()
{
    // a CTA's B columns share one y; a box side is at most 256 elements
    return P::B <= P::L && P::L <= 256 && sizeof(float2) * P::B * P::L <= 64 * 1024;
}

template <class P, int MODE>
constexpr size_t zpass_smem()
{
    if constexpr (!zpass_tma<P>()) return fftl::plan_smem<P>();
    else return 128 + sizeof(float2) * P::B * P::L + (MODE ? (size_t)P::B * P::L : 0) + fftl::plan_smem<P>() + 16;
}

template <class P, int MODE>
__global__ void __launch_bounds__(P::THREADS, fftl::plan_min_ctas<P>(3))
    zpass_kernel(LoopArgs a, const float2 *__restrict__ tw, const __grid_constant__ CUtensorMap f2map,
                 const __grid_constant__ CUtensorMap maskmap, long ahead)
{
    constexpr int L = P::L;
    constexpr bool TMA = zpass_tma<P>();
    const bool staged = TMA && a.staged;   // uniform over the grid
    extern __shared__ float4 smem4[];
    // [F2 tile, z-major: B*L float2][mask tile B*L bytes][FFT buffer][mbarrier], 128-byte aligned
    char *base0 = reinterpret_cast<char *>(smem4);
    char *al = TMA ? base0 + ((128 - (tma::smem_addr(base0) & 127)) & 127) : base0;
    float2 *sf2 = reinterpret_cast<float2 *>(al);
    uint8_t *smask = reinterpret_cast<uint8_t *>(sf2 + (TMA ? P::B * L : 0));
    float2 *buf = reinterpret_cast<float2 *>(smask + ((TMA && MODE) ? P::B * L : 0));
    uint64_t *bar = reinterpret_cast<uint64_t *>(buf + P::B * P::LP);
    const long nl = (long)L * L;
    const long line0 = (long)blockIdx.x * P::B;   // line = x + L y
    if (staged) {
        if (threadIdx.x == 0) {
            tma::prefetch_map(&f2map);
            if (MODE) tma::prefetch_map(&maskmap);
            tma::mbar_init(bar, 1);
            tma::fence_barrier_init();
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            const int x0 = (int)(line0 % L), y = (int)(line0 / L);
            tma::mbar_expect_tx(bar, (uint32_t)(P::B * L * (sizeof(float2) + (MODE ? 1 : 0))));
            tma::tma_load_3d(sf2, &f2map, x0, y, 0, bar);
            if (MODE) tma::tma_load_3d(smask, &maskmap, x0, y, 0, bar);
        }
    }
    const int b = threadIdx.x % P::B, t = threadIdx.x / P::B;
    const long base = line0 + b;
    prefetch_next_wave<P>(a.G, line0, ahead);
    float2 v[P::E];
#pragma unroll
    for (int i = 0; i < P::E; i++) v[i] = __ldcs(&a.G[base + (long)fftl::slot_pos<L, P::T, P::F0>(i, t) * nl]);
    P::template seq<false, false, false>(buf, v, tw);
    if (staged) tma::mbar_wait(bar, 0, a.err, 1);
#pragma unroll
    for (int i = 0; i < P::E; i++) {
        const int z = fftl::slot_pos<L, P::T, P::RV0>(i, t);
        float2 f2;
        bool keep;
        if (staged) {
            f2 = sf2[z * P::B + b];
            if (MODE == 0) keep = (f2.x != 0.0f && f2.y != 0.0f);
            else keep = smask[z * P::B + b] != 0;
        } else {
            const long idx = base + (long)z * nl;
            f2 = __ldcs(&a.F2[idx]);
            if (MODE == 0) keep = (f2.x != 0.0f && f2.y != 0.0f);
            else keep = a.mask[idx] != 0;
        }
        if (keep) v[i] = f2;
    }
    P::template seqr<true, false, false>(buf, v, tw);
#pragma unroll
    for (int i = 0; i < P::E; i++) __stcs(&a.G[base + (long)fftl::slot_pos<L, P::T, P::F0>(i, t) * nl], v[i]);
}

// ------------------------------------------------------------ z pass on packed measured samples
// The same pass reading only the measured samples: the tile's keep masks (one word
// per z) and its packed values arrive by bulk copies issued before the forward
// transform; the replacement indexes the packed values by a prefix count over z.
// The first ZCAP packed values of a tile are staged (8 KiB; the Ewald caps fill 5% of
// a 256^3 volume, about 200 values per 16-line tile), the rest are read from L2 at the
// replacement.  With that staging and 64 registers 4 CTAs fit per SM instead of 3:
// 69.1 -> 65.4 us per launch at 256^3 in the headline step.
constexpr int ZCAP = 1024;

template <class P>
constexpr bool zpass_packable()
{
    return (P::B == 8 || P::B == 16 || P::B == 32) && P::B <= P::L &&
           sizeof(float2) * P::B * P::L <= 64 * 1024 && (P::L * 4) % 16 == 0;
}

template <class P>
constexpr size_t zpass_packed_smem()
{
    return 128 + sizeof(float2) * ZCAP + sizeof(uint32_t) * P::L + sizeof(int) * P::L + 64 +
           fftl::plan_smem<P>() + 16;
}

template <class P>
__global__ void __launch_bounds__(P::THREADS, fftl::plan_min_ctas<P>(4))
    zpass_packed_kernel(LoopArgs a, const float2 *__restrict__ tw, long ahead)
{
    constexpr int L = P::L;
    extern __shared__ float4 smem4[];
    char *base0 = reinterpret_cast<char *>(smem4);
    char *al = base0 + ((128 - (tma::smem_addr(base0) & 127)) & 127);
    float2 *svals = reinterpret_cast<float2 *>(al);                          // ZCAP
    uint32_t *smask = reinterpret_cast<uint32_t *>(svals + ZCAP);            // L
    int *spre = reinterpret_cast<int *>(smask + L);                          // L (+16 spare)
    float2 *buf = reinterpret_cast<float2 *>(spre + L + 16);
    uint64_t *bar = reinterpret_cast<uint64_t *>(buf + P::B * P::LP);
    const long nl = (long)L * L;
    const long line0 = (long)blockIdx.x * P::B;   // line = x + L y; tile = line0 / B
    const long tile = line0 / P::B;
    if (threadIdx.x == 0) {
        tma::mbar_init(bar, 1);
        tma::fence_barrier_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const int cnt = a.tcount[tile];
        const uint32_t vbytes = (uint32_t)(((min(cnt, ZCAP) + 1) & ~1) * sizeof(float2));
        tma::mbar_expect_tx(bar, (uint32_t)(2 * L * sizeof(uint32_t)) + vbytes);
        tma::bulk_load(smask, a.tmask + tile * L, (uint32_t)(L * sizeof(uint32_t)), bar);
        tma::bulk_load(spre, a.tprefix + tile * L, (uint32_t)(L * sizeof(int)), bar);
        if (vbytes) tma::bulk_load(svals, a.tvals + tile * (long)P::B * L, vbytes, bar);
    }
    const int b = threadIdx.x % P::B, t = threadIdx.x / P::B;
    const long base = line0 + b;
    prefetch_next_wave<P>(a.G, line0, ahead);
    float2 v[P::E];
#pragma unroll
    for (int i = 0; i < P::E; i++) v[i] = __ldcs(&a.G[base + (long)fftl::slot_pos<L, P::T, P::F0>(i, t) * nl]);
    P::template seq<false, false, false>(buf, v, tw);
    tma::mbar_wait(bar, 0, a.err, 3);   // masks, row prefixes (from the packing) and values
    const uint32_t below = (1u << b) - 1u;
#pragma unroll
    for (int i = 0; i < P::E; i++) {
        const int z = fftl::slot_pos<L, P::T, P::RV0>(i, t);
        const uint32_t m = smask[z];
        if ((m >> b) & 1u) {
            const int q = spre[z] + __popc(m & below);
            v[i] = q < ZCAP ? svals[q] : a.tvals[tile * (long)P::B * L + q];
        }
    }
    P::template seqr<true, false, false>(buf, v, tw);
#pragma unroll
    for (int i = 0; i < P::E; i++) __stcs(&a.G[base + (long)fftl::slot_pos<L, P::T, P::F0>(i, t) * nl], v[i]);
}

// ------------------------------------------------------------ launchers
// kind: LOOP_X, LOOP_X_FINAL, LOOP_Y_FWD, LOOP_Y_INV, LOOP_Z (flag = check mode)
template <class P>
static cudaError_t run_loop_pass(int kind, const LoopArgs &a, int flag, cudaStream_t s)
{
    constexpr int L = P::L;
    const unsigned grid = (unsigned)((long)L * L / P::B);
    cudaError_t e;
    if (kind == LOOP_X || kind == LOOP_X_FINAL) {
        const size_t smem = fftl::plan_smem_row<P>();
        auto k = kind == LOOP_X_FINAL ? xpass_kernel<P, true>
                                      : (a.xprev ? xpass_kernel<P, false, true> : xpass_kernel<P, false>);
        e = prep_plan_kernel(k, L, smem);
        if (e != cudaSuccess) return e;
        k<<<grid, P::THREADS, smem, s>>>(a, twiddles(L));
    } else if (kind == LOOP_Y_FWD || kind == LOOP_Y_INV) {
        const size_t smem = fftl::plan_smem<P>();
        auto k = kind == LOOP_Y_INV ? ypass_kernel<P, true> : ypass_kernel<P, false>;
        e = prep_plan_kernel(k, L, smem);
        if (e != cudaSuccess) return e;
        k<<<grid, P::THREADS, smem, s>>>(a, twiddles(L));
    } else if (a.packed && zpass_packable<P>()) {
        const size_t smem = zpass_packed_smem<P>();
        auto k = zpass_packed_kernel<P>;
        e = prep_plan_kernel(k, L, smem);
        if (e != cudaSuccess) return e;
        k<<<grid, P::THREADS, smem, s>>>(a, twiddles(L), zpass_ahead<P>(k, smem));
    } else {
        const size_t smem = flag ? zpass_smem<P, 1>() : zpass_smem<P, 0>();
        auto k = flag ? zpass_kernel<P, 1> : zpass_kernel<P, 0>;
        e = prep_plan_kernel(k, L, smem);
        if (e != cudaSuccess) return e;
        CUtensorMap f2map = {}, maskmap = {};
        LoopArgs la = a;
        la.staged = 0;
        if (zpass_tma<P>()) {
            // F2 and the mask viewed as (x, y, z) arrays; a box is B columns of one y by R
            // planes.  Tiles are staged when both arrays meet the tensor-map alignment (any
            // cudaMalloc base does); otherwise the kernel reads them directly.
            const uint64_t dims[3] = {(uint64_t)L, (uint64_t)L, (uint64_t)L};
            const uint32_t box[3] = {(uint32_t)P::B, 1u, (uint32_t)L};
            bool okmap = tma::make_map_3d(&f2map, a.F2, 8, dims, box) == cudaSuccess;
            if (okmap && flag) okmap = tma::make_map_3d(&maskmap, a.mask, 1, dims, box) == cudaSuccess;
            la.staged = okmap ? 1 : 0;
        }
        k<<<grid, P::THREADS, smem, s>>>(la, twiddles(L), f2map, maskmap, zpass_ahead<P>(k, smem));
    }
    note_launch();
    return cudaGetLastError();
}

// Lines per z-pass CTA when that plan reads packed measured samples, else 0.
template <class P>
constexpr int zpass_tile()
{
    return zpass_packable<P>() ? P::B : 0;
}

}  // namespace ctdm

// One translation unit per volume side: loop_pass_<R>(kind, variant, args, flag, stream).
#define CTDM_LOOP_SIZE_1(LL)                                                                              \
    namespace ctdm {                                                                                      \
    cudaError_t loop_pass_##LL(int kind, int variant, const LoopArgs &a, int flag, cudaStream_t s)        \
    {                                                                                                     \
        (void)variant;                                                                                    \
        return run_loop_pass<fftl::PV<LL, 0>>(kind, a, flag, s);                                         \
    }                                                                                                     \
    int loop_ztile_##LL(int variant)                                                                      \
    {                                                                                                     \
        (void)variant;                                                                                    \
        return zpass_tile<fftl::PV<LL, 0>>();                                                             \
    }                                                                                                     \
    }
#define CTDM_LOOP_SIZE_3(LL)                                                                              \
    namespace ctdm {                                                                                      \
    cudaError_t loop_pass_##LL(int kind, int variant, const LoopArgs &a, int flag, cudaStream_t s)        \
    {                                                                                                     \
        switch (variant) {                                                                                \
        case 1: return run_loop_pass<fftl::PV<LL, 1>>(kind, a, flag, s);                                  \
        case 2: return run_loop_pass<fftl::PV<LL, 2>>(kind, a, flag, s);                                  \
        default: return run_loop_pass<fftl::PV<LL, 0>>(kind, a, flag, s);                                 \
        }                                                                                                 \
    }                                                                                                     \
    int loop_ztile_##LL(int variant)                                                                      \
    {                                                                                                     \
        return variant == 1 ? zpass_tile<fftl::PV<LL, 1>>()                                               \
                            : (variant == 2 ? zpass_tile<fftl::PV<LL, 2>>() : zpass_tile<fftl::PV<LL, 0>>()); \
    }                                                                                                     \
    }
