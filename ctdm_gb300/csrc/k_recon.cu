// Fourier-domain ODT kernels: batched line transforms, Ewald-cap mapping and
// the fused positivity-loop passes over a complex64 R^3 volume.
//
// Reference path (y-h-Lin/cTDM): BatchRecon (cTDM/HilbertTransform.cu:1825-2047)
// calls EdwardSphere/fillEdwardSphere (cTDM/Recon_kernel.cu:171-229),
// Initial_F_F2 (:253-276), cuFFT3D (cTDM/FFT.cu:807-838), calculate_n3D
// (:305-342), Modify_F3D (:370-383) and check_F3D (:396-412) as separate
// full-volume passes.  Here one loop body {modify, FFT3, replace, IFFT3, est_n}
// is four line passes over HBM:
//   x pass: IFFT_x, 1/R^3, est_n, modify, FFT_x   (the real-space operators)
//   y pass: FFT_y
//   z pass: FFT_z, replace with the measured data, IFFT_z   (k-space operator)
//   y pass: IFFT_y
// The mapping kernel owns whole z columns, so it accumulates the Ewald samples,
// forms F2 = F/C/dx and applies the first z inverse transform in shared memory.
#include <cmath>

#include <cudaTypedefs.h>

#include "fft_line.cuh"
#include "kernels.cuh"
#include "point_ops.cuh"
#include "tma.cuh"

// ------------------------------------------------------------ TMA tensor maps (host)
namespace tma {

static PFN_cuTensorMapEncodeTiled_v12000 encode_fn()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    return fn;
}

cudaError_t make_map_3d(CUtensorMap *map, const void *base, int elem_bytes, const uint64_t dims[3], const uint32_t box[3])
{
    auto fn = encode_fn();
    if (!fn) return cudaErrorNotSupported;
    if ((reinterpret_cast<uintptr_t>(base) & 15) || (box[0] * (uint32_t)elem_bytes) % 16) return cudaErrorInvalidValue;
    const CUtensorMapDataType ty = elem_bytes == 8 ? CU_TENSOR_MAP_DATA_TYPE_INT64 : CU_TENSOR_MAP_DATA_TYPE_UINT8;
    const cuuint64_t gdim[3] = {dims[0], dims[1], dims[2]};
    const cuuint64_t gstride[2] = {dims[0] * elem_bytes, dims[0] * dims[1] * elem_bytes};
    const cuuint32_t bdim[3] = {box[0], box[1], box[2]};
    const cuuint32_t estride[3] = {1, 1, 1};
    CUresult r = fn(map, ty, 3, const_cast<void *>(base), gdim, gstride, bdim, estride, CU_TENSOR_MAP_INTERLEAVE_NONE,
                    CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

}  // namespace tma

namespace ctdm {

using fftl::Plan;

// ------------------------------------------------------------ load / store
// Contiguous lines: line l occupies data[l*L .. l*L+L).
template <int L>
__device__ __forceinline__ void load_rows(float2 *buf, const float2 *__restrict__ src, long line0, long nlines)
{
    using P = Plan<L>;
    const float4 *s4 = reinterpret_cast<const float4 *>(src);
#pragma unroll 4
    for (int e = threadIdx.x; e < P::B * L / 2; e += P::THREADS) {
        const int b = (2 * e) / L, p = 2 * e - b * L;
        const long l = line0 + b;
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (l < nlines) v = __ldcs(&s4[(l * L + p) / 2]);
        buf[b * P::LP + p] = make_float2(v.x, v.y);
        buf[b * P::LP + p + 1] = make_float2(v.z, v.w);
    }
}

template <int L>
__device__ __forceinline__ void store_rows(float2 *dst, const float2 *buf, long line0, long nlines)
{
    using P = Plan<L>;
    float4 *d4 = reinterpret_cast<float4 *>(dst);
#pragma unroll 4
    for (int e = threadIdx.x; e < P::B * L / 2; e += P::THREADS) {
        const int b = (2 * e) / L, p = 2 * e - b * L;
        const long l = line0 + b;
        if (l < nlines) {
            float2 a = buf[b * P::LP + p], c = buf[b * P::LP + p + 1];
            __stcs(&d4[(l * L + p) / 2], make_float4(a.x, a.y, c.x, c.y));
        }
    }
}

// Strided lines: element p of line l at (l % nx) + (l / nx) * plane + p * ld.
// Threads are b-fastest so B consecutive lines give coalesced segments.
template <int L>
__device__ __forceinline__ long col_base(long line0, int nx, long plane, long nlines, bool &ok)
{
    using P = Plan<L>;
    const int b = threadIdx.x % P::B;
    const long l = line0 + b;
    ok = l < nlines;
    return (l % nx) + (l / nx) * plane;
}

template <int L>
__device__ __forceinline__ void load_cols(float2 *buf, const float2 *__restrict__ src, long base, bool ok, long ld)
{
    using P = Plan<L>;
    const int b = threadIdx.x % P::B, t = threadIdx.x / P::B;
#pragma unroll 4
    for (int p = t; p < L; p += P::T) buf[b * P::LP + p] = ok ? __ldcs(&src[base + p * ld]) : make_float2(0.f, 0.f);
}

template <int L>
__device__ __forceinline__ void store_cols(float2 *dst, const float2 *buf, long base, bool ok, long ld)
{
    using P = Plan<L>;
    const int b = threadIdx.x % P::B, t = threadIdx.x / P::B;
    if (!ok) return;
#pragma unroll 4
    for (int p = t; p < L; p += P::T) __stcs(&dst[base + p * ld], buf[b * P::LP + p]);
}

// ------------------------------------------------------------ generic passes
template <int L, bool INV>
__global__ void __launch_bounds__(Plan<L>::THREADS) rows_kernel(float2 *data, const float2 *__restrict__ tw, long nlines)
{
    extern __shared__ float4 smem4[];
    float2 *buf = reinterpret_cast<float2 *>(smem4);
    const long line0 = (long)blockIdx.x * Plan<L>::B;
    load_rows<L>(buf, data, line0, nlines);
    __syncthreads();
    Plan<L>::template run<INV>(buf, tw);
    store_rows<L>(data, buf, line0, nlines);
}

template <int L, bool INV>
__global__ void __launch_bounds__(Plan<L>::THREADS) cols_kernel(float2 *data, const float2 *__restrict__ tw, long nlines,
                                                                int nx, long plane, long ld)
{
    using P = Plan<L>;
    using En = fftl::Ends<L>;
    extern __shared__ float4 smem4[];
    float2 *buf = reinterpret_cast<float2 *>(smem4);
    const long line0 = (long)blockIdx.x * P::B;
    bool ok;
    const long base = col_base<L>(line0, nx, plane, nlines, ok);
    const int t = threadIdx.x / P::B;
    float2 v[P::E];
#pragma unroll
    for (int i = 0; i < P::E; i++)
        v[i] = ok ? __ldcs(&data[base + (long)fftl::slot_pos<L, P::T, En::F>(i, t) * ld]) : make_float2(0.f, 0.f);
    P::template seq<INV, false, false>(buf, v, tw);
    if (!ok) return;
#pragma unroll
    for (int i = 0; i < P::E; i++) __stcs(&data[base + (long)fftl::slot_pos<L, P::T, En::Rv>(i, t) * ld], v[i]);
}

// Large dynamic shared memory opt-in and the largest shared-memory carveout, so
// that several line-batch CTAs stay resident per SM.
template <int L, class K>
static cudaError_t prep_launch(K kernel, size_t smem)
{
    if (!twiddles(L)) return cudaErrorInitializationError;   // device tables not built on this device
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    return cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                                (int)cudaSharedmemCarveoutMaxShared);
}

template <int L>
static cudaError_t rows_launch(float2 *data, long nlines, bool inv, cudaStream_t s)
{
    using P = Plan<L>;
    const size_t smem = fftl::smem_bytes<L>();
    const long grid = (nlines + P::B - 1) / P::B;
    auto k = inv ? rows_kernel<L, true> : rows_kernel<L, false>;
    cudaError_t e = prep_launch<L>(k, smem);
    if (e != cudaSuccess) return e;
    k<<<(unsigned)grid, P::THREADS, smem, s>>>(data, twiddles(L), nlines); note_launch();
    return cudaGetLastError();
}

template <int L>
static cudaError_t cols_launch(float2 *data, long nlines, int nx, long plane, long ld, bool inv, cudaStream_t s)
{
    using P = Plan<L>;
    const size_t smem = fftl::smem_bytes<L>();
    const long grid = (nlines + P::B - 1) / P::B;
    auto k = inv ? cols_kernel<L, true> : cols_kernel<L, false>;
    cudaError_t e = prep_launch<L>(k, smem);
    if (e != cudaSuccess) return e;
    k<<<(unsigned)grid, P::THREADS, smem, s>>>(data, twiddles(L), nlines, nx, plane, ld); note_launch();
    return cudaGetLastError();
}

cudaError_t fft_rows(float2 *data, int L, long nlines, bool inverse, cudaStream_t s)
{
    CTDM_DISPATCH_L(L, rows_launch, data, nlines, inverse, s)
}

cudaError_t fft_cols(float2 *data, int L, long nlines, int nx, long plane, long ld, bool inverse, cudaStream_t s)
{
    CTDM_DISPATCH_L(L, cols_launch, data, nlines, nx, plane, ld, inverse, s)
}

__global__ void scale_kernel(float2 *d, long n, float s, bool conj)
{
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        float2 v = d[i];
        d[i] = make_float2(v.x * s, conj ? -v.y * s : v.y * s);
    }
}

cudaError_t scale_complex(float2 *data, long n, float s, bool conjugate, cudaStream_t st)
{
    long blocks = (n + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    scale_kernel<<<(unsigned)blocks, 256, 0, st>>>(data, n, s, conjugate); note_launch();
    return cudaGetLastError();
}

cudaError_t fft3d(float2 *data, int R, bool inverse, cudaStream_t s)
{
    const long r2 = (long)R * R;
    cudaError_t e = fft_rows(data, R, r2, inverse, s);
    if (e == cudaSuccess) e = fft_cols(data, R, r2, R, r2, R, inverse, s);
    if (e == cudaSuccess) e = fft_cols(data, R, r2, R, R, r2, inverse, s);
    if (e == cudaSuccess && inverse) e = scale_complex(data, r2 * R, 1.0f / (float)(r2 * R), false, s);
    return e;
}

// ------------------------------------------------------------ x pass
// Rows are contiguous, so the pass runs under the row mapping: each thread loads
// its first-stage points straight from HBM (unit stride across the warp), the
// inverse transform ends in registers, the point operators run on the registers,
// and the forward transform in the reversed radix order stores straight back.
template <int L, bool FINAL>
__global__ void __launch_bounds__(Plan<L>::THREADS, fftl::min_ctas<L>(4)) xpass_kernel(LoopArgs a, const float2 *__restrict__ tw)
{
    using P = Plan<L>;
    using En = fftl::Ends<L>;
    extern __shared__ float4 smem4[];
    float2 *buf = reinterpret_cast<float2 *>(smem4);
    const int t = threadIdx.x % P::T, b = threadIdx.x / P::T;
    const long l = (long)blockIdx.x * P::B + b;   // row y + L z (the grid covers the L^2 rows exactly)
    const float2 *src = a.G + l * L;
    float2 v[P::E];
#pragma unroll
    for (int i = 0; i < P::E; i++) v[i] = __ldcs(&src[fftl::slot_pos<L, P::T, En::F>(i, t)]);
    P::template seq_row<true>(buf, v, tw);
    if constexpr (FINAL) {
        // est_n then the octant shift (cuFFT3Dshift, cTDM/FFT.cu:324-350) on the write
        const int y = (int)(l % L), z = (int)(l / L);
        float2 *dst = a.out + (long)L * ((y + L / 2) % L) + (long)L * L * ((z + L / 2) % L);
#pragma unroll
        for (int i = 0; i < P::E; i++) {
            const int p = fftl::slot_pos<L, P::T, En::Rv>(i, t);
            dst[(p + L / 2) % L] = est_n_scaled(v[i], a.s1, a.n_med);
        }
    } else {
#pragma unroll
        for (int i = 0; i < P::E; i++) v[i] = modify_f_scaled(est_n_scaled(v[i], a.s1, a.n_med), a.s2, a.k2);
        P::template seqr_row<false>(buf, v, tw);
        float2 *dst = a.G + l * L;
#pragma unroll
        for (int i = 0; i < P::E; i++) __stcs(&dst[fftl::slot_pos<L, P::T, En::F>(i, t)], v[i]);
    }
}

// ------------------------------------------------------------ y pass
template <int L, bool INV>
__global__ void __launch_bounds__(Plan<L>::THREADS) ypass_kernel(LoopArgs a, const float2 *__restrict__ tw)
{
    using P = Plan<L>;
    using En = fftl::Ends<L>;
    extern __shared__ float4 smem4[];
    float2 *buf = reinterpret_cast<float2 *>(smem4);
    const long nl = (long)L * L;
    // planes in descending z: the x pass runs them ascending, so each pass starts on
    // the planes the previous one wrote last (still in L2)
    const long line0 = (long)(gridDim.x - 1 - blockIdx.x) * P::B;
    bool ok;
    const long base = col_base<L>(line0, L, (long)L * L, nl, ok);
    const int t = threadIdx.x / P::B;
    float2 v[P::E];
#pragma unroll
    for (int i = 0; i < P::E; i++) v[i] = __ldcs(&a.G[base + (long)fftl::slot_pos<L, P::T, En::F>(i, t) * L]);
    P::template seq<INV, false, false>(buf, v, tw);
#pragma unroll
    for (int i = 0; i < P::E; i++) __stcs(&a.G[base + (long)fftl::slot_pos<L, P::T, En::Rv>(i, t) * L], v[i]);
}

// ------------------------------------------------------------ z pass
// check_F3D (cTDM/Recon_kernel.cu:396-412): F <- F2 where F2.re != 0 and F2.im != 0
// (mode 0, the reference predicate) or where the voxel was hit (mode 1).
//
// For R <= 256 the CTA's F2 tile (B columns x R planes, and the hit-mask tile in
// mode 1) is staged into shared memory by TMA bulk tensor loads issued before the
// forward transform, so the measured data arrive while the transform runs instead
// of as a second dependent round trip to HBM.  Larger R keeps direct loads (the
// tile would cost the pass its second resident CTA).
template <int L>
constexpr bool zpass_tma()
{
    return L <= 256 && Plan<L>::B <= L;   // a CTA's B columns share one y
}
// z extent of one TMA box (a box side is at most 256 elements)
template <int L>
constexpr int zpass_box()
{
    return L <= 256 ? L : 256;
}

template <int L, int MODE>
constexpr size_t zpass_smem()
{
    using P = Plan<L>;
    if constexpr (!zpass_tma<L>()) return fftl::smem_bytes<L>();
    else
        return 128 + sizeof(float2) * P::B * L + (MODE ? (size_t)P::B * L : 0) + fftl::smem_bytes<L>() + 16;
}

template <int L, int MODE>
__global__ void __launch_bounds__(Plan<L>::THREADS, fftl::min_ctas<L>(3))
    zpass_kernel(LoopArgs a, const float2 *__restrict__ tw, const __grid_constant__ CUtensorMap f2map,
                 const __grid_constant__ CUtensorMap maskmap)
{
    using P = Plan<L>;
    using En = fftl::Ends<L>;
    constexpr bool TMA = zpass_tma<L>();
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
    const long line0 = (long)blockIdx.x * P::B;
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
            constexpr int ZB = zpass_box<L>();
            tma::mbar_expect_tx(bar, (uint32_t)(P::B * L * (sizeof(float2) + (MODE ? 1 : 0))));
            for (int z0 = 0; z0 < L; z0 += ZB) {
                tma::tma_load_3d(sf2 + (long)z0 * P::B, &f2map, x0, y, z0, bar);
                if (MODE) tma::tma_load_3d(smask + (long)z0 * P::B, &maskmap, x0, y, z0, bar);
            }
        }
    }
    bool ok;
    const long base = col_base<L>(line0, L, L, nl, ok);
    const int b = threadIdx.x % P::B, t = threadIdx.x / P::B;
    float2 v[P::E];
#pragma unroll
    for (int i = 0; i < P::E; i++) v[i] = __ldcs(&a.G[base + (long)fftl::slot_pos<L, P::T, En::F>(i, t) * nl]);
    P::template seq<false, false, false>(buf, v, tw);
    if (staged) tma::mbar_wait(bar, 0, a.err, 1);
#pragma unroll
    for (int i = 0; i < P::E; i++) {
        const int z = fftl::slot_pos<L, P::T, En::Rv>(i, t);
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
    for (int i = 0; i < P::E; i++) __stcs(&a.G[base + (long)fftl::slot_pos<L, P::T, En::F>(i, t) * nl], v[i]);
}

template <int L>
static cudaError_t xpass_launch(const LoopArgs &a, bool fin, cudaStream_t s)
{
    using P = Plan<L>;
    const size_t smem = fftl::smem_bytes_row<L>();
    auto k = fin ? xpass_kernel<L, true> : xpass_kernel<L, false>;
    cudaError_t e = prep_launch<L>(k, smem);
    if (e != cudaSuccess) return e;
    k<<<(unsigned)((long)L * L / P::B), P::THREADS, smem, s>>>(a, twiddles(L)); note_launch();
    return cudaGetLastError();
}

template <int L>
static cudaError_t ypass_launch(const LoopArgs &a, bool inv, cudaStream_t s)
{
    using P = Plan<L>;
    const size_t smem = fftl::smem_bytes<L>();
    auto k = inv ? ypass_kernel<L, true> : ypass_kernel<L, false>;
    cudaError_t e = prep_launch<L>(k, smem);
    if (e != cudaSuccess) return e;
    k<<<(unsigned)((long)L * L / P::B), P::THREADS, smem, s>>>(a, twiddles(L)); note_launch();
    return cudaGetLastError();
}

template <int L>
static cudaError_t zpass_launch(const LoopArgs &a, int mode, cudaStream_t s)
{
    using P = Plan<L>;
    const size_t smem = mode ? zpass_smem<L, 1>() : zpass_smem<L, 0>();
    auto k = mode ? zpass_kernel<L, 1> : zpass_kernel<L, 0>;
    cudaError_t e = prep_launch<L>(k, smem);
    if (e != cudaSuccess) return e;
    CUtensorMap f2map = {}, maskmap = {};
    LoopArgs la = a;
    la.staged = 0;
    if (zpass_tma<L>()) {
        // F2 and the mask viewed as (x, y, z) arrays; a box is B columns of one y by R planes.
        // Tiles are staged when both arrays meet the tensor-map alignment (any cudaMalloc
        // base does); otherwise the kernel reads them directly.
        const uint64_t dims[3] = {(uint64_t)L, (uint64_t)L, (uint64_t)L};
        const uint32_t box[3] = {(uint32_t)P::B, 1u, (uint32_t)zpass_box<L>()};
        bool okmap = tma::make_map_3d(&f2map, a.F2, 8, dims, box) == cudaSuccess;
        if (okmap && mode) okmap = tma::make_map_3d(&maskmap, a.mask, 1, dims, box) == cudaSuccess;
        la.staged = okmap ? 1 : 0;
    }
    k<<<(unsigned)((long)L * L / P::B), P::THREADS, smem, s>>>(la, twiddles(L), f2map, maskmap); note_launch();
    return cudaGetLastError();
}

// Volume sides supported by the reconstruction passes.
#define CTDM_DISPATCH_R(Rrt, FN, ...)                  \
    switch (Rrt) {                                     \
    case 32: return FN<32>(__VA_ARGS__);               \
    case 64: return FN<64>(__VA_ARGS__);               \
    case 128: return FN<128>(__VA_ARGS__);             \
    case 256: return FN<256>(__VA_ARGS__);             \
    case 384: return FN<384>(__VA_ARGS__);             \
    case 512: return FN<512>(__VA_ARGS__);             \
    case 768: return FN<768>(__VA_ARGS__);             \
    default: return cudaErrorInvalidValue;             \
    }

cudaError_t launch_xpass(const LoopArgs &a, bool final_pass, cudaStream_t s)
{
    CTDM_DISPATCH_R(a.R, xpass_launch, a, final_pass, s)
}
cudaError_t launch_ypass(const LoopArgs &a, bool inverse, cudaStream_t s)
{
    CTDM_DISPATCH_R(a.R, ypass_launch, a, inverse, s)
}
cudaError_t launch_zpass(const LoopArgs &a, int check_mode, cudaStream_t s)
{
    CTDM_DISPATCH_R(a.R, zpass_launch, a, check_mode, s)
}

// ------------------------------------------------------------ Ewald mapping
template <int L>
__global__ void __launch_bounds__(Plan<L>::THREADS) ewald_kernel(EwaldArgs a, const float2 *__restrict__ tw)
{
    using P = Plan<L>;
    constexpr int R = L;
    extern __shared__ float4 smem4[];
    float2 *buf = reinterpret_cast<float2 *>(smem4);
    uint32_t *cnt = reinterpret_cast<uint32_t *>(buf + P::B * P::LP);
    AngleGeom *geo = reinterpret_cast<AngleGeom *>(cnt + P::B * L);
    const long line0 = (long)blockIdx.x * P::B;   // line = x + R*y, B consecutive x
    for (int e = threadIdx.x; e < P::B * P::LP; e += P::THREADS) buf[e] = make_float2(0.f, 0.f);
    for (int e = threadIdx.x; e < P::B * L; e += P::THREADS) cnt[e] = 0u;
    for (int e = threadIdx.x; e < a.A; e += P::THREADS) geo[e] = a.geom[e];
    __syncthreads();

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = P::THREADS >> 5;
    const long rr = (long)R * R;
    const float four_pi = 4.0f * CTDM_PI_F;
    for (int b = warp; b < P::B; b += nwarps) {
        const long l = line0 + b;
        const int x = (int)(l % R), y = (int)(l / R);
        const int ii = x < R / 2 ? x : x - R;
        const int jj = y < R / 2 ? y : y - R;
        const float2 *ucol = a.U + x + (long)R * y;
        float2 *col = buf + b * P::LP;
        uint32_t *ccol = cnt + b * L;
        for (int a0 = 0; a0 < a.A; a0 += 32) {
            const int ang = a0 + lane;
            int nz = -1;
            float2 val = make_float2(0.f, 0.f);
            if (ang < a.A && geo[ang].valid) {
                float fz;
                nz = ewald_nz(ii, jj, geo[ang], a.df, a.fm02, a.fm02s, R, fz);
                if (nz >= 0) {
                    const float2 u = __ldg(&ucol[ang * rr]);
                    val = make_float2(-fz * four_pi * u.y, fz * four_pi * u.x);
                }
            }
            // angle order per voxel: lanes are applied one after another
            unsigned pending = __ballot_sync(0xffffffffu, nz >= 0);
            while (pending) {
                const int q = __ffs(pending) - 1;
                if (lane == q) {
                    float2 c = col[nz];
                    col[nz] = make_float2(c.x + val.x, c.y + val.y);
                    ccol[nz] += 1u;
                }
                __syncwarp();
                pending &= pending - 1;
            }
        }
    }
    __syncthreads();
    // Initial_F_F2 (cTDM/Recon_kernel.cu:253-276): F2 = (F / C where C != 0) / dx
    {
        const int b = threadIdx.x % P::B, t = threadIdx.x / P::B;
        const long l = line0 + b;
        const long base = l;   // (x + R*y)
        for (int p = t; p < L; p += P::T) {
            float2 v = buf[b * P::LP + p];
            const uint32_t c = cnt[b * L + p];
            if (c != 0u) v = make_float2(v.x / (float)c, v.y / (float)c);
            v = make_float2(v.x / a.dx, v.y / a.dx);
            buf[b * P::LP + p] = v;
            const long idx = base + (long)p * rr;
            a.F2[idx] = v;
            if (a.counts) a.counts[idx] = c;
            if (a.mask) a.mask[idx] = c != 0u;
        }
    }
    __syncthreads();
    {
        float2 v[P::E];
        P::template seq<true, true, false>(buf, v, tw);
        const int b = threadIdx.x % P::B, t = threadIdx.x / P::B;
        const long base = line0 + b;
#pragma unroll
        for (int i = 0; i < P::E; i++) a.G[base + (long)fftl::slot_pos<L, P::T, fftl::Ends<L>::Rv>(i, t) * rr] = v[i];
    }
}

template <int L>
static cudaError_t ewald_launch(const EwaldArgs &a, cudaStream_t s)
{
    using P = Plan<L>;
    const size_t smem = fftl::smem_bytes<L>() + sizeof(uint32_t) * P::B * L + sizeof(AngleGeom) * a.A;
    auto k = ewald_kernel<L>;
    cudaError_t e = prep_launch<L>(k, smem);
    if (e != cudaSuccess) return e;
    k<<<(unsigned)((long)L * L / P::B), P::THREADS, smem, s>>>(a, twiddles(L)); note_launch();
    return cudaGetLastError();
}

cudaError_t launch_ewald(const EwaldArgs &a, cudaStream_t s)
{
    CTDM_DISPATCH_R(a.R, ewald_launch, a, s)
}

}  // namespace ctdm
