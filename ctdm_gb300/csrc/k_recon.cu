// Fourier-domain ODT kernels: batched line transforms of the FFT core and the
// Ewald-cap mapping.  The positivity-loop passes are in loop_passes.cuh.
//
// Reference path (y-h-Lin/cTDM): BatchRecon (cTDM/HilbertTransform.cu:1825-2047)
// calls EdwardSphere/fillEdwardSphere (cTDM/Recon_kernel.cu:171-229),
// Initial_F_F2 (:253-276) and cuFFT3D (cTDM/FFT.cu:807-838).  The mapping kernel
// owns whole z columns, so it accumulates the Ewald samples, forms F2 = F/C/dx and
// applies the first z inverse transform in shared memory.
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

// ------------------------------------------------------------ Ewald mapping
// Frequency interpolation between scan angles (FrquencyInterpolation, FI_kernel and
// calF, cTDM/Recon_kernel.cu:471-731, with the mathematics fixed).  A frame puts its
// detector frequency (Fx, Fy) on the voxel of its own cap, Fz = nz df after rounding.
// The illumination angle theta' (tilt in the y-z plane, the scan axis AngX) whose cap
// passes through that voxel centre satisfies Fy sin(theta') + Fz cos(theta') =
// -|K|^2 / (2 fm), i.e. theta' = atan2(Fy, Fz) +- acos(-|K|^2 / (2 fm rho)) with
// rho = |(Fy, Fz)|; the root nearer the frame's own angle is taken.  The spectra of the
// two scan angles around theta' are interpolated linearly in angle at the same
// detector frequency (the detector-plane part of the reference's trilinear
// interpolation is the identity there, since theta' maps the voxel back onto (Fx, Fy))
// and scaled by i 4 pi fz' with fz' = Fz + fm cos(theta').  Outside the scanned range
// the edge angle's spectrum is used; where no theta' exists, the frame's own sample.
__device__ __forceinline__ float2 fi_sample(int ii, int jj, int nzs, double df, double fm0, double theta_own,
                                            const double *th, const int *fr, int A, const float2 *ucol, long rr,
                                            float2 u_own, float fz_own)
{
    const double Fx = ii * df, Fy = jj * df, Fz = nzs * df;
    const double rho = sqrt(Fy * Fy + Fz * Fz);
    const double c = -(Fx * Fx + Fy * Fy + Fz * Fz) / (2.0 * fm0 * rho);
    const float four_pi = 4.0f * CTDM_PI_F;
    if (!(rho > 0.0) || c < -1.0 || c > 1.0)
        return make_float2(-fz_own * four_pi * u_own.y, fz_own * four_pi * u_own.x);
    const double phi = atan2(Fy, Fz), dth = acos(c);
    const double t1 = phi + dth, t2 = phi - dth;
    const double tp = fabs(t1 - theta_own) <= fabs(t2 - theta_own) ? t1 : t2;
    const float fzp = (float)(Fz + fm0 * cos(tp));
    int s = 0;
    double w = 0.0;
    if (tp >= th[A - 1]) {
        s = A - 1;
    } else if (tp > th[0]) {
        int lo = 0, hi = A - 1;   // th[lo] <= tp < th[hi]
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (th[mid] <= tp) lo = mid;
            else hi = mid;
        }
        s = lo;
        w = (tp - th[lo]) / (th[hi] - th[lo]);
    }
    float2 u = __ldg(&ucol[fr[s] * rr]);
    if (w > 0.0) {
        const float2 u2 = __ldg(&ucol[fr[s + 1] * rr]);
        const float wf = (float)w, vf = (float)(1.0 - w);
        u = make_float2(vf * u.x + wf * u2.x, vf * u.y + wf * u2.y);
    }
    return make_float2(-fzp * four_pi * u.y, fzp * four_pi * u.x);
}

template <int L, bool FI>
__global__ void __launch_bounds__(Plan<L>::THREADS) ewald_kernel(EwaldArgs a, const float2 *__restrict__ tw)
{
    using P = Plan<L>;
    constexpr int R = L;
    extern __shared__ float4 smem4[];
    float2 *buf = reinterpret_cast<float2 *>(smem4);
    uint32_t *cnt = reinterpret_cast<uint32_t *>(buf + P::B * P::LP);
    float2 *stage = reinterpret_cast<float2 *>(cnt + P::B * L);              // 32 values per warp
    AngleGeom *geo = reinterpret_cast<AngleGeom *>(stage + P::THREADS);
    double *th = reinterpret_cast<double *>(geo + a.A);   // FI: sorted scan angles
    int *fr = reinterpret_cast<int *>(th + a.A);          // FI: their frames
    const long line0 = (long)blockIdx.x * P::B;   // line = x + R*y, B consecutive x
    for (int e = threadIdx.x; e < P::B * P::LP; e += P::THREADS) buf[e] = make_float2(0.f, 0.f);
    for (int e = threadIdx.x; e < P::B * L; e += P::THREADS) cnt[e] = 0u;
    for (int e = threadIdx.x; e < a.A; e += P::THREADS) {
        geo[e] = a.geom[e];
        if constexpr (FI) {
            th[e] = a.fi_theta[e];
            fr[e] = a.fi_frame[e];
        }
    }
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
                if constexpr (FI) {
                    const int nzs = ewald_nz_signed(ii, jj, geo[ang], a.df, a.fm02, a.fm02s, fz);
                    if (nzs != kNoSample) {
                        nz = imod(nzs, R);
                        const float2 u = __ldg(&ucol[ang * rr]);
                        val = fi_sample(ii, jj, nzs, a.df, a.fm0, asin(geo[ang].fy0 / a.fm0), th, fr, a.A, ucol, rr,
                                        u, fz);
                    }
                } else {
                    nz = ewald_nz(ii, jj, geo[ang], a.df, a.fm02, a.fm02s, R, fz);
                    if (nz >= 0) {
                        const float2 u = __ldg(&ucol[ang * rr]);
                        val = make_float2(-fz * four_pi * u.y, fz * four_pi * u.x);
                    }
                }
            }
            // angle order per voxel: lanes hitting the same voxel form a group whose
            // lowest lane adds the members' values in lane (= angle) order, the same
            // sequence of float additions as applying the lanes one after another
            if (__ballot_sync(0xffffffffu, nz >= 0) == 0u) continue;
            const unsigned grp = __match_any_sync(0xffffffffu, nz);
            stage[warp * 32 + lane] = val;
            __syncwarp();
            if (nz >= 0 && (__ffs(grp) - 1) == lane) {
                float2 c = col[nz];
                for (unsigned m = grp; m; m &= m - 1) {
                    const float2 w = stage[warp * 32 + __ffs(m) - 1];
                    c = make_float2(c.x + w.x, c.y + w.y);
                }
                col[nz] = c;
                ccol[nz] += (uint32_t)__popc(grp);
            }
            __syncwarp();
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
    const bool fi = a.fi_theta != nullptr;
    const size_t smem = fftl::smem_bytes<L>() + sizeof(uint32_t) * P::B * L + sizeof(float2) * P::THREADS +
                        sizeof(AngleGeom) * a.A + (fi ? (sizeof(double) + sizeof(int)) * a.A : 0);
    auto k = fi ? ewald_kernel<L, true> : ewald_kernel<L, false>;
    cudaError_t e = prep_launch<L>(k, smem);
    if (e != cudaSuccess) return e;
    k<<<(unsigned)((long)L * L / P::B), P::THREADS, smem, s>>>(a, twiddles(L)); note_launch();
    return cudaGetLastError();
}

// ------------------------------------------------------------ packed measured samples
// One CTA per z-pass tile (TB consecutive x of one y, all z): the keep bits of each
// z row by a warp ballot, an exclusive prefix of the per-row counts, then the kept
// values in (z, b) order at the tile's fixed offset.
template <int TB>
__global__ void __launch_bounds__(256) pack_measured_kernel(const float2 *__restrict__ F2,
                                                           const uint8_t *__restrict__ mask, int R, uint32_t *tmask,
                                                           int *tcount, int *tprefix, float2 *tvals)
{
    extern __shared__ int spre[];   // R prefixes, then 8 warp totals
    int *swarp = spre + R;
    constexpr int ZR = 256 / TB;    // z rows per step
    const long tile = blockIdx.x;
    const long line0 = tile * TB;
    const long rr = (long)R * R;
    const int b = threadIdx.x % TB, zr = threadIdx.x / TB;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int sub = lane / TB;
    uint32_t *tm = tmask + tile * R;
    for (int z0 = 0; z0 < R; z0 += ZR) {
        const int z = z0 + zr;
        bool keep = false;
        if (z < R) {
            const long idx = line0 + b + (long)z * rr;
            if (mask) {
                keep = mask[idx] != 0;
            } else {
                const float2 f = F2[idx];
                keep = f.x != 0.0f && f.y != 0.0f;
            }
        }
        const unsigned bal = __ballot_sync(0xffffffffu, keep);
        const uint32_t m = TB == 32 ? bal : (bal >> (sub * TB)) & ((1u << TB) - 1u);
        if (b == 0 && z < R) {
            tm[z] = m;
            spre[z] = __popc(m);
        }
    }
    __syncthreads();
    // exclusive prefix of the row counts: up to 3 consecutive rows per thread
    constexpr int IT = 3;
    int own[IT], sum = 0;
#pragma unroll
    for (int k = 0; k < IT; k++) {
        const int z = threadIdx.x * IT + k;
        own[k] = z < R ? spre[z] : 0;
        sum += own[k];
    }
    int incl = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int n = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += n;
    }
    if (lane == 31) swarp[warp] = incl;
    __syncthreads();
    int before = 0;
    for (int w = 0; w < warp; w++) before += swarp[w];
    int run = before + incl - sum;
    __syncthreads();
#pragma unroll
    for (int k = 0; k < IT; k++) {
        const int z = threadIdx.x * IT + k;
        if (z < R) spre[z] = run;
        run += own[k];
    }
    if (threadIdx.x == 255) tcount[tile] = run;
    __syncthreads();
    for (int z = threadIdx.x; z < R; z += 256) tprefix[tile * R + z] = spre[z];
    float2 *tv = tvals + tile * (long)TB * R;
    const uint32_t below = (1u << b) - 1u;
    for (int z0 = 0; z0 < R; z0 += ZR) {
        const int z = z0 + zr;
        if (z >= R) continue;
        const uint32_t m = tm[z];
        if (!((m >> b) & 1u)) continue;
        tv[spre[z] + __popc(m & below)] = F2[line0 + b + (long)z * rr];
    }
}

cudaError_t pack_measured(const float2 *F2, const uint8_t *mask, int R, int TB, uint32_t *tmask, int *tcount,
                          int *tprefix, float2 *tvals, cudaStream_t s)
{
    if (R > 768) return cudaErrorInvalidValue;
    const unsigned tiles = (unsigned)((long)R * R / TB);
    const size_t smem = sizeof(int) * (R + 8);
    switch (TB) {
    case 8: pack_measured_kernel<8><<<tiles, 256, smem, s>>>(F2, mask, R, tmask, tcount, tprefix, tvals); break;
    case 16: pack_measured_kernel<16><<<tiles, 256, smem, s>>>(F2, mask, R, tmask, tcount, tprefix, tvals); break;
    case 32: pack_measured_kernel<32><<<tiles, 256, smem, s>>>(F2, mask, R, tmask, tcount, tprefix, tvals); break;
    default: return cudaErrorInvalidValue;
    }
    note_launch();
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

cudaError_t launch_ewald(const EwaldArgs &a, cudaStream_t s)
{
    CTDM_DISPATCH_R(a.R, ewald_launch, a, s)
}

}  // namespace ctdm
