// Off-axis phase retrieval, QPI Algorithm A (y-h-Lin/cTDM extractQPI_AlgorithmA,
// cTDM/HilbertTransform.cu:1546-1585, get1stOrder_new :3566-3586, calcWrapPhase
// :3618-3639, scaleFFT2D cTDM/FFT.cu:853-868).
//
// The reference transforms the whole N x N hologram, swaps quadrants, copies an
// M x M window around the carrier, swaps again and inverse-transforms.  Only the
// window's +-radius box around the carrier survives get1stOrder_new's mask, so the
// forward transform is pruned to it: a row pass computes full N-point row transforms
// (two real rows packed in one complex transform) and keeps the box's columns of
// the window; a column pass transforms those columns and keeps the window rows,
// masks to the box and writes them at their ifftshifted positions (zeros elsewhere).
// The M x M inverse transform follows: rows, skipping the rows outside the box, then
// columns with the 1/M^2 scale, conjugate and the phase/amplitude epilogue fused.
// On 1024^2 holograms with a 256 window and radius 42 the box holds 85 of the 256
// columns and rows.
#include <cmath>

#include "fft_line.cuh"
#include "kernels_front.cuh"

namespace ctdm {

using fftl::Plan;

template <int L, class K>
static cudaError_t set_smem(K kernel, size_t smem)
{
    if (!twiddles(L)) return cudaErrorInitializationError;   // device tables not built on this device
    if (smem > 48 * 1024)
        return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    return cudaSuccess;
}

// ------------------------------------------------------------ carrier search
// obtainRadius (cTDM/HilbertTransform.cu:3425-3455): argmax of |X| over rows
// j >= start of the quadrant-swapped spectrum, first maximum in raster order.
// Packed key: (bits of |X|^2) << 32 | ~(raster index) so that atomicMax picks the
// largest magnitude and, among equal ones, the smallest index.
__global__ void carrier_argmax_kernel(const float2 *__restrict__ spec, int N, int start, unsigned long long *key)
{
    unsigned long long best = 0ull;
    const long total = (long)(N - start) * N;
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total; e += (long)gridDim.x * blockDim.x) {
        const int js = start + (int)(e / N), is = (int)(e % N);
        const int iu = (is + N / 2) % N, ju = (js + N / 2) % N;
        const float2 v = spec[iu + (long)N * ju];
        const float m = v.x * v.x + v.y * v.y;
        const unsigned idx = (unsigned)(is + N * js);
        const unsigned long long k = ((unsigned long long)__float_as_uint(m) << 32) | (unsigned long long)(~idx);
        if (k > best) best = k;
    }
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long other = __shfl_xor_sync(0xffffffffu, best, o);
        if (other > best) best = other;
    }
    if ((threadIdx.x & 31) == 0) atomicMax(key, best);
}

__global__ void carrier_finish_kernel(const unsigned long long *key, int N, int *carrier)
{
    const unsigned idx = ~(unsigned)(*key & 0xffffffffull);
    const int r = (int)(idx / (unsigned)N), c = (int)(idx % (unsigned)N);
    carrier[0] = r;
    carrier[1] = c;
    carrier[2] = abs(r - N / 2) / 3;
}

__global__ void real_to_complex_kernel(const float *__restrict__ in, float2 *out, long n)
{
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        out[i] = make_float2(in[i], 0.f);
}

cudaError_t qpi_find_carrier(const float *bg, int N, float2 *scratch, unsigned long long *key, int *carrier,
                             cudaStream_t s)
{
    const long n2 = (long)N * N;
    real_to_complex_kernel<<<1024, 256, 0, s>>>(bg, scratch, n2); note_launch();
    cudaError_t e = fft_rows(scratch, N, N, false, s);
    if (e == cudaSuccess) e = fft_cols(scratch, N, N, N, 0, N, false, s);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(key, 0, sizeof(unsigned long long), s);
    if (e != cudaSuccess) return e;
    carrier_argmax_kernel<<<256, 256, 0, s>>>(scratch, N, (600 * N) / 1024, key); note_launch();
    carrier_finish_kernel<<<1, 1, 0, s>>>(key, N, carrier); note_launch();
    return cudaGetLastError();
}

// ------------------------------------------------------------ forward row pass
// holo: A holograms N x N (float, [a][y][x]); T1: A x N x M complex ([a][y][m]).
// Column m of the window is spectrum column k = (c - N/2 + m - M/2) mod N of the
// unshifted transform (the quadrant swap folded into the index).
//
// Row mapping (threads along the row pair, 16-point register tiles): every thread
// loads its first-stage points of the two packed rows straight from HBM (unit
// stride across the warp), the transform ends in registers, and the spectrum is
// parked in shared memory only for the symmetric window extraction.
template <int N>
struct QRows : fftl::Plan<N> {};
template <> struct QRows<512> : fftl::PlanT<512, 8, 32, fftl::Radices<8, 8, 8>, fftl::Radices<8, 8, 8>> {};
template <> struct QRows<1024> : fftl::PlanT<1024, 4, 64, fftl::Radices<16, 16, 4>, fftl::Radices<4, 16, 16>> {};
template <> struct QRows<2048> : fftl::PlanT<2048, 2, 128, fftl::Radices<16, 16, 8>, fftl::Radices<8, 16, 16>> {};

// Holograms arrive as float or as 16- / 8-bit camera counts (read as they are and
// converted on load, exact: every count is an integer below 2^24).  4 CTAs per SM (64
// registers, no spills) instead of the 3 that 78 registers allowed: 412 -> 399 us for
// QPI A over 121 x 1024^2 holograms.
template <int N, class T>
__global__ void __launch_bounds__(QRows<N>::THREADS, 1024 / QRows<N>::THREADS)
    qpi_rows_kernel(const T *__restrict__ holo, float2 *T1, const int *__restrict__ carrier, long npairs, int M,
                    const float2 *__restrict__ tw)
{
    using P = QRows<N>;
    using Y = fftl::Lay<N, P::LP, true>;
    extern __shared__ float4 smem4[];
    float2 *buf = reinterpret_cast<float2 *>(smem4);
    const int t = threadIdx.x % P::T, b = threadIdx.x / P::T;
    const long q = (long)blockIdx.x * P::B + b;   // pair q covers rows 2q, 2q+1 of the stack
    const bool ok = q < npairs;
    const T *r0 = holo + (ok ? 2 * q : 0) * N;
    float2 v[P::E];
#pragma unroll
    for (int i = 0; i < P::E; i++) {
        const int p = fftl::slot_pos<N, P::T, P::F0>(i, t);
        v[i] = ok ? make_float2((float)__ldcs(&r0[p]), (float)__ldcs(&r0[N + p])) : make_float2(0.f, 0.f);
    }
    P::template seq_row<false>(buf, v, tw);
    float2 *line = buf + b * Y::LINE;
    // Only the columns of the radius box survive the column pass's mask: window
    // columns m in [mlo, mhi] (|m - M/2| <= radius), spectrum columns k in
    // [kb, kb + W) mod N.  Park those points and their mirrors.
    const int c = __ldg(&carrier[1]), rad = __ldg(&carrier[2]);
    const int mlo = max(0, M / 2 - rad), mhi = min(M - 1, M / 2 + rad), W = mhi - mlo + 1;
    const int kb = (c - N / 2 - M / 2 + mlo + 2 * N) & (N - 1);
#pragma unroll
    for (int i = 0; i < P::E; i++) {
        const int k = fftl::slot_pos<N, P::T, P::RV0>(i, t);
        if (((k - kb + N) & (N - 1)) < W || ((((N - k) & (N - 1)) - kb + N) & (N - 1)) < W) line[Y::at(k)] = v[i];
    }
    __syncthreads();
    if (!ok) return;
    for (int m = mlo + t; m <= mhi; m += P::T) {
        int k = (c - N / 2 + m - M / 2) % N;
        if (k < 0) k += N;
        const float2 z1 = line[Y::at(k)];
        const float2 z2 = line[Y::at((N - k) % N)];
        // two real rows from one complex transform: Xa = (Z_k + conj Z_{N-k})/2,
        // Xb = (Z_k - conj Z_{N-k})/(2i)
        const float2 xa = make_float2(0.5f * (z1.x + z2.x), 0.5f * (z1.y - z2.y));
        const float2 xb = make_float2(0.5f * (z1.y + z2.y), -0.5f * (z1.x - z2.x));
        T1[(2 * q) * M + m] = xa;
        T1[(2 * q + 1) * M + m] = xb;
    }
}

// ------------------------------------------------------------ forward column pass
// Lines l = m + M*a, element y at T1[a*N*M + y*M + m].  Keeps window rows
// ky = (r - N/2 + j - M/2) mod N, masks to |offsets| <= radius and stores at the
// ifftshifted position of S (A x M x M).  T1 is L2-resident (one chunk of
// holograms), the first stage loads straight into registers and the spectrum is
// parked in shared memory only for the window extraction.  The row pass wrote only
// the radius box's columns: a CTA whose lines all lie outside it writes their zero
// columns and skips the transform (a line outside the box in a CTA that transforms
// reads stale T1 values and masks them).
template <int N>
struct QCols : fftl::Plan<N> {};
template <> struct QCols<1024> : fftl::PlanT<1024, 4, 64, fftl::Radices<16, 16, 4>, fftl::Radices<4, 16, 16>> {};
template <> struct QCols<2048> : fftl::PlanT<2048, 2, 128, fftl::Radices<16, 16, 8>, fftl::Radices<8, 16, 16>> {};

template <int N>
__global__ void __launch_bounds__(QCols<N>::THREADS, 1024 / QCols<N>::THREADS)
    qpi_cols_kernel(const float2 *__restrict__ T1, float2 *S, const int *__restrict__ carrier, long nlines, int M,
                    const float2 *__restrict__ tw)
{
    using P = QCols<N>;
    extern __shared__ float4 smem4[];
    float2 *buf = reinterpret_cast<float2 *>(smem4);
    const long line0 = (long)blockIdx.x * P::B;
    const int b = threadIdx.x % P::B, t = threadIdx.x / P::B;
    const long l = line0 + b;
    const bool ok = l < nlines;
    const int m = ok ? (int)(l % M) : 0;
    const long a = ok ? l / M : 0;
    const int r = carrier[0], rad = carrier[2];
    const int ox = m - M / 2;
    const int io = (m + M / 2) % M;
    float2 *dst = S + a * (long)M * M;
    bool any_in = false;   // the same for every thread of the CTA
    for (int bb = 0; bb < P::B; bb++) {
        const long lb = line0 + bb;
        any_in |= lb < nlines && abs((int)(lb % M) - M / 2) <= rad;
    }
    if (!any_in) {
        if (ok)
            for (int j = t; j < M; j += P::T) dst[(long)((j + M / 2) % M) * M + io] = make_float2(0.f, 0.f);
        return;
    }
    const float2 *src = T1 + a * (long)N * M + m;
    float2 v[P::E];
#pragma unroll
    for (int i = 0; i < P::E; i++)
        v[i] = ok ? __ldcs(&src[(long)fftl::slot_pos<N, P::T, P::F0>(i, t) * M]) : make_float2(0.f, 0.f);
    P::template seq<false, false, false>(buf, v, tw);
    float2 *line = buf + b * P::LP;
#pragma unroll
    for (int i = 0; i < P::E; i++) line[fftl::slot_pos<N, P::T, P::RV0>(i, t)] = v[i];
    __syncthreads();
    if (!ok) return;
    for (int j = t; j < M; j += P::T) {
        const int oy = j - M / 2;
        int ky = (r - N / 2 + oy) % N;
        if (ky < 0) ky += N;
        float2 vv = line[ky];
        if (abs(ox) > rad || abs(oy) > rad) vv = make_float2(0.f, 0.f);
        dst[(long)((j + M / 2) % M) * M + io] = vv;
    }
}

// ------------------------------------------------------------ inverse row pass
// Rows j' of S (ifftshifted window rows) outside the radius box, rad < j' < M - rad,
// are zero (the column pass wrote them so) and stay zero: a CTA whose rows all lie
// there returns at once.  Row mapping: the first stage loads straight from S, the
// last one stores straight back.
template <int M>
__global__ void __launch_bounds__(Plan<M>::THREADS) qpi_rows_inv_kernel(float2 *S, long nlines,
                                                                       const int *__restrict__ carrier,
                                                                       const float2 *__restrict__ tw)
{
    using P = Plan<M>;
    extern __shared__ float4 smem4[];
    float2 *buf = reinterpret_cast<float2 *>(smem4);
    const long line0 = (long)blockIdx.x * P::B;
    const int rad = __ldg(&carrier[2]);
    bool any_in = false;   // the same for every thread of the CTA
    for (int bb = 0; bb < P::B; bb++) {
        const long lb = line0 + bb;
        const int j = (int)(lb % M);
        any_in |= lb < nlines && (j <= rad || j >= M - rad);
    }
    if (!any_in) return;
    const int t = threadIdx.x % P::T, b = threadIdx.x / P::T;
    const long l = line0 + b;
    const bool ok = l < nlines;
    float2 *row = S + (ok ? l : 0) * (long)M;
    float2 v[P::E];
#pragma unroll
    for (int i = 0; i < P::E; i++)
        v[i] = ok ? __ldcs(&row[fftl::slot_pos<M, P::T, P::F0>(i, t)]) : make_float2(0.f, 0.f);
    P::template seq_row<true>(buf, v, tw);
    if (!ok) return;
#pragma unroll
    for (int i = 0; i < P::E; i++) __stcg(&row[fftl::slot_pos<M, P::T, P::RV0>(i, t)], v[i]);
}

// ------------------------------------------------------------ inverse column pass
// Lines are the M columns of each M x M spectrum (rows already inverse
// transformed; the rows outside the radius box are zero and not read).  Epilogue:
// x 1/M^2 and conjugate (scaleFFT2D), then either store the complex field
// (background) or the phase arg BG - arg SP and amplitude |SP|/|BG| with NaN/inf -> 0
// (calcWrapPhase).
template <int M>
__global__ void __launch_bounds__(Plan<M>::THREADS) qpi_final_kernel(const float2 *__restrict__ S, long nlines,
                                                                    const int *__restrict__ carrier,
                                                                    float2 *field_out, const float2 *__restrict__ bgf,
                                                                    long bg_stride, float *phase, float *amp,
                                                                    const float2 *__restrict__ tw)
{
    using P = Plan<M>;
    extern __shared__ float4 smem4[];
    float2 *buf = reinterpret_cast<float2 *>(smem4);
    const long line0 = (long)blockIdx.x * P::B;
    const int b = threadIdx.x % P::B, t = threadIdx.x / P::B;
    const long l = line0 + b;
    const bool ok = l < nlines;
    const int x = ok ? (int)(l % M) : 0;
    const long a = ok ? l / M : 0;
    const long mm = (long)M * M;
    const float2 *src = S + a * mm + x;
    const int rad = __ldg(&carrier[2]);
    for (int p = t; p < M; p += P::T)
        buf[b * P::LP + p] = ok && (p <= rad || p >= M - rad) ? src[(long)p * M] : make_float2(0.f, 0.f);
    __syncthreads();
    P::template run<true>(buf, tw);
    if (!ok) return;
    const float sc = 1.0f / (float)mm;
    for (int y = t; y < M; y += P::T) {
        const float2 raw = buf[b * P::LP + y];
        const float2 v = make_float2(raw.x * sc, -raw.y * sc);
        const long o = a * mm + x + (long)M * y;
        if (field_out) {
            field_out[o] = v;
        } else {
            const float2 g = bgf[a * bg_stride + x + (long)M * y];
            float ph = atan2f(g.y, g.x) - atan2f(v.y, v.x);
            if (isnan(ph) || isinf(ph)) ph = 0.f;
            float am = sqrtf(v.x * v.x + v.y * v.y) / sqrtf(g.x * g.x + g.y * g.y);
            if (isnan(am) || isinf(am)) am = 0.f;
            phase[o] = ph;
            amp[o] = am;
        }
    }
}

template <int N, class T>
static cudaError_t qpi_rows_launch(const T *holo, long npairs, int M, const int *carrier, float2 *T1, cudaStream_t s)
{
    using PR = QRows<N>;
    const size_t smem_r = fftl::plan_smem_row<PR>();
    cudaError_t e = set_smem<N>(qpi_rows_kernel<N, T>, smem_r);
    if (e != cudaSuccess) return e;
    qpi_rows_kernel<N, T><<<(unsigned)((npairs + PR::B - 1) / PR::B), PR::THREADS, smem_r, s>>>(holo, T1, carrier,
                                                                                              npairs, M, twiddles(N));
    note_launch();
    return cudaGetLastError();
}

template <int N>
static cudaError_t qpi_fwd_launch(const void *holo, int bpc, int A, int M, const int *carrier, float2 *T1, float2 *S,
                                  cudaStream_t s)
{
    const long npairs = (long)A * N / 2;
    cudaError_t e;
    if (bpc == 2) e = qpi_rows_launch<N>(static_cast<const uint16_t *>(holo), npairs, M, carrier, T1, s);
    else if (bpc == 1) e = qpi_rows_launch<N>(static_cast<const uint8_t *>(holo), npairs, M, carrier, T1, s);
    else e = qpi_rows_launch<N>(static_cast<const float *>(holo), npairs, M, carrier, T1, s);
    if (e != cudaSuccess) return e;
    using PC = QCols<N>;
    const long nl = (long)A * M;
    const size_t smem = fftl::plan_smem<PC>();
    e = set_smem<N>(qpi_cols_kernel<N>, smem);
    if (e != cudaSuccess) return e;
    qpi_cols_kernel<N><<<(unsigned)((nl + PC::B - 1) / PC::B), PC::THREADS, smem, s>>>(T1, S, carrier, nl, M,
                                                                                      twiddles(N)); note_launch();
    return cudaGetLastError();
}

template <int M>
static cudaError_t qpi_inv_launch(float2 *S, int A, const int *carrier, float2 *field_out, const float2 *bgf,
                                  long bg_stride, float *phase, float *amp, cudaStream_t s)
{
    using P = Plan<M>;
    const long nl = (long)A * M;
    const size_t smem_r = fftl::plan_smem_row<P>();
    cudaError_t e = set_smem<M>(qpi_rows_inv_kernel<M>, smem_r);
    if (e != cudaSuccess) return e;
    qpi_rows_inv_kernel<M><<<(unsigned)((nl + P::B - 1) / P::B), P::THREADS, smem_r, s>>>(S, nl, carrier,
                                                                                         twiddles(M)); note_launch();
    const size_t smem = fftl::smem_bytes<M>();
    e = set_smem<M>(qpi_final_kernel<M>, smem);
    if (e != cudaSuccess) return e;
    qpi_final_kernel<M><<<(unsigned)((nl + P::B - 1) / P::B), P::THREADS, smem, s>>>(S, nl, carrier, field_out, bgf,
                                                                                    bg_stride, phase, amp, twiddles(M));
    note_launch();
    return cudaGetLastError();
}

cudaError_t qpi_forward_window(const void *holo, int bpc, int A, int N, int M, const int *carrier, float2 *T1,
                               float2 *S, cudaStream_t s)
{
    CTDM_DISPATCH_L(N, qpi_fwd_launch, holo, bpc, A, M, carrier, T1, S, s)
}

cudaError_t qpi_inverse_window(float2 *S, int A, int M, const int *carrier, float2 *field_out, const float2 *bgf,
                               long bg_stride, float *phase, float *amp, cudaStream_t s)
{
    CTDM_DISPATCH_L(M, qpi_inv_launch, S, A, carrier, field_out, bgf, bg_stride, phase, amp, s)
}

// ------------------------------------------------------------ QPI Algorithm B
// extractQPI_AlgorithmB / sequence1DFFT (cTDM/HilbertTransform.cu:1587-1660): rows
// resampled N -> N/4 by the bilinear tap rule (:3658-3723; x ratio (N-1)/N, y ratio
// (N-1)/(N/4), taps past the edge read 0), an N-point transform along x per row, the
// swap of the x halves (shiftArray :1745-1758).  Frame 1 takes the carrier column
// from the column sums of |X| (HistogramFT :1727-1743, thrust::max_element over
// [int(0.6 N), N), mirrored when within N/8 of the edge); every frame keeps N/4
// columns from c - N/8 (CropFTdomain :1800-1812), swaps their halves, inverse
// transforms them (N/4 points) and stores them scaled by 1/(N/4), conjugated and
// transposed (copySharedMem :1704-1724).
//
// Row pass: two output rows packed in one complex transform (row mapping, first
// stage straight from the bilinear taps), the spectrum parked in shared memory for
// the unpacking; it either records |X| of both rows (histogram frames) or writes the
// cropped, half-swapped window rows.

__device__ __forceinline__ float qpib_tap(const float *__restrict__ h, int N, float xr, float yr, int i, int j)
{
    const int ix = (int)(xr * (float)i), iy = (int)(yr * (float)j);
    const float a = xr * (float)i - (float)ix, b = yr * (float)j - (float)iy;
    const float d00 = (ix < N && iy < N) ? __ldg(&h[(long)iy * N + ix]) : 0.f;
    const float d10 = (ix + 1 < N && iy < N) ? __ldg(&h[(long)iy * N + ix + 1]) : 0.f;
    const float d01 = (ix < N && iy + 1 < N) ? __ldg(&h[(long)(iy + 1) * N + ix]) : 0.f;
    const float d11 = (ix + 1 < N && iy + 1 < N) ? __ldg(&h[(long)(iy + 1) * N + ix + 1]) : 0.f;
    const float t1 = a * d10 + (-d00 * a + d00);
    const float t2 = a * d11 + (-d01 * a + d01);
    return b * t2 + (-t1 * b + t1);
}

// holo: A holograms N x N; pairs q cover output rows (2q, 2q+1) of the A * N/4 rows.
// mag != NULL: |X| of the shifted spectrum rows (N floats per row).  Else T gets
// the M = N/4 window columns per row, half-swapped.  center: device int.
template <int N>
__global__ void __launch_bounds__(QRows<N>::THREADS) qpib_rows_kernel(const float *__restrict__ holo, long npairs,
                                                                     float *mag, float2 *T,
                                                                     const int *__restrict__ center,
                                                                     const float2 *__restrict__ tw)
{
    using P = QRows<N>;
    using Y = fftl::Lay<N, P::LP, true>;
    constexpr int H = N / 4, M = N / 4;
    extern __shared__ float4 smem4[];
    float2 *buf = reinterpret_cast<float2 *>(smem4);
    const int t = threadIdx.x % P::T, b = threadIdx.x / P::T;
    const long q = (long)blockIdx.x * P::B + b;
    const bool ok = q < npairs;
    const long r0 = ok ? 2 * q : 0;                 // global output row (a * H + j)
    const float *h0 = holo + (r0 / H) * (long)N * N, *h1 = holo + ((r0 + 1) / H) * (long)N * N;
    const int j0 = (int)(r0 % H), j1 = (int)((r0 + 1) % H);
    const float xr = (float)(N - 1) / (float)N, yr = (float)(N - 1) / (float)H;
    float2 v[P::E];
#pragma unroll
    for (int i = 0; i < P::E; i++) {
        const int p = fftl::slot_pos<N, P::T, P::F0>(i, t);
        v[i] = ok ? make_float2(qpib_tap(h0, N, xr, yr, p, j0), qpib_tap(h1, N, xr, yr, p, j1))
                  : make_float2(0.f, 0.f);
    }
    P::template seq_row<false>(buf, v, tw);
    float2 *line = buf + b * Y::LINE;
#pragma unroll
    for (int i = 0; i < P::E; i++) line[Y::at(fftl::slot_pos<N, P::T, P::RV0>(i, t))] = v[i];
    __syncthreads();
    if (!ok) return;
    if (mag) {
        for (int x = t; x < N; x += P::T) {
            const int k = (x + N / 2) % N;          // shifted position x holds bin k
            const float2 z1 = line[Y::at(k)], z2 = line[Y::at((N - k) % N)];
            const float2 xa = make_float2(0.5f * (z1.x + z2.x), 0.5f * (z1.y - z2.y));
            const float2 xb = make_float2(0.5f * (z1.y + z2.y), -0.5f * (z1.x - z2.x));
            mag[r0 * N + x] = sqrtf(xa.x * xa.x + xa.y * xa.y);
            mag[(r0 + 1) * N + x] = sqrtf(xb.x * xb.x + xb.y * xb.y);
        }
        return;
    }
    const int c = *center;
    for (int x2 = t; x2 < M; x2 += P::T) {
        const int x = (x2 + M / 2) % M;             // half swap of the window
        const int ks = x - N / 8 + c;               // column of the shifted spectrum
        float2 xa = make_float2(0.f, 0.f), xb = make_float2(0.f, 0.f);
        if (ks >= 0 && ks < N) {
            const int k = (ks + N / 2) % N;
            const float2 z1 = line[Y::at(k)], z2 = line[Y::at((N - k) % N)];
            xa = make_float2(0.5f * (z1.x + z2.x), 0.5f * (z1.y - z2.y));
            xb = make_float2(0.5f * (z1.y + z2.y), -0.5f * (z1.x - z2.x));
        }
        T[r0 * M + x2] = xa;
        T[(r0 + 1) * M + x2] = xb;
    }
}

// Column sums of |X| over the H rows of one hologram's spectrum, in row order, and
// the first maximum over [int(0.6 N), N), mirrored to N - c when N - c < N/8.
__global__ void qpib_center_kernel(const float *__restrict__ mag, int N, int H, int *center)
{
    __shared__ unsigned long long best[32];
    unsigned long long key = 0ull;
    const int lo = (int)(N * 0.6);
    for (int i = lo + threadIdx.x; i < N; i += blockDim.x) {
        float s = 0.f;
        for (int j = 0; j < H; j++) s += mag[(long)j * N + i];
        const unsigned long long k2 = ((unsigned long long)__float_as_uint(s) << 32) | (unsigned long long)(~(unsigned)i);
        if (k2 > key) key = k2;
    }
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long other = __shfl_xor_sync(0xffffffffu, key, o);
        if (other > key) key = other;
    }
    if ((threadIdx.x & 31) == 0) best[threadIdx.x >> 5] = key;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long k = best[0];
        for (int w = 1; w < (int)(blockDim.x >> 5); w++)
            if (best[w] > k) k = best[w];
        int c = (int)(~(unsigned)(k & 0xffffffffull));
        if (N - c < (N / 4) / 2) c = N - c;
        *center = c;
    }
}

// Inverse M-point transforms of the window rows, 1/M, conjugate, transposed store:
// field[a][X * M + Y] from row Y, column X; with bgf the phase / amplitude epilogue
// of calcWrapPhase instead (cTDM/HilbertTransform.cu:3618-3639).
template <int M>
__global__ void __launch_bounds__(Plan<M>::THREADS) qpib_inv_kernel(const float2 *__restrict__ T, long nrows,
                                                                   float2 *field_out, const float2 *__restrict__ bgf,
                                                                   long bg_stride, float *phase, float *amp,
                                                                   const float2 *__restrict__ tw)
{
    using P = Plan<M>;
    extern __shared__ float4 smem4[];
    float2 *buf = reinterpret_cast<float2 *>(smem4);
    const long row0 = (long)blockIdx.x * P::B;
    for (int e = threadIdx.x; e < P::B * M; e += P::THREADS) {
        const int bb = e / M, x = e - bb * M;
        const long r = row0 + bb;
        buf[bb * P::LP + x] = r < nrows ? T[r * M + x] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    float2 v[P::E];
    P::template seq<true, true, false>(buf, v, tw);
    const int b = threadIdx.x % P::B, t = threadIdx.x / P::B;
    const long r = row0 + b;
    if (r >= nrows) return;
    const long a = r / M;
    const int yy = (int)(r % M);
    const long mm = (long)M * M;
    const float sc = 1.0f / (float)M;
#pragma unroll
    for (int i = 0; i < P::E; i++) {
        const int X = fftl::slot_pos<M, P::T, P::RV0>(i, t);
        const float2 f = make_float2(v[i].x * sc, -v[i].y * sc);
        const long o = a * mm + (long)X * M + yy;
        if (field_out) {
            field_out[o] = f;
        } else {
            const float2 g = bgf[a * bg_stride + (long)X * M + yy];
            float ph = atan2f(g.y, g.x) - atan2f(f.y, f.x);
            if (isnan(ph) || isinf(ph)) ph = 0.f;
            float am = sqrtf(f.x * f.x + f.y * f.y) / sqrtf(g.x * g.x + g.y * g.y);
            if (isnan(am) || isinf(am)) am = 0.f;
            phase[o] = ph;
            amp[o] = am;
        }
    }
}

template <int N>
static cudaError_t qpib_rows_launch(const float *holo, int A, float *mag, float2 *T, const int *center, cudaStream_t s)
{
    using PR = QRows<N>;
    if constexpr (N < 64) {
        return cudaErrorInvalidValue;
    } else {
        const size_t smem = fftl::plan_smem_row<PR>();
        const long npairs = (long)A * (N / 4) / 2;
        cudaError_t e = set_smem<N>(qpib_rows_kernel<N>, smem);
        if (e != cudaSuccess) return e;
        qpib_rows_kernel<N><<<(unsigned)((npairs + PR::B - 1) / PR::B), PR::THREADS, smem, s>>>(holo, npairs, mag, T,
                                                                                              center, twiddles(N));
        note_launch();
        return cudaGetLastError();
    }
}

template <int M>
static cudaError_t qpib_inv_launch(const float2 *T, int A, float2 *field_out, const float2 *bgf, long bg_stride,
                                   float *phase, float *amp, cudaStream_t s)
{
    using P = Plan<M>;
    const size_t smem = fftl::smem_bytes<M>();
    cudaError_t e = set_smem<M>(qpib_inv_kernel<M>, smem);
    if (e != cudaSuccess) return e;
    const long nrows = (long)A * M;
    qpib_inv_kernel<M><<<(unsigned)((nrows + P::B - 1) / P::B), P::THREADS, smem, s>>>(T, nrows, field_out, bgf,
                                                                                      bg_stride, phase, amp,
                                                                                      twiddles(M));
    note_launch();
    return cudaGetLastError();
}

// ------------------------------------------------------------ angle camera (AngCal_GPU)
// AngCal_GPU (cTDM/HilbertTransform.cu:2920-2983): forward 2-D transform of the
// angle-camera image, quadrant swap, log10 |X| with NaN/inf -> 0 (cufftComplex2Real
// :2986-2996), first maximum over the flattened range [int(0.53 N^2), int(0.79 N^2)).
// spec: the transformed image (N x N complex, unshifted).  pos: device int (index).
__device__ __forceinline__ unsigned order_key(float v)
{
    const unsigned u = __float_as_uint(v);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);   // unsigned order = float order
}

__global__ void angcal_argmax_kernel(const float2 *__restrict__ spec, int N, long lo, long hi, unsigned long long *key)
{
    unsigned long long best = 0ull;
    for (long e = lo + blockIdx.x * (long)blockDim.x + threadIdx.x; e < hi; e += (long)gridDim.x * blockDim.x) {
        const int xs = (int)(e % N), ys = (int)(e / N);
        const float2 v = spec[(long)((xs + N / 2) % N) + (long)N * ((ys + N / 2) % N)];
        float m = log10f(sqrtf(v.x * v.x + v.y * v.y));
        if (isnan(m) || isinf(m)) m = 0.f;
        const unsigned long long k = ((unsigned long long)order_key(m) << 32) | (unsigned long long)(~(unsigned)e);
        if (k > best) best = k;
    }
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long other = __shfl_xor_sync(0xffffffffu, best, o);
        if (other > best) best = other;
    }
    if ((threadIdx.x & 31) == 0) atomicMax(key, best);
}

cudaError_t angcal_peak(const float *img, int N, float2 *scratch, unsigned long long *key, cudaStream_t s)
{
    const long n2 = (long)N * N;
    real_to_complex_kernel<<<1024, 256, 0, s>>>(img, scratch, n2); note_launch();
    cudaError_t e = fft_rows(scratch, N, N, false, s);
    if (e == cudaSuccess) e = fft_cols(scratch, N, N, N, 0, N, false, s);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(key, 0, sizeof(unsigned long long), s);
    if (e != cudaSuccess) return e;
    angcal_argmax_kernel<<<256, 256, 0, s>>>(scratch, N, (long)(n2 * 0.53), (long)(n2 * 0.79), key); note_launch();
    return cudaGetLastError();
}

cudaError_t qpib_spectrum_center(const float *holo, int N, float *mag, int *center, cudaStream_t s)
{
    cudaError_t e;
    switch (N) {
    case 64: e = qpib_rows_launch<64>(holo, 1, mag, nullptr, nullptr, s); break;
    case 128: e = qpib_rows_launch<128>(holo, 1, mag, nullptr, nullptr, s); break;
    case 256: e = qpib_rows_launch<256>(holo, 1, mag, nullptr, nullptr, s); break;
    case 512: e = qpib_rows_launch<512>(holo, 1, mag, nullptr, nullptr, s); break;
    case 1024: e = qpib_rows_launch<1024>(holo, 1, mag, nullptr, nullptr, s); break;
    case 2048: e = qpib_rows_launch<2048>(holo, 1, mag, nullptr, nullptr, s); break;
    default: return cudaErrorInvalidValue;
    }
    if (e != cudaSuccess) return e;
    qpib_center_kernel<<<1, 1024, 0, s>>>(mag, N, N / 4, center);
    note_launch();
    return cudaGetLastError();
}

cudaError_t qpib_window(const float *holo, int A, int N, const int *center, float2 *T, cudaStream_t s)
{
    CTDM_DISPATCH_L(N, qpib_rows_launch, holo, A, nullptr, T, center, s)
}

cudaError_t qpib_inverse(const float2 *T, int A, int M, float2 *field_out, const float2 *bgf, long bg_stride,
                         float *phase, float *amp, cudaStream_t s)
{
    CTDM_DISPATCH_L(M, qpib_inv_launch, T, A, field_out, bgf, bg_stride, phase, amp, s)
}

}  // namespace ctdm

namespace ctdm {
__global__ void set_carrier_kernel(int *carrier, int r, int c, int rad)
{
    carrier[0] = r;
    carrier[1] = c;
    carrier[2] = rad;
}

cudaError_t set_carrier(int *carrier, int r, int c, int rad, cudaStream_t s)
{
    set_carrier_kernel<<<1, 1, 0, s>>>(carrier, r, c, rad); note_launch();
    return cudaGetLastError();
}
}  // namespace ctdm
