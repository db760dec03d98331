// Least-squares phase unwrapping by a DCT Poisson solve
// (y-h-Lin/cTDM DCT_UWLS_Unwrapped, cTDM/DCT_Unwrapping.cu:10-59).
//
// The reference runs 14 launches and 4 cuFFT calls per map: wrapped
// derivatives (NumericDerivative1 :336), divergence (SumDerivative :394), a
// row DCT-II through a 2M-point FFT of the mirrored row (float2cufft :144,
// countFDCT :202), a transpose (:179), the same for columns, the Poisson divide
// (devConstant :300) and the inverse (countIDCT :218, cufft2float :164) twice.
// Here it is three line passes:
//   rows:    wrapped Laplacian (fused load) -> mirror -> FFT_2M -> DCT-II
//   columns: mirror -> FFT_2M -> DCT-II -> divide -> IDCT build -> IFFT_2M
//   rows:    IDCT build -> IFFT_2M -> real part
// The inverse keeps the reference's twiddle on the mirrored half ((i+1) pi/2M,
// mode 0) or uses the exact DCT-III (i pi/2M, mode 1).
#include <cmath>

#include "fft_line.cuh"
#include "kernels_front.cuh"

namespace ctdm {

using fftl::Plan;

// Line plan of the three passes: 256 threads per CTA and at most 16 points per
// thread, so that four CTAs fit on an SM.  The passes are latency-bound (a few
// loads and a transform per line between barriers), and at 512 points moving from
// 16 lines x 16 threads at 128 registers (2 CTAs per SM) to 8 lines x 32 threads
// at 64 registers (4 CTAs) cut the three passes from 369 to 219 us on 121 maps
// of 256 x 256.
template <int L2>
struct DctPlan : Plan<L2> {};
template <>
struct DctPlan<512> : fftl::PV<512, 2> {};
template <>
struct DctPlan<768> : fftl::PV<768, 1> {};
template <>
struct DctPlan<1024> : fftl::PlanT<1024, 4, 64, fftl::Radices<16, 16, 4>, fftl::Radices<4, 16, 16>> {};

// Resident CTAs per SM the register allocation aims for.
template <class P>
__host__ __device__ constexpr int dct_min_ctas()
{
    return P::E <= 16 ? 1024 / P::THREADS : (P::E <= 24 ? 768 / P::THREADS : 512 / P::THREADS);
}

// NumericDerivative1 wrap: t - 2 pi sign(t) floor(|pi sign(t) + t| / 2 pi), which
// the reference evaluates in double; it is exactly t when |t| < pi.  For a wrapped
// difference (|t| < 4 pi, so the floor q is 0, 1 or 2) the float form
// |t| - q fl(2 pi) is exact (Sterbenz) and subtracting q (2 pi - fl(2 pi)) rounds
// once, which is the double expression's value; the double expression itself runs
// only where q is in doubt (the quotient within 1e-5 of an integer).  GB300's FP64
// rate made the double form the most expensive part of the row pass.
__device__ __forceinline__ float wrap_grad(float t)
{
    if (fabsf(t) < 3.14159f) return t;
    const float u = fabsf(t);
    const float v = (u + (float)CTDM_PI_D) * (float)(0.5 / CTDM_PI_D);
    const float qf = floorf(v), f = v - qf;
    if (u < 15.0f && f > 1e-5f && f < 1.0f - 1e-5f) {
        const float p1 = (float)(2 * CTDM_PI_D);
        const float p2 = (float)(2 * CTDM_PI_D - (double)(float)(2 * CTDM_PI_D));
        const float r = (u - qf * p1) - qf * p2;
        return t < 0.f ? -r : r;
    }
    const double s = t > 0.f ? 1.0 : (t < 0.f ? -1.0 : 0.0);
    const double td = (double)t;
    const double q = floor(fabs(__dadd_rn(CTDM_PI_D * s, td)) / (CTDM_PI_D * 2));
    return (float)__dsub_rn(td, 2 * CTDM_PI_D * s * q);
}

__device__ __forceinline__ float lap_at(const float *__restrict__ phi, int x, int y, int M)
{
    const long i = x + (long)M * y;
    const float c = phi[i];
    // SumDerivative (:394-417): (gx(x) - gx(x-1)) + (gy(y) - gy(y-1)) with zero edges
    const float c1 = (x == M - 1) ? 0.f : wrap_grad(phi[i + 1] - c);
    float c2 = 0.f;
    if (x > 0) {
        const float l = phi[i - 1];
        c2 = wrap_grad(c - l);
    }
    const float c3 = (y == M - 1) ? 0.f : wrap_grad(phi[i + M] - c);
    float c4 = 0.f;
    if (y > 0) {
        const float u = phi[i - M];
        c4 = wrap_grad(c - u);
    }
    return (c1 - c2) + (c3 - c4);
}

// lap_at on staged rows: r points at row y, rows y - 1 and y + 1 lie M before and after.
__device__ __forceinline__ float lap_rows(const float *r, int x, int y, int M)
{
    const float c = r[x];
    const float c1 = (x == M - 1) ? 0.f : wrap_grad(r[x + 1] - c);
    const float c2 = (x > 0) ? wrap_grad(c - r[x - 1]) : 0.f;
    const float c3 = (y == M - 1) ? 0.f : wrap_grad(r[x + M] - c);
    const float c4 = (y > 0) ? wrap_grad(c - r[x - M]) : 0.f;
    return (c1 - c2) + (c3 - c4);
}

// countFDCT (:202-216): X_k from the 2M-point transform Y of the mirrored line.
__device__ __forceinline__ float dct_from_fft(float2 Y, int k, const float2 *__restrict__ dtw, float dT)
{
    if (k == 0) return Y.x * dT * 0.70710678118654752440f;
    const float2 w = __ldg(&dtw[k]);
    return (Y.x * w.x + Y.y * w.y) * dT;
}

// countIDCT (:218-246) element p of the 2M-point input built from X[0..M).
__device__ __forceinline__ float2 idct_input(const float *X, int p, int M, const float2 *__restrict__ dtw, float dT,
                                             int mode)
{
    if (p < M) {
        const float2 w = __ldg(&dtw[p]);
        float v = X[p] * dT;
        float2 r = make_float2(w.x * v, w.y * v);
        if (p == 0) r = make_float2(r.x * 1.41421356237309504880f, r.y * 1.41421356237309504880f);
        return r;
    }
    const int i = p - M;
    if (i == 0) return make_float2(0.f, 0.f);
    const float2 w = __ldg(&dtw[mode == 0 ? i + 1 : i]);
    const float v2 = X[M - i] * dT;
    return make_float2(w.y * v2, -w.x * v2);
}

// Two real lines per complex transform.  Every line of the three passes is real (the
// mirrored rows and columns of the forward transforms) or has only its real part kept
// (the inverse transforms), so a CTA of the plan's B complex lines covers 2B real
// lines, line 2b in the real and line 2b + 1 in the imaginary part of complex line b.
// Forward: Z = FFT(z_a + i z_b) gives Y_a[k] = (Z[k] + conj Z[-k]) / 2 and
// Y_b[k] = (Z[k] - conj Z[-k]) / 2i.  Inverse: the reference keeps Re IFFT(V) of the
// countIDCT input V, and Re IFFT(V) = IFFT(H) with H[p] = (V[p] + conj V[-p]) / 2
// (Hermitian, so its transform is real); IFFT(H_a + i H_b) = x_a + i x_b.  Half the
// transforms of the one-line-per-transform form, the same results up to float rounding.
template <int L2>
__host__ __device__ constexpr int dct_lines_per_cta()
{
    return 2 * DctPlan<L2>::B;
}

// Y_a, Y_b of the two real lines packed in complex line `line` (length L2, stride 1).
__device__ __forceinline__ void unpack_pair(const float2 *line, int k, int L2, float2 &ya, float2 &yb)
{
    const float2 z = line[k];
    const float2 r = line[k == 0 ? 0 : L2 - k];   // Z[-k]
    ya = make_float2(0.5f * (z.x + r.x), 0.5f * (z.y - r.y));
    yb = make_float2(0.5f * (z.y + r.y), -0.5f * (z.x - r.x));
}

// H_a + i H_b at point p of the inverse input of the two coefficient rows Xa, Xb.
__device__ __forceinline__ float2 idct_pair_input(const float *Xa, const float *Xb, int p, int M,
                                                  const float2 *__restrict__ dtw, float dT, int mode)
{
    const int q = p == 0 ? 0 : 2 * M - p;
    const float2 a0 = idct_input(Xa, p, M, dtw, dT, mode), a1 = idct_input(Xa, q, M, dtw, dT, mode);
    const float2 b0 = idct_input(Xb, p, M, dtw, dT, mode), b1 = idct_input(Xb, q, M, dtw, dT, mode);
    const float2 ha = make_float2(0.5f * (a0.x + a1.x), 0.5f * (a0.y - a1.y));
    const float2 hb = make_float2(0.5f * (b0.x + b1.x), 0.5f * (b0.y - b1.y));
    return make_float2(ha.x - hb.y, ha.y + hb.x);
}

// Pass 1: rows.  phi: A x M x M; T: A x M x M (row DCT coefficients, [a][y][kx]).
template <int L2>
__global__ void __launch_bounds__(DctPlan<L2>::THREADS, dct_min_ctas<DctPlan<L2>>())
    dct_rows_kernel(const float *__restrict__ phi, float *T, long nlines, int /* M = L2 / 2 */,
                    const float2 *__restrict__ dtw, const float2 *__restrict__ tw)
{
    using P = DctPlan<L2>;
    constexpr int M = L2 / 2, RL = dct_lines_per_cta<L2>();
    extern __shared__ float4 smem4[];
    float2 *buf = reinterpret_cast<float2 *>(smem4);
    const long line0 = (long)blockIdx.x * RL;
    // map and row of the CTA's first line; a line j further on is y0 + j rows later
    const long a0 = line0 / M;
    const int y0 = (int)(line0 - a0 * M);
    if constexpr (RL <= M) {
        // RL divides M, so the CTA's lines are rows y0 .. y0 + RL - 1 of one map: rows
        // y0 - 1 .. y0 + RL are staged in shared memory by independent coalesced loads
        // (a thread's loads are all in flight together), and the Laplacian is taken
        // from there.  The staging fits in the line buffer: (RL + 2) M floats <= 4 B M.
        constexpr int SR = RL + 2, NS = (SR * M + P::THREADS - 1) / P::THREADS, PER = M / P::T;
        float *S = reinterpret_cast<float *>(buf);
        const float *map = phi + a0 * (long)M * M;
        const bool live = line0 < nlines;
#pragma unroll
        for (int k = 0; k < NS; ++k) {
            const int e = threadIdx.x + k * P::THREADS;
            if (e < SR * M) {
                const int y = y0 - 1 + e / M;
                S[e] = (live && y >= 0 && y < M) ? __ldg(map + (long)y0 * M - M + e) : 0.f;
            }
        }
        __syncthreads();
        float2 v[PER];
#pragma unroll
        for (int k = 0; k < PER; ++k) {
            const int e = threadIdx.x + k * P::THREADS;
            const int b = e / M, x = e - b * M;
            v[k] = make_float2(lap_rows(S + (2 * b + 1) * M, x, y0 + 2 * b, M),
                               lap_rows(S + (2 * b + 2) * M, x, y0 + 2 * b + 1, M));
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < PER; ++k) {
            const int e = threadIdx.x + k * P::THREADS;
            const int b = e / M, x = e - b * M;
            buf[b * P::LP + x] = v[k];
            buf[b * P::LP + (L2 - 1 - x)] = v[k];
        }
    } else {
        // maps smaller than RL lines: the CTA covers several maps
        for (int e = threadIdx.x; e < P::B * M; e += P::THREADS) {
            const int b = e / M, x = e - b * M;
            float v[2];
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const long l = line0 + 2 * b + h;
                v[h] = 0.f;
                if (l < nlines) {
                    int y = y0 + 2 * b + h;
                    long a = a0;
                    while (y >= M) {
                        y -= M;
                        a++;
                    }
                    v[h] = lap_at(phi + a * (long)M * M, x, y, M);
                }
            }
            buf[b * P::LP + x] = make_float2(v[0], v[1]);
            buf[b * P::LP + (L2 - 1 - x)] = make_float2(v[0], v[1]);
        }
    }
    __syncthreads();
    P::template run<false>(buf, tw);
    const float dT = 1.0f / sqrtf((float)L2);
    for (int e = threadIdx.x; e < P::B * M; e += P::THREADS) {
        const int b = e / M, k = e - b * M;
        const long l = line0 + 2 * b;   // nlines is even: l < nlines covers both lines
        if (l < nlines) {
            float2 ya, yb;
            unpack_pair(buf + b * P::LP, k, L2, ya, yb);
            T[l * M + k] = dct_from_fft(ya, k, dtw, dT);
            T[(l + 1) * M + k] = dct_from_fft(yb, k, dtw, dT);
        }
    }
}

// Row stride of the column pass's coefficient staging (2B rows, rows 2b and 2b + 1 for
// complex line b): a warp holds min(B, 32) complex lines at 32 / B consecutive
// positions each, so rows 2b need 2 x stride = 32 / B (mod 32), a stride of M (a
// multiple of 16) plus 16 / B, to fall on distinct banks.
template <int L2>
__host__ __device__ constexpr int x_stride(int M)
{
    return M + (DctPlan<L2>::B >= 16 ? 1 : 16 / DctPlan<L2>::B);
}

// Pass 2: columns.  Real line l = kx + M*a, element y at T[a*M*M + y*M + kx]; complex
// line b holds columns kx, kx + 1 (kx even), read and written as float2.
template <int L2>
__global__ void __launch_bounds__(DctPlan<L2>::THREADS, dct_min_ctas<DctPlan<L2>>())
    dct_cols_kernel(float *T, long nlines, int /* M = L2 / 2 */, int mode, const float2 *__restrict__ dtw,
                    const float *__restrict__ eig, const float2 *__restrict__ tw)
{
    using P = DctPlan<L2>;
    constexpr int M = L2 / 2, RL = dct_lines_per_cta<L2>();
    extern __shared__ float4 smem4[];
    float2 *buf = reinterpret_cast<float2 *>(smem4);
    float *X = reinterpret_cast<float *>(buf + P::B * P::LP);   // 2B rows of x_stride(M)
    const long line0 = (long)blockIdx.x * RL;
    const int b = threadIdx.x % P::B, t = threadIdx.x / P::B;
    float *Xa = X + (2 * b) * x_stride<L2>(M), *Xb = Xa + x_stride<L2>(M);
    const long l = line0 + 2 * b;   // nlines is even: l < nlines covers both lines
    const bool ok = l < nlines;
    const int kx = ok ? (int)(l % M) : 0;
    const long a = ok ? l / M : 0;
    float2 *col = reinterpret_cast<float2 *>(T + a * (long)M * M + kx);   // kx even: 8-byte aligned
    for (int y = t; y < M; y += P::T) {
        const float2 v = ok ? col[(long)y * (M / 2)] : make_float2(0.f, 0.f);
        buf[b * P::LP + y] = v;
        buf[b * P::LP + (L2 - 1 - y)] = v;
    }
    __syncthreads();
    P::template run<false>(buf, tw);
    const float dT = 1.0f / sqrtf((float)L2);
    const float exa = __ldg(&eig[kx]), exb = __ldg(&eig[kx + 1]);
    for (int ky = t; ky < M; ky += P::T) {
        float2 ya, yb;
        unpack_pair(buf + b * P::LP, ky, L2, ya, yb);
        float va = dct_from_fft(ya, ky, dtw, dT), vb = dct_from_fft(yb, ky, dtw, dT);
        // devConstant (:300-311): / (2cos(4 pi i/(4M-1)) + 2cos(4 pi j/(4M-1)) - 4), (0,0) -> 0;
        // the denominator is -(4 sin^2(2 pi i/(4M-1)) + 4 sin^2(2 pi j/(4M-1))), free of cancellation
        const float ey = __ldg(&eig[ky]);
        if (kx == 0 && ky == 0) va = 0.f;
        else va = va / (-(exa + ey));
        vb = vb / (-(exb + ey));
        Xa[ky] = va;
        Xb[ky] = vb;
    }
    __syncthreads();
    for (int p = t; p < L2; p += P::T) buf[b * P::LP + p] = idct_pair_input(Xa, Xb, p, M, dtw, dT, mode);
    __syncthreads();
    P::template run<true>(buf, tw);
    if (!ok) return;
    for (int y = t; y < M; y += P::T) col[(long)y * (M / 2)] = buf[b * P::LP + y];
}

// Pass 3: rows inverse.  T: [a][y][kx] -> out [a][y][x].
template <int L2>
__global__ void __launch_bounds__(DctPlan<L2>::THREADS, dct_min_ctas<DctPlan<L2>>())
    dct_rows_inv_kernel(const float *__restrict__ T, float *out, long nlines, int /* M = L2 / 2 */, int mode,
                        const float2 *__restrict__ dtw, const float2 *__restrict__ tw)
{
    using P = DctPlan<L2>;
    constexpr int M = L2 / 2, RL = dct_lines_per_cta<L2>();
    extern __shared__ float4 smem4[];
    float2 *buf = reinterpret_cast<float2 *>(smem4);
    float *X = reinterpret_cast<float *>(buf + P::B * P::LP);   // 2B rows of M
    const long line0 = (long)blockIdx.x * RL;
    for (int e = threadIdx.x; e < RL * M; e += P::THREADS) {
        const int j = e / M, k = e - j * M;
        const long l = line0 + j;
        X[j * M + k] = (l < nlines) ? T[l * M + k] : 0.f;
    }
    __syncthreads();
    const float dT = 1.0f / sqrtf((float)L2);
    for (int e = threadIdx.x; e < P::B * L2; e += P::THREADS) {
        const int b = e / L2, p = e - b * L2;
        buf[b * P::LP + p] = idct_pair_input(X + (2 * b) * M, X + (2 * b + 1) * M, p, M, dtw, dT, mode);
    }
    __syncthreads();
    P::template run<true>(buf, tw);
    for (int e = threadIdx.x; e < P::B * M; e += P::THREADS) {
        const int b = e / M, x = e - b * M;
        const long l = line0 + 2 * b;
        if (l < nlines) {
            const float2 o = buf[b * P::LP + x];
            out[l * M + x] = o.x;
            out[(l + 1) * M + x] = o.y;
        }
    }
}

template <int L2, class K>
static cudaError_t set_smem2(K kernel, size_t smem)
{
    if (smem > 48 * 1024)
        return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    return cudaSuccess;
}

template <int L2>
static cudaError_t dct_launch(const float *phi, float *out, float *T, int A, int M, int mode, cudaStream_t s)
{
    using P = DctPlan<L2>;
    const long nl = (long)A * M;
    constexpr int RL = dct_lines_per_cta<L2>();
    const unsigned grid = (unsigned)((nl + RL - 1) / RL);
    const size_t smem1 = fftl::plan_smem<P>();
    const size_t smem2 = smem1 + sizeof(float) * RL * x_stride<L2>(M);
    const float2 *dtw = dct_twiddles(M);
    const float2 *tw = twiddles(L2);
    if (!dtw || !tw || !dct_eigen(M)) return cudaErrorInitializationError;   // device tables not built
    cudaError_t e = set_smem2<L2>(dct_rows_kernel<L2>, smem1);
    if (e != cudaSuccess) return e;
    dct_rows_kernel<L2><<<grid, P::THREADS, smem1, s>>>(phi, T, nl, M, dtw, tw); note_launch();
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    e = set_smem2<L2>(dct_cols_kernel<L2>, smem2);
    if (e != cudaSuccess) return e;
    dct_cols_kernel<L2><<<grid, P::THREADS, smem2, s>>>(T, nl, M, mode, dtw, dct_eigen(M), tw); note_launch();
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    e = set_smem2<L2>(dct_rows_inv_kernel<L2>, smem2);
    if (e != cudaSuccess) return e;
    dct_rows_inv_kernel<L2><<<grid, P::THREADS, smem2, s>>>(T, out, nl, M, mode, dtw, tw); note_launch();
    return cudaGetLastError();
}

cudaError_t dct_unwrap(const float *phi, float *out, float *T, int A, int M, int mode, cudaStream_t s)
{
    CTDM_DISPATCH_L(2 * M, dct_launch, phi, out, T, A, M, mode, s)
}

}  // namespace ctdm

namespace ctdm {

// The same three passes with caller-supplied tables and scratch (no lookups in
// the per-device table registry).
template <int L2>
static cudaError_t dct_launch_explicit(const float *phi, float *out, float *T, int A, int M, int mode,
                                       const float2 *tw, const float2 *dtw, const float *eig, cudaStream_t s)
{
    using P = DctPlan<L2>;
    const long nl = (long)A * M;
    constexpr int RL = dct_lines_per_cta<L2>();
    const unsigned grid = (unsigned)((nl + RL - 1) / RL);
    const size_t smem1 = fftl::plan_smem<P>();
    const size_t smem2 = smem1 + sizeof(float) * RL * x_stride<L2>(M);
    cudaError_t e = set_smem2<L2>(dct_rows_kernel<L2>, smem1);
    if (e != cudaSuccess) return e;
    dct_rows_kernel<L2><<<grid, P::THREADS, smem1, s>>>(phi, T, nl, M, dtw, tw); note_launch();
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    e = set_smem2<L2>(dct_cols_kernel<L2>, smem2);
    if (e != cudaSuccess) return e;
    dct_cols_kernel<L2><<<grid, P::THREADS, smem2, s>>>(T, nl, M, mode, dtw, eig, tw); note_launch();
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    e = set_smem2<L2>(dct_rows_inv_kernel<L2>, smem2);
    if (e != cudaSuccess) return e;
    dct_rows_inv_kernel<L2><<<grid, P::THREADS, smem2, s>>>(T, out, nl, M, mode, dtw, tw); note_launch();
    return cudaGetLastError();
}

cudaError_t dct_unwrap_explicit(const float *phi, float *out, float *T, int A, int M, int mode, const float2 *tw,
                                const float2 *dtw, const float *eig, cudaStream_t s)
{
    CTDM_DISPATCH_L(2 * M, dct_launch_explicit, phi, out, T, A, M, mode, tw, dtw, eig, s)
}

}  // namespace ctdm
