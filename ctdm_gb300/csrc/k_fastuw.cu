// FFT-based least-squares unwrapping (y-h-Lin/cTDM FastUnwrapping,
// cTDM/FastUnwrapping.cu:5-117).  The Laplacian of the true phase is formed
// from sin/cos of the wrapped phase, cos L(sin) - sin L(cos), on the mirrored
// 2M x 2M extension, inverted by a division by k^2 in the Fourier domain, and
// the wrapped phase is moved by the nearest multiple of 2 pi onto it.  The
// reference's plans are (M/2)^2 for (2M)^2 arrays; the intended (2M)^2
// transform is used.  sin and cos are transformed together as sin + i cos:
// k^2 is even, so the inverse gives L(sin) + i L(cos).
#include <cfloat>
#include <cmath>

#include "kernels_front.cuh"

namespace ctdm {

// PhaseNormalize (:119-130): per-map min/max, then 2 pi (x - min)/(max - min).
__global__ void normalize_kernel(float *phi, int M, float *minmax)
{
    const long n = (long)M * M;
    float *p = phi + blockIdx.x * n;
    float lo = FLT_MAX, hi = -FLT_MAX;
    for (long i = threadIdx.x; i < n; i += blockDim.x) {
        lo = fminf(lo, p[i]);
        hi = fmaxf(hi, p[i]);
    }
    __shared__ float slo[32], shi[32];
    for (int o = 16; o > 0; o >>= 1) {
        lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    if ((threadIdx.x & 31) == 0) { slo[threadIdx.x >> 5] = lo; shi[threadIdx.x >> 5] = hi; }
    __syncthreads();
    if (threadIdx.x < 32) {
        const int nw = blockDim.x >> 5;
        lo = threadIdx.x < nw ? slo[threadIdx.x] : FLT_MAX;
        hi = threadIdx.x < nw ? shi[threadIdx.x] : -FLT_MAX;
        for (int o = 16; o > 0; o >>= 1) {
            lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
            hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
        }
        if (threadIdx.x == 0) { slo[0] = lo; shi[0] = hi; }
    }
    __syncthreads();
    lo = slo[0];
    hi = shi[0];
    if (minmax && threadIdx.x == 0) { minmax[2 * blockIdx.x] = lo; minmax[2 * blockIdx.x + 1] = hi; }
    for (long i = threadIdx.x; i < n; i += blockDim.x)
        p[i] = (float)(2 * CTDM_PI_D * (double)(p[i] - lo) / (double)(hi - lo));
}

// makeSimmetric (:144-169) into one complex array: sin + i cos, mirrored.
__global__ void mirror_sincos_kernel(const float *__restrict__ phi, float2 *W, int M)
{
    const int a = blockIdx.z;
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= M || j >= M) return;
    const int M2 = 2 * M;
    float s, c;
    sincosf(phi[a * (long)M * M + i + (long)M * j], &s, &c);
    float2 *w = W + a * (long)M2 * M2;
    const float2 v = make_float2(s, c);
    w[i + (long)M2 * j] = v;
    w[(M2 - 1 - i) + (long)M2 * j] = v;
    w[i + (long)M2 * (M2 - 1 - j)] = v;
    w[(M2 - 1 - i) + (long)M2 * (M2 - 1 - j)] = v;
}

// k^2 of the signed frequency (MultiplyPosition :263-279 / MultiplyInvPosition :281-306)
template <bool INV>
__global__ void k2_kernel(float2 *W, int M2, long total)
{
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total; e += (long)gridDim.x * blockDim.x) {
        const long q = e % ((long)M2 * M2);
        const int i = (int)(q % M2), j = (int)(q / M2);
        const int fi = i < M2 / 2 ? i : i - M2, fj = j < M2 / 2 ? j : j - M2;
        const float con = (float)(fi * fi + fj * fj);
        float2 v = W[e];
        if (INV) v = con == 0.f ? make_float2(0.f, 0.f) : make_float2(v.x / con, v.y / con);
        else v = make_float2(v.x * con, v.y * con);
        W[e] = v;
    }
}

// cos L(sin) - sin L(cos) (MultiplyComplex + SubtractComplex), real.
__global__ void combine_kernel(float2 *W, const float *__restrict__ phi, int M, float scale)
{
    const int a = blockIdx.z;
    const int M2 = 2 * M;
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= M2 || j >= M2) return;
    const int si = i < M ? i : M2 - 1 - i, sj = j < M ? j : M2 - 1 - j;
    float s, c;
    sincosf(phi[a * (long)M * M + si + (long)M * sj], &s, &c);
    float2 *w = W + a * (long)M2 * M2;
    const float2 v = w[i + (long)M2 * j];
    w[i + (long)M2 * j] = make_float2((c * v.x - s * v.y) * scale, 0.f);
}

// ObtainUnwrap (:333-345): phi + 2 pi round((phi_LS - phi) / 2 pi).
__global__ void obtain_kernel(const float2 *__restrict__ W, const float *__restrict__ phi, float *out, int M, float scale)
{
    const int a = blockIdx.z;
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= M || j >= M) return;
    const int M2 = 2 * M;
    const float cont = W[a * (long)M2 * M2 + i + (long)M2 * j].x * scale;
    const long o = a * (long)M * M + i + (long)M * j;
    const float src = phi[o];
    out[o] = src + 2.0f * CTDM_PI_F * roundf((cont - src) * (0.5f / CTDM_PI_F));
}

// subtractMin (:347-359)
__global__ void submin_kernel(float *out, int M)
{
    const long n = (long)M * M;
    float *p = out + blockIdx.x * n;
    float lo = FLT_MAX;
    for (long i = threadIdx.x; i < n; i += blockDim.x) lo = fminf(lo, p[i]);
    __shared__ float sl[32];
    for (int o = 16; o > 0; o >>= 1) lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    if ((threadIdx.x & 31) == 0) sl[threadIdx.x >> 5] = lo;
    __syncthreads();
    if (threadIdx.x < 32) {
        lo = threadIdx.x < (int)(blockDim.x >> 5) ? sl[threadIdx.x] : FLT_MAX;
        for (int o = 16; o > 0; o >>= 1) lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        if (threadIdx.x == 0) sl[0] = lo;
    }
    __syncthreads();
    lo = sl[0];
    for (long i = threadIdx.x; i < n; i += blockDim.x) p[i] -= lo;
}

static cudaError_t fft2_batch(float2 *W, int L, int A, bool inv, cudaStream_t s)
{
    cudaError_t e = fft_rows(W, L, (long)A * L, inv, s);
    if (e == cudaSuccess) e = fft_cols(W, L, (long)A * L, L, (long)L * L, L, inv, s);
    return e;
}

// work: 4*M*M complex per map (processed one map at a time beyond that).
cudaError_t fast_unwrap(float *phi, float *out, float2 *work, int A, int M, cudaStream_t s)
{
    const int M2 = 2 * M;
    const long n2 = (long)M2 * M2;
    const float sc = 1.0f / (float)n2;
    normalize_kernel<<<A, 512, 0, s>>>(phi, M, nullptr); note_launch();
    cudaError_t e = cudaGetLastError();
    for (int a = 0; a < A && e == cudaSuccess; a++) {
        float *pa = phi + (long)a * M * M;
        float *oa = out + (long)a * M * M;
        dim3 b(32, 8), g1((M + 31) / 32, (M + 7) / 8, 1), g2((M2 + 31) / 32, (M2 + 7) / 8, 1);
        mirror_sincos_kernel<<<g1, b, 0, s>>>(pa, work, M); note_launch();
        e = fft2_batch(work, M2, 1, false, s);
        if (e != cudaSuccess) break;
        k2_kernel<false><<<1024, 256, 0, s>>>(work, M2, n2); note_launch();
        e = fft2_batch(work, M2, 1, true, s);
        if (e != cudaSuccess) break;
        combine_kernel<<<g2, b, 0, s>>>(work, pa, M, sc); note_launch();
        e = fft2_batch(work, M2, 1, false, s);
        if (e != cudaSuccess) break;
        k2_kernel<true><<<1024, 256, 0, s>>>(work, M2, n2); note_launch();
        e = fft2_batch(work, M2, 1, true, s);
        if (e != cudaSuccess) break;
        obtain_kernel<<<g1, b, 0, s>>>(work, pa, oa, M, sc); note_launch();
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) return e;
    submin_kernel<<<A, 512, 0, s>>>(out, M); note_launch();
    return cudaGetLastError();
}

}  // namespace ctdm
