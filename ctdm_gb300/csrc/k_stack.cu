// Per-angle preparation of the Rytov data for the Fourier mapping.
//
// Reference chain (y-h-Lin/cTDM): bilinear_interpolation_kernel M -> N
// (cTDM/HilbertTransform.cu:3658-3723), Combine2Stack centre crop N -> R with the
// NaN/inf scrub (:1394-1427), MedianFilter_gpu + checkMaps per slice
// (cTDM/Recon_kernel.cu:7-27,65-142), cuCopyArray u = log A + i phi transposed
// (:154-169) and cuFFT2Dshift (cTDM/FFT.cu:220).  One kernel per 32 x 32 tile:
// only the R x R window of the upsampled map is interpolated (into shared
// memory with a one-pixel halo), the median is taken out of place (the
// reference filters in place and races), and the transposed, quadrant-swapped
// complex value is written coalesced.
#include <cmath>

#include "kernels_front.cuh"

namespace ctdm {

// bilinear_interpolation_kernel tap rule; taps past the input edge read 0 (the
// reference leaves d10_2 unset there; it is defined as 0).
__device__ __forceinline__ float resize_at(const float *__restrict__ d, int M1, float xr, int i, int j)
{
    const int ix = (int)(xr * (float)i);
    const float a = xr * (float)i - (float)ix;
    const int iy = (int)(xr * (float)j);
    const float b = xr * (float)j - (float)iy;
    const float d00 = (ix < M1 && iy < M1) ? d[iy * M1 + ix] : 0.f;
    const float d10 = (ix + 1 < M1 && iy < M1) ? d[iy * M1 + ix + 1] : 0.f;
    const float d01 = (ix < M1 && iy + 1 < M1) ? d[(iy + 1) * M1 + ix] : 0.f;
    const float d11 = (ix + 1 < M1 && iy + 1 < M1) ? d[(iy + 1) * M1 + ix + 1] : 0.f;
    const float t1 = a * d10 + (-d00 * a + d00);
    const float t2 = a * d11 + (-d01 * a + d01);
    return b * t2 + (-t1 * b + t1);
}

#define CTDM_SORT2(a, b)               \
    {                                  \
        const float lo_ = fminf(a, b); \
        b = fmaxf(a, b);               \
        a = lo_;                       \
    }

// Median of nine by the 19-exchange network published by Paeth (Graphics Gems).
__device__ __forceinline__ float median9(float p0, float p1, float p2, float p3, float p4, float p5, float p6,
                                         float p7, float p8)
{
    CTDM_SORT2(p1, p2); CTDM_SORT2(p4, p5); CTDM_SORT2(p7, p8);
    CTDM_SORT2(p0, p1); CTDM_SORT2(p3, p4); CTDM_SORT2(p6, p7);
    CTDM_SORT2(p1, p2); CTDM_SORT2(p4, p5); CTDM_SORT2(p7, p8);
    CTDM_SORT2(p0, p3); CTDM_SORT2(p5, p8); CTDM_SORT2(p4, p7);
    CTDM_SORT2(p3, p6); CTDM_SORT2(p1, p4); CTDM_SORT2(p2, p5);
    CTDM_SORT2(p4, p7); CTDM_SORT2(p4, p2); CTDM_SORT2(p6, p4);
    CTDM_SORT2(p4, p2);
    return p4;
}

__device__ __forceinline__ float tile_median(float (*s)[35], int ly, int lx)
{
    return median9(s[ly - 1][lx - 1], s[ly - 1][lx], s[ly - 1][lx + 1], s[ly][lx - 1], s[ly][lx], s[ly][lx + 1],
                   s[ly + 1][lx - 1], s[ly + 1][lx], s[ly + 1][lx + 1]);
}

__device__ __forceinline__ float med3(float a, float b, float c) { return fmaxf(fminf(a, b), fminf(fmaxf(a, b), c)); }

// The three values of a window column in order.
__device__ __forceinline__ void sort3(float a, float b, float c, float &lo, float &md, float &hi)
{
    const float l = fminf(a, b), h = fmaxf(a, b);
    lo = fminf(l, c);
    hi = fmaxf(h, c);
    md = fmaxf(l, fminf(h, c));
}

// The same taps read from a staged block of the source map: rows sy0 .. sy0 + SS - 1 and
// columns sx0 .. sx0 + SS - 1 at s[row - sy0][col - sx0] (taps past the map's edge were
// staged as 0).
constexpr int PREP_SS = 40;
__device__ __forceinline__ float resize_staged(const float (*t)[PREP_SS + 1], int sx0, int sy0, float xr, int i,
                                               int j)
{
    const int ix = (int)(xr * (float)i);
    const float a = xr * (float)i - (float)ix;
    const int iy = (int)(xr * (float)j);
    const float b = xr * (float)j - (float)iy;
    const int x = ix - sx0, y = iy - sy0;
    const float d00 = t[y][x], d10 = t[y][x + 1], d01 = t[y + 1][x], d11 = t[y + 1][x + 1];
    const float t1 = a * d10 + (-d00 * a + d00);
    const float t2 = a * d11 + (-d01 * a + d01);
    return b * t2 + (-t1 * b + t1);
}

// MODE 0: resize+crop from M x M maps.  MODE 1: input is already an R x R stack.
// OUT 0: Rytov complex (transposed, swapped).  OUT 1: phase/amp stack.
// MODE 0 stages the source block that a tile's taps read (once per source pixel instead
// of four times per resized pixel) when it fits PREP_SS x PREP_SS, which holds for every
// enlargement and slight shrink ((M - 1) / N up to about 1.1); else the taps read the
// maps directly.
template <int MODE, int OUT>
__global__ void __launch_bounds__(256) prep_kernel(const float *__restrict__ phase, const float *__restrict__ amp,
                                                  int M, int N, int R, float2 *U0, float *ph_out, float *am_out)
{
    __shared__ float sp[34][35], sa[34][35];
    __shared__ float tp[MODE == 0 ? PREP_SS : 1][PREP_SS + 1], ta[MODE == 0 ? PREP_SS : 1][PREP_SS + 1];
    const int a = blockIdx.z;
    const int tx0 = blockIdx.x * 32, ty0 = blockIdx.y * 32;
    const long in_sz = MODE == 0 ? (long)M * M : (long)R * R;
    const float *P = phase + a * in_sz;
    const float *Am = amp + a * in_sz;
    const float xr = (float)(M - 1) / (float)N;
    const int off = (N - R) / 2;
    const int tid = threadIdx.y * 32 + threadIdx.x;
    // source block of the tile's taps: the tap index (int)(xr i) grows with i, so the
    // block spans the taps of the tile's first and last (halo) pixels plus one
    const int ia = max(tx0 - 1, 0) + off, ib = min(tx0 + 32, R - 1) + off;
    const int ja = max(ty0 - 1, 0) + off, jb = min(ty0 + 32, R - 1) + off;
    const int sx0 = (int)(xr * (float)ia), sy0 = (int)(xr * (float)ja);
    const int sw = (int)(xr * (float)ib) + 2 - sx0, sh = (int)(xr * (float)jb) + 2 - sy0;
    const bool staged = MODE == 0 && sw <= PREP_SS && sh <= PREP_SS;   // the same for the whole CTA
    if (staged) {
        for (int e = tid; e < sw * sh; e += 256) {
            const int lx = e % sw, ly = e / sw;
            const int x = sx0 + lx, y = sy0 + ly;
            const bool in = x < M && y < M;
            tp[ly][lx] = in ? __ldg(&P[(long)y * M + x]) : 0.f;
            ta[ly][lx] = in ? __ldg(&Am[(long)y * M + x]) : 0.f;
        }
        __syncthreads();
    }
    for (int e = tid; e < 34 * 34; e += 256) {
        const int lx = e % 34, ly = e / 34;
        const int i = tx0 - 1 + lx, j = ty0 - 1 + ly;
        float pv = 0.f, av = 1.f;
        if (i >= 0 && i < R && j >= 0 && j < R) {
            if (MODE == 0) {
                if (staged) {
                    pv = resize_staged(tp, sx0, sy0, xr, i + off, j + off);
                    av = resize_staged(ta, sx0, sy0, xr, i + off, j + off);
                } else {
                    pv = resize_at(P, M, xr, i + off, j + off);
                    av = resize_at(Am, M, xr, i + off, j + off);
                }
                if (isnan(pv) || isinf(pv)) pv = 0.f;   // Combine2Stack scrub
                if (isnan(av) || isinf(av)) av = 1.f;
            } else {
                pv = P[i + (long)R * j];
                av = Am[i + (long)R * j];
            }
        }
        sp[ly][lx] = pv;
        sa[ly][lx] = av;
    }
    __syncthreads();
    const long rr = (long)R * R;
    // MODE 0 (values scrubbed of NaN and inf above): a thread takes 4 adjacent pixels of
    // one tile row, sorts the 6 window columns they span once, and takes each median as
    // med3(max of the column minima, med3 of the column middles, min of the column
    // maxima) over its 3 columns, the median of the 9 values.  MODE 1 keeps the
    // 19-exchange network per pixel.
    const int li0 = MODE == 0 ? 4 * (int)threadIdx.y : (int)threadIdx.y, lstep = MODE == 0 ? 1 : 8;
    float plo[6], pmd[6], phv[6], alo[6], amd[6], ahv[6];
    if constexpr (MODE == 0) {
        const int lj = threadIdx.x;
#pragma unroll
        for (int c = 0; c < 6; c++) {
            sort3(sp[lj][li0 + c], sp[lj + 1][li0 + c], sp[lj + 2][li0 + c], plo[c], pmd[c], phv[c]);
            sort3(sa[lj][li0 + c], sa[lj + 1][li0 + c], sa[lj + 2][li0 + c], alo[c], amd[c], ahv[c]);
        }
    }
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const int li = li0 + lstep * k, lj = threadIdx.x;
        const int i = tx0 + li, j = ty0 + lj;
        if (i >= R || j >= R) continue;
        float pv, av;
        if (i == 0 || i == R - 1 || j == 0 || j == R - 1) {
            pv = sp[lj + 1][li + 1];
            av = sa[lj + 1][li + 1];
        } else if constexpr (MODE == 0) {
            pv = med3(fmaxf(fmaxf(plo[k], plo[k + 1]), plo[k + 2]), med3(pmd[k], pmd[k + 1], pmd[k + 2]),
                      fminf(fminf(phv[k], phv[k + 1]), phv[k + 2]));
            av = med3(fmaxf(fmaxf(alo[k], alo[k + 1]), alo[k + 2]), med3(amd[k], amd[k + 1], amd[k + 2]),
                      fminf(fminf(ahv[k], ahv[k + 1]), ahv[k + 2]));
        } else {
            pv = tile_median(sp, lj + 1, li + 1);
            av = tile_median(sa, lj + 1, li + 1);
        }
        // checkMaps (cTDM/Recon_kernel.cu:122-142)
        if (isnan(pv) || isinf(pv)) pv = 0.f;
        if (isnan(av) || isinf(av)) av = 1.0f;
        else if (av == 0.f) av = 0.01f;
        else av = fabsf(av);
        if (OUT == 0) {
            const int xs = (j + R / 2) % R, ys = (i + R / 2) % R;
            U0[a * rr + xs + (long)R * ys] = make_float2(logf(av), pv);
        } else {
            ph_out[a * rr + i + (long)R * j] = pv;
            am_out[a * rr + i + (long)R * j] = av;
        }
    }
}

// bilinear_interpolation_kernel M -> N over whole maps (the per-frame resize of the
// job driver, cTDM/HilbertTransform.cu:1044-1047), phase and amplitude.
__global__ void resize_maps_kernel(const float *__restrict__ ph, const float *__restrict__ am, int A, int M, int N,
                                   float *ph_out, float *am_out)
{
    const long nn = (long)N * N, total = (long)A * nn;
    const float xr = (float)(M - 1) / (float)N;
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total; e += (long)gridDim.x * blockDim.x) {
        const long a = e / nn;
        const int p = (int)(e - a * nn), i = p % N, j = p / N;
        ph_out[e] = resize_at(ph + a * (long)M * M, M, xr, i, j);
        am_out[e] = resize_at(am + a * (long)M * M, M, xr, i, j);
    }
}

cudaError_t resize_maps(const float *ph, const float *am, int A, int M, int N, float *ph_out, float *am_out,
                        cudaStream_t s)
{
    long blocks = ((long)A * N * N + 255) / 256;
    if (blocks > 8192) blocks = 8192;
    resize_maps_kernel<<<(unsigned)blocks, 256, 0, s>>>(ph, am, A, M, N, ph_out, am_out);
    note_launch();
    return cudaGetLastError();
}

// Camera counts (8- or 16-bit) to float, four per thread (n a multiple of 4, both
// buffers 16-byte aligned): the host-buffer entries widen the backgrounds, and the
// holograms when QPI Algorithm B reads them, here.
template <class T>
__global__ void __launch_bounds__(256) widen_kernel(const T *__restrict__ in, float *out, long n4)
{
    for (long i = blockIdx.x * 256l + threadIdx.x; i < n4; i += (long)gridDim.x * 256) {
        if constexpr (sizeof(T) == 1) {
            const uchar4 v = reinterpret_cast<const uchar4 *>(in)[i];
            reinterpret_cast<float4 *>(out)[i] = make_float4(v.x, v.y, v.z, v.w);
        } else {
            const ushort4 v = reinterpret_cast<const ushort4 *>(in)[i];
            reinterpret_cast<float4 *>(out)[i] = make_float4(v.x, v.y, v.z, v.w);
        }
    }
}

cudaError_t widen_counts(const void *in, int bytes_per_count, long n, float *out, cudaStream_t s)
{
    if (n % 4 != 0 || (bytes_per_count != 1 && bytes_per_count != 2)) return cudaErrorInvalidValue;
    const long n4 = n / 4;
    long blocks = (n4 + 255) / 256;
    if (blocks > 8 * 152) blocks = 8 * 152;
    if (bytes_per_count == 1) widen_kernel<uint8_t><<<(unsigned)blocks, 256, 0, s>>>((const uint8_t *)in, out, n4);
    else widen_kernel<uint16_t><<<(unsigned)blocks, 256, 0, s>>>((const uint16_t *)in, out, n4);
    note_launch();
    return cudaGetLastError();
}

cudaError_t prep_rytov(const float *phase, const float *amp, int A, int M, int N, int R, float2 *U0, cudaStream_t s)
{
    dim3 grid((R + 31) / 32, (R + 31) / 32, A), block(32, 8);
    prep_kernel<0, 0><<<grid, block, 0, s>>>(phase, amp, M, N, R, U0, nullptr, nullptr); note_launch();
    return cudaGetLastError();
}

cudaError_t prep_stack(const float *phase, const float *amp, int A, int M, int N, int R, float *ph_out,
                       float *am_out, cudaStream_t s)
{
    dim3 grid((R + 31) / 32, (R + 31) / 32, A), block(32, 8);
    prep_kernel<0, 1><<<grid, block, 0, s>>>(phase, amp, M, N, R, nullptr, ph_out, am_out); note_launch();
    return cudaGetLastError();
}

cudaError_t stack_to_rytov(const float *ph, const float *am, int A, int R, float2 *U0, cudaStream_t s)
{
    dim3 grid((R + 31) / 32, (R + 31) / 32, A), block(32, 8);
    prep_kernel<1, 0><<<grid, block, 0, s>>>(ph, am, R, R, R, U0, nullptr, nullptr); note_launch();
    return cudaGetLastError();
}

}  // namespace ctdm

namespace ctdm {
// MedianFilter on R x R stacks (stack in, stack out).
cudaError_t median_stack(const float *ph, const float *am, int A, int R, float *ph_out, float *am_out, cudaStream_t s)
{
    dim3 grid((R + 31) / 32, (R + 31) / 32, A), block(32, 8);
    prep_kernel<1, 1><<<grid, block, 0, s>>>(ph, am, R, R, R, nullptr, ph_out, am_out); note_launch();
    return cudaGetLastError();
}
}  // namespace ctdm
