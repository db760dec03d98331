/*
 * ctdm_oracle.c -- FP64 host restatement of the cTDM hologram -> RI path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity oracle: it is built into
 * oracle/_build/libctdm_oracle.so and loaded by tests/, by the smoke check and by
 * the CPU-baseline leg of bench.py.  The product library (ctdm_gb300/csrc) never
 * links, calls or falls back to it.
 *
 * Every function restates the reference algorithm (y-h-Lin/cTDM) and cites the
 * file:line it follows.  Floating-point stages run in double precision.  Stages
 * whose outputs are integers (residue charges, branch-cut masks, voxel indices,
 * hit counts, carrier position) follow the exact float/int semantics written here
 * so that the CUDA kernels can be compared bit for bit.
 *
 * Pinning: the DCT unwrap chain is checked against the float32 dumps the
 * reference ships (cTDM/src, Laplace, DCT, DCT2, IDCT .256.256.raw) in
 * tests/test_oracle_golden.py.  The remaining stages have no reference golden
 * vectors; they are pinned by closed-form known answers (FFT of impulses and
 * tones, DCT against the textbook definition, round trips) in the same tests.
 *
 * Layout conventions (reference, cTDM/HilbertTransform.cu): 2-D arrays are
 * x-fastest, element (i, j) at i + W*j; 3-D arrays at i + W*j + W*H*k.
 * Complex arrays are interleaved (re, im) doubles (C99 double complex).
 */
#include <complex.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef double complex cplx;

#define OR_PI 3.14159265358979323846

/* ------------------------------------------------------------------------- */
/* threads                                                                    */
/* ------------------------------------------------------------------------- */
void or_set_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

int or_get_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------------- */
/* FFT: mixed radix (4, 2, 3, generic) recursive Cooley-Tukey, FP64.           */
/* Semantics of cuFFT C2C used by the reference (cTDM/FFT.cu:697-838):          */
/* forward = exp(-i 2 pi k n / N), unnormalised; inverse = exp(+i ...),       */
/* unnormalised (callers scale).                                              */
/* ------------------------------------------------------------------------- */
/* tw[e] = exp(sign * 2 pi i e / N) for the top-level size N; a sub-transform of
 * size n uses W_n^e = tw[e * N / n]. */
static cplx *make_tw(int N, int sign)
{
    cplx *tw = (cplx *)malloc(sizeof(cplx) * N);
    for (int e = 0; e < N; e++) {
        double a = sign * 2.0 * OR_PI * (double)e / N;
        tw[e] = cos(a) + I * sin(a);
    }
    return tw;
}

static void dft_rec(const cplx *in, cplx *out, int n, int stride, const cplx *tw, int N, int sign)
{
    if (n == 1) { out[0] = in[0]; return; }
    int p;
    if (n % 4 == 0) p = 4; else if (n % 2 == 0) p = 2; else if (n % 3 == 0) p = 3; else p = n;
    int m = n / p, step = N / n;
    if (p == n) {
        for (int k = 0; k < n; k++) {
            cplx s = 0;
            for (int j = 0; j < n; j++) s += in[j * stride] * tw[(int)(((long)j * k) % n) * step];
            out[k] = s;
        }
        return;
    }
    for (int q = 0; q < p; q++) dft_rec(in + q * stride, out + q * m, m, stride * p, tw, N, sign);
    if (p == 4) {
        for (int k = 0; k < m; k++) {
            cplx a0 = out[k], a1 = out[m + k] * tw[k * step], a2 = out[2 * m + k] * tw[2 * k * step],
                 a3 = out[3 * m + k] * tw[3 * k * step];
            cplx t0 = a0 + a2, t1 = a0 - a2, t2 = a1 + a3, t3 = (a1 - a3) * (sign < 0 ? -I : I);
            out[k] = t0 + t2;
            out[m + k] = t1 + t3;
            out[2 * m + k] = t0 - t2;
            out[3 * m + k] = t1 - t3;
        }
    } else if (p == 2) {
        for (int k = 0; k < m; k++) {
            cplx a0 = out[k], a1 = out[m + k] * tw[k * step];
            out[k] = a0 + a1;
            out[m + k] = a0 - a1;
        }
    } else {
        const double s3 = 0.86602540378443864676;
        for (int k = 0; k < m; k++) {
            cplx a0 = out[k], a1 = out[m + k] * tw[k * step], a2 = out[2 * m + k] * tw[2 * k * step];
            cplx t1 = a1 + a2, t2 = (a1 - a2) * (sign < 0 ? -I * s3 : I * s3);
            out[k] = a0 + t1;
            out[m + k] = a0 - 0.5 * t1 + t2;
            out[2 * m + k] = a0 - 0.5 * t1 - t2;
        }
    }
}

/* 1-D transform of one contiguous line (in place). sign = -1 forward, +1 inverse. */
void or_fft1d(cplx *a, int n, int sign)
{
    cplx *tmp = (cplx *)malloc(sizeof(cplx) * n);
    cplx *tw = make_tw(n, sign);
    dft_rec(a, tmp, n, 1, tw, n, sign);
    memcpy(a, tmp, sizeof(cplx) * n);
    free(tmp);
    free(tw);
}

/* Transform along one axis of an (nx, ny, nz) array, in place. */
static void fft_axis(cplx *a, int nx, int ny, int nz, int axis, int sign)
{
    long n = axis == 0 ? nx : (axis == 1 ? ny : nz);
    long nlines = (long)nx * ny * nz / n;
    cplx *tw = make_tw((int)n, sign);
#pragma omp parallel
    {
        cplx *line = (cplx *)malloc(sizeof(cplx) * n);
        cplx *out = (cplx *)malloc(sizeof(cplx) * n);
#pragma omp for schedule(static)
        for (long l = 0; l < nlines; l++) {
            long base, step;
            if (axis == 0) { base = l * nx; step = 1; }
            else if (axis == 1) { long x = l % nx, z = l / nx; base = x + (long)nx * ny * z; step = nx; }
            else { base = l; step = (long)nx * ny; }
            for (long p = 0; p < n; p++) line[p] = a[base + p * step];
            dft_rec(line, out, (int)n, 1, tw, (int)n, sign);
            for (long p = 0; p < n; p++) a[base + p * step] = out[p];
        }
        free(line);
        free(out);
    }
    free(tw);
}

/* 2-D unnormalised transform of an nx-by-ny (x fastest) array. */
void or_fft2d(cplx *a, int nx, int ny, int sign)
{
    fft_axis(a, nx, ny, 1, 0, sign);
    fft_axis(a, nx, ny, 1, 1, sign);
}

/* 3-D transform, cuFFT3D semantics (cTDM/FFT.cu:807-838, scaleFFT3D :900-916):
 * dir = -1 forward unnormalised; dir = +1 inverse times 1/(nx ny nz), no conjugate. */
void or_fft3d(cplx *a, int nx, int ny, int nz, int dir)
{
    int sign = dir < 0 ? -1 : 1;
    fft_axis(a, nx, ny, nz, 0, sign);
    fft_axis(a, nx, ny, nz, 1, sign);
    fft_axis(a, nx, ny, nz, 2, sign);
    if (dir > 0) {
        double s = 1.0 / ((double)nx * ny * nz);
        long tot = (long)nx * ny * nz;
#pragma omp parallel for schedule(static)
        for (long i = 0; i < tot; i++) a[i] *= s;
    }
}

/* Quadrant swap (cuFFT2Dshift, cTDM/FFT.cu:220-236).  For even sizes it is both
 * fftshift and ifftshift. */
void or_shift2d(cplx *a, int w, int h)
{
    for (int j = 0; j < h / 2; j++)
        for (int i = 0; i < w / 2; i++) {
            cplx t = a[i + j * w];
            a[i + j * w] = a[(i + w / 2) + (j + h / 2) * w];
            a[(i + w / 2) + (j + h / 2) * w] = t;
            t = a[(i + w / 2) + j * w];
            a[(i + w / 2) + j * w] = a[i + (j + h / 2) * w];
            a[i + (j + h / 2) * w] = t;
        }
}

/* Octant swap (cuFFT3Dshift, cTDM/FFT.cu:324-350), out of place. */
void or_shift3d(const cplx *in, cplx *out, int nx, int ny, int nz)
{
    for (int k = 0; k < nz; k++)
        for (int j = 0; j < ny; j++)
            for (int i = 0; i < nx; i++) {
                int i2 = (i + nx / 2) % nx, j2 = (j + ny / 2) % ny, k2 = (k + nz / 2) % nz;
                out[i2 + (long)nx * j2 + (long)nx * ny * k2] = in[i + (long)nx * j + (long)nx * ny * k];
            }
}

/* ------------------------------------------------------------------------- */
/* QPI Algorithm A                                                            */
/* ------------------------------------------------------------------------- */

/* First search row of the carrier argmax.  obtainRadius (cTDM/HilbertTransform.cu:
 * 3439) hard-codes row 600 for 1024-pixel holograms; the rule is scaled to N. */
int or_carrier_start_row(int n) { return (600 * n) / 1024; }

/* obtainRadius (cTDM/HilbertTransform.cu:3425-3455): argmax of |X| over rows
 * j >= start of the fftshifted spectrum, first maximum in raster order;
 * radius = |r - N/2| / 3 (integer division). r = row (y), c = column (x). */
void or_qpi_carrier(const float *holo, int n, int *r, int *c, int *radius)
{
    cplx *a = (cplx *)malloc(sizeof(cplx) * n * n);
    for (long i = 0; i < (long)n * n; i++) a[i] = holo[i];
    or_fft2d(a, n, n, -1);
    or_shift2d(a, n, n);
    double best = -1.0;
    int br = 0, bc = 0;
    for (int j = or_carrier_start_row(n); j < n; j++)
        for (int i = 0; i < n; i++) {
            double m = creal(a[i + (long)j * n]) * creal(a[i + (long)j * n]) +
                       cimag(a[i + (long)j * n]) * cimag(a[i + (long)j * n]);
            if (m > best) { best = m; br = j; bc = i; }
        }
    *r = br;
    *c = bc;
    *radius = abs(br - n / 2) / 3;
    free(a);
}

/* extractQPI_AlgorithmA (cTDM/HilbertTransform.cu:1546-1585): FFT2 (N), fftshift,
 * get1stOrder_new crop of an M x M box around (c, r) with the +-radius mask
 * (:3566-3586), ifftshift (M), IFFT2 (M), scale 1/M^2 and conjugate
 * (scaleFFT2D, cTDM/FFT.cu:853-868).  field: M*M complex. */
void or_qpi_field(const float *holo, int n, int m, int r, int c, int radius, cplx *field)
{
    cplx *a = (cplx *)malloc(sizeof(cplx) * n * n);
    for (long i = 0; i < (long)n * n; i++) a[i] = holo[i];
    or_fft2d(a, n, n, -1);
    or_shift2d(a, n, n);
    for (int j = 0; j < m; j++)
        for (int i = 0; i < m; i++) {
            int ii = i + (c - m / 2), jj = j + (r - m / 2);
            cplx v = 0;
            if (ii >= c - radius && ii <= c + radius && jj >= r - radius && jj <= r + radius &&
                ii >= 0 && ii < n && jj >= 0 && jj < n)
                v = a[ii + (long)jj * n];
            field[i + j * m] = v;
        }
    or_shift2d(field, m, m);
    or_fft2d(field, m, m, +1);
    double s = 1.0 / ((double)m * m);
    for (int i = 0; i < m * m; i++) field[i] = conj(field[i] * s);
    free(a);
}

/* ------------------------------------------------------------------------- */
/* QPI Algorithm B                                                            */
/* ------------------------------------------------------------------------- */

/* The y-downsampled row spectra of Algorithm B (extractQPI_AlgorithmB and
 * sequence1DFFT, cTDM/HilbertTransform.cu:1587-1660): bilinear resample of the N x N
 * hologram to N x N/4 by the tap rule of bilinear_interpolation_kernel (:3658-3723;
 * x ratio (N-1)/N, y ratio (N-1)/(N/4), taps past the edge read 0), an N-point
 * forward transform of every row, then the swap of the two x halves (shiftArray
 * :1745-1758).  spec: N/4 rows of N. */
static void qpib_spectra(const float *holo, int n, cplx *spec)
{
    const int h = n / 4;
    const float xr = (float)(n - 1) / (float)n, yr = (float)(n - 1) / (float)h;
    for (int j = 0; j < h; j++) {
        cplx *row = spec + (long)j * n;
        for (int i = 0; i < n; i++) {
            int ix = (int)(xr * (float)i), iy = (int)(yr * (float)j);
            double a = (double)(xr * (float)i - (float)ix), b = (double)(yr * (float)j - (float)iy);
            double d00 = (ix < n && iy < n) ? holo[(long)iy * n + ix] : 0;
            double d10 = (ix + 1 < n && iy < n) ? holo[(long)iy * n + ix + 1] : 0;
            double d01 = (ix < n && iy + 1 < n) ? holo[(long)(iy + 1) * n + ix] : 0;
            double d11 = (ix + 1 < n && iy + 1 < n) ? holo[(long)(iy + 1) * n + ix + 1] : 0;
            double t1 = a * d10 + (-d00 * a + d00);
            double t2 = a * d11 + (-d01 * a + d01);
            row[i] = b * t2 + (-t1 * b + t1);
        }
        or_fft1d(row, n, -1);
        for (int i = 0; i < n / 2; i++) {
            cplx t = row[i];
            row[i] = row[i + n / 2];
            row[i + n / 2] = t;
        }
    }
}

/* Carrier column of Algorithm B (frame 1 of sequence1DFFT, :1626-1641): the column
 * sums of |X| over the N/4 rows (HistogramFT :1727-1743), the first maximum over
 * columns [int(0.6 N), N) (thrust::max_element), mirrored to N - c when N - c < N/8. */
int or_qpib_center(const float *holo, int n)
{
    const int h = n / 4;
    cplx *spec = (cplx *)malloc(sizeof(cplx) * (long)n * h);
    qpib_spectra(holo, n, spec);
    int best = (int)(n * 0.6);
    double bv = -1.0;
    for (int i = (int)(n * 0.6); i < n; i++) {
        double s = 0;
        for (int j = 0; j < h; j++) s += cabs(spec[i + (long)j * n]);
        if (s > bv) { bv = s; best = i; }
    }
    free(spec);
    if (n - best < (n / 4) / 2) best = n - best;
    return best;
}

/* Algorithm B field (:1643-1659): N/4 columns of each row spectrum from c - N/8
 * (CropFTdomain :1800-1812; columns outside the spectrum read 0, where the reference
 * would read past its array), swap of the halves (N/4), inverse N/4-point transform,
 * scale 1/(N/4) with conjugation and a transpose (copySharedMem :1704-1724).
 * field: M x M, M = N/4, field[X * M + Y] from row Y, column X. */
void or_qpib_field(const float *holo, int n, int center, cplx *field)
{
    const int m = n / 4;
    cplx *spec = (cplx *)malloc(sizeof(cplx) * (long)n * m);
    cplx *row = (cplx *)malloc(sizeof(cplx) * m);
    qpib_spectra(holo, n, spec);
    for (int y = 0; y < m; y++) {
        for (int x = 0; x < m; x++) {
            int k = x - n / 8 + center;
            row[x] = (k >= 0 && k < n) ? spec[k + (long)y * n] : 0;
        }
        for (int x = 0; x < m / 2; x++) {
            cplx t = row[x];
            row[x] = row[x + m / 2];
            row[x + m / 2] = t;
        }
        or_fft1d(row, m, +1);
        for (int x = 0; x < m; x++) field[(long)x * m + y] = conj(row[x] / (double)m);
    }
    free(row);
    free(spec);
}

/* calcWrapPhase (cTDM/HilbertTransform.cu:3618-3639): phase = arg BG - arg SP (not
 * rewrapped), amp = |SP| / |BG|; NaN/inf -> 0 for both. */
void or_wrap_phase(const cplx *sp, const cplx *bg, int count, double *phase, double *amp)
{
    for (int i = 0; i < count; i++) {
        double p = atan2(cimag(bg[i]), creal(bg[i])) - atan2(cimag(sp[i]), creal(sp[i]));
        if (isnan(p) || isinf(p)) p = 0;
        double a = cabs(sp[i]) / cabs(bg[i]);
        if (isnan(a) || isinf(a)) a = 0;
        phase[i] = p;
        amp[i] = a;
    }
}

/* ------------------------------------------------------------------------- */
/* DCT least-squares unwrapping (cTDM/DCT_Unwrapping.cu)                       */
/* ------------------------------------------------------------------------- */

/* NumericDerivative1 wrap (cTDM/DCT_Unwrapping.cu:336-358), evaluated in double
 * as the reference expression is (M_PI is a double). */
static double wrap_grad(double t)
{
    double s = t > 0 ? 1.0 : (t < 0 ? -1.0 : 0.0);
    return t - 2 * OR_PI * s * floor(fabs(OR_PI * s + t) / (OR_PI * 2));
}

/* Wrapped Laplacian rho (NumericDerivative1 + SumDerivative, :336-417). */
void or_wrapped_laplacian(const double *phi, int w, int h, double *rho)
{
    double *gx = (double *)malloc(sizeof(double) * w * h);
    double *gy = (double *)malloc(sizeof(double) * w * h);
    for (int j = 0; j < h; j++)
        for (int i = 0; i < w; i++) {
            int idx = i + w * j;
            double tx = (i == w - 1) ? -phi[idx] : phi[idx + 1] - phi[idx];
            double ty = (j == h - 1) ? -phi[idx] : phi[idx + w] - phi[idx];
            gx[idx] = wrap_grad(tx);
            gy[idx] = wrap_grad(ty);
        }
    for (int j = 0; j < h; j++)
        for (int i = 0; i < w; i++) {
            int idx = i + w * j;
            double c1 = (i == w - 1) ? 0 : gx[idx];
            double c2 = (i == 0) ? 0 : gx[idx - 1];
            double c3 = (j == h - 1) ? 0 : gy[idx];
            double c4 = (j == 0) ? 0 : gy[idx - w];
            rho[idx] = (c1 - c2) + (c3 - c4);
        }
    free(gx);
    free(gy);
}

/* Orthonormal DCT-II of every line along one axis, computed the way myDCT does
 * (cTDM/DCT_Unwrapping.cu:61-83): mirror-extend to 2L (float2cufft :144), 2L-point
 * forward FFT, countFDCT twiddle (:202-216). */
static void dct2_axis(double *a, int w, int h, int axis)
{
    int L = axis == 0 ? w : h, nl = axis == 0 ? h : w;
#pragma omp parallel
    {
        cplx *z = (cplx *)malloc(sizeof(cplx) * 2 * L);
        cplx *o = (cplx *)malloc(sizeof(cplx) * 2 * L);
        cplx *tw = make_tw(2 * L, -1);
#pragma omp for schedule(static)
        for (int l = 0; l < nl; l++) {
            for (int p = 0; p < L; p++) {
                double v = axis == 0 ? a[p + w * l] : a[l + w * p];
                z[p] = v;
                z[2 * L - 1 - p] = v;
            }
            dft_rec(z, o, 2 * L, 1, tw, 2 * L, -1);
            double dt = 1.0 / sqrt(2.0 * L);
            for (int k = 0; k < L; k++) {
                double v = k == 0 ? creal(o[0]) * dt / sqrt(2.0)
                                  : (creal(o[k]) * cos(k * OR_PI / (2.0 * L)) +
                                     cimag(o[k]) * sin(k * OR_PI / (2.0 * L))) * dt;
                if (axis == 0) a[k + w * l] = v; else a[l + w * k] = v;
            }
        }
        free(z);
        free(o);
        free(tw);
    }
}

/* Inverse used by myIDCT (cTDM/DCT_Unwrapping.cu:85-107, countIDCT :218-246):
 * the left half holds X_i e^{i pi i/2L} (times sqrt 2 at i = 0), the right half at
 * L + i holds X_{L-i} (sin t, -cos t) with t = (i+1) pi/2L in the reference
 * (mode 0, ref_compat) or t = i pi/2L (mode 1, exact DCT-III); 2L-point inverse
 * FFT, real part of the first L outputs (cufft2float :164). */
static void dct3_axis(double *a, int w, int h, int axis, int mode)
{
    int L = axis == 0 ? w : h, nl = axis == 0 ? h : w;
#pragma omp parallel
    {
        cplx *z = (cplx *)malloc(sizeof(cplx) * 2 * L);
        cplx *o = (cplx *)malloc(sizeof(cplx) * 2 * L);
        double *x = (double *)malloc(sizeof(double) * L);
        cplx *tw = make_tw(2 * L, +1);
#pragma omp for schedule(static)
        for (int l = 0; l < nl; l++) {
            double dt = 1.0 / sqrt(2.0 * L);
            for (int p = 0; p < L; p++) x[p] = axis == 0 ? a[p + w * l] : a[l + w * p];
            for (int i = 0; i < L; i++) {
                double th = i * OR_PI / (2.0 * L);
                double v = x[i] * dt;
                z[i] = (i == 0) ? (cos(th) * v * sqrt(2.0) + I * sin(th) * v * sqrt(2.0))
                                : (cos(th) * v + I * sin(th) * v);
                if (i == 0) {
                    z[L] = 0;
                } else {
                    double t2 = (mode == 0 ? (i + 1.0) : (double)i) * OR_PI / (2.0 * L);
                    double v2 = x[L - i] * dt;
                    z[L + i] = sin(t2) * v2 + I * (-cos(t2)) * v2;
                }
            }
            dft_rec(z, o, 2 * L, 1, tw, 2 * L, +1);
            for (int p = 0; p < L; p++) {
                if (axis == 0) a[p + w * l] = creal(o[p]); else a[l + w * p] = creal(o[p]);
            }
        }
        free(z);
        free(o);
        free(x);
        free(tw);
    }
}

/* 2-D orthonormal DCT-II (x then y), as myDCT. */
void or_dct2d(double *a, int w, int h)
{
    dct2_axis(a, w, h, 0);
    dct2_axis(a, w, h, 1);
}

/* 2-D inverse as myIDCT (y first, then x). */
void or_idct2d(double *a, int w, int h, int mode)
{
    dct3_axis(a, w, h, 1, mode);
    dct3_axis(a, w, h, 0, mode);
}

/* devConstant (cTDM/DCT_Unwrapping.cu:300-311): divide by
 * 2cos(4 pi i/(4W-1)) + 2cos(4 pi j/(4H-1)) - 4, (0,0) -> 0 (quirk Q2 kept). */
void or_poisson_divide(double *a, int w, int h)
{
    for (int j = 0; j < h; j++)
        for (int i = 0; i < w; i++) {
            int idx = i + w * j;
            if (i == 0 && j == 0) { a[idx] = 0; continue; }
            double d = 2 * cos(4 * OR_PI * i / (4.0 * w - 1)) + 2 * cos(4 * OR_PI * j / (4.0 * h - 1)) - 4;
            a[idx] = a[idx] / d;
        }
}

/* DCT_UWLS_Unwrapped (cTDM/DCT_Unwrapping.cu:10-59). mode 0 = ref_compat IDCT
 * twiddle (quirk Q1), mode 1 = exact DCT-III. */
void or_dct_unwrap(const double *phi, int w, int h, int mode, double *out)
{
    or_wrapped_laplacian(phi, w, h, out);
    or_dct2d(out, w, h);
    or_poisson_divide(out, w, h);
    or_idct2d(out, w, h, mode);
}

/* ------------------------------------------------------------------------- */
/* FFT-based least-squares unwrapping (cTDM/FastUnwrapping.cu:5-117)           */
/* The intended (2W x 2H) transforms are used (quirk Q8: the reference's plans   */
/* are (W/2)^2).  phi is normalised in place like PhaseNormalize (:119-130).   */
/* ------------------------------------------------------------------------- */
void or_fast_unwrap(double *phi, int w, int h, double *out)
{
    long n = (long)w * h;
    double mn = phi[0], mx = phi[0];
    for (long i = 0; i < n; i++) { if (phi[i] < mn) mn = phi[i]; if (phi[i] > mx) mx = phi[i]; }
    for (long i = 0; i < n; i++) phi[i] = 2 * OR_PI * (phi[i] - mn) / (mx - mn);   /* RescalePhaseMap :132-142 */
    int W2 = 2 * w, H2 = 2 * h;
    long n2 = (long)W2 * H2;
    double *sn = (double *)malloc(sizeof(double) * n2), *cs = (double *)malloc(sizeof(double) * n2);
    cplx *t1 = (cplx *)malloc(sizeof(cplx) * n2), *t2 = (cplx *)malloc(sizeof(cplx) * n2);
    for (int j = 0; j < h; j++)                                                    /* makeSimmetric :144-169 */
        for (int i = 0; i < w; i++) {
            double s = sin(phi[i + w * j]), c = cos(phi[i + w * j]);
            long id[4] = {i + (long)W2 * j, (W2 - 1 - i) + (long)W2 * j, i + (long)W2 * (H2 - 1 - j),
                          (W2 - 1 - i) + (long)W2 * (H2 - 1 - j)};
            for (int q = 0; q < 4; q++) { sn[id[q]] = s; cs[id[q]] = c; }
        }
    for (long i = 0; i < n2; i++) { t1[i] = sn[i]; t2[i] = cs[i]; }
    or_fft2d(t1, W2, H2, -1);
    or_fft2d(t2, W2, H2, -1);
    /* MultiplyPosition (:263-279) in the shifted frame: con = (i-W)^2 + (j-H)^2 at the
     * shifted index, i.e. k^2 of the signed frequency at the unshifted index. */
    for (int j = 0; j < H2; j++)
        for (int i = 0; i < W2; i++) {
            int fi = i < w ? i : i - W2, fj = j < h ? j : j - H2;
            double con = (double)fi * fi + (double)fj * fj;
            t1[i + (long)W2 * j] *= con;
            t2[i + (long)W2 * j] *= con;
        }
    or_fft2d(t1, W2, H2, +1);
    or_fft2d(t2, W2, H2, +1);
    double sc = 1.0 / (double)n2;
    for (long i = 0; i < n2; i++) {                       /* scaleFFT2D (conj) then MultiplyComplex */
        t1[i] = conj(t1[i] * sc) * cs[i];
        t2[i] = conj(t2[i] * sc) * sn[i];
    }
    or_fft2d(t1, W2, H2, -1);
    or_fft2d(t2, W2, H2, -1);
    for (int j = 0; j < H2; j++)                           /* MultiplyInvPosition :281-306, SubtractComplex */
        for (int i = 0; i < W2; i++) {
            int fi = i < w ? i : i - W2, fj = j < h ? j : j - H2;
            double con = (double)fi * fi + (double)fj * fj;
            long k = i + (long)W2 * j;
            t1[k] = con == 0 ? 0 : (t1[k] - t2[k]) / con;
        }
    or_fft2d(t1, W2, H2, +1);
    double mnu = 1e300;
    for (int j = 0; j < h; j++)                            /* transferQuarter + ObtainUnwrap :333-345 */
        for (int i = 0; i < w; i++) {
            double cont = creal(conj(t1[i + (long)W2 * j] * sc));
            double src = phi[i + w * j];
            double k = round((cont - src) * (0.5 / OR_PI));
            double v = src + 2 * OR_PI * k;
            out[i + w * j] = v;
            if (v < mnu) mnu = v;
        }
    for (long i = 0; i < n; i++) out[i] -= mnu;            /* subtractMin :347-359 */
    free(sn); free(cs); free(t1); free(t2);
}

/* ------------------------------------------------------------------------- */
/* Goldstein (cTDM/Goldstein.cu).  Float semantics, serial specification.     */
/* ------------------------------------------------------------------------- */

/* cudaMod (cTDM/Goldstein.cu:1193-1201) applied to the expression of
 * cudaPhaseResidues: the float difference is promoted to double, M_PI added,
 * rounded to float for fmodf; the remainder minus M_PI is rounded to float. */
static float res_term(float a, float b)
{
    float d = a - b;
    float x = (float)((double)d + OR_PI);
    float m = (float)(OR_PI * 2);
    float r = fmodf(x, m);
    if (r < 0) r = r + m;
    return (float)((double)r - OR_PI);
}

/* cudaPhaseResidues (cTDM/Goldstein.cu:52-103). charges in {-1, 0, +1}. */
void or_goldstein_residues(const float *phi, int w, int h, int8_t *charges)
{
    for (int c = 0; c < h; c++)
        for (int r = 0; r < w; r++) {
            int8_t q = 0;
            if (r != w - 1 && c != h - 1) {
                float r1 = res_term(phi[r + c * w], phi[(r + 1) + c * w]);
                float r2 = res_term(phi[(r + 1) + c * w], phi[(r + 1) + (c + 1) * w]);
                float r3 = res_term(phi[(r + 1) + (c + 1) * w], phi[r + (c + 1) * w]);
                float r4 = res_term(phi[r + (c + 1) * w], phi[r + c * w]);
                float t = r1 + r2;
                t = t + r3;
                t = t + r4;
                if (t >= 6.0f) q = 1;
                else if (t <= -6.0f) q = -1;
            }
            charges[r + c * w] = q;
        }
}

/* cuPlaceBranchCutInternal (cTDM/Goldstein.cu:224-248) with its unsigned index
 * arithmetic: a fill pixel is kept only when min(r1,r2)-1 < rFill < max(r1,r2)+1
 * in unsigned 32-bit arithmetic (so segments touching index 0 keep only their end
 * points).  __float2int_rn = round half to even. */
static void place_cut(uint8_t *cut, int w, unsigned r1, unsigned c1, unsigned r2, unsigned c2)
{
    cut[r1 + (unsigned)w * c1] = 1;
    cut[r2 + (unsigned)w * c2] = 1;
    float dR = (float)(int)(r2 - r1);
    float dC = (float)(int)(c2 - c1);
    float radius = sqrtf(dR * dR + dC * dC);
    float ct = dR / radius;
    float st = dC / radius;
    int nr = (int)rintf(radius);
    unsigned rlo = (r1 < r2 ? r1 : r2) - 1u, rhi = (r1 > r2 ? r1 : r2) + 1u;
    unsigned clo = (c1 < c2 ? c1 : c2) - 1u, chi = (c1 > c2 ? c1 : c2) + 1u;
    for (int ii = 1; ii <= nr; ii++) {
        unsigned rf = r1 + (unsigned)(int)rintf((float)ii * ct);
        unsigned cf = c1 + (unsigned)(int)rintf((float)ii * st);
        if (rf > rlo && rf < rhi && cf > clo && cf < chi) cut[rf + (unsigned)w * cf] = 1;
    }
}

/* Serial specification of cuBranchCuts / cudaBC (cTDM/Goldstein.cu:105-201): the
 * residues are visited in raster order idx = i + w*j ascending, each executing the
 * body of cudaBC with the shared arrays updated in that order (the reference runs
 * them concurrently without synchronisation).  Unsigned box bounds are kept as
 * written (max(i-r,0) on unsigned wraps, leaving the box empty).  The branch-cut
 * mask starts all zero (inverseLogic on an all-ones IM_Mask, :208-222). */
void or_goldstein_cuts(const int8_t *charges, int w, int h, uint8_t *cut)
{
    long n = (long)w * h;
    int8_t *masked = (int8_t *)malloc(n);
    memcpy(masked, charges, n);
    memset(cut, 0, n);
    int maxBox = 901;
    int half = (int)floorf((float)(w / 2));
    if (half < maxBox) maxBox = half;
    unsigned maxR = (unsigned)maxBox;
    unsigned hr = (unsigned)(int)rintf((float)w * 0.5f);
    if (hr < maxR) maxR = hr;
    for (unsigned j = 0; j < (unsigned)h; j++)
        for (unsigned i = 0; i < (unsigned)w; i++) {
            unsigned idx = i + (unsigned)w * j;
            int charge = masked[idx];
            if (charge == 0) continue;
            if (i <= 0 || i >= (unsigned)w - 1 || j <= 0 || j >= (unsigned)h - 1) {
                cut[idx] = 1;
                masked[idx] = 0;
            }
            for (unsigned r = 1; r < maxR; r++) {
                unsigned m1 = i - r, m2 = i + r, n1 = j - r, n2 = j + r;
                if (m2 > (unsigned)w - 1) m2 = (unsigned)w - 1;
                if (n2 > (unsigned)h - 1) n2 = (unsigned)h - 1;
                for (unsigned mm = m1; mm <= m2; mm++) {
                    if (charge == 0) continue;
                    unsigned ndel = (mm == m1 || mm == m2) ? 1u : n2 - n1;
                    for (unsigned nn = n1; nn <= n2; nn += ndel) {
                        if (mm <= 0 || mm >= (unsigned)w - 1) {
                            place_cut(cut, w, i, j, mm, j);
                            charge = 0;
                            masked[idx] = 0;
                            masked[i + (unsigned)w * nn] = 0;
                        } else if (nn <= 0 || nn >= (unsigned)h - 1) {
                            place_cut(cut, w, i, j, i, nn);
                            charge = 0;
                            masked[idx] = 0;
                            masked[mm + (unsigned)w * j] = 0;
                        } else if ((int)masked[idx] * (int)masked[mm + (unsigned)w * nn] == -1) {
                            place_cut(cut, w, i, j, mm, nn);
                            charge = 0;
                            masked[idx] = 0;
                            masked[mm + (unsigned)w * nn] = 0;
                        }
                        if (ndel == 0) break;
                    }
                }
            }
        }
    free(masked);
}

/* One pass of FloodFill's inner loop body over a raster-ordered list
 * (cTDM/Goldstein.cu:758-913 and :946-1077).  use_cuts selects the main loop
 * (neighbours must not be cut pixels) or the final cut-pixel fill. */
static void ff_visit(long p, int w, int h, const uint8_t *cut, const float *phi, float *um,
                     uint8_t *ub, uint8_t *adj, int use_cuts)
{
    int rr = (int)(p % w), cc = (int)(p / w);
    long nb[4] = {p + 1, p - 1, p + w, p - w};
    int ok[4] = {rr + 1 <= w - 1, rr - 1 >= 0, cc + 1 <= h - 1, cc - 1 >= 0};
    int chosen = -1;
    for (int k = 0; k < 4; k++) {
        if (!ok[k]) continue;
        if (use_cuts && cut[nb[k]] != 0) continue;
        if (ub[nb[k]] == 1) {
            if (chosen < 0) chosen = k;
        } else {
            adj[nb[k]] = 1;
        }
    }
    if (chosen >= 0) {
        float ref = um[nb[chosen]];
        float d = phi[p] - ref;
        /* the reference calls sin/cos/atan2 on floats, which C++ resolves to the
         * float overloads */
        float dp = atan2f(sinf(d), cosf(d));
        um[p] = ref + dp;
        ub[p] = 1;
    }
    adj[p] = 0;
}

/* FloodFill (cTDM/Goldstein.cu:643-1095), the serial CPU flood fill.  Returns 0
 * when it completes, 1 when the 5000-sweep limit stops it (the reference returns
 * early and skips the final cut fill), 2 when the sweeps stall with a non-empty
 * adjoin set (the reference spins forever there; the fill stops and the final
 * cut fill runs).  out: unwrapped phase, 0 where never reached.  um_mask gets 1
 * where a value was assigned. */
int or_goldstein_floodfill(const uint8_t *cut, const float *phi, int w, int h, float *out, uint8_t *ub)
{
    long n = (long)w * h;
    uint8_t *adj = (uint8_t *)calloc(n, 1);
    long *list = (long *)malloc(sizeof(long) * n);
    long *stuck = (long *)malloc(sizeof(long) * n);
    memset(ub, 0, n);
    for (long i = 0; i < n; i++) out[i] = 0.0f;
    /* The seed is (rowRef, colRef) = (2, W/2), index rowRef + W colRef: the reference
     * sets it (:656-657) before it walks the diagonal from (W/2, 2) off the cuts
     * (:659-663), so the walk changes nothing (it only reads, past the image when the
     * whole diagonal is cut) and the seed may lie on a cut.  A seed outside the image
     * stops the fill here. */
    const int rowRef = 2, colRef = w / 2;
    if (rowRef >= w || colRef >= h) { free(adj); free(list); free(stuck); return 2; }
    long nbc = 0;
    for (long i = 0; i < n; i++) nbc += cut[i] != 0;
    if (rowRef > 0) adj[(rowRef - 1) + (long)w * colRef] = 1;
    if (rowRef < w - 1) adj[(rowRef + 1) + (long)w * colRef] = 1;
    if (colRef > 0) adj[rowRef + (long)w * (colRef - 1)] = 1;
    if (colRef < h - 1) adj[rowRef + (long)w * (colRef + 1)] = 1;
    out[rowRef + (long)w * colRef] = phi[rowRef + (long)w * colRef];
    ub[rowRef + (long)w * colRef] = 1;
    int first = 1, countLimit = 0, status = 0;
    long L1 = 0, L2 = 0;
    for (;;) {
        long sum = 0;
        for (long i = 0; i < n; i++) sum += adj[i] == 1;
        if (sum == 0) break;
        if (countLimit >= 2) { status = 2; break; }
        int term = 0;
        while (countLimit < 2) {
            if (++term > 5000) { free(adj); free(list); free(stuck); return 1; }
            if (!first) { L1 = L2; memcpy(stuck, list, sizeof(long) * L2); }
            first = 0;
            L2 = 0;
            for (long i = 0; i < n; i++) if (adj[i] != 0) list[L2++] = i;
            if (L1 == L2) {
                int same = 1;
                for (long q = 0; q < L1; q++) if (stuck[q] != list[q]) { same = 0; break; }
                if (same) countLimit++;
            } else {
                countLimit = 0;
            }
            for (long q = 0; q < L2; q++) ff_visit(list[q], w, h, cut, phi, out, ub, adj, 1);
        }
    }
    if (nbc > 0) {
        for (int cc = 1; cc < h - 1; cc++)
            for (int rr = 1; rr < w - 1; rr++) {
                long p = rr + (long)w * cc;
                if (cut[p] == 1 && (cut[p + 1] == 0 || cut[p - 1] == 0 || cut[p - w] == 0 || cut[p + w] == 0))
                    adj[p] = 1;
            }
        L2 = 0;
        for (long i = 0; i < n; i++) if (adj[i] != 0) list[L2++] = i;
        for (long q = 0; q < L2; q++) ff_visit(list[q], w, h, cut, phi, out, ub, adj, 0);
    }
    free(adj); free(list); free(stuck);
    return status;
}

/* ------------------------------------------------------------------------- */
/* Resize, stack assembly, median, Rytov spectrum                              */
/* ------------------------------------------------------------------------- */

/* bilinear_interpolation_kernel (cTDM/HilbertTransform.cu:3658-3723) producing only
 * the centred R x R window of the M2 x N2 result that Combine2Stack with
 * ResizeFlag = 1 keeps (:1394-1427); NaN/inf scrub of Combine2Stack applied
 * (phase -> 0, amp -> 1).  Out-of-range taps read 0 (the reference leaves d10_2
 * unset, quirk Q18; it is defined as 0 here). */
void or_resize_crop(const double *p_in, const double *a_in, int m1, int n1, int m2, int n2, int r,
                    double *p_out, double *a_out)
{
    float xr = (float)(m1 - 1) / (float)m2, yr = (float)(n1 - 1) / (float)n2;
    int ox = (m2 - r) / 2, oy = (n2 - r) / 2;
    for (int jj = 0; jj < r; jj++)
        for (int ii = 0; ii < r; ii++) {
            int i = ii + ox, j = jj + oy;
            int ix = (int)(xr * (float)i), iy = (int)(yr * (float)j);
            double a = (double)xr * i - ix, b = (double)yr * j - iy;
            for (int q = 0; q < 2; q++) {
                const double *d = q == 0 ? p_in : a_in;
                double d00 = (ix < m1 && iy < n1) ? d[iy * m1 + ix] : 0;
                double d10 = (ix + 1 < m1 && iy < n1) ? d[iy * m1 + ix + 1] : 0;
                double d01 = (ix < m1 && iy + 1 < n1) ? d[(iy + 1) * m1 + ix] : 0;
                double d11 = (ix + 1 < m1 && iy + 1 < n1) ? d[(iy + 1) * m1 + ix + 1] : 0;
                double t1 = a * d10 + (-d00 * a + d00);
                double t2 = a * d11 + (-d01 * a + d01);
                double v = b * t2 + (-t1 * b + t1);
                if (q == 0) { if (isnan(v) || isinf(v)) v = 0; p_out[ii + r * jj] = v; }
                else { if (isnan(v) || isinf(v)) v = 1; a_out[ii + r * jj] = v; }
            }
        }
}

static double med9(double *v)
{
    for (int i = 1; i < 9; i++) {
        double x = v[i];
        int j = i - 1;
        while (j >= 0 && v[j] > x) { v[j + 1] = v[j]; j--; }
        v[j + 1] = x;
    }
    return v[4];
}

/* MedianFilter (cTDM/Recon_kernel.cu:7-27): 3x3 median of the interior of each
 * slice (MedianFilter_gpu :65-120 skips x in {0, W-1}, y in {0, H-1}), computed out
 * of place (the reference filters in place and races, quirk Q5), then checkMaps
 * (:122-142): phase NaN/inf -> 0; amp NaN/inf -> 1, 0 -> 0.01, else |amp|. */
void or_median_check(const double *ph, const double *am, int w, int h, double *ph_out, double *am_out)
{
    for (int q = 0; q < 2; q++) {
        const double *in = q == 0 ? ph : am;
        double *o = q == 0 ? ph_out : am_out;
        for (int y = 0; y < h; y++)
            for (int x = 0; x < w; x++) {
                if (x == 0 || x == w - 1 || y == 0 || y == h - 1) { o[x + w * y] = in[x + w * y]; continue; }
                double v[9];
                int k = 0;
                for (int dx = -1; dx <= 1; dx++)
                    for (int dy = -1; dy <= 1; dy++) v[k++] = in[(x + dx) + w * (y + dy)];
                o[x + w * y] = med9(v);
            }
    }
    for (long i = 0; i < (long)w * h; i++) {
        if (isnan(ph_out[i]) || isinf(ph_out[i])) ph_out[i] = 0;
        double a = am_out[i];
        if (isnan(a) || isinf(a)) a = 1.0;
        else if (a == 0) a = 0.01;
        else a = fabs(a);
        am_out[i] = a;
    }
}

/* CopyDataArray (cTDM/Recon_kernel.cu:144-169, transposed: u[j + i*W] from pixel
 * (i, j)), cuFFT2Dshift, cuFFT2D forward (BatchRecon :1909-1913). */
void or_rytov_spectrum(const double *ph, const double *am, int w, cplx *u)
{
    for (int j = 0; j < w; j++)
        for (int i = 0; i < w; i++) u[j + i * w] = log(am[i + j * w]) + I * ph[i + j * w];
    or_shift2d(u, w, w);
    or_fft2d(u, w, w, -1);
}

/* ------------------------------------------------------------------------- */
/* Fourier mapping onto the Ewald cap (cTDM/Recon_kernel.cu:171-239)           */
/* ------------------------------------------------------------------------- */

/* Voxel index rule of fillEdwardSphere (:187-229) evaluated in IEEE double with
 * no contraction (the reference computes it in float under fast math; the FP64
 * rule is what both implementations here share).  fx0 = fm0 sin(AngY),
 * fy0 = fm0 sin(AngX) (quirk Q4).  Writes, per spectrum bin q = Nx + R*Ny, the
 * voxel index or -1 when the cap has no sample there, and fz (for the value). */
void or_ewald_index(int r, double fm0, double df, double angx, double angy, int64_t *vox, double *fzo)
{
    double fx0 = fm0 * sin(angy);
    double fy0 = fm0 * sin(angx);
    double fm02 = fm0 * fm0;
    double rad0 = fm02 - fx0 * fx0;
    rad0 = rad0 - fy0 * fy0;
    double fz0 = sqrt(rad0);
    for (long q = 0; q < (long)r * r; q++) { vox[q] = -1; if (fzo) fzo[q] = 0; }
    for (int j = 0; j < r; j++)
        for (int i = 0; i < r; i++) {
            int ii = i - r / 2, jj = j - r / 2;
            double fx = (double)ii * df;
            fx = fx + fx0;
            double fy = (double)jj * df;
            fy = fy + fy0;
            double s = fx * fx;
            s = s + fy * fy;
            double rad = fm02 - s;
            if (rad0 < 0 || rad < 0) continue;
            double fz = sqrt(rad);
            double Fz = fz - fz0;
            double t = Fz / df;
            double rn = t > 0.0 ? floor(t + 0.5) : ceil(t - 0.5);
            long nz = (long)rn;
            int nx = ((ii % r) + r) % r, ny = ((jj % r) + r) % r;
            long nzm = ((nz % r) + r) % r;
            long qi = nx + (long)r * ny;
            vox[qi] = nx + (long)r * ny + (long)r * r * nzm;
            if (fzo) fzo[qi] = fz;
        }
}

/* EdwardSphere accumulation over all angles in order (F += i 4 pi fz u, C += 1)
 * followed by Initial_F_F2 (:253-276): F2 = (F / C where C != 0) / dx.
 * U: A spectra of R*R; F2: R^3 (output); counts: R^3 (output, may be NULL). */
void or_ewald_map(const cplx *U, const float *angx, const float *angy, int na, int r, double fm0,
                  double df, double dx, cplx *F2, uint32_t *counts)
{
    long n3 = (long)r * r * r, n2 = (long)r * r;
    uint32_t *C = counts ? counts : (uint32_t *)malloc(sizeof(uint32_t) * n3);
    memset(C, 0, sizeof(uint32_t) * n3);
    for (long i = 0; i < n3; i++) F2[i] = 0;
    int64_t *vox = (int64_t *)malloc(sizeof(int64_t) * n2);
    double *fz = (double *)malloc(sizeof(double) * n2);
    for (int a = 0; a < na; a++) {
        or_ewald_index(r, fm0, df, angx[a], angy[a], vox, fz);
        for (long q = 0; q < n2; q++) {
            if (vox[q] < 0) continue;
            cplx u = U[(long)a * n2 + q];
            F2[vox[q]] += (-fz[q] * 4 * OR_PI * cimag(u)) + I * (fz[q] * 4 * OR_PI * creal(u));
            C[vox[q]] += 1;
        }
    }
    for (long i = 0; i < n3; i++) {
        cplx f = F2[i];
        if (C[i] != 0) f = f / (double)C[i];
        F2[i] = f / dx;
    }
    free(vox);
    free(fz);
    if (!counts) free(C);
}

/* ------------------------------------------------------------------------- */
/* Positivity loop (cTDM/HilbertTransform.cu:1943-1975, Recon_kernel.cu:278-412) */
/* ------------------------------------------------------------------------- */

/* calculate_n3D (:305-342): principal square root; clamp Re n >= n_med, Im n >= 0. */
static cplx est_n(cplx F, double k2, double nmed)
{
    double c = creal(F) / (-k2) + 1, d = cimag(F) / (-k2);
    double mod = sqrt(c * c + d * d);
    double a = sqrt((mod + c) / 2);
    double b = d != 0 ? sqrt((mod - c) / 2) * (d / fabs(d)) : 0.0;
    double nr = a * nmed, ni = b * nmed;
    if (nr < nmed) nr = nmed;
    if (ni < 0) ni = 0;
    return nr + I * ni;
}

/* Modify_F3D (:370-383) called with n_med^2 (HilbertTransform.cu:1962). */
static cplx modify_f(cplx n, double k2, double nmed2)
{
    double nr = creal(n), ni = cimag(n);
    return ((nr * nr - ni * ni) / nmed2 - 1) * (-k2) + I * ((nr * ni * 2) / nmed2 * (-k2));
}

/* Full plain reconstruction from F2: F = F2, IFFT3, n = est_n, then `iters` loop
 * bodies {modify, FFT3, replace, IFFT3, est_n}, final octant shift.  check_mode 0
 * keeps the reference predicate (F2.re != 0 and F2.im != 0, quirk Q10); 1 uses the
 * hit mask counts > 0.  n_out: R^3 complex, fftshifted. */
void or_positivity(const cplx *F2, const uint32_t *counts, int r, int iters, double k2, double nmed,
                   int check_mode, cplx *n_out)
{
    long n3 = (long)r * r * r;
    cplx *F = (cplx *)malloc(sizeof(cplx) * n3);
    cplx *n = (cplx *)malloc(sizeof(cplx) * n3);
    memcpy(F, F2, sizeof(cplx) * n3);
    or_fft3d(F, r, r, r, +1);
#pragma omp parallel for schedule(static)
    for (long i = 0; i < n3; i++) n[i] = est_n(F[i], k2, nmed);
    double nmed2 = nmed * nmed;
    for (int it = 0; it < iters; it++) {
#pragma omp parallel for schedule(static)
        for (long i = 0; i < n3; i++) F[i] = modify_f(n[i], k2, nmed2);
        or_fft3d(F, r, r, r, -1);
#pragma omp parallel for schedule(static)
        for (long i = 0; i < n3; i++) {
            int keep = check_mode == 0 ? (creal(F2[i]) != 0.0 && cimag(F2[i]) != 0.0) : (counts[i] > 0);
            if (keep) F[i] = F2[i];
        }
        or_fft3d(F, r, r, r, +1);
#pragma omp parallel for schedule(static)
        for (long i = 0; i < n3; i++) n[i] = est_n(F[i], k2, nmed);
    }
    or_shift3d(n, n_out, r, r, r);
    free(F);
    free(n);
}

/* ------------------------------------------------------------------------- */
/* Whole path: holograms -> RI volume                                          */
/* ------------------------------------------------------------------------- */
typedef struct {
    int n;            /* hologram side N */
    int m;            /* crop side M */
    int r;            /* volume side R */
    int iters;        /* positivity loop bodies */
    int unwrap_mode;  /* 0 ref_compat, 1 exact */
    int check_mode;   /* 0 ref_compat predicate, 1 hit mask */
    int carrier_r, carrier_c, carrier_radius; /* < 0: detect from the background */
    double fm0, df, dx, k2, n_med;
    int qpi_method;   /* reference QPI_Method numbering: 0 Algorithm B, 1 Algorithm A */
} or_params;

/* Phase and amplitude stacks for A angles (R*R each, after resize+crop and
 * median/check), from SP holograms (A*N*N) and BG holograms (1 or A). */
void or_front_end(const or_params *p, const float *sp, const float *bg, int na, int bg_per_angle,
                  double *phase_out, double *amp_out, int *carrier /* r, c, radius */)
{
    int n = p->n, m = p->m, r = p->r;
    const int method_b = p->qpi_method == 0;
    int cr = p->carrier_r, cc = p->carrier_c, rad = p->carrier_radius;
    int cb = -1, cs0 = -1;   /* Algorithm B: carrier columns of the background and of frame 1 */
    if (method_b) {
        m = n / 4;
        if (cc >= 0) {
            cb = cs0 = cc;
        } else {
            /* frame 1 of sequence1DFFT computes the column from its own spectrum, the
             * SP first and then the BG; later frames keep the BG's */
            cs0 = or_qpib_center(sp, n);
            cb = or_qpib_center(bg, n);
        }
        if (carrier) { carrier[0] = cb; carrier[1] = cs0; carrier[2] = -1; }
    } else {
        if (cr < 0 || cc < 0 || rad < 0) or_qpi_carrier(bg, n, &cr, &cc, &rad);
        if (carrier) { carrier[0] = cr; carrier[1] = cc; carrier[2] = rad; }
    }
    long mm = (long)m * m;
    cplx *bgf = (cplx *)malloc(sizeof(cplx) * mm);
    if (!bg_per_angle) {
        if (method_b) or_qpib_field(bg, n, cb, bgf);
        else or_qpi_field(bg, n, m, cr, cc, rad, bgf);
    }
    for (int a = 0; a < na; a++) {
        cplx *spf = (cplx *)malloc(sizeof(cplx) * mm);
        double *ph = (double *)malloc(sizeof(double) * mm), *am = (double *)malloc(sizeof(double) * mm);
        double *uw = (double *)malloc(sizeof(double) * mm);
        double *pr = (double *)malloc(sizeof(double) * r * r), *ar = (double *)malloc(sizeof(double) * r * r);
        if (method_b) {
            or_qpib_field(sp + (long)a * n * n, n, a == 0 ? cs0 : cb, spf);
            if (bg_per_angle) or_qpib_field(bg + (long)a * n * n, n, cb, bgf);
        } else {
            or_qpi_field(sp + (long)a * n * n, n, m, cr, cc, rad, spf);
            if (bg_per_angle) or_qpi_field(bg + (long)a * n * n, n, m, cr, cc, rad, bgf);
        }
        or_wrap_phase(spf, bgf, (int)mm, ph, am);
        or_dct_unwrap(ph, m, m, p->unwrap_mode, uw);
        or_resize_crop(uw, am, m, m, n, n, r, pr, ar);
        or_median_check(pr, ar, r, r, phase_out + (long)a * r * r, amp_out + (long)a * r * r);
        free(spf); free(ph); free(am); free(uw); free(pr); free(ar);
    }
    free(bgf);
}

/* Plain pipeline: BatchRecon after the per-frame loop.  Returns the fftshifted RI
 * volume.  counts may be NULL unless check_mode == 1. */
void or_pipeline(const or_params *p, const float *sp, const float *bg, int na, int bg_per_angle,
                 const float *angx, const float *angy, cplx *n_out, int *carrier)
{
    int r = p->r;
    long r2 = (long)r * r, r3 = r2 * r;
    double *ph = (double *)malloc(sizeof(double) * na * r2), *am = (double *)malloc(sizeof(double) * na * r2);
    or_front_end(p, sp, bg, na, bg_per_angle, ph, am, carrier);
    cplx *U = (cplx *)malloc(sizeof(cplx) * na * r2);
    for (int a = 0; a < na; a++) or_rytov_spectrum(ph + a * r2, am + a * r2, r, U + a * r2);
    cplx *F2 = (cplx *)malloc(sizeof(cplx) * r3);
    uint32_t *C = (uint32_t *)malloc(sizeof(uint32_t) * r3);
    or_ewald_map(U, angx, angy, na, r, p->fm0, p->df, p->dx, F2, C);
    or_positivity(F2, C, r, p->iters, p->k2, p->n_med, p->check_mode, n_out);
    free(ph); free(am); free(U); free(F2); free(C);
}

/* A whole tomogram as the reference runs it (cTDM/HilbertTransform.cu:963-976 per
 * frame: QPI Algorithm A, calcWrapPhase, the unwrap; Combine2Stack; BatchRecon
 * :1825-2047), for the timed CPU baseline: the per-angle chain (QPI A, wrapped phase,
 * Goldstein residues / cuts / flood fill on the float phase when run_goldstein, DCT
 * unwrap, resize + crop, median + checkMaps, Rytov spectrum) runs in parallel over the
 * angles, then the Ewald mapping and the positivity loop.  Same results as
 * or_pipeline; charges (may be NULL) receive the residue maps (na * M * M). */
void or_tomogram(const or_params *p, const float *sp, const float *bg, int na, const float *angx, const float *angy,
                 int run_goldstein, cplx *n_out, int8_t *charges, int *carrier)
{
    int n = p->n, m = p->m, r = p->r;
    int cr = p->carrier_r, cc = p->carrier_c, rad = p->carrier_radius;
    if (cr < 0 || cc < 0 || rad < 0) or_qpi_carrier(bg, n, &cr, &cc, &rad);
    if (carrier) { carrier[0] = cr; carrier[1] = cc; carrier[2] = rad; }
    long mm = (long)m * m, r2 = (long)r * r, r3 = r2 * r;
    cplx *bgf = (cplx *)malloc(sizeof(cplx) * mm);
    or_qpi_field(bg, n, m, cr, cc, rad, bgf);
    cplx *U = (cplx *)malloc(sizeof(cplx) * na * r2);
#pragma omp parallel for schedule(dynamic, 1)
    for (int a = 0; a < na; a++) {
        cplx *spf = (cplx *)malloc(sizeof(cplx) * mm);
        double *ph = (double *)malloc(sizeof(double) * mm), *am = (double *)malloc(sizeof(double) * mm);
        double *uw = (double *)malloc(sizeof(double) * mm);
        double *pr = (double *)malloc(sizeof(double) * r2), *ar = (double *)malloc(sizeof(double) * r2);
        double *pm = (double *)malloc(sizeof(double) * r2), *amd = (double *)malloc(sizeof(double) * r2);
        or_qpi_field(sp + (long)a * n * n, n, m, cr, cc, rad, spf);
        or_wrap_phase(spf, bgf, (int)mm, ph, am);
        if (run_goldstein) {
            float *phf = (float *)malloc(sizeof(float) * mm), *gout = (float *)malloc(sizeof(float) * mm);
            int8_t *q = charges ? charges + (long)a * mm : (int8_t *)malloc(mm);
            uint8_t *cut = (uint8_t *)malloc(mm), *ub = (uint8_t *)malloc(mm);
            for (long i = 0; i < mm; i++) phf[i] = (float)ph[i];
            or_goldstein_residues(phf, m, m, q);
            or_goldstein_cuts(q, m, m, cut);
            or_goldstein_floodfill(cut, phf, m, m, gout, ub);
            if (!charges) free(q);
            free(phf); free(gout); free(cut); free(ub);
        }
        or_dct_unwrap(ph, m, m, p->unwrap_mode, uw);
        or_resize_crop(uw, am, m, m, n, n, r, pr, ar);
        or_median_check(pr, ar, r, r, pm, amd);
        or_rytov_spectrum(pm, amd, r, U + a * r2);
        free(spf); free(ph); free(am); free(uw); free(pr); free(ar); free(pm); free(amd);
    }
    cplx *F2 = (cplx *)malloc(sizeof(cplx) * r3);
    uint32_t *C = (uint32_t *)malloc(sizeof(uint32_t) * r3);
    or_ewald_map(U, angx, angy, na, r, p->fm0, p->df, p->dx, F2, C);
    or_positivity(F2, C, r, p->iters, p->k2, p->n_med, p->check_mode, n_out);
    free(bgf); free(U); free(F2); free(C);
}

/* ------------------------------------------------------------------------- */
/* ASD-POCS with total variation (BatchReconPOCS, cTDM/HilbertTransform.cu:    */
/* 2049-2402; FrquencyInterpolation / FI_kernel / calF and the POCS kernels,   */
/* cTDM/Recon_kernel.cu:414-1106), with the mathematics fixed as the product   */
/* defines it: see ctdm_gb300/csrc/k_pocs.cu and the FI notes of k_recon.cu.   */
/* ------------------------------------------------------------------------- */

/* Frequency-interpolation mapping for a one-axis scan of tilts angx (AngY = 0).
 * Voxel rule of or_ewald_index (unwrapped z index kept for Fz = nz df); the angle
 * theta' whose cap passes through the voxel centre, Fy sin t + Fz cos t =
 * -|K|^2 / (2 fm), root nearer the frame's own angle; spectra of the two scan angles
 * around theta' interpolated linearly in angle; value i 4 pi fz' u,
 * fz' = Fz + fm cos(theta'); per-voxel mean over frames, / dx. */
void or_fi_map(const cplx *U, const float *angx, int na, int r, double fm0, double df, double dx, cplx *F2,
               uint32_t *counts)
{
    long n3 = (long)r * r * r, n2 = (long)r * r;
    uint32_t *C = counts ? counts : (uint32_t *)malloc(sizeof(uint32_t) * n3);
    memset(C, 0, sizeof(uint32_t) * n3);
    for (long i = 0; i < n3; i++) F2[i] = 0;
    int *order = (int *)malloc(sizeof(int) * na);
    double *th = (double *)malloc(sizeof(double) * na);
    for (int a = 0; a < na; a++) order[a] = a;
    for (int a = 1; a < na; a++) {   /* stable insertion sort by angle */
        int v = order[a], b = a - 1;
        while (b >= 0 && angx[order[b]] > angx[v]) { order[b + 1] = order[b]; b--; }
        order[b + 1] = v;
    }
    for (int k = 0; k < na; k++) th[k] = (double)angx[order[k]];
    double fm02 = fm0 * fm0;
    for (int a = 0; a < na; a++) {
        double fx0 = fm0 * sin(0.0), fy0 = fm0 * sin((double)angx[a]);
        double rad0 = fm02 - fx0 * fx0;
        rad0 = rad0 - fy0 * fy0;
        if (rad0 < 0) continue;
        double fz0 = sqrt(rad0);
        double theta_own = asin(fy0 / fm0);
        for (int j = 0; j < r; j++)
            for (int i = 0; i < r; i++) {
                int ii = i - r / 2, jj = j - r / 2;
                double fx = (double)ii * df;
                fx = fx + fx0;
                double fy = (double)jj * df;
                fy = fy + fy0;
                double s = fx * fx;
                s = s + fy * fy;
                double rad = fm02 - s;
                if (rad < 0) continue;
                double fz = sqrt(rad);
                double t = (fz - fz0) / df;
                double rn = t > 0.0 ? floor(t + 0.5) : ceil(t - 0.5);
                long nzs = (long)rn;
                int nx = ((ii % r) + r) % r, ny = ((jj % r) + r) % r;
                long nzm = ((nzs % r) + r) % r;
                long q = nx + (long)r * ny;
                long vox = q + n2 * nzm;
                cplx u_own = U[(long)a * n2 + q];
                double Fx = ii * df, Fy = jj * df, Fz = (double)nzs * df;
                double rho = sqrt(Fy * Fy + Fz * Fz);
                double c = -(Fx * Fx + Fy * Fy + Fz * Fz) / (2.0 * fm0 * rho);
                cplx val;
                if (!(rho > 0.0) || c < -1.0 || c > 1.0) {
                    val = I * (4 * OR_PI * fz) * u_own;
                } else {
                    double phi = atan2(Fy, Fz), dth = acos(c);
                    double t1 = phi + dth, t2 = phi - dth;
                    double tp = fabs(t1 - theta_own) <= fabs(t2 - theta_own) ? t1 : t2;
                    double fzp = Fz + fm0 * cos(tp);
                    int sidx = 0;
                    double w = 0.0;
                    if (tp >= th[na - 1]) {
                        sidx = na - 1;
                    } else if (tp > th[0]) {
                        int lo = 0, hi = na - 1;
                        while (hi - lo > 1) {
                            int mid = (lo + hi) / 2;
                            if (th[mid] <= tp) lo = mid;
                            else hi = mid;
                        }
                        sidx = lo;
                        w = (tp - th[lo]) / (th[hi] - th[lo]);
                    }
                    cplx u = U[(long)order[sidx] * n2 + q];
                    if (w > 0.0) u = (1.0 - w) * u + w * U[(long)order[sidx + 1] * n2 + q];
                    val = I * (4 * OR_PI * fzp) * u;
                }
                F2[vox] += val;
                C[vox] += 1;
            }
    }
    for (long i = 0; i < n3; i++) {
        cplx f = F2[i];
        if (C[i] != 0) f = f / (double)C[i];
        F2[i] = f / dx;
    }
    free(order);
    free(th);
    if (!counts) free(C);
}

typedef struct {
    int iterations, tv_steps;
    double beta, beta_red, alpha, alpha_red, r_max, eps_data, tv_eps;
} or_pocs_params;

/* Gradient of the isotropic TV (backward differences, periodic) of V at every voxel. */
static void tv_gradient(const double *V, int r, double eps, double *g)
{
    long rr = (long)r * r;
#pragma omp parallel for schedule(static)
    for (int z = 0; z < r; z++)
        for (int y = 0; y < r; y++)
            for (int x = 0; x < r; x++) {
                int xm = (x + r - 1) % r, xp = (x + 1) % r, ym = (y + r - 1) % r, yp = (y + 1) % r;
                int zm = (z + r - 1) % r, zp = (z + 1) % r;
#define VV(a, b, c) V[(a) + (long)r * (b) + rr * (c)]
                double v = VV(x, y, z);
                double a0 = v - VV(xm, y, z), b0 = v - VV(x, ym, z), c0 = v - VV(x, y, zm);
                double d0 = sqrt(eps + a0 * a0 + b0 * b0 + c0 * c0);
                double vxp = VV(xp, y, z), vyp = VV(x, yp, z), vzp = VV(x, y, zp);
                double ax = vxp - v, bx = vxp - VV(xp, ym, z), cx = vxp - VV(xp, y, zm);
                double ay = vyp - VV(xm, yp, z), by = vyp - v, cy = vyp - VV(x, yp, zm);
                double az = vzp - VV(xm, y, zp), bz = vzp - VV(x, ym, zp), cz = vzp - v;
#undef VV
                double dx = sqrt(eps + ax * ax + bx * bx + cx * cx);
                double dy = sqrt(eps + ay * ay + by * by + cy * cy);
                double dz = sqrt(eps + az * az + bz * bz + cz * cz);
                g[x + (long)r * y + rr * z] = (a0 + b0 + c0) / d0 - ax / dx - by / dy - cz / dz;
            }
}

static double norm2(const double *a, long n)
{
    double s = 0;
    for (long i = 0; i < n; i++) s += a[i] * a[i];
    return sqrt(s);
}

/* ASD-POCS on the contrast V = n^2 / n_med^2 - 1 from F2 (zero where unmeasured):
 * data step F = beta Y + (1 - beta) F at the measured voxels (Y = F2 / -k^2),
 * projection V+ = max(Re sqrt(1 + V), 1)^2 - 1, Dp = |V+ - V_start|,
 * Dd = |FFT3(V+) - Y| over the measured voxels (want_dd, else +inf), TV steepest
 * descent (dtvg = alpha Dp on the first iteration; tv_steps normalised-gradient steps),
 * Dg = |V - V+|, dtvg *= alpha_red when Dg > r_max Dp and Dd > eps_data,
 * beta *= beta_red.  Output: one more data step, n = est_n, octant shifted.
 * hist: 4 doubles per iteration (Dp, Dd, Dg, dtvg used). */
void or_pocs(const cplx *F2, int r, const or_pocs_params *p, double k2, double nmed, int want_dd, cplx *n_out,
             double *hist)
{
    long n3 = (long)r * r * r;
    double *V = (double *)calloc(n3, sizeof(double)), *Vp = (double *)malloc(sizeof(double) * n3);
    double *g = (double *)malloc(sizeof(double) * n3), *d = (double *)malloc(sizeof(double) * n3);
    cplx *G = (cplx *)malloc(sizeof(cplx) * n3);
    double beta = p->beta, dtvg = 0;
    int first = 1;
    for (int it = 0; it <= p->iterations; it++) {
        for (long i = 0; i < n3; i++) G[i] = V[i];
        or_fft3d(G, r, r, r, -1);
        for (long i = 0; i < n3; i++)
            if (creal(F2[i]) != 0.0 || cimag(F2[i]) != 0.0) G[i] = beta * (F2[i] / (-k2)) + (1 - beta) * G[i];
        or_fft3d(G, r, r, r, +1);
        if (it == p->iterations) break;   /* the output's data step */
        double dp = 0;
        for (long i = 0; i < n3; i++) {
            double u = creal(csqrt(1.0 + G[i])) - 1.0;
            double vn = u > 0 ? u * (2 + u) : 0;
            dp += (vn - V[i]) * (vn - V[i]);
            V[i] = vn;
            Vp[i] = vn;
        }
        dp = sqrt(dp);
        double dd = HUGE_VAL;
        if (want_dd) {
            for (long i = 0; i < n3; i++) G[i] = Vp[i];
            or_fft3d(G, r, r, r, -1);
            double s = 0;
            for (long i = 0; i < n3; i++)
                if (creal(F2[i]) != 0.0 || cimag(F2[i]) != 0.0) {
                    cplx e = G[i] - F2[i] / (-k2);
                    s += creal(e) * creal(e) + cimag(e) * cimag(e);
                }
            dd = sqrt(s);
        }
        tv_gradient(V, r, p->tv_eps, g);
        double gn = norm2(g, n3);
        if (first) { dtvg = p->alpha * dp; first = 0; }
        for (int t = 0; t < p->tv_steps; t++) {
            double s = gn > 0 ? dtvg / gn : 0;
            for (long i = 0; i < n3; i++) V[i] -= s * g[i];
            if (t + 1 < p->tv_steps) {
                tv_gradient(V, r, p->tv_eps, g);
                gn = norm2(g, n3);
            }
        }
        for (long i = 0; i < n3; i++) d[i] = V[i] - Vp[i];
        double dg = norm2(d, n3);
        if (hist) {
            hist[4 * it] = dp;
            hist[4 * it + 1] = dd;
            hist[4 * it + 2] = dg;
            hist[4 * it + 3] = dtvg;
        }
        if (dg > p->r_max * dp && dd > p->eps_data) dtvg *= p->alpha_red;
        beta *= p->beta_red;
    }
    cplx *n = (cplx *)malloc(sizeof(cplx) * n3);
    for (long i = 0; i < n3; i++) n[i] = est_n(G[i] * (-k2), k2, nmed);
    or_shift3d(n, n_out, r, r, r);
    free(V); free(Vp); free(g); free(d); free(G); free(n);
}
