// Declarations of the per-angle (2-D) stage launchers.
#pragma once
#include "kernels.cuh"

namespace ctdm {

// QPI Algorithm A --------------------------------------------------------
// Carrier of one background hologram (N x N float): carrier = {r, c, radius}
// on the device.  scratch: N*N complex; key: one 64-bit word.
cudaError_t qpi_find_carrier(const float *bg, int N, float2 *scratch, unsigned long long *key, int *carrier,
                             cudaStream_t s);
// Pruned forward transform of A holograms into their M x M window spectra S
// (ifftshifted, masked to the carrier's radius box: every entry of S is written, the
// rows and columns outside the box with zeros).  T1: A*N*M complex scratch, of which
// only the box's columns are used.
// holo: A holograms of N x N pixels, bpc bytes each (4 float, 2 uint16, 1 uint8 counts)
cudaError_t qpi_forward_window(const void *holo, int bpc, int A, int N, int M, const int *carrier, float2 *T1,
                               float2 *S, cudaStream_t s);
// Inverse M x M transform of an S written by qpi_forward_window with the same carrier
// (destroyed; its zero rows are skipped) and the epilogue: field_out != NULL stores
// the complex field, otherwise phase/amp against bgf[a * bg_stride].
cudaError_t qpi_inverse_window(float2 *S, int A, int M, const int *carrier, float2 *field_out, const float2 *bgf,
                               long bg_stride, float *phase, float *amp, cudaStream_t s);

// QPI Algorithm B --------------------------------------------------------
// Carrier column of one hologram from its y-downsampled row spectra (mag: N/4 * N
// floats of scratch; center: device int).
cudaError_t qpib_spectrum_center(const float *holo, int N, float *mag, int *center, cudaStream_t s);
// Window rows of A holograms (T: A * (N/4) rows of N/4 complex) for the carrier column.
cudaError_t qpib_window(const float *holo, int A, int N, const int *center, float2 *T, cudaStream_t s);
// Inverse window transforms into transposed fields, or phase/amp against bgf.
cudaError_t qpib_inverse(const float2 *T, int A, int M, float2 *field_out, const float2 *bgf, long bg_stride,
                         float *phase, float *amp, cudaStream_t s);

// Angle camera: index of the spectrum peak of AngCal_GPU in *key's low word
// (complemented; see angcal_peak).  scratch: N*N complex.
cudaError_t angcal_peak(const float *img, int N, float2 *scratch, unsigned long long *key, cudaStream_t s);
// Integer camera counts (1 or 2 bytes each, n a multiple of 4) to float.
cudaError_t widen_counts(const void *in, int bytes_per_count, long n, float *out, cudaStream_t s);
// Whole-map bilinear resize M -> N of phase and amplitude stacks.
cudaError_t resize_maps(const float *ph, const float *am, int A, int M, int N, float *ph_out, float *am_out,
                        cudaStream_t s);

// DCT least-squares unwrap -----------------------------------------------
// A phase maps M x M (float) -> unwrapped maps.  T: A*M*M float scratch.
// mode 0 = reference IDCT twiddle, 1 = exact DCT-III.
cudaError_t dct_unwrap(const float *phi, float *out, float *T, int A, int M, int mode, cudaStream_t s);

// FFT-based unwrap (FastUnwrapping) ---------------------------------------
cudaError_t fast_unwrap(float *phi, float *out, float2 *work, int A, int M, cudaStream_t s);

// Resize + centre crop + median + checkMaps + log/complex + transpose + shift
// into the per-angle Rytov arrays U0 (A x R x R complex), ready for FFT2.
cudaError_t prep_rytov(const float *phase, const float *amp, int A, int M, int N, int R, float2 *U0,
                       cudaStream_t s);
// Same stage, writing the phase/amp stack instead (for inspection / tests):
// resized+cropped then median+checkMaps, A x R x R each.
cudaError_t prep_stack(const float *phase, const float *amp, int A, int M, int N, int R, float *ph_out,
                       float *am_out, cudaStream_t s);
// Median + checkMaps on an existing R x R stack, then Rytov arrays.
cudaError_t stack_to_rytov(const float *ph, const float *am, int A, int R, float2 *U0, cudaStream_t s);

// Goldstein ---------------------------------------------------------------
cudaError_t goldstein_residues(const float *phi, int A, int W, int H, int8_t *charges, cudaStream_t s);
cudaError_t goldstein_cuts(const int8_t *charges, int A, int W, int H, uint8_t *cuts, int8_t *work,
                           cudaStream_t s);
cudaError_t goldstein_floodfill(const uint8_t *cuts, const float *phi, int A, int W, int H, float *out,
                                uint8_t *state, int *lists, int *status, cudaStream_t s);

}  // namespace ctdm
