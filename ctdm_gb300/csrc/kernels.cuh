// Declarations of the kernel launchers shared between translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "ctdm_common.cuh"

namespace ctdm {

// Counts kernel launches issued by the library (process-wide, for instrumentation).
void note_launch();

// Builds the current device's tables once (contexts and tapes call it at creation).
cudaError_t device_tables();
// Twiddle table for an FFT length (exp(-2 pi i e / L), e < L), device resident;
// NULL until device_tables() has run on the current device.
const float2 *twiddles(int L);
// DCT helper tables for crop side M: dct_tw[k] = (cos(k pi/2M), sin(k pi/2M)),
// k = 0..2M; eig[k] = 4 sin^2(2 pi k/(4M-1)).
const float2 *dct_twiddles(int M);
const float *dct_eigen(int M);

// ---- per-angle Ewald geometry (host computed, FP64 rule inputs)
struct AngleGeom {
    double fx0, fy0, fz0;  // illumination frequency (1/m); fx0 = fm0 sin(AngY), fy0 = fm0 sin(AngX)
    float fx0s, fy0s, fz0s;  // the same divided by df (FP32 fast path)
    int valid;             // 0 when fm0^2 - fx0^2 - fy0^2 < 0 (the whole angle is skipped)
};

struct EwaldArgs {
    const float2 *U;        // A spectra, R*R each, [a][Ny][Nx]
    const AngleGeom *geom;  // A entries
    int A, R;
    double fm0, df, fm02;
    float fm02s;            // (fm0/df)^2
    float dx;
    float2 *F2;             // R^3 out (k-space data, F/C/dx)
    float2 *G;              // R^3 out (F2 after the z inverse transform)
    uint32_t *counts;       // optional R^3 hit counts
    uint8_t *mask;          // optional R^3 hit mask (1 where counts > 0)
    // frequency interpolation between scan angles (FI mapping) when fi_theta is set:
    // fi_theta = the A scan angles ascending (rad), fi_frame = the frame of each
    const double *fi_theta;
    const int *fi_frame;
};

struct LoopArgs {
    float2 *G;
    const float2 *F2;
    const uint8_t *mask;
    float2 *out;            // final RI volume (octant shifted), only for the final pass
    int R;
    float inv_n3, k2, n_med, n_med2;
    float s1;   // -1 / (R^3 k^2)
    float s2;   // -k^2 / n_med^2
    int *err;   // device status word: a bounded wait that ran out records a nonzero code
    int staged; // z pass: F2 / mask tiles staged by TMA (set by the launcher)
    // measured samples packed per z-pass tile (TB = the z plan's lines per CTA):
    // tmask[tile * R + z] bit b = voxel (x0 + b, y, z) keeps its measured value,
    // tcount[tile] = kept samples, tvals + tile * TB * R = the kept values in (z, b)
    // order.  packed = 0: the z pass reads F2 / mask instead.
    const uint32_t *tmask;
    const int *tcount;
    const int *tprefix;     // tprefix[tile * R + z]: kept samples of the tile before row z
    const float2 *tvals;
    int packed;
    // accelerated loop (projected FISTA): the pass that applies est_n and modify keeps
    // the projected iterate x_k in xprev and sends w_k = x_k + beta (x_k - x_{k-1}) on
    // to the forward transform; xprev == nullptr: the plain loop
    float2 *xprev;
    float beta;
};

// Packs F2 (mode 0: re != 0 && im != 0; mode 1: mask != 0) into per-tile masks,
// counts, row prefixes and values for the z pass (TB lines per tile, 8, 16 or 32).
cudaError_t pack_measured(const float2 *F2, const uint8_t *mask, int R, int TB, uint32_t *tmask, int *tcount,
                          int *tprefix, float2 *tvals, cudaStream_t s);

cudaError_t launch_ewald(const EwaldArgs &a, cudaStream_t s);
cudaError_t launch_xpass(const LoopArgs &a, bool final_pass, cudaStream_t s);
cudaError_t launch_ypass(const LoopArgs &a, bool inverse, cudaStream_t s);
cudaError_t launch_zpass(const LoopArgs &a, int check_mode, cudaStream_t s);

// Positivity-loop passes by plan variant (one translation unit per volume side).
enum LoopKind { LOOP_X = 0, LOOP_X_FINAL = 1, LOOP_Y_FWD = 2, LOOP_Y_INV = 3, LOOP_Z = 4 };
cudaError_t loop_pass_32(int kind, int variant, const LoopArgs &a, int flag, cudaStream_t s);
cudaError_t loop_pass_64(int kind, int variant, const LoopArgs &a, int flag, cudaStream_t s);
cudaError_t loop_pass_128(int kind, int variant, const LoopArgs &a, int flag, cudaStream_t s);
cudaError_t loop_pass_256(int kind, int variant, const LoopArgs &a, int flag, cudaStream_t s);
cudaError_t loop_pass_384(int kind, int variant, const LoopArgs &a, int flag, cudaStream_t s);
cudaError_t loop_pass_512(int kind, int variant, const LoopArgs &a, int flag, cudaStream_t s);
cudaError_t loop_pass_768(int kind, int variant, const LoopArgs &a, int flag, cudaStream_t s);
int loop_ztile_32(int variant);
int loop_ztile_64(int variant);
int loop_ztile_128(int variant);
int loop_ztile_256(int variant);
int loop_ztile_384(int variant);
int loop_ztile_512(int variant);
int loop_ztile_768(int variant);
// Tile width (lines per CTA) of the z pass in use for side R when it reads packed
// measured samples, else 0.
int loop_ztile(int R);
// Number of plan variants of the loop passes for volume side R (0: unsupported).
int loop_plan_count(int R);
cudaError_t loop_pass_variant(int kind, int variant, const LoopArgs &a, int flag, cudaStream_t s);
// Autotuner (tune.cu): tunes volume side R on this device on first use.
cudaError_t ensure_tuned(int R, int check_mode, cudaStream_t s);
// (kernel, device) pairs whose launch attributes have been set.
bool kernel_configured(const void *fn, int dev);
void mark_kernel_configured(const void *fn, int dev);

// Plane pass (plane_pass.cuh): x and y transforms of whole planes in thread-block
// clusters; sides without one return cudaErrorNotSupported / 0 clusters.
cudaError_t plane_pass_256(const LoopArgs &a, bool final_pass, int variant, cudaStream_t s);
int plane_clusters_256();
cudaError_t plane_pass_512(const LoopArgs &a, bool final_pass, int variant, cudaStream_t s);
int plane_clusters_512();
// Loop scheme of side R on this device: 0 = x / y / z / y passes, 1 and 2 = plane + z
// passes (two cluster sizes per plane: 8 and 4 CTAs at R = 256, 16 and 8 at R = 512).
int loop_scheme(int R);
cudaError_t launch_plane(const LoopArgs &a, bool final_pass, cudaStream_t s);

// ---- ASD-POCS with total-variation steepest descent (k_pocs.cu)
// Controller of one run in device memory: kernels read the step sizes from it and the
// last block of each reduction updates it, so an iteration launches no host work.
struct PocsCtl {
    double beta, dtvg, dp, dd, dg, gnorm;
    double alpha, alpha_red, r_max, eps_data, beta_red;
    int first, it, n_hist, pad_;
    unsigned int ticket;
};
struct PocsBufs {
    float *V, *g, *V2, *g2, *Vp;   // real R^3 volumes (contrast, TV gradient, ping-pong, POCS result)
    float2 *G;                     // complex R^3 work volume
    const float2 *F2;              // measured k-space data (zero where nothing was measured)
    double *part;                  // per-block partial sums (pocs_partials(R))
    PocsCtl *ctl;
    double *hist;                  // 4 doubles per iteration: Dp, Dd, Dg, the TV step used
    int R;
    float y_scale;                 // -1 / k^2: F2 -> spectrum of the contrast
    float tv_eps;
};
// Partial-sum slots a run of side R needs.
int pocs_partials(int R);
cudaError_t pocs_iteration(const PocsBufs &b, int tv_steps, bool want_dd, cudaStream_t s);
// After the last iteration: one more data-consistency step, then n = n_med sqrt(1 + V)
// with Re n >= n_med, Im n >= 0, octant shifted into ri.
cudaError_t pocs_finish(const PocsBufs &b, float n_med, float2 *ri, cudaStream_t s);

// Generic batched transforms.  rows: nlines contiguous lines of length L.
// cols: lines of length L with element p at (l % nx) + (l / nx) * plane + p * ld.
cudaError_t fft_rows(float2 *data, int L, long nlines, bool inverse, cudaStream_t s);
cudaError_t fft_cols(float2 *data, int L, long nlines, int nx, long plane, long ld, bool inverse,
                     cudaStream_t s);
// 3-D transform in place (cuFFT3D semantics: inverse scaled by 1/(R^3)).
cudaError_t fft3d(float2 *data, int R, bool inverse, cudaStream_t s);
cudaError_t scale_complex(float2 *data, long n, float s, bool conjugate, cudaStream_t st);

}  // namespace ctdm
