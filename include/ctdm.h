/*
 * ctdm.h -- C ABI of the GB300-native cTDM reconstruction library (libctdm_gb300.so).
 *
 * Two groups of entry points:
 *
 *  1. Drop-in symbols with the names and argument lists of the reference
 *     (y-h-Lin/cTDM) functions on the hologram -> refractive-index path, so a
 *     reference driver links against this library instead of its own .cu files.
 *     Like the reference they return void; failures are reported through
 *     ctdm_last_error() (thread-local, empty string when the last call succeeded).
 *     They run on the legacy default stream and synchronise before returning.
 *
 *  2. The native API (ctdm_*): explicit context, explicit stream, status codes,
 *     caller-owned buffers, no hidden global state.
 *
 * Complex data is interleaved float32 (re, im), layout-compatible with
 * cufftComplex / float2.  2-D arrays are x-fastest (element (i, j) at i + W*j),
 * volumes at i + W*j + W*H*k, as in the reference.
 */
#ifndef CTDM_H
#define CTDM_H

#include <stddef.h>
#include <stdint.h>
#ifndef __cplusplus
#include <stdbool.h>
#endif

#if defined(CTDM_BUILD) && defined(__GNUC__)
#define CTDM_API __attribute__((visibility("default")))
#else
#define CTDM_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    float x, y;
} ctdm_cfloat;

typedef enum {
    CTDM_OK = 0,
    CTDM_ERR_INVALID = 1,     /* bad argument or unsupported size */
    CTDM_ERR_CUDA = 2,        /* CUDA runtime error (message in ctdm_last_error) */
    CTDM_ERR_NOMEM = 3,       /* device or host allocation failed */
    CTDM_ERR_IO = 4,          /* file could not be read or written */
    CTDM_ERR_STALLED = 5,     /* Goldstein flood fill stopped early (see ctdm_goldstein) */
    CTDM_ERR_TIMEOUT = 6      /* a bounded device-side wait ran out */
} ctdm_status;

typedef struct ctdm_ctx ctdm_ctx;

/* Unwrap modes: the reference's inverse DCT twiddle (quirk kept) or the exact DCT-III. */
#define CTDM_UNWRAP_REF 0
#define CTDM_UNWRAP_EXACT 1
/* Data-replacement predicate in the positivity loop: the reference's
 * (F2.re != 0 && F2.im != 0) or the Ewald hit mask. */
#define CTDM_CHECK_REF 0
#define CTDM_CHECK_MASK 1
/* Phase retrieval (the reference's QPI_Method values, cTDM/HilbertTransform.cu:27):
 * Algorithm B = 1-D filtering of y-downsampled rows (the reference's default), Algorithm A
 * = 2-D window of the hologram spectrum (the default here). */
#define CTDM_QPI_B 0
#define CTDM_QPI_A 1
/* Which unwrapped phase feeds the reconstruction. */
#define CTDM_METHOD_DCT 0
#define CTDM_METHOD_FAST 1
#define CTDM_METHOD_GOLDSTEIN 2

typedef struct {
    int n_holo;          /* hologram side N (power of two, 64..2048) */
    int m_crop;          /* window side M (0: N/4) */
    int r_vol;           /* volume side R (32, 64, 128, 256, 384, 512, 768) */
    int iterations;      /* positivity loop bodies (the reference runs IterTime + 1) */
    int unwrap_mode;     /* CTDM_UNWRAP_REF / CTDM_UNWRAP_EXACT */
    int check_mode;      /* CTDM_CHECK_REF / CTDM_CHECK_MASK */
    int unwrap_method;   /* CTDM_METHOD_* */
    int run_goldstein;   /* 1: also run Goldstein residues, cuts and flood fill per angle */
    int bg_per_angle;    /* 1: one background hologram per angle, 0: one shared */
    int carrier_r, carrier_c, carrier_radius; /* window centre row/col and radius; < 0: detect */
    double n_med;        /* medium refractive index */
    double wavelength;   /* vacuum wavelength (m) */
    double dx;           /* reconstruction voxel (m) */
    int qpi_method;      /* reference QPI_Method numbering: CTDM_QPI_B (0) or CTDM_QPI_A (1, default) */
    int accelerated;     /* 0: the reference's positivity loop; 1: the same projection step with
                            Nesterov momentum (see ctdm_positivity_ex); no reference counterpart */
} ctdm_params;

/* Default parameters (reference defaults where they exist). */
CTDM_API void ctdm_params_default(ctdm_params *p);
/* Upper bound of the device memory a context holds for one device-buffer reconstruction
 * of this job (ctdm_reconstruct_device; host-buffer calls add the uploaded holograms and
 * two volumes), for a caller's own admission of tomograms by free memory.  No reference
 * counterpart. */
CTDM_API ctdm_status ctdm_workspace_bytes(const ctdm_params *p, int n_angles, size_t *bytes);

CTDM_API const char *ctdm_last_error(void);
CTDM_API const char *ctdm_version(void);

CTDM_API ctdm_status ctdm_ctx_create(int device, ctdm_ctx **out);
CTDM_API void ctdm_ctx_destroy(ctdm_ctx *ctx);
/* Carrier {row, col, radius} used by the last pipeline / ctdm_qpi call. */
CTDM_API ctdm_status ctdm_ctx_carrier(ctdm_ctx *ctx, int *carrier3);
/* Device buffers of the last pipeline call (valid until the next call or destroy):
 * which = 0 phase (A*M*M f32), 1 amp, 2 unwrapped phase, 3 Goldstein charges (i8),
 * 4 Goldstein cuts (u8), 5 Goldstein unwrapped (f32), 6 spectra U (A*R*R c64),
 * 7 F2 (R^3 c64), 8 hit counts (R^3 u32, only with CTDM_CHECK_MASK). */
CTDM_API ctdm_status ctdm_ctx_buffer(ctdm_ctx *ctx, int which, void **dptr, size_t *bytes);
/* Copies min(bytes, size) of buffer `which` (see ctdm_ctx_buffer) to host memory (synchronous). */
CTDM_API ctdm_status ctdm_ctx_read_buffer(ctdm_ctx *ctx, int which, void *host, size_t bytes);
/* Stage timing with CUDA events on the call's stream (off by default).  Stages:
 * 0 QPI, 1 unwrap, 2 Goldstein, 3 spectra (prep + FFT2), 4 Ewald mapping,
 * 5 y inverse pass, 6 x pass (loop), 7 y forward pass, 8 z pass, 9 final x pass.
 * ms[i]: device time of stage i summed over the pipeline calls made since timing was
 * switched on (set_timing(1) restarts the sums); counts[i]: number of launches of
 * that stage (may be NULL).  Up to 16383 stage marks and 1024 side-stream intervals
 * are kept; later ones are not recorded. */
CTDM_API ctdm_status ctdm_ctx_set_timing(ctdm_ctx *ctx, int on);
CTDM_API ctdm_status ctdm_ctx_stage_times(ctdm_ctx *ctx, double *ms, int *counts, int n);
/* Status word of the context's bounded device-side waits: 0, or the code of a wait
 * that ran out since the last read (1: a TMA tile of the positivity loop's dense z
 * pass did not arrive, 3: one of its packed z pass, 9: ctdm_ctx_probe_wait).
 * Synchronises the device; reading clears it.  A submitted call that saw a code makes
 * ctdm_wait return CTDM_ERR_TIMEOUT (and clears it). */
CTDM_API ctdm_status ctdm_ctx_device_status(ctdm_ctx *ctx, int *status);
/* Device bytes the context's workspace holds now (its buffers grow to the largest call
 * and are kept). */
CTDM_API ctdm_status ctdm_ctx_workspace(ctdm_ctx *ctx, size_t *bytes);
/* Diagnostic (no reference counterpart): one device-side wait that nothing completes,
 * on an mbarrier with the bounded wait the z pass uses for its TMA tiles, `polls`
 * polls long (<= 0: that wait's production bound).  The wait runs out, records code 9
 * in the status word above and the kernel returns (no copy was issued, so none is left
 * in flight); the context stays usable.  ms (may be NULL) receives the wait's length.
 * Synchronises the device. */
CTDM_API ctdm_status ctdm_ctx_probe_wait(ctdm_ctx *ctx, int polls, double *ms);
/* Number of kernels this library has launched in the process so far (a batch graph
 * launch counts the kernels captured in it). */
CTDM_API unsigned long long ctdm_launch_count(void);

/* --- whole path (replaces HilbertTransform's per-frame loop + BatchRecon) --- */
/* Device-resident inputs: d_holo (A*N*N f32), d_bg (N*N or A*N*N f32), angles on
 * the host (A f32 each, radians).  d_ri: R^3 complex RI volume, octant-shifted like
 * the reference's output.  stream: cudaStream_t (NULL = legacy default). */
CTDM_API ctdm_status ctdm_reconstruct_device(ctdm_ctx *ctx, const ctdm_params *p, int n_angles, const float *d_holo,
                                    const float *d_bg, const float *h_angx, const float *h_angy,
                                    ctdm_cfloat *d_ri, void *stream);
/* Same with host buffers: copies in, reconstructs, copies the volume out, waits.  The
 * holograms go over the host link in chunks of angles while the front end of the
 * earlier chunks runs; pinned host memory lets the copies overlap. */
CTDM_API ctdm_status ctdm_reconstruct(ctdm_ctx *ctx, const ctdm_params *p, int n_angles, const float *h_holo,
                             const float *h_bg, const float *h_angx, const float *h_angy, ctdm_cfloat *h_ri);
/* The same for integer camera frames (16- or 8-bit counts, as the reference's BMP frames
 * are): uploaded as they are (a half or a quarter of the float bytes) and converted to
 * float on the GPU; the result equals ctdm_reconstruct on the same values as floats. */
CTDM_API ctdm_status ctdm_reconstruct_u16(ctdm_ctx *ctx, const ctdm_params *p, int n_angles, const uint16_t *h_holo,
                                          const uint16_t *h_bg, const float *h_angx, const float *h_angy,
                                          ctdm_cfloat *h_ri);
CTDM_API ctdm_status ctdm_reconstruct_u8(ctdm_ctx *ctx, const ctdm_params *p, int n_angles, const uint8_t *h_holo,
                                         const uint8_t *h_bg, const float *h_angx, const float *h_angy,
                                         ctdm_cfloat *h_ri);
/* The host-buffer call without the wait, for a stream of tomograms (no reference
 * counterpart): enqueues the reconstruction and returns.  bytes_per_count: 4 (float),
 * 2 (uint16) or 1 (uint8) per hologram pixel.  The host buffers must stay valid, and
 * h_ri unread, until ctdm_wait returns.  Calls in flight overlap: a call's uploads run
 * beside the previous call's loop once that call's front end has read the inputs, and
 * its volume download beside the next call's loop (the last call's in ctdm_wait); with
 * pageable buffers the copies do not overlap, the results are the same.  A refused call
 * leaves nothing in flight.  Submitted calls share the context's device buffers: until
 * ctdm_wait returns, the context serves ctdm_submit alone, and its other entry points
 * (stages, device-buffer reconstructions, buffer reads) return CTDM_ERR_INVALID without
 * doing anything (another context serves other work meanwhile).  ctdm_reconstruct* is
 * ctdm_submit + ctdm_wait. */
CTDM_API ctdm_status ctdm_submit(ctdm_ctx *ctx, const ctdm_params *p, int n_angles, const void *h_holo,
                                 const void *h_bg, int bytes_per_count, const float *h_angx, const float *h_angy,
                                 ctdm_cfloat *h_ri);
/* Waits for every call submitted on ctx; CTDM_ERR_TIMEOUT when a bounded device-side
 * wait ran out in any of them. */
CTDM_API ctdm_status ctdm_wait(ctdm_ctx *ctx);

/* --- batched reconstruction (no reference counterpart) ----------------------------
 * Many independent tomograms, each with its own sizes and angle count, scheduled over
 * `lanes` concurrent workspaces and captured into one CUDA graph: ctdm_batch_run is a
 * single graph launch for the whole batch.  ctdm_batch_plan validates every job, runs
 * the batch once eagerly (allocating each lane's workspace for its largest job; the
 * outputs of that run are valid results), then captures the same launches.  The plan
 * keeps the job pointers: to reconstruct new data, overwrite the same input buffers
 * and run again.  Angles are copied at plan time.  The reference's one-tomogram path
 * is BatchRecon (cTDM/HilbertTransform.cu:1825-2047). */
typedef struct {
    ctdm_params params;
    int n_angles;
    const float *d_holo;   /* A*N*N f32, device */
    const float *d_bg;     /* N*N (or A*N*N with bg_per_angle) f32, device */
    const float *h_angx;   /* A f32 radians, host */
    const float *h_angy;
    ctdm_cfloat *d_ri;     /* R^3 complex out, device, octant-shifted */
} ctdm_job;
typedef struct ctdm_batch ctdm_batch;
CTDM_API ctdm_status ctdm_batch_create(int device, int lanes, ctdm_batch **out);
CTDM_API void ctdm_batch_destroy(ctdm_batch *batch);
CTDM_API ctdm_status ctdm_batch_plan(ctdm_batch *batch, const ctdm_job *jobs, int n_jobs);
/* One graph launch on `stream` (cudaStream_t, NULL = legacy default). */
CTDM_API ctdm_status ctdm_batch_run(ctdm_batch *batch, void *stream);
/* The planned schedule launched kernel by kernel (no graph), for comparison. */
CTDM_API ctdm_status ctdm_batch_run_eager(ctdm_batch *batch, void *stream);
/* Admission by free device memory (no reference counterpart; the reference chooses its
 * ReconMode from free memory, cTDM/HilbertTransform.cu:1932-1939): ctdm_batch_plan bounds
 * every job's workspace (ctdm_workspace_bytes), keeps back 24 R^3 + 256 MiB bytes for
 * the autotuner's scratch volumes, and uses only as many of the batch's lanes as fit in
 * the device memory that is free plus what its lanes already hold, at most `bytes` when a
 * limit is set (0: no limit); lanes left out give their buffers back.  A plan whose
 * largest job does not fit alone returns CTDM_ERR_NOMEM before it allocates anything. */
CTDM_API ctdm_status ctdm_batch_set_memory_limit(ctdm_batch *batch, size_t bytes);
/* The last plan's admission: lanes used, workspace bound of its largest job, and the
 * memory the plan could use. */
CTDM_API ctdm_status ctdm_batch_admission(const ctdm_batch *batch, int *lanes_used, size_t *bytes_per_lane,
                                          size_t *bytes_available);
/* Lane each job was assigned to (longest job first onto the least-loaded lane). */
CTDM_API ctdm_status ctdm_batch_lanes(const ctdm_batch *batch, int *lane_of_job, int n_jobs);

/* --- autotuner of the positivity-loop passes (no reference counterpart) -------------
 * Each volume side has ctdm_plan_count(R) FFT plan variants (lines per CTA, threads per
 * line, radix sequence) for each of the x, y and z passes.  The first reconstruction
 * of a side on a device times them all on scratch volumes and keeps the fastest per
 * pass (the call synchronises the device once; set CTDM_AUTOTUNE=0 to keep variant 0).
 * Variants differ in rounding at the float32 ulp level only. */
CTDM_API int ctdm_plan_count(int R);
/* Tune now: variants3 (may be NULL) receives the x, y, z choice; ms (may be NULL)
 * receives the median time of pass p, variant v at ms[3 * p + v] (n_ms entries). */
CTDM_API ctdm_status ctdm_autotune(int device, int R, int check_mode, int *variants3, double *ms, int n_ms);
/* Current choice for (device, R); tuned = 1 when it came from the autotuner. */
/* Lines per tile of the z pass's packed measured samples with the current plan of
 * (device, R); 0 when that plan reads the measured data densely. */
CTDM_API ctdm_status ctdm_z_tile(int device, int R, int *lines);
CTDM_API ctdm_status ctdm_plans(int device, int R, int *variants3, int *tuned);
/* Pin a choice (also disables tuning of that side on that device). */
CTDM_API ctdm_status ctdm_set_plans(int device, int R, const int *variants3);
/* Loop scheme of side R: 0 = x / y / z / y line passes (72 R^3 bytes per iteration);
 * 1, 2 = plane pass (x and y transforms of whole planes by 8-CTA thread-block clusters,
 * each plane kept in L2 between its row and column phases; register targets of 3 and
 * 4 CTAs per SM) + z pass (40 R^3 bytes).  The plane schemes exist for R = 256; scheme 1
 * is the default where the device can co-schedule the clusters, and the autotuner
 * keeps the fastest.  ctdm_autotune's ms[9..11] (when n_ms > 11) receive one
 * iteration of schemes 0, 1 and 2. */
CTDM_API ctdm_status ctdm_loop_scheme(int device, int R, int *scheme);
CTDM_API ctdm_status ctdm_set_loop_scheme(int device, int R, int scheme);

/* --- stages (device pointers) --- */
/* QPI Algorithm A.  carrier3: in {row, col, radius} (any < 0: detect from the first
 * background), out: the carrier used. */
CTDM_API ctdm_status ctdm_qpi(ctdm_ctx *ctx, int N, int M, int A, const float *d_holo, const float *d_bg, int bg_per_angle,
                     int *carrier3, float *d_phase, float *d_amp, void *stream);
/* QPI Algorithm B (extractQPI_AlgorithmB, cTDM/HilbertTransform.cu:1587-1660): phase and
 * amplitude maps of M = N/4 side, transposed like the reference's copySharedMem.
 * center2: in {column, column} (any < 0: detect), out {background column, frame-1
 * column}: the reference takes frame 1's column from frame 1's own spectrum and every
 * later frame's from the background's.  Synchronises the stream. */
CTDM_API ctdm_status ctdm_qpi_b(ctdm_ctx *ctx, int N, int A, const float *d_holo, const float *d_bg, int bg_per_angle,
                                int *center2, float *d_phase, float *d_amp, void *stream);
CTDM_API ctdm_status ctdm_unwrap_dct(ctdm_ctx *ctx, int A, int M, int mode, const float *d_phi, float *d_out, void *stream);
/* FastUnwrapping: d_phi is normalised in place like the reference. */
CTDM_API ctdm_status ctdm_unwrap_fast(ctdm_ctx *ctx, int A, int M, float *d_phi, float *d_out, void *stream);
/* Goldstein: residue charges (-1/0/+1), branch-cut mask (0/1), flood-filled phase.
 * h_status (A ints, may be NULL): 0 done, 1 sweep limit reached, 2 stalled. */
CTDM_API ctdm_status ctdm_goldstein(ctdm_ctx *ctx, int A, int W, int H, const float *d_phi, int8_t *d_charges,
                           uint8_t *d_cuts, float *d_out, int *h_status, void *stream);
/* Flood fill alone with caller-provided branch cuts (0/1 per pixel). */
CTDM_API ctdm_status ctdm_goldstein_fill(ctdm_ctx *ctx, int A, int W, int H, const uint8_t *d_cuts, const float *d_phi,
                                         float *d_out, int *h_status, void *stream);
/* Entries per list (16..3072; 0: the default 1024) that the flood fill of maps of up
 * to 96 Ki pixels keeps in shared memory; a fill whose list outgrows them starts over
 * on global lists, with the same result.  Applies to later launches in the process. */
CTDM_API ctdm_status ctdm_set_fill_list_capacity(int capacity);
/* Resize M -> N, centre crop R, median + checkMaps, u = log A + i phi (transposed,
 * quadrant-swapped), forward FFT2: d_U (A*R*R complex). */
CTDM_API ctdm_status ctdm_prepare_spectra(ctdm_ctx *ctx, int A, int M, int N, int R, const float *d_phase,
                                 const float *d_amp, ctdm_cfloat *d_U, void *stream);
/* The same from R x R phase/amp stacks (BatchRecon's input). */
CTDM_API ctdm_status ctdm_stack_spectra(ctdm_ctx *ctx, int A, int R, const float *d_ph, const float *d_am,
                               ctdm_cfloat *d_U, void *stream);
/* Resize + crop + median + checkMaps only (phase/amp stacks out). */
CTDM_API ctdm_status ctdm_prepare_stack(ctdm_ctx *ctx, int A, int M, int N, int R, const float *d_phase, const float *d_amp,
                               float *d_ph_out, float *d_am_out, void *stream);
/* Ewald-cap mapping of all angles + F2 = F/C/dx.  d_counts may be NULL. */
CTDM_API ctdm_status ctdm_map_ewald(ctdm_ctx *ctx, int A, int R, const ctdm_cfloat *d_U, const float *h_angx,
                           const float *h_angy, double fm0, double df, double dx, ctdm_cfloat *d_F2,
                           uint32_t *d_counts, void *stream);
/* Positivity loop from F2: iterations loop bodies, octant-shifted RI out.
 * d_counts required for CTDM_CHECK_MASK (else may be NULL). */
CTDM_API ctdm_status ctdm_positivity(ctdm_ctx *ctx, int R, int iterations, int check_mode, double k2, double n_med,
                            const ctdm_cfloat *d_F2, const uint32_t *d_counts, ctdm_cfloat *d_ri, void *stream);
/* The same loop with accelerated = 1 (no reference counterpart): projected FISTA at
 * lambda 0 and unit step, fused into the loop passes.  The pass that applies est_n and
 * modify keeps the projected iterate x_k and sends x_k + beta_k (x_k - x_{k-1}) to the
 * forward transform, beta_k = (t_{k-1} - 1) / t_k, t_0 = 1,
 * t_k = (1 + sqrt(1 + 4 t_{k-1}^2)) / 2 (beta_1 = 0); the output is the RI of the next
 * projected iterate.  It is ctdm_reconstruct_gradient_ex(positivity = 1, lambda = 0,
 * step = 1) run with iterations + 1 steps, at one extra read and write of R^3 values
 * per iteration.  accelerated = 0 is ctdm_positivity. */
CTDM_API ctdm_status ctdm_positivity_ex(ctdm_ctx *ctx, int R, int iterations, int check_mode, int accelerated,
                                        double k2, double n_med, const ctdm_cfloat *d_F2, const uint32_t *d_counts,
                                        ctdm_cfloat *d_ri, void *stream);
/* --- ASD-POCS with total variation (BatchReconPOCS, cTDM/HilbertTransform.cu:2049-2402,
 * cTDM/Recon_kernel.cu:414-1106, with its mathematics fixed) -------------------------
 * Frequency-interpolation mapping: like ctdm_map_ewald for a one-axis scan of tilts
 * h_angx (AngY taken as zero), each voxel's value interpolated linearly in angle
 * between the two scan angles around the angle whose cap passes exactly through the
 * voxel centre (FrquencyInterpolation / FI_kernel). */
CTDM_API ctdm_status ctdm_map_fi(ctdm_ctx *ctx, int A, int R, const ctdm_cfloat *d_U, const float *h_angx, double fm0,
                                 double df, double dx, ctdm_cfloat *d_F2, uint32_t *d_counts, void *stream);
typedef struct {
    int iterations;                  /* outer iterations (reference 100) */
    int tv_steps;                    /* TV steepest-descent steps per iteration (20) */
    double beta, beta_red;           /* data-step relaxation and its decay (1.0, 0.995) */
    double alpha, alpha_red, r_max;  /* TV step = alpha Dp, reduced by alpha_red when Dg > r_max Dp */
    double eps_data;                 /* data tolerance of the reduction rule (0) */
    double tv_eps;                   /* TV smoothing in contrast units (1e-8) */
} ctdm_pocs_params;
CTDM_API void ctdm_pocs_defaults(ctdm_pocs_params *p);
/* ASD-POCS from F2 (zero where nothing was measured): octant-shifted RI volume like
 * ctdm_positivity.  h_hist (may be NULL; synchronises when given): 4 doubles per
 * iteration, the data-step distance Dp, the data residual Dd, the TV distance Dg and
 * the TV step used. */
CTDM_API ctdm_status ctdm_pocs(ctdm_ctx *ctx, int R, const ctdm_pocs_params *p, double k2, double n_med,
                               const ctdm_cfloat *d_F2, ctdm_cfloat *d_ri, double *h_hist, void *stream);

/* --- differentiable form (no reference counterpart) ---------------------------------
 * Measurement operator A = P F~: unitary 3-D FFT (F / R^{3/2}) then sampling at the
 * measured voxels of the Ewald caps.  V is the contrast f / (-k^2) of the reference's
 * scattering potential (n = n_med sqrt(1 + V)).  The tape keeps the sorted measured
 * voxel indices and the data y = F2 / (-k^2 R^{3/2}); forward/backward are shaped like
 * a torch.autograd.Function (backward = A^H, recomputing the transform).  Gradients
 * use the conjugate-Wirtinger convention dL/dRe V + i dL/dIm V. */
typedef struct ctdm_tape ctdm_tape;
/* Measured voxels: d_counts > 0 when given, else the reference predicate on F2. */
CTDM_API ctdm_status ctdm_tape_create(int device, int R, const ctdm_cfloat *d_F2, const uint32_t *d_counts, double k2,
                                      ctdm_tape **out);
CTDM_API void ctdm_tape_destroy(ctdm_tape *tape);
CTDM_API long ctdm_tape_samples(const ctdm_tape *tape);
CTDM_API ctdm_status ctdm_tape_data(const ctdm_tape *tape, ctdm_cfloat *h_y, uint32_t *h_idx);
/* y (S complex) = A V */
CTDM_API ctdm_status ctdm_forward(ctdm_tape *tape, const ctdm_cfloat *d_V, ctdm_cfloat *d_y, void *stream);
/* dL/dV (R^3 complex) = A^H dL/dy */
CTDM_API ctdm_status ctdm_backward(ctdm_tape *tape, const ctdm_cfloat *d_gy, ctdm_cfloat *d_gV, void *stream);
/* L = 1/2 ||A V - y||^2 + lambda TV_eps(V) and its gradient (synchronous). */
CTDM_API ctdm_status ctdm_loss_grad(ctdm_tape *tape, const ctdm_cfloat *d_V, double lambda, double eps,
                                    ctdm_cfloat *d_grad, double *loss);
/* Accelerated gradient descent (FISTA) on L from d_V (updated in place).  step <= 0
 * picks 1 / (1 + 12 lambda / eps).  h_loss (iterations doubles, may be NULL) receives
 * the objective per iteration (synchronises each iteration when given). */
CTDM_API ctdm_status ctdm_reconstruct_gradient(ctdm_tape *tape, int iterations, double lambda, double eps, double step,
                                               ctdm_cfloat *d_V, double *h_loss, void *stream);
/* The same with the positivity constraint of the reference's loop as a proximal step
 * (positivity = 1): each update is projected onto Re n >= n_med, Im n >= 0 for
 * n = n_med sqrt(1 + V).  With lambda = 0 and step 1 the iteration is the reference's
 * data-replacement / positivity loop with Nesterov momentum. */
CTDM_API ctdm_status ctdm_reconstruct_gradient_ex(ctdm_tape *tape, int iterations, double lambda, double eps,
                                                  double step, int positivity, ctdm_cfloat *d_V, double *h_loss,
                                                  void *stream);
/* n = n_med sqrt(1 + V), optional positivity clamp, octant-shifted like the reference output. */
CTDM_API ctdm_status ctdm_contrast_to_ri(int R, const ctdm_cfloat *d_V, double n_med, int clamp, ctdm_cfloat *d_ri,
                                         void *stream);

/* DCT least-squares unwrap that allocates nothing -- no counterpart in the reference.
 * For callers that cannot allocate device memory: an acquisition loop that must not
 * allocate once it runs, or a host that owns all GPU memory through its own pool.
 * The scratch map and the transform tables are file-scope __device__ arrays of the
 * library (about 16.1 MiB per GPU, held until the process exits).
 * Limits: M in {16, 32, 64, 128, 256}, A * M * M <= 4194304 points and mode 0 or 1;
 * other requests return CTDM_ERR_INVALID with a message in ctdm_last_error().  The
 * first call on a device loads the arrays there (under CUDA's default lazy module
 * loading that is when their 16.1 MiB is taken, not when the library is opened),
 * resolves their device addresses and fills the tables with synchronous copies: make
 * it as a warm-up before a memory pool claims the device's memory, before the loop
 * that must not allocate starts, and before any stream capture on that device.  All
 * calls share one scratch array, which keeps the last call's contents (nothing in
 * it needs clearing); calls that overlap on the GPU (other streams or threads) race
 * on it, so serialise them. */
CTDM_API ctdm_status ctdm_unwrap_dct_noalloc(int A, int M, int mode, const float *d_phi, float *d_out, void *stream);
/* Unnormalised batched FFT of the library's line lengths.  rank 1..3, dims
 * fastest-first; inverse = 1 uses exp(+i), no scaling. */
CTDM_API ctdm_status ctdm_fft(ctdm_cfloat *d_data, int rank, const int *dims, int batch, int inverse, void *stream);

/* --- on-disk formats and the JobList driver (cTDM/HilbertTransform.cu:70-175,
 * 327-1230, 1316-1544, 2437-2455, 2680-2731) ------------------------------------- */
/* 8-bit grey BMP as the reference's read_bmp stores it: header width at byte 18 read as
 * nr, height at 22 as nc, palette skipped, nr lines of nc bytes (padded to 4), bottom
 * line first, image[j * nr + i] = byte j of line i counted from the top.  image NULL:
 * only *width / *height are filled (bmp_header). */
CTDM_API ctdm_status ctdm_read_bmp(const char *path, int *width, int *height, uint8_t *image);
/* Per-frame map file (outputImg / openImage): 1-byte status, angle x and y (float64),
 * size x and y (int32), then size_x * size_y (phase, amp) float32 pairs, no padding. */
CTDM_API ctdm_status ctdm_write_phimap(const char *path, int status, double angle_x, double angle_y, int size_x,
                                       int size_y, const float *phase, const float *amp);
/* phase / amp may be NULL (header only). */
CTDM_API ctdm_status ctdm_read_phimap(const char *path, int *status, double *angle_x, double *angle_y, int *size_x,
                                      int *size_y, float *phase, float *amp);
/* dir/3D-RI-{Complex,Real,Imag}_RxRxR.rimap from a host R^3 volume; save_mode 0 complex64,
 * 1 real part, 2 imaginary part (float32). */
CTDM_API ctdm_status ctdm_write_rimap(const char *dir, int R, int save_mode, const ctdm_cfloat *h_ri);
/* Frame check (checkArray on the centre half of an N x N phase map with limit_std and
 * limit_range when resize_flag = 1, on the whole map with 0.5 and 5 pi when 0):
 * 1 when the frame is rejected. */
CTDM_API int ctdm_check_frame(const float *phase, int N, int resize_flag, double limit_std, double limit_range);
/* Illumination angle from an N x N angle-camera image (row-major, x fastest): the
 * first maximum of log10 |FFT2| (quadrant-swapped) over flat indices
 * [int(0.53 N^2), int(0.79 N^2)), fx = (N/2 - 1 - column) / (N pixel), sin theta =
 * mag fx n_med^-1 wavelength, angle = -sign(sin theta) |asin| (AngCal_GPU,
 * cTDM/HilbertTransform.cu:2920-2983, whose 511 and 1024 are N/2 - 1 and N at N = 1024).
 * peak (may be NULL) receives the flat index of the maximum. */
CTDM_API ctdm_status ctdm_angle_from_image(const float *h_img, int N, double n_med, double wavelength_nm, double mag,
                                           double camera_pixel_um, float *angle, long *peak);

/* One job of a JobList: the 20 ordered key=value fields of a parameter file
 * (cTDM/HilbertTransform.cu:96-120) and two optional trailing keys, QPI_Method and
 * IterTime, which the reference fixes at compile time (:25, :35). */
typedef struct {
    char sp_dir[256], bg_dir[256], ang_dir[256], save_dir[256];
    int row_pts[2], col_pts[2];
    int recon_flag;        /* 0 maps only, 1 maps + reconstruction, 2 reconstruction from saved maps */
    int recon_save;        /* .rimap content: 0 complex, 1 real, 2 imaginary */
    int size_type;         /* 0: R = 256, 1: R = 512 */
    int resize_flag;       /* 1: centre R x R window of the map, 0: bilinear resize to R */
    double n_med, mag, camera_pixel_um, wavelength_nm;
    int save_phase_stack, save_amp_stack; /* 1: also write Phase%03d_NxN.raw / Amp%03d_NxN.raw */
    double criteria_range, criteria_std;
    int qpi_method;        /* reference numbering: 0 Algorithm B (default), 1 Algorithm A */
    int iter_time;         /* BatchRecon runs iter_time + 1 loop bodies (default 100) */
} ctdm_job_file;

typedef struct {
    int frames;            /* frames found (Buffer*.bmp pairs, or saved buffer*.phimap files) */
    int rejected;          /* frames that failed the check */
    int recon_frames;      /* frames reconstructed (0: no reconstruction ran) */
    int n_holo;            /* hologram side */
    int recon_size;        /* volume side */
} ctdm_job_result;

/* The reference's defaults (cTDM/HilbertTransform.cu:11-35). */
CTDM_API void ctdm_job_defaults(ctdm_job_file *job);
/* Parses one parameter file (fields in the reference's order; spaces after '=' are
 * allowed; values end at white space, and a value containing '=' keeps its last
 * '='-separated piece, as the reference's obtainParameter does). */
CTDM_API ctdm_status ctdm_parse_job_file(const char *path, ctdm_job_file *job);
/* Runs one job like HilbertTransform with SpeedTestFlag = 0 (the mode that writes maps
 * and reconstructs): all frames' QPI, unwrapping and resizing run batched on the GPU;
 * buffer%03d.phimap per frame; reconstruction of the frames that pass the check.
 * Folders use '/'.  result may be NULL. */
CTDM_API ctdm_status ctdm_run_job(const ctdm_job_file *job, ctdm_job_result *result);

/* ------------------------------------------------------------------------- */
/* Drop-in replacements for the reference entry points (void, default stream) */
/* ------------------------------------------------------------------------- */
/* Reference globals consumed by BatchRecon / HilbertTransform
 * (cTDM/HilbertTransform.cu:11-35): ReconX=Y=Z, Nmed, wavelength (nm),
 * CameraPixelSize (um), Mag, IterTime, ReconSave, SaveDir. */
CTDM_API void ctdm_set_recon_globals(int recon_size, double n_med, double wavelength_nm, double camera_pixel_um, double mag,
                            int iter_time, int recon_save, const char *save_dir);

/* cTDM/HilbertTransform.cuh:170 (defined at HilbertTransform.cu:1546) -- host SP/BG
 * holograms as complex Nx*Ny arrays whose imaginary parts are zero (the reference's job
 * loop fills them that way; the imaginary parts are not read), Nx == Ny a power of two
 * of 64..2048.  The M x M fields (M = Nx/4) after the inverse transform, 1/M^2 and the
 * conjugation go to the device arrays cuSP_FFT / cuBG_FFT (the reference writes its
 * globals cuSP2 / cuBG2, which its call sites pass as these arguments).  frame == 1
 * detects the carrier from BG (rows from 600*N/1024, as obtainRadius does at N = 1024)
 * and keeps it per device for the later frames. */
CTDM_API void extractQPI_AlgorithmA(ctdm_cfloat *SP, ctdm_cfloat *BG, ctdm_cfloat *cuSP_FFT, ctdm_cfloat *cuBG_FFT, int Nx,
                                    int Ny, int frame);
/* cTDM/HilbertTransform.cu:1587 (declared in HilbertTransform.cuh) -- host SP/BG
 * holograms (Nx*Ny float, Nx == Ny), device fields out (Nx/4 * Ny/4).  frame == 1
 * detects the carrier columns (kept per device for the later frames). */
CTDM_API void extractQPI_AlgorithmB(float *SP, float *BG, ctdm_cfloat *cuSP_FFT, ctdm_cfloat *cuBG_FFT, int Nx, int Ny,
                                    int frame);
/* cTDM/DCT_Unwrapping.cuh:106 -- device pointers, sizeX == sizeY. */
CTDM_API void DCT_UWLS_Unwrapped(float *ImgDst, float *ImgSrc, int sizeX, int sizeY);
/* cTDM/FastUnwrapping.cuh:12 -- (src, dst) order; src is normalised in place. */
CTDM_API void FastUnwrapping(float *ImgSrc, float *ImgDst, int sizeX, int sizeY);
/* cTDM/Goldstein.cuh:41 */
CTDM_API void cudaGoldsteinUnwrap2D(float *cu_phi, float *cu_UnWrapPhase, int sizeX, int sizeY, int frameNumber);
/* cTDM/Recon_kernel.cuh:31 -- host stacks in, filtered device stacks out. */
CTDM_API void MedianFilter(float *PhaseData, float *AmpData, float *Phase_img, float *Amp_img, int nx, int ny, int nz);
/* cTDM/Recon_kernel.cuh:37 */
CTDM_API void CopyDataArray(ctdm_cfloat *u_sp, float *phase, float *amp, int sizeX, int sizeY, int sizeZ, int numZ);
/* cTDM/Recon_kernel.cuh:41 */
CTDM_API void EdwardSphere(ctdm_cfloat *u_sp, ctdm_cfloat *F, float *C, float fm0, float df, float AngX, float AngY, int sizeX,
                  int sizeY, int sizeZ);
/* cTDM/Recon_kernel.cuh:51 */
CTDM_API void initial_F_and_F2(float *C, ctdm_cfloat *cuF, ctdm_cfloat *cuF2, float recon_dx, int Image_Width,
                      int Image_Height, int Image_Slice);
/* cTDM/Recon_kernel.cuh:56 (device n; the reference's host mode 1 is not kept) */
CTDM_API void est_n_3D(ctdm_cfloat *n, ctdm_cfloat *F, float recon_k2, float recon_med, int Image_Width, int Image_Height,
              int Image_Slice);
/* cTDM/Recon_kernel.cuh:63 */
CTDM_API void modify_F_3D(ctdm_cfloat *n, ctdm_cfloat *F, float recon_k2, float recon_med, int Image_Width, int Image_Height,
                 int Image_Slice);
/* cTDM/Recon_kernel.cuh:70 */
CTDM_API void check_F_3D(ctdm_cfloat *F, ctdm_cfloat *F2, int Image_Width, int Image_Height, int Image_Slice);
/* cTDM/FFT.cuh:29 -- dir -1 forward, +1 inverse scaled by 1/(XYZ). */
CTDM_API void cuFFT3D(ctdm_cfloat *ImgArray, int sizeX, int sizeY, int sizeZ, int dir);
/* cTDM/FFT.cuh:25 -- dir -1 forward, +1 inverse scaled by 1/(XY) and conjugated. */
CTDM_API void cuFFT2D(ctdm_cfloat *ImgArray, int sizeX, int sizeY, int dir);
/* cTDM/HilbertTransform.cuh:133 (defined at HilbertTransform.cu:2049) --
 * host stacks and AngX scan angles; ASD-POCS with the reference's constants; writes
 * 3D-RI-*.raw into SaveDir as the reference does. */
CTDM_API void BatchReconPOCS(float *PhaseStack, float *AmpStack, float *sampleAngleRadX, float *sampleAngleRadY,
                             int ReconFrame);
/* cTDM/HilbertTransform.cu:70 -- each white-space separated entry of the job list is a
 * parameter file, parsed and run in turn.  Returns 0 when the list cannot be opened,
 * else 1; a failed job leaves its message in ctdm_last_error and the next job runs. */
CTDM_API int scriptFileRead(char *script);
/* cTDM/HilbertTransform.cuh:127 -- one job with the folders given and every other
 * field from the parameter file scriptFileRead parsed last (the reference's file-scope
 * globals), or the defaults.  rowSize, colSize, StartNo, SpaceNo and EndNo are not
 * used (the reference uses them only on its unreachable half-size branch). */
CTDM_API void HilbertTransform(char *SPDir, char *BGDir, char *AngDir, char *SaveDir, int rowPts[], int colPts[],
                               int rowSize, int colSize, int StartNo, int SpaceNo, int EndNo);
/* cTDM/HilbertTransform.cu:2920 -- host N x N angle image (sizeX == sizeY), optics
 * from the last parsed parameter file or the defaults. */
CTDM_API float AngCal_GPU(float *src, int sizeX, int sizeY, int frame, int totalFrame);
/* cTDM/HilbertTransform.cuh:158 (defined at HilbertTransform.cu:3056) -- true when the
 * standard deviation or the range exceeds its limit (also for NULL or size < 1). */
CTDM_API bool checkArray(float *array2D, float limitSTD, float limitRange, int size);
/* cTDM/HilbertTransform.cuh:132 -- host stacks (R*R*frames) and angles (radians);
 * reconstructs with the globals above and writes 3D-RI-*.rimap into SaveDir. */
CTDM_API void BatchRecon(float *PhaseStack, float *AmpStack, float *sampleAngleRadX, float *sampleAngleRadY, int ReconFrame);

#ifdef __cplusplus
}
#endif

#endif /* CTDM_H */
