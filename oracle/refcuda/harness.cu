// Comparison harness: runs the reference's own CUDA pipeline (y-h-Lin/cTDM, cuFFT) on a
// tomogram read from a file and writes the RI volume it produces, with its wall time.
//
// COMPARISON INFRASTRUCTURE ONLY: the product never links or runs it.  The compute is
// the reference's code, assembled unmodified by oracle/refcuda/assemble.py (whole
// FFT.cu, Recon_kernel.cu, DCT_Unwrapping.cu; extractQPI_AlgorithmA, obtainRadius,
// get1stOrder_new, calcWrapPhase and bilinear_interpolation_kernel cut from
// HilbertTransform.cu).  This file supplies what the reference's driver would: the
// file-scope globals those functions use (cTDM/HilbertTransform.cuh:68-110,
// cTDM/HilbertTransform.cu:11-51), their allocation and cuFFT plans
// (cTDM/HilbertTransform.cu:376-414,545-574), and the call sequence of the job loop
// for QPI_Method = 1 with SpeedTestFlag = 0 (:940-1130: QPI A, wrapped phase, DCT
// unwrap, bilinear resize, maps back to the host, Combine2Stack with ResizeFlag = 1,
// :1397-1427) followed by BatchRecon (:1825-2047, ReconMode 0).
//
// Two departures, both forced: the carrier (row, column, radius) is taken from the
// input instead of obtainRadius (:3425-3455), whose search starts at row 600 and finds
// nothing below 1024-pixel holograms (the input carries the same rule's result,
// rows from 600 N / 1024); and dx is taken from the input instead of
// CameraPixelSize / Mag * 1024 / ReconZ (:1854), so both sides reconstruct on one grid.
//
// Input (little-endian): "CTDMREF1", int32 N, R, A, iterations, carrier row, column,
// radius; float64 n_med, wavelength (m), dx (m); float32 angx[A], angy[A],
// background[N*N], holograms[A][N*N].  Output: R^3 complex64 (octant-shifted n, as
// BatchRecon exports it).  Usage: ref_pipeline <in> <out> <repetitions> [dump folder]
//
// With a dump folder the first repetition also writes the reference's intermediate
// arrays there (it is then left out of the timing): phase.f32 and amp.f32 (the wrapped
// phase and amplitude of calcWrapPhase, A * M * M), unwrapped.f32 (DCT_UWLS_Unwrapped),
// counts.f32 (the Ewald hit counts C, R^3) and f2.c64 (initial_F_and_F2's F2, R^3).
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <string>
#include <vector>

#include <cuda_runtime.h>
#include <cufft.h>

#include "DCT_Unwrapping.cuh"
#include "FFT.cuh"
#include "Recon_kernel.cuh"

// ---- file-scope globals of the reference's driver (cTDM/HilbertTransform.cuh:68-110)
int blocksInX, blocksInY, blocksInX2, blocksInY2, blocksInX3, blocksInY3, blocksInX4, blocksInY4;
int Nx2, Ny2;
int rCircle, cCircle, radiusCircle;
cufftComplex *cuSP, *cuBG, *cuSP2, *cuBG2;
cufftHandle plan_1D_C2C_FORWARD, plan_1D_C2C_INVERSE, plan_2D_C2C_FORWARD_s1, plan_2D_C2C_INVERSE_s2;
clock_t s_datatransfer, e_datatransfer, s_wrap, e_wrap, s_unwrap, e_unwrap;
float dataTransfer_time, wrap_time, unwrap_time;
float *LaplaceArray, *outX, *outY, *inX, *inY, *dst_DCT;
cufftComplex *dSrc_DCT_FORWARD, *dSrc_DCT_INVERSE;
int ReconSave = 0;
extern int ReconMode;   // defined in cTDM/Recon_kernel.cu:4

// ---- the reference's functions cut from cTDM/HilbertTransform.cu (qpi_a.cu)
void extractQPI_AlgorithmA(cufftComplex *SP, cufftComplex *BG, cufftComplex *cuSP_FFT, cufftComplex *cuBG_FFT, int Nx,
                           int Ny, int frame);
__global__ void calcWrapPhase(float *Phase, float *Amp, cufftComplex *SP, cufftComplex *BG, int sizeX, int sizeY);
__global__ void bilinear_interpolation_kernel(float *__restrict__ d_result_1, const float *__restrict__ d_data_1,
                                              float *__restrict__ d_result_2, const float *__restrict__ d_data_2,
                                              const int M1, const int N1, const int M2, const int N2);

#define CK(x)                                                                                   \
    do {                                                                                        \
        cudaError_t e_ = (x);                                                                   \
        if (e_ != cudaSuccess) {                                                                \
            std::fprintf(stderr, "%s:%d %s: %s\n", __FILE__, __LINE__, #x, cudaGetErrorString(e_)); \
            std::exit(3);                                                                       \
        }                                                                                       \
    } while (0)
#define CKF(x)                                                                                  \
    do {                                                                                        \
        cufftResult r_ = (x);                                                                   \
        if (r_ != CUFFT_SUCCESS) {                                                              \
            std::fprintf(stderr, "%s:%d %s: cuFFT error %d\n", __FILE__, __LINE__, #x, (int)r_); \
            std::exit(3);                                                                       \
        }                                                                                       \
    } while (0)

struct Input {
    int N = 0, R = 0, A = 0, iters = 0, car[3] = {0, 0, 0};
    double n_med = 0, wavelength = 0, dx = 0;
    std::vector<float> angx, angy, bg, holo;
};

static bool read_input(const char *path, Input &in)
{
    FILE *f = std::fopen(path, "rb");
    if (!f) return false;
    char magic[8];
    int32_t h[7];
    double d[3];
    bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, "CTDMREF1", 8) == 0 &&
              std::fread(h, sizeof h, 1, f) == 1 && std::fread(d, sizeof d, 1, f) == 1;
    if (ok) {
        in.N = h[0], in.R = h[1], in.A = h[2], in.iters = h[3];
        in.car[0] = h[4], in.car[1] = h[5], in.car[2] = h[6];
        in.n_med = d[0], in.wavelength = d[1], in.dx = d[2];
        const size_t nn = (size_t)in.N * in.N;
        ok = in.N >= 128 && in.N <= 2048 && (in.N & (in.N - 1)) == 0 && in.R >= 32 && in.R <= in.N &&
             in.R % 32 == 0 && in.A >= 1 && in.A <= 1024 && in.iters >= 1;
        if (ok) {
            in.angx.resize(in.A), in.angy.resize(in.A), in.bg.resize(nn), in.holo.resize(nn * in.A);
            ok = std::fread(in.angx.data(), 4, in.A, f) == (size_t)in.A &&
                 std::fread(in.angy.data(), 4, in.A, f) == (size_t)in.A && std::fread(in.bg.data(), 4, nn, f) == nn &&
                 std::fread(in.holo.data(), 4, nn * in.A, f) == nn * in.A;
        }
    }
    std::fclose(f);
    return ok;
}

int main(int argc, char **argv)
{
    if (argc != 4 && argc != 5) {
        std::fprintf(stderr, "usage: %s <input> <output> <repetitions> [dump folder]\n", argv[0]);
        return 2;
    }
    Input in;
    if (!read_input(argv[1], in)) {
        std::fprintf(stderr, "cannot read %s\n", argv[1]);
        return 2;
    }
    const int reps = std::atoi(argv[3]);
    const char *dump_dir = argc == 5 ? argv[4] : nullptr;
    if (reps < (dump_dir ? 2 : 1)) {
        std::fprintf(stderr, "repetitions must be at least %d\n", dump_dir ? 2 : 1);
        return 2;
    }
    const int Nx = in.N, Ny = in.N, R = in.R, A = in.A;
    const long nn = (long)Nx * Ny;
    // the window the carrier selects must lie inside the spectrum (get1stOrder_new reads it)
    const int M = Nx / 4;
    if (in.car[0] - M / 2 < 0 || in.car[0] + M / 2 > Ny || in.car[1] - M / 2 < 0 || in.car[1] + M / 2 > Nx ||
        in.car[2] < 0 || in.car[2] > M / 2) {
        std::fprintf(stderr, "carrier (%d, %d, %d) outside the spectrum\n", in.car[0], in.car[1], in.car[2]);
        return 2;
    }
    rCircle = in.car[0], cCircle = in.car[1], radiusCircle = in.car[2];

    // sizes and launch grids as the driver sets them (cTDM/HilbertTransform.cu:376-414)
    Nx2 = Nx >> 2, Ny2 = Ny >> 2;
    blocksInX = (Nx + 31) / 32, blocksInY = (Ny + 31) / 32;
    blocksInX2 = (Nx / 2 + 31) / 32, blocksInY2 = (Ny / 2 + 31) / 32;
    blocksInX3 = (Nx2 + 31) / 32, blocksInY3 = (Ny2 + 31) / 32;
    blocksInX4 = (Nx2 / 2 + 31) / 32, blocksInY4 = (Ny2 / 2 + 31) / 32;
    dim3 grid(blocksInX, blocksInY), grid3(blocksInX3, blocksInY3), block(32, 32);

    // device buffers and plans (:520-574)
    float *UnWrapPhaseSP2, *cuAmpMap2, *cuPhaseMap2, *cuPhaseMap, *cuAmpMap;
    CK(cudaMalloc(&cuSP, sizeof(cufftComplex) * nn));
    CK(cudaMalloc(&cuBG, sizeof(cufftComplex) * nn));
    CK(cudaMalloc(&cuSP2, sizeof(cufftComplex) * Nx2 * Ny2));
    CK(cudaMalloc(&cuBG2, sizeof(cufftComplex) * Nx2 * Ny2));
    CK(cudaMalloc(&UnWrapPhaseSP2, sizeof(float) * Nx2 * Ny2));
    CK(cudaMalloc(&cuAmpMap2, sizeof(float) * Nx2 * Ny2));
    CK(cudaMalloc(&cuPhaseMap2, sizeof(float) * Nx2 * Ny2));
    CK(cudaMalloc(&cuPhaseMap, sizeof(float) * nn));
    CK(cudaMalloc(&cuAmpMap, sizeof(float) * nn));
    CK(cudaMalloc(&LaplaceArray, sizeof(float) * Nx2 * Ny2));
    CK(cudaMalloc(&inX, sizeof(float) * Nx2 * Ny2));
    CK(cudaMalloc(&inY, sizeof(float) * Nx2 * Ny2));
    size_t pitch = 0;
    CK(cudaMallocPitch(&dst_DCT, &pitch, Nx2 * sizeof(float), Ny2));
    CK(cudaMalloc(&dSrc_DCT_FORWARD, sizeof(cufftComplex) * Nx2 * 2 * Ny2));
    CK(cudaMalloc(&dSrc_DCT_INVERSE, sizeof(cufftComplex) * Nx2 * 2 * Ny2));
    CKF(cufftPlan1d(&plan_1D_C2C_FORWARD, Ny2 * 2, CUFFT_C2C, Nx2));
    CKF(cufftPlan1d(&plan_1D_C2C_INVERSE, Nx2 * 2, CUFFT_C2C, Ny2));
    CKF(cufftPlan2d(&plan_2D_C2C_FORWARD_s1, Nx, Ny, CUFFT_C2C));
    CKF(cufftPlan2d(&plan_2D_C2C_INVERSE_s2, Nx2, Ny2, CUFFT_C2C));
    ReconMode = 0;   // device-resident n (BatchRecon picks it when free memory allows, :1932-1939)

    // host holograms as the job loop keeps them: complex with zero imaginary parts (:711-716)
    std::vector<cufftComplex> sp_cu((size_t)A * nn), bg_cu(nn);
    for (long i = 0; i < nn * A; i++) sp_cu[i] = make_cuComplex(in.holo[i], 0.f);
    for (long i = 0; i < nn; i++) bg_cu[i] = make_cuComplex(in.bg[i], 0.f);
    std::vector<float> final_phase(nn), final_amp(nn);
    const long r2 = (long)R * R, r3 = r2 * R;
    std::vector<cufftComplex> n3d(r3);

    // BatchRecon's constants, in float as it computes them (:1839-1863), with the input dx
    const float n_med = (float)in.n_med, n_med2 = (float)(in.n_med * in.n_med);
    const float lambda = (float)in.wavelength;
    const float f0 = 1 / lambda, fm0 = f0 * n_med;
    const double dx = in.dx;
    const float k = 2 * (float)M_PI * n_med / lambda, k2 = k * k;
    const float df = (float)(1 / (R * dx));
    dim3 grid2D((R / 2 + 31) / 32, (R / 2 + 31) / 32), block2D(32, 32);
    dim3 grid3D((R / 2 + 7) / 8, (R / 2 + 7) / 8, (R / 2 + 15) / 16), block3D(8, 8, 16);

    double best_ms = 1e30, sum_ms = 0, front_ms = 0, recon_ms = 0;
    long bad_maps = 0, bad_stack = 0;   // non-finite map values before / after the Combine2Stack fix-up
    const long mm = (long)Nx2 * Ny2;
    std::vector<float> d_phase, d_amp, d_unw, d_counts;
    std::vector<cufftComplex> d_f2;
    if (dump_dir) d_phase.resize(mm * A), d_amp.resize(mm * A), d_unw.resize(mm * A);
    int timed = 0;
    for (int rep = 0; rep < reps; rep++) {
        const bool dumping = dump_dir && rep == 0;
        CK(cudaDeviceSynchronize());
        const auto t0 = std::chrono::steady_clock::now();
        std::vector<float> phase_stack(r2 * A), amp_stack(r2 * A);
        for (int frame = 1; frame <= A; frame++) {
            // frame 2 onwards keeps the carrier (obtainRadius runs for frame 1 only, :1572)
            extractQPI_AlgorithmA(sp_cu.data() + (size_t)(frame - 1) * nn, bg_cu.data(), cuSP2, cuBG2, Nx, Ny, 2);
            calcWrapPhase<<<grid3, block>>>(UnWrapPhaseSP2, cuAmpMap2, cuSP2, cuBG2, Nx2, Ny2);
            DCT_UWLS_Unwrapped(cuPhaseMap2, UnWrapPhaseSP2, Nx2, Ny2);
            if (dumping) {   // the DCT reads the wrapped phase without changing it
                const long o = (long)(frame - 1) * mm;
                CK(cudaMemcpy(d_phase.data() + o, UnWrapPhaseSP2, sizeof(float) * mm, cudaMemcpyDeviceToHost));
                CK(cudaMemcpy(d_amp.data() + o, cuAmpMap2, sizeof(float) * mm, cudaMemcpyDeviceToHost));
                CK(cudaMemcpy(d_unw.data() + o, cuPhaseMap2, sizeof(float) * mm, cudaMemcpyDeviceToHost));
            }
            bilinear_interpolation_kernel<<<grid, block>>>(cuPhaseMap, cuPhaseMap2, cuAmpMap, cuAmpMap2, Nx2, Ny2, Nx,
                                                           Ny);
            CK(cudaMemcpy(final_phase.data(), cuPhaseMap, sizeof(float) * nn, cudaMemcpyDeviceToHost));
            CK(cudaMemcpy(final_amp.data(), cuAmpMap, sizeof(float) * nn, cudaMemcpyDeviceToHost));
            // Combine2Stack, ResizeFlag 1: the centre R x R of the N x N maps (:1397-1427)
            for (int j = (Nx - R) / 2; j < (Nx + R) / 2; j++)
                for (int i = (Ny - R) / 2; i < (Ny + R) / 2; i++) {
                    const long o = (i - (Nx - R) / 2) + (long)(j - (Ny - R) / 2) * R + (long)(frame - 1) * r2;
                    float p = final_phase[i + (long)j * Nx], a = final_amp[i + (long)j * Nx];
                    if (rep == 0) bad_maps += !std::isfinite(p) + !std::isfinite(a);
                    phase_stack[o] = (std::isnan(p) || std::isinf(p)) ? 0.f : p;
                    amp_stack[o] = (std::isnan(a) || std::isinf(a)) ? 1.f : a;
                }
        }
        CK(cudaDeviceSynchronize());
        const auto t1 = std::chrono::steady_clock::now();

        if (rep == 0)
            for (long i = 0; i < r2 * A; i++) bad_stack += !std::isfinite(phase_stack[i]) + !std::isfinite(amp_stack[i]);
        // BatchRecon (:1825-2047)
        float *CUDA_Phase, *CUDA_Amp, *CUDA_C;
        cufftComplex *CUDA_F, *u_sp_device, *CUDA_F2, *CUDA_n;
        CK(cudaMalloc(&CUDA_Phase, sizeof(float) * r2 * A));
        CK(cudaMalloc(&CUDA_Amp, sizeof(float) * r2 * A));
        MedianFilter(CUDA_Phase, CUDA_Amp, phase_stack.data(), amp_stack.data(), R, R, A);
        CK(cudaMalloc(&CUDA_F, sizeof(cufftComplex) * r3));
        CK(cudaMalloc(&u_sp_device, sizeof(cufftComplex) * r2));
        CK(cudaMalloc(&CUDA_C, sizeof(float) * r3));
        CK(cudaMemset(CUDA_C, 0, sizeof(float) * r3));
        {
            std::vector<cufftComplex> zeros(r3, make_cuComplex(0.f, 0.f));
            CK(cudaMemcpy(CUDA_F, zeros.data(), sizeof(cufftComplex) * r3, cudaMemcpyHostToDevice));
        }
        for (int z = 0; z < A; z++) {
            CopyDataArray(u_sp_device, CUDA_Phase, CUDA_Amp, R, R, R, z);
            cuFFT2Dshift<<<grid2D, block2D>>>(u_sp_device, R, R);
            cuFFT2D(u_sp_device, R, R, -1);
            EdwardSphere(u_sp_device, CUDA_F, CUDA_C, fm0, df, in.angx[z], in.angy[z], R, R, R);
        }
        CK(cudaFree(u_sp_device));
        CK(cudaFree(CUDA_Phase));
        CK(cudaFree(CUDA_Amp));
        CK(cudaMalloc(&CUDA_F2, sizeof(cufftComplex) * r3));
        initial_F_and_F2(CUDA_C, CUDA_F, CUDA_F2, (float)dx, R, R, R);
        if (dumping) {
            d_counts.resize(r3), d_f2.resize(r3);
            CK(cudaMemcpy(d_counts.data(), CUDA_C, sizeof(float) * r3, cudaMemcpyDeviceToHost));
            CK(cudaMemcpy(d_f2.data(), CUDA_F2, sizeof(cufftComplex) * r3, cudaMemcpyDeviceToHost));
        }
        CK(cudaFree(CUDA_C));
        cuFFT3D(CUDA_F, R, R, R, 1);
        CK(cudaMalloc(&CUDA_n, sizeof(cufftComplex) * r3));
        est_n_3D(CUDA_n, CUDA_F, k2, n_med, R, R, R);
        for (int iter = 0; iter < in.iters; iter++) {   // IterTime + 1 loop bodies (:1957)
            modify_F_3D(CUDA_n, CUDA_F, k2, n_med2, R, R, R);
            cuFFT3D(CUDA_F, R, R, R, -1);
            check_F_3D(CUDA_F, CUDA_F2, R, R, R);
            cuFFT3D(CUDA_F, R, R, R, 1);
            est_n_3D(CUDA_n, CUDA_F, k2, n_med, R, R, R);
        }
        cuFFT3Dshift<<<grid3D, block3D>>>(CUDA_n, R, R, R);
        CK(cudaMemcpy(n3d.data(), CUDA_n, sizeof(cufftComplex) * r3, cudaMemcpyDeviceToHost));
        CK(cudaFree(CUDA_n));
        CK(cudaFree(CUDA_F));
        CK(cudaFree(CUDA_F2));
        CK(cudaDeviceSynchronize());
        CK(cudaGetLastError());
        const auto t2 = std::chrono::steady_clock::now();
        const double ms = std::chrono::duration<double, std::milli>(t2 - t0).count();
        if (dumping) continue;   // the dumps' copies are not part of the pipeline
        timed++;
        best_ms = ms < best_ms ? ms : best_ms;
        sum_ms += ms;
        front_ms += std::chrono::duration<double, std::milli>(t1 - t0).count();
        recon_ms += std::chrono::duration<double, std::milli>(t2 - t1).count();
    }
    FILE *f = std::fopen(argv[2], "wb");
    if (!f || std::fwrite(n3d.data(), sizeof(cufftComplex), r3, f) != (size_t)r3) {
        std::fprintf(stderr, "cannot write %s\n", argv[2]);
        return 2;
    }
    std::fclose(f);
    if (dump_dir) {
        auto put = [&](const char *name, const void *data, size_t bytes) {
            std::string path = std::string(dump_dir) + "/" + name;
            FILE *g = std::fopen(path.c_str(), "wb");
            const bool ok = g && std::fwrite(data, 1, bytes, g) == bytes;
            if (g) std::fclose(g);
            if (!ok) std::fprintf(stderr, "cannot write %s\n", path.c_str());
            return ok;
        };
        if (!put("phase.f32", d_phase.data(), sizeof(float) * d_phase.size()) ||
            !put("amp.f32", d_amp.data(), sizeof(float) * d_amp.size()) ||
            !put("unwrapped.f32", d_unw.data(), sizeof(float) * d_unw.size()) ||
            !put("counts.f32", d_counts.data(), sizeof(float) * d_counts.size()) ||
            !put("f2.c64", d_f2.data(), sizeof(cufftComplex) * d_f2.size()))
            return 2;
    }
    long bad_out = 0;
    for (long i = 0; i < r3; i++) bad_out += !std::isfinite(n3d[i].x) || !std::isfinite(n3d[i].y);
    std::printf("{\"reps\": %d, \"ms_mean\": %.3f, \"ms_best\": %.3f, \"front_ms_mean\": %.3f, "
                "\"recon_ms_mean\": %.3f, \"non_finite_map_values\": %ld, \"non_finite_stack_values\": %ld, "
                "\"non_finite_voxels\": %ld}\n",
                timed, sum_ms / timed, best_ms, front_ms / timed, recon_ms / timed, bad_maps, bad_stack, bad_out);
    return 0;
}
