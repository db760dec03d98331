// Comparison harness for QPI Algorithm B (the reference's default QPI_Method = 0): runs
// the reference's own extractQPI_AlgorithmB and calcWrapPhase on the holograms of a
// tomogram read from a file and writes the wrapped phase and amplitude it produces.
//
// COMPARISON INFRASTRUCTURE ONLY: the product never links or runs it.  The compute is the
// reference's code, cut unmodified from cTDM/HilbertTransform.cu into qpi_b.cu by
// oracle/refcuda/assemble.py (extractQPI_AlgorithmB, sequence1DFFT, real2cufft,
// copySharedMem, HistogramFT, shiftArray, CropFTdomain, calcWrapPhase,
// bilinear_interpolation_kernel; thrust for the carrier's max_element).  This file
// supplies what the reference's driver would: the file-scope globals
// (cTDM/HilbertTransform.cuh:68-110), their allocation and the two 1-D cuFFT plans
// (cTDM/HilbertTransform.cu:376-414,545-564), and the job loop's call for method 0
// (:951-963): one background for every frame, frame numbers from 1 (frame 1 sets the
// carrier column from its own spectrum, and the background's call then resets it).
//
// Input: the "CTDMREF1" file of oracle/refcuda/harness.cu (the carrier fields are not
// used).  Output (A * M * M floats each, M = N / 4): <out>.phase.f32, <out>.amp.f32;
// stdout: one JSON line with the wall time per frame and the carrier column in use.
// Usage: ref_qpib <input> <output prefix>
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <string>
#include <vector>

#include <cuda_runtime.h>
#include <cufft.h>

// ---- file-scope globals of the reference's driver (cTDM/HilbertTransform.cuh:68-110)
int blocksInX, blocksInY, blocksInX2, blocksInY2, blocksInX3, blocksInY3, blocksInX4, blocksInY4;
int Nx2, Ny2;
int max_idx_seq1D;
float *cuSP_PE_temp, *cuBG_PE_temp, *cuSP_PE_resample, *cuBG_PE_resample;
cufftComplex *device_PE_FFT, *out_PE_FFT;
float *sumFFT_PE_1D;
cufftHandle plan_1D_C2C_FORWARD_FT, plan_1D_C2C_INVERSE_FT;
clock_t s_datatransfer, e_datatransfer, s_wrap, e_wrap;
float dataTransfer_time, wrap_time;

// ---- the reference's functions cut from cTDM/HilbertTransform.cu (qpi_b.cu)
void extractQPI_AlgorithmB(float *SP, float *BG, cufftComplex *cuSP_FFT, cufftComplex *cuBG_FFT, int Nx, int Ny,
                           int frame);
__global__ void calcWrapPhase(float *Phase, float *Amp, cufftComplex *SP, cufftComplex *BG, int sizeX, int sizeY);

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

int main(int argc, char **argv)
{
    if (argc != 3) {
        std::fprintf(stderr, "usage: %s <input> <output prefix>\n", argv[0]);
        return 2;
    }
    FILE *f = std::fopen(argv[1], "rb");
    if (!f) {
        std::fprintf(stderr, "cannot open %s\n", argv[1]);
        return 2;
    }
    char magic[8];
    int32_t h[7];
    double d[3];
    bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, "CTDMREF1", 8) == 0 &&
              std::fread(h, sizeof h, 1, f) == 1 && std::fread(d, sizeof d, 1, f) == 1;
    const int N = ok ? h[0] : 0, A = ok ? h[2] : 0;
    ok = ok && N >= 128 && N <= 2048 && (N & (N - 1)) == 0 && A >= 1 && A <= 1024;
    const long nn = (long)N * N;
    std::vector<float> ang(2 * (size_t)(ok ? A : 0)), bg(ok ? nn : 0), holo(ok ? nn * A : 0);
    ok = ok && std::fread(ang.data(), 4, 2 * (size_t)A, f) == 2 * (size_t)A && std::fread(bg.data(), 4, nn, f) == (size_t)nn &&
         std::fread(holo.data(), 4, nn * A, f) == (size_t)(nn * A);
    std::fclose(f);
    if (!ok) {
        std::fprintf(stderr, "cannot read %s\n", argv[1]);
        return 2;
    }
    const int Nx = N, Ny = N;
    // sizes and launch grids as the driver sets them (cTDM/HilbertTransform.cu:376-414)
    Nx2 = Nx >> 2, Ny2 = Ny >> 2;
    blocksInX = (Nx + 31) / 32, blocksInY = (Ny + 31) / 32;
    blocksInX2 = (Nx / 2 + 31) / 32, blocksInY2 = (Ny / 2 + 31) / 32;
    blocksInX3 = (Nx2 + 31) / 32, blocksInY3 = (Ny2 + 31) / 32;
    blocksInX4 = (Nx2 / 2 + 31) / 32, blocksInY4 = (Ny2 / 2 + 31) / 32;
    const long mm = (long)Nx2 * Ny2;
    // buffers and plans of Algorithm B (:545-564)
    CK(cudaMalloc(&cuSP_PE_temp, sizeof(float) * nn));
    CK(cudaMalloc(&cuBG_PE_temp, sizeof(float) * nn));
    CK(cudaMalloc(&cuSP_PE_resample, sizeof(float) * Nx * (Ny / 4)));
    CK(cudaMalloc(&cuBG_PE_resample, sizeof(float) * Nx * (Ny / 4)));
    CK(cudaMalloc(&device_PE_FFT, sizeof(cufftComplex) * Nx * (Ny / 4)));
    CK(cudaMalloc(&out_PE_FFT, sizeof(cufftComplex) * (Nx / 4) * (Ny / 4)));
    CK(cudaMalloc(&sumFFT_PE_1D, sizeof(float) * Nx));
    CKF(cufftPlan1d(&plan_1D_C2C_FORWARD_FT, Nx, CUFFT_C2C, Ny / 4));
    CKF(cufftPlan1d(&plan_1D_C2C_INVERSE_FT, Nx / 4, CUFFT_C2C, Ny / 4));
    cufftComplex *cuSP2, *cuBG2;
    float *phase, *amp;
    CK(cudaMalloc(&cuSP2, sizeof(cufftComplex) * mm));
    CK(cudaMalloc(&cuBG2, sizeof(cufftComplex) * mm));
    CK(cudaMalloc(&phase, sizeof(float) * mm));
    CK(cudaMalloc(&amp, sizeof(float) * mm));
    dim3 grid3(blocksInX3, blocksInY3), block(32, 32);

    std::vector<float> h_phase(mm * A), h_amp(mm * A);
    int carrier = -1;
    CK(cudaDeviceSynchronize());
    const auto t0 = std::chrono::steady_clock::now();
    for (int frame = 1; frame <= A; frame++) {
        extractQPI_AlgorithmB(holo.data() + (size_t)(frame - 1) * nn, bg.data(), cuSP2, cuBG2, Nx, Ny, frame);
        calcWrapPhase<<<grid3, block>>>(phase, amp, cuSP2, cuBG2, Nx2, Ny2);
        CK(cudaGetLastError());
        CK(cudaMemcpy(h_phase.data() + (size_t)(frame - 1) * mm, phase, sizeof(float) * mm, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(h_amp.data() + (size_t)(frame - 1) * mm, amp, sizeof(float) * mm, cudaMemcpyDeviceToHost));
        carrier = max_idx_seq1D;
    }
    CK(cudaDeviceSynchronize());
    const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    for (const char *suffix : {".phase.f32", ".amp.f32"}) {
        const std::string path = std::string(argv[2]) + suffix;
        const std::vector<float> &v = suffix[1] == 'p' ? h_phase : h_amp;
        FILE *g = std::fopen(path.c_str(), "wb");
        const bool wrote = g && std::fwrite(v.data(), sizeof(float), v.size(), g) == v.size();
        if (g) std::fclose(g);
        if (!wrote) {
            std::fprintf(stderr, "cannot write %s\n", path.c_str());
            return 2;
        }
    }
    // the carrier column the later frames used: the background's, set by frame 1's second call
    std::printf("{\"frames\": %d, \"ms_per_frame\": %.4f, \"carrier_column\": %d}\n", A, ms / A, carrier);
    return 0;
}
