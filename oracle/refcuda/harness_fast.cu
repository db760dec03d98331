// Comparison harness for FastUnwrapping (cTDM/FastUnwrapping.cu:5-117): runs the
// reference's own function on wrapped phase maps read from a file and writes the
// unwrapped maps and the in-place normalised inputs it leaves behind.
//
// COMPARISON INFRASTRUCTURE ONLY: the product never links or runs it.  The compute is the
// reference's whole FastUnwrapping.cu and FFT.cu, unmodified.  One forced departure: the
// reference's driver creates the FTUP plans at (M/2)^2 (cTDM/HilbertTransform.cu:555-556)
// while FastUnwrapping transforms (2M)^2 arrays with them, so only a corner of each array
// would be transformed; this harness creates them at the (2M)^2 the function needs, the
// transform its code intends.
//
// Input (little-endian): "CTDMFU01", int32 M, A; float32 maps[A][M][M].  Output:
// <out>.unwrapped.f32 and <out>.normalised.f32 (A * M * M floats each); stdout: one JSON
// line with the time per map.  Usage: ref_fastuw <input> <output prefix>
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

#include "FastUnwrapping.cuh"

// ---- file-scope globals of the reference's driver that FastUnwrapping uses
clock_t s_unwrap, e_unwrap;
float unwrap_time;
cufftHandle plan_2D_C2C_FORWARD_FTUP, plan_2D_C2C_INVERSE_FTUP;

#define CK(x)                                                                                   \
    do {                                                                                        \
        cudaError_t e_ = (x);                                                                   \
        if (e_ != cudaSuccess) {                                                                \
            std::fprintf(stderr, "%s:%d %s: %s\n", __FILE__, __LINE__, #x, cudaGetErrorString(e_)); \
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
    int32_t h[2];
    bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, "CTDMFU01", 8) == 0 &&
              std::fread(h, sizeof h, 1, f) == 1;
    const int M = ok ? h[0] : 0, A = ok ? h[1] : 0;
    ok = ok && M >= 32 && M <= 2048 && M % 32 == 0 && A >= 1 && A <= 1024;
    const long mm = (long)M * M;
    std::vector<float> maps(ok ? mm * A : 0);
    ok = ok && std::fread(maps.data(), 4, mm * A, f) == (size_t)(mm * A);
    std::fclose(f);
    if (!ok) {
        std::fprintf(stderr, "cannot read %s\n", argv[1]);
        return 2;
    }
    if (cufftPlan2d(&plan_2D_C2C_FORWARD_FTUP, 2 * M, 2 * M, CUFFT_C2C) != CUFFT_SUCCESS ||
        cufftPlan2d(&plan_2D_C2C_INVERSE_FTUP, 2 * M, 2 * M, CUFFT_C2C) != CUFFT_SUCCESS) {
        std::fprintf(stderr, "cufftPlan2d failed\n");
        return 3;
    }
    float *src, *dst;
    CK(cudaMalloc(&src, sizeof(float) * mm));
    CK(cudaMalloc(&dst, sizeof(float) * mm));
    std::vector<float> unw(mm * A), norm(mm * A);
    CK(cudaDeviceSynchronize());
    const auto t0 = std::chrono::steady_clock::now();
    for (int a = 0; a < A; a++) {
        CK(cudaMemcpy(src, maps.data() + (size_t)a * mm, sizeof(float) * mm, cudaMemcpyHostToDevice));
        FastUnwrapping(src, dst, M, M);
        CK(cudaGetLastError());
        CK(cudaMemcpy(unw.data() + (size_t)a * mm, dst, sizeof(float) * mm, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(norm.data() + (size_t)a * mm, src, sizeof(float) * mm, cudaMemcpyDeviceToHost));
    }
    CK(cudaDeviceSynchronize());
    const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    for (const char *suffix : {".unwrapped.f32", ".normalised.f32"}) {
        const std::string path = std::string(argv[2]) + suffix;
        const std::vector<float> &v = suffix[1] == 'u' ? unw : norm;
        FILE *g = std::fopen(path.c_str(), "wb");
        const bool wrote = g && std::fwrite(v.data(), sizeof(float), v.size(), g) == v.size();
        if (g) std::fclose(g);
        if (!wrote) {
            std::fprintf(stderr, "cannot write %s\n", path.c_str());
            return 2;
        }
    }
    std::printf("{\"maps\": %d, \"ms_per_map\": %.4f}\n", A, ms / A);
    return 0;
}
