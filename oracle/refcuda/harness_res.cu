// Comparison harness for the Goldstein residues: runs the reference's own
// cudaPhaseResidues on wrapped phase maps read from a file and writes the charges it
// produces.
//
// COMPARISON INFRASTRUCTURE ONLY: the product never links or runs it.  The compute is the
// reference's code, cut unmodified from cTDM/Goldstein.cu into gold_res.cu by
// oracle/refcuda/assemble.py (cudaPhaseResidues and the cudaMod it calls).  The launch is
// the reference's: 32 x 32 threads, ceil(W / 32) x ceil(H / 32) blocks
// (cTDM/Goldstein.cuh:37-38, cTDM/Goldstein.cu:22), a float charge map per phase map.
// The residue kernel is the one deterministic stage of the reference's Goldstein path
// (cudaBC's boxes grow from every residue at once and race on shared flags), so it is the
// stage pinned bit-exactly.
//
// Input: "CTDMRS01", int32 W, H, A, then A maps of W * H float32 (x fastest).
// Output: <out>.charges.f32 (A * W * H floats in {-1, 0, 1}); stdout: one JSON line.
// Usage: ref_residues <input> <output prefix>
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

// ---- the reference's kernel cut from cTDM/Goldstein.cu (gold_res.cu)
__global__ void cudaPhaseResidues(float *phi, int sizeX, int sizeY, float *ResiduesCharge);

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
    int32_t h[3];
    bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, "CTDMRS01", 8) == 0 &&
              std::fread(h, sizeof h, 1, f) == 1;
    const int W = ok ? h[0] : 0, H = ok ? h[1] : 0, A = ok ? h[2] : 0;
    ok = ok && W >= 2 && W <= 4096 && H >= 2 && H <= 4096 && A >= 1 && A <= 1024;
    const size_t wh = (size_t)W * H;
    std::vector<float> maps(ok ? wh * A : 0);
    ok = ok && std::fread(maps.data(), 4, wh * A, f) == wh * A;
    std::fclose(f);
    if (!ok) {
        std::fprintf(stderr, "cannot read %s\n", argv[1]);
        return 2;
    }
    float *phi, *charges;
    CK(cudaMalloc(&phi, sizeof(float) * wh));
    CK(cudaMalloc(&charges, sizeof(float) * wh));
    const dim3 grid((W + 31) / 32, (H + 31) / 32), block(32, 32);
    std::vector<float> out(wh * A);
    double ms = 0;
    for (int a = 0; a < A; a++) {
        CK(cudaMemcpy(phi, maps.data() + a * wh, sizeof(float) * wh, cudaMemcpyHostToDevice));
        // the reference zeroes the charge map before the launch (cTDM/Goldstein.cu:14-15)
        CK(cudaMemset(charges, 0, sizeof(float) * wh));
        CK(cudaDeviceSynchronize());
        const auto t0 = std::chrono::steady_clock::now();
        cudaPhaseResidues<<<grid, block>>>(phi, W, H, charges);
        CK(cudaGetLastError());
        CK(cudaDeviceSynchronize());
        ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        CK(cudaMemcpy(out.data() + a * wh, charges, sizeof(float) * wh, cudaMemcpyDeviceToHost));
    }
    const std::string path = std::string(argv[2]) + ".charges.f32";
    FILE *g = std::fopen(path.c_str(), "wb");
    const bool wrote = g && std::fwrite(out.data(), sizeof(float), out.size(), g) == out.size();
    if (g) std::fclose(g);
    if (!wrote) {
        std::fprintf(stderr, "cannot write %s\n", path.c_str());
        return 2;
    }
    std::printf("{\"maps\": %d, \"ms_per_map\": %.4f}\n", A, ms / A);
    return 0;
}
