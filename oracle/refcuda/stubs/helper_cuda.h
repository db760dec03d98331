// Minimal stand-in for the CUDA samples' helper_cuda.h, which the reference's
// sources include for checkCudaErrors (comparison build only).
#pragma once
#include <cstdio>
#include <cstdlib>
#include <cuda_runtime.h>
#include <cufft.h>
static inline void ref_check(cudaError_t e, const char *what, const char *file, int line)
{
    if (e != cudaSuccess) {
        std::fprintf(stderr, "%s:%d %s: %s\n", file, line, what, cudaGetErrorString(e));
        std::exit(3);
    }
}
static inline void ref_check(cufftResult r, const char *what, const char *file, int line)
{
    if (r != CUFFT_SUCCESS) {
        std::fprintf(stderr, "%s:%d %s: cuFFT error %d\n", file, line, what, (int)r);
        std::exit(3);
    }
}
#define checkCudaErrors(x) ref_check((x), #x, __FILE__, __LINE__)
#define getLastCudaError(msg) ref_check(cudaGetLastError(), (msg), __FILE__, __LINE__)
