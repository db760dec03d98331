// DCT least-squares unwrapping for callers that cannot allocate device memory.
//
// Some hosts of this library own every byte of device memory themselves: an
// instrument's acquisition loop that must not allocate once it is running, or an
// application that hands out all GPU memory from its own pool and forbids hidden
// cudaMalloc calls.  ctdm_unwrap_dct_noalloc serves them.  Its intermediate map and
// its transform tables live in file-scope __device__ arrays that are part of the
// loaded module, so a call allocates nothing; the caller passes only the input and
// output maps.  The price: every GPU on which the library's kernels are loaded
// holds these arrays (about 16.1 MiB) until the process exits, the size is capped,
// and all calls share one scratch array, so two calls that overlap on the GPU (on
// different streams, or from different threads) race on it.  Each .cu file of the
// library is its own module; under CUDA's default lazy module loading this file's
// module, arrays included, is loaded on a device by the first call there (the
// address look-up below), not when the library is opened.  That first call is the
// one that takes device memory, so a caller makes it as a warm-up before its pool
// claims the memory or its loop starts.
#include <cmath>
#include <cstdio>
#include <mutex>
#include <vector>

#include "ctdm.h"
#include "kernels_front.cuh"

namespace ctdm {
void set_error_message(const char *msg);
cudaError_t dct_unwrap_explicit(const float *phi, float *out, float *T, int A, int M, int mode, const float2 *tw,
                                const float2 *dtw, const float *eig, cudaStream_t s);
}  // namespace ctdm

namespace {

// Capacity: maps of side M in {16, 32, 64, 128, 256}, A * M * M <= 4194304 points.
constexpr long kScratchFloats = 4194304;
constexpr int kMinM = 16, kMaxM = 256;
static_assert(kMinM << (5 - 1) == kMaxM, "five sides, 16 to 256");
constexpr int kSides = 5;                     // 16, 32, 64, 128, 256
constexpr int kTwTotal = 32 + 64 + 128 + 256 + 512;          // FFT tables of length 2M
constexpr int kDctTotal = 33 + 65 + 129 + 257 + 513;         // cos/sin(k pi / 2M), k = 0..2M
constexpr int kEigTotal = 16 + 32 + 64 + 128 + 256;          // 4 sin^2(2 pi k / (4M - 1))

// Scratch: the row-transformed map between the three passes.  Every element a
// pass reads was written by the previous pass of the same call, so it needs no
// clearing; it keeps the last call's contents.
static __device__ __align__(256) float g_noalloc_scratch[kScratchFloats];
static __device__ __align__(256) float2 g_noalloc_tw[kTwTotal];
static __device__ __align__(256) float2 g_noalloc_dct[kDctTotal];
static __device__ __align__(256) float g_noalloc_eig[kEigTotal];

struct DeviceSymbols {
    bool ready = false;
    float *scratch = nullptr;
    float2 *tw = nullptr, *dct = nullptr;
    float *eig = nullptr;
};
std::mutex g_mu;
DeviceSymbols g_dev[64];
thread_local char g_msg[256];

ctdm_status fail(ctdm_status st)
{
    ctdm::set_error_message(g_msg);
    return st;
}

int side_index(int M)
{
    for (int i = 0, m = kMinM; i < kSides; i++, m *= 2)
        if (m == M) return i;
    return -1;
}

// Offsets of side M's tables inside the packed arrays.
void offsets(int idx, int &tw, int &dct, int &eig)
{
    tw = dct = eig = 0;
    for (int i = 0, m = kMinM; i < idx; i++, m *= 2) {
        tw += 2 * m;
        dct += 2 * m + 1;
        eig += m;
    }
}

// Once per device, with that device current: resolve the device addresses of the
// arrays (the host-side names are only stand-ins) and fill the tables.
cudaError_t setup_current_device(DeviceSymbols *&out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_mu);
    DeviceSymbols &d = g_dev[dev];
    if (!d.ready) {
        if ((e = cudaGetSymbolAddress((void **)&d.scratch, g_noalloc_scratch)) != cudaSuccess) return e;
        if ((e = cudaGetSymbolAddress((void **)&d.tw, g_noalloc_tw)) != cudaSuccess) return e;
        if ((e = cudaGetSymbolAddress((void **)&d.dct, g_noalloc_dct)) != cudaSuccess) return e;
        if ((e = cudaGetSymbolAddress((void **)&d.eig, g_noalloc_eig)) != cudaSuccess) return e;
        std::vector<float2> tw(kTwTotal), dct(kDctTotal);
        std::vector<float> eig(kEigTotal);
        const double pi = 3.14159265358979323846;
        for (int i = 0, m = kMinM; i < kSides; i++, m *= 2) {
            int otw, odct, oeig;
            offsets(i, otw, odct, oeig);
            const int L = 2 * m;
            for (int k = 0; k < L; k++) {
                const double a = -2.0 * pi * (double)k / (double)L;
                tw[otw + k] = make_float2((float)cos(a), (float)sin(a));
            }
            for (int k = 0; k <= L; k++) {
                const double a = (double)k * pi / (2.0 * m);
                dct[odct + k] = make_float2((float)cos(a), (float)sin(a));
            }
            for (int k = 0; k < m; k++) {
                const double s = sin(2.0 * pi * (double)k / (4.0 * m - 1.0));
                eig[oeig + k] = (float)(4.0 * s * s);
            }
        }
        if ((e = cudaMemcpy(d.tw, tw.data(), sizeof(float2) * kTwTotal, cudaMemcpyHostToDevice)) != cudaSuccess)
            return e;
        if ((e = cudaMemcpy(d.dct, dct.data(), sizeof(float2) * kDctTotal, cudaMemcpyHostToDevice)) != cudaSuccess)
            return e;
        if ((e = cudaMemcpy(d.eig, eig.data(), sizeof(float) * kEigTotal, cudaMemcpyHostToDevice)) != cudaSuccess)
            return e;
        d.ready = true;
    }
    out = &d;
    return cudaSuccess;
}

}  // namespace

extern "C" ctdm_status ctdm_unwrap_dct_noalloc(int A, int M, int mode, const float *d_phi, float *d_out, void *stream)
{
    g_msg[0] = 0;
    if (!d_phi || !d_out) {
        snprintf(g_msg, sizeof g_msg, "ctdm_unwrap_dct_noalloc: NULL map pointer");
        return fail(CTDM_ERR_INVALID);
    }
    const int idx = side_index(M);
    if (idx < 0) {
        snprintf(g_msg, sizeof g_msg, "ctdm_unwrap_dct_noalloc: map side %d not in {16, 32, 64, 128, 256}", M);
        return fail(CTDM_ERR_INVALID);
    }
    if (mode != CTDM_UNWRAP_REF && mode != CTDM_UNWRAP_EXACT) {
        snprintf(g_msg, sizeof g_msg, "ctdm_unwrap_dct_noalloc: unknown mode %d (0 reference IDCT, 1 exact DCT-III)",
                 mode);
        return fail(CTDM_ERR_INVALID);
    }
    if (A < 1 || (long)A * M * M > kScratchFloats) {
        snprintf(g_msg, sizeof g_msg,
                 "ctdm_unwrap_dct_noalloc: %d maps of %dx%d exceed the fixed scratch of %ld points", A, M, M,
                 kScratchFloats);
        return fail(CTDM_ERR_INVALID);
    }
    DeviceSymbols *d = nullptr;
    cudaError_t e = setup_current_device(d);
    if (e != cudaSuccess) {
        snprintf(g_msg, sizeof g_msg, "ctdm_unwrap_dct_noalloc: set-up failed: %s", cudaGetErrorString(e));
        return fail(CTDM_ERR_CUDA);
    }
    int otw, odct, oeig;
    offsets(idx, otw, odct, oeig);
    e = ctdm::dct_unwrap_explicit(d_phi, d_out, d->scratch, A, M, mode, d->tw + otw, d->dct + odct, d->eig + oeig,
                                  (cudaStream_t)stream);
    if (e != cudaSuccess) {
        snprintf(g_msg, sizeof g_msg, "ctdm_unwrap_dct_noalloc: %s", cudaGetErrorString(e));
        return fail(CTDM_ERR_CUDA);
    }
    ctdm::set_error_message("");
    return CTDM_OK;
}
