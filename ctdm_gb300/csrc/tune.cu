// Autotuner of the positivity-loop passes: per device and volume side it times
// every FFT plan variant (lines per CTA, threads per line, radix sequence; see
// fft_line.cuh PV<R, v>) of the x, y and z passes on scratch volumes and keeps the
// fastest per pass.  The first reconstruction of a new volume side tunes it
// (unless CTDM_AUTOTUNE=0 in the environment, or the stream is being captured);
// ctdm_autotune runs it explicitly and ctdm_set_plans pins a choice.
//
// No reference counterpart: the reference calls cuFFT with a fixed plan per call
// (cTDM/FFT.cu:807-838).
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <set>
#include <utility>
#include <vector>

#include "api_internal.h"

namespace ctdm {

struct PlanChoice {
    int v[3] = {0, 0, 0};   // x, y, z pass
    int scheme = -1;        // -1 default, 0 x / y / z / y passes, 1 / 2 plane + z passes
    bool tuned = false;
};
static std::mutex g_tune_mu;
static std::map<std::pair<int, int>, PlanChoice> g_choice;   // (device, R)

static std::mutex g_cfg_mu;
static std::set<std::pair<const void *, int>> g_configured;   // (kernel, device) with attributes set
bool kernel_configured(const void *fn, int dev)
{
    std::lock_guard<std::mutex> lk(g_cfg_mu);
    return g_configured.count({fn, dev}) != 0;
}
void mark_kernel_configured(const void *fn, int dev)
{
    std::lock_guard<std::mutex> lk(g_cfg_mu);
    g_configured.insert({fn, dev});
}

int loop_plan_count(int R)
{
    switch (R) {
    case 32: case 64: case 128: return 1;
    case 256: case 384: case 512: case 768: return 3;
    default: return 0;
    }
}

cudaError_t loop_pass_variant(int kind, int variant, const LoopArgs &a, int flag, cudaStream_t s)
{
    switch (a.R) {
    case 32: return loop_pass_32(kind, variant, a, flag, s);
    case 64: return loop_pass_64(kind, variant, a, flag, s);
    case 128: return loop_pass_128(kind, variant, a, flag, s);
    case 256: return loop_pass_256(kind, variant, a, flag, s);
    case 384: return loop_pass_384(kind, variant, a, flag, s);
    case 512: return loop_pass_512(kind, variant, a, flag, s);
    case 768: return loop_pass_768(kind, variant, a, flag, s);
    default: return cudaErrorInvalidValue;
    }
}

static PlanChoice choice_of(int R);

// Lines per packed z-pass tile of variant v at side R (0: that plan reads F2 densely).
static int ztile_of(int R, int v)
{
    const char *env = std::getenv("CTDM_PACKED_Z");
    if (env && std::strcmp(env, "0") == 0) return 0;
    switch (R) {
    case 32: return loop_ztile_32(v);
    case 64: return loop_ztile_64(v);
    case 128: return loop_ztile_128(v);
    case 256: return loop_ztile_256(v);
    case 384: return loop_ztile_384(v);
    case 512: return loop_ztile_512(v);
    case 768: return loop_ztile_768(v);
    default: return 0;
    }
}

int loop_ztile(int R)
{
    int v = 0;
    {
        int dev = 0;
        cudaGetDevice(&dev);
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_choice.find({dev, R});
        if (it != g_choice.end()) v = it->second.v[2];
    }
    return ztile_of(R, v);
}

static PlanChoice choice_of(int R)
{
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_choice.find({dev, R});
    return it == g_choice.end() ? PlanChoice() : it->second;
}

static std::map<std::pair<int, int>, int> g_plane_ok;   // (device, R) -> clusters resident

static bool plane_available(int R)
{
    if (R != 256 && R != 512) return false;
    int dev = 0;
    cudaGetDevice(&dev);
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_plane_ok.find({dev, R});
        if (it != g_plane_ok.end()) return it->second > 0;
    }
    const int n = R == 256 ? plane_clusters_256() : plane_clusters_512();
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_plane_ok[{dev, R}] = n;
    return n > 0;
}

int loop_scheme(int R)
{
    const PlanChoice pc = choice_of(R);
    if (pc.scheme >= 0) return pc.scheme >= 1 && plane_available(R) ? pc.scheme : 0;
    return plane_available(R) ? 1 : 0;
}

static cudaError_t plane_variant(const LoopArgs &a, bool final_pass, int scheme, cudaStream_t s)
{
    if (a.R == 256) return plane_pass_256(a, final_pass, scheme, s);
    if (a.R == 512) return plane_pass_512(a, final_pass, scheme, s);
    return cudaErrorNotSupported;
}

cudaError_t launch_plane(const LoopArgs &a, bool final_pass, cudaStream_t s)
{
    return plane_variant(a, final_pass, loop_scheme(a.R), s);
}

cudaError_t launch_xpass(const LoopArgs &a, bool final_pass, cudaStream_t s)
{
    return loop_pass_variant(final_pass ? LOOP_X_FINAL : LOOP_X, choice_of(a.R).v[0], a, 0, s);
}
cudaError_t launch_ypass(const LoopArgs &a, bool inverse, cudaStream_t s)
{
    return loop_pass_variant(inverse ? LOOP_Y_INV : LOOP_Y_FWD, choice_of(a.R).v[1], a, 0, s);
}
cudaError_t launch_zpass(const LoopArgs &a, int check_mode, cudaStream_t s)
{
    return loop_pass_variant(LOOP_Z, choice_of(a.R).v[2], a, check_mode, s);
}

// Median time (ms) of `reps` launches of one pass variant on stream s.
static cudaError_t time_variant(int kind, int v, const LoopArgs &a, int flag, cudaStream_t s, int reps, double &ms)
{
    cudaEvent_t e0, e1;
    cudaError_t e = cudaEventCreate(&e0);
    if (e != cudaSuccess) return e;
    e = cudaEventCreate(&e1);
    if (e != cudaSuccess) {
        cudaEventDestroy(e0);
        return e;
    }
    std::vector<double> t;
    e = loop_pass_variant(kind, v, a, flag, s);   // warm-up (module load, attributes)
    for (int r = 0; r < reps && e == cudaSuccess; r++) {
        cudaEventRecord(e0, s);
        e = loop_pass_variant(kind, v, a, flag, s);
        cudaEventRecord(e1, s);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        float dt = 0.f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&dt, e0, e1);
        t.push_back(dt);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) return e;
    std::sort(t.begin(), t.end());
    ms = t[t.size() / 2];
    return cudaSuccess;
}

// Times every variant of every pass at volume side R on zero-filled scratch volumes
// (the passes are data-independent in cost) and records the fastest.
cudaError_t autotune_loop(int R, int check_mode, int *chosen, double *ms_out, int n_ms)
{
    const int nv = loop_plan_count(R);
    if (nv == 0) return cudaErrorInvalidValue;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const size_t r3 = (size_t)R * R * R;
    float2 *G = nullptr, *F2 = nullptr;
    uint8_t *mask = nullptr;
    int *err = nullptr;
    cudaStream_t s = nullptr;
    e = cudaMalloc(&G, sizeof(float2) * r3);
    if (e == cudaSuccess) e = cudaMalloc(&F2, sizeof(float2) * r3);
    if (e == cudaSuccess && check_mode) e = cudaMalloc(&mask, r3);
    if (e == cudaSuccess) e = cudaMalloc(&err, sizeof(int));
    // packed z passes are timed as the loop runs them, on empty tiles (no measured
    // samples: the same transforms, loads and stores, none of the few value loads)
    int tbmin = 0;
    for (int v = 0; v < nv; v++) {
        const int tb = ztile_of(R, v);
        if (tb > 0 && (tbmin == 0 || tb < tbmin)) tbmin = tb;
    }
    uint32_t *tmask = nullptr;
    int *tcount = nullptr, *tprefix = nullptr;
    const size_t tiles = tbmin ? (size_t)R * R / tbmin : 0;
    if (e == cudaSuccess && tiles) e = cudaMalloc(&tmask, sizeof(uint32_t) * tiles * R);
    if (e == cudaSuccess && tiles) e = cudaMalloc(&tcount, sizeof(int) * tiles);
    if (e == cudaSuccess && tiles) e = cudaMalloc(&tprefix, sizeof(int) * tiles * R);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (e == cudaSuccess && tiles) e = cudaMemsetAsync(tmask, 0, sizeof(uint32_t) * tiles * R, s);
    if (e == cudaSuccess && tiles) e = cudaMemsetAsync(tcount, 0, sizeof(int) * tiles, s);
    if (e == cudaSuccess && tiles) e = cudaMemsetAsync(tprefix, 0, sizeof(int) * tiles * R, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(G, 0, sizeof(float2) * r3, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(F2, 0, sizeof(float2) * r3, s);
    if (e == cudaSuccess && mask) e = cudaMemsetAsync(mask, 0, r3, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(err, 0, sizeof(int), s);
    PlanChoice pc;
    if (e == cudaSuccess) {
        LoopArgs a = {};
        a.G = G;
        a.F2 = F2;
        a.mask = mask;
        a.out = F2;   // the final x pass is not timed
        a.R = R;
        const double k2 = 1.0e14, nm = 1.337;
        a.inv_n3 = (float)(1.0 / (double)r3);
        a.k2 = (float)k2;
        a.n_med = (float)nm;
        a.n_med2 = (float)(nm * nm);
        a.s1 = (float)(-1.0 / ((double)r3 * k2));
        a.s2 = (float)(-k2 / (nm * nm));
        a.err = err;
        a.tmask = tmask;
        a.tcount = tcount;
        a.tprefix = tprefix;
        a.tvals = G;   // never read: every tile is empty
        // the z pass of variant v as the loop would run it
        auto zargs = [&](int v) {
            LoopArgs z = a;
            z.packed = tiles && ztile_of(R, v) > 0 ? 1 : 0;
            return z;
        };
        const int kinds[3] = {LOOP_X, LOOP_Y_FWD, LOOP_Z};
        for (int p = 0; p < 3 && e == cudaSuccess; p++) {
            double best = 1e30;
            for (int v = 0; v < nv && e == cudaSuccess; v++) {
                double ms = 0;
                e = time_variant(kinds[p], v, kinds[p] == LOOP_Z ? zargs(v) : a, check_mode, s, 5, ms);
                if (ms_out && p * 3 + v < n_ms) ms_out[p * 3 + v] = ms;
                if (e == cudaSuccess && ms < best) {
                    best = ms;
                    pc.v[p] = v;
                }
            }
        }
        // loop scheme: one iteration of x / y / z / y against plane + z (both plane variants)
        if (e == cudaSuccess && plane_available(R)) {
            cudaEvent_t e0, e1;
            e = cudaEventCreate(&e0);
            if (e == cudaSuccess) e = cudaEventCreate(&e1);
            double best[3] = {1e30, 1e30, 1e30};
            for (int rep = 0; rep < 4 && e == cudaSuccess; rep++) {
                for (int sc = 0; sc < 3 && e == cudaSuccess; sc++) {
                    float d = 0.f;
                    cudaEventRecord(e0, s);
                    if (sc == 0) {
                        e = loop_pass_variant(LOOP_X, pc.v[0], a, 0, s);
                        if (e == cudaSuccess) e = loop_pass_variant(LOOP_Y_FWD, pc.v[1], a, 0, s);
                        if (e == cudaSuccess) e = loop_pass_variant(LOOP_Z, pc.v[2], zargs(pc.v[2]), check_mode, s);
                        if (e == cudaSuccess) e = loop_pass_variant(LOOP_Y_INV, pc.v[1], a, 0, s);
                    } else {
                        e = plane_variant(a, false, sc, s);
                        if (e == cudaSuccess) e = loop_pass_variant(LOOP_Z, pc.v[2], zargs(pc.v[2]), check_mode, s);
                    }
                    cudaEventRecord(e1, s);
                    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
                    if (e == cudaSuccess) e = cudaEventElapsedTime(&d, e0, e1);
                    if (rep > 0) best[sc] = std::min(best[sc], (double)d);
                }
            }
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            pc.scheme = (int)(std::min_element(best, best + 3) - best);
            for (int sc = 0; sc < 3; sc++)
                if (ms_out && 9 + sc < n_ms) ms_out[9 + sc] = best[sc];
        }
        pc.tuned = e == cudaSuccess;
    }
    if (s) {
        cudaStreamSynchronize(s);
        cudaStreamDestroy(s);
    }
    cudaFree(G);
    cudaFree(F2);
    cudaFree(mask);
    cudaFree(err);
    cudaFree(tmask);
    cudaFree(tcount);
    cudaFree(tprefix);
    if (e != cudaSuccess) return e;
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_choice[{dev, R}] = pc;
    }
    if (chosen)
        for (int p = 0; p < 3; p++) chosen[p] = pc.v[p];
    return cudaSuccess;
}

// Tunes R on first use on this device (see the file comment).
cudaError_t ensure_tuned(int R, int check_mode, cudaStream_t s)
{
    const char *env = std::getenv("CTDM_AUTOTUNE");
    if (env && std::strcmp(env, "0") == 0) return cudaSuccess;
    if (loop_plan_count(R) <= 1) return cudaSuccess;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_choice.find({dev, R});
        if (it != g_choice.end()) return cudaSuccess;   // tuned or pinned
    }
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    e = cudaStreamIsCapturing(s, &cs);
    if (e != cudaSuccess || cs != cudaStreamCaptureStatusNone) return cudaSuccess;
    return autotune_loop(R, check_mode, nullptr, nullptr, 0);
}

}  // namespace ctdm

using namespace ctdm;

extern "C" int ctdm_plan_count(int R) { return loop_plan_count(R); }

extern "C" ctdm_status ctdm_autotune(int device, int R, int check_mode, int *variants3, double *ms, int n_ms)
{
    if (loop_plan_count(R) == 0) return fail_invalid("ctdm_autotune: unsupported volume side");
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return fail_cuda(e, "cudaSetDevice");
    e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = autotune_loop(R, check_mode != 0, variants3, ms, n_ms);
    if (e != cudaSuccess) return fail_cuda(e, "autotune");
    clear_error();
    return CTDM_OK;
}

extern "C" ctdm_status ctdm_z_tile(int device, int R, int *lines)
{
    if (!lines || loop_plan_count(R) == 0) return fail_invalid("ctdm_z_tile: bad argument");
    int v = 0;
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_choice.find({device, R});
        if (it != g_choice.end()) v = it->second.v[2];
    }
    *lines = ztile_of(R, v);
    clear_error();
    return CTDM_OK;
}

extern "C" ctdm_status ctdm_plans(int device, int R, int *variants3, int *tuned)
{
    if (!variants3 || loop_plan_count(R) == 0) return fail_invalid("ctdm_plans: bad argument");
    PlanChoice pc;
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_choice.find({device, R});
        if (it != g_choice.end()) pc = it->second;
    }
    for (int p = 0; p < 3; p++) variants3[p] = pc.v[p];
    if (tuned) *tuned = pc.tuned ? 1 : 0;
    clear_error();
    return CTDM_OK;
}

extern "C" ctdm_status ctdm_set_plans(int device, int R, const int *variants3)
{
    const int nv = loop_plan_count(R);
    if (!variants3 || nv == 0) return fail_invalid("ctdm_set_plans: bad argument");
    for (int p = 0; p < 3; p++)
        if (variants3[p] < 0 || variants3[p] >= nv) return fail_invalid("ctdm_set_plans: variant out of range");
    std::lock_guard<std::mutex> lk(g_tune_mu);
    PlanChoice &pc = g_choice[{device, R}];
    for (int p = 0; p < 3; p++) pc.v[p] = variants3[p];
    pc.tuned = false;
    clear_error();
    return CTDM_OK;
}

extern "C" ctdm_status ctdm_loop_scheme(int device, int R, int *scheme)
{
    if (!scheme || loop_plan_count(R) == 0) return fail_invalid("ctdm_loop_scheme: bad argument");
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return fail_cuda(e, "cudaSetDevice");
    *scheme = loop_scheme(R);
    clear_error();
    return CTDM_OK;
}

extern "C" ctdm_status ctdm_set_loop_scheme(int device, int R, int scheme)
{
    if (loop_plan_count(R) == 0 || scheme < 0 || scheme > 2) return fail_invalid("ctdm_set_loop_scheme: bad argument");
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_choice[{device, R}].scheme = scheme;
    clear_error();
    return CTDM_OK;
}
