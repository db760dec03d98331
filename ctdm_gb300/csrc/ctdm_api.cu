// Host runtime and C ABI of libctdm_gb300: device tables, contexts, workspace,
// the fused hologram -> RI pipeline and the reference-named entry points.
#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "api_internal.h"
#include "ctdm.h"
#include "ctdm_common.cuh"
#include "kernels_front.cuh"

namespace ctdm {
cudaError_t compat_copy_data_array(float2 *u, const float *ph, const float *am, int W, int H, int numZ,
                                   cudaStream_t s);
cudaError_t compat_edward_sphere(const float2 *u, float2 *F, float *C, const AngleGeom &g, double df, double fm02,
                                 float fm02s, int W, int H, int Z, cudaStream_t s);
cudaError_t compat_initial_f(const float *C, float2 *F, float2 *F2, float dx, long n, cudaStream_t s);
cudaError_t compat_est_n(float2 *n, const float2 *F, float k2, float nm, long cnt, cudaStream_t s);
cudaError_t compat_modify(const float2 *n, float2 *F, float k2, float nm2, long cnt, cudaStream_t s);
cudaError_t compat_check(float2 *F, const float2 *F2, long cnt, cudaStream_t s);
cudaError_t counts_to_mask(const uint32_t *c, uint8_t *m, long n, cudaStream_t s);
cudaError_t real_parts(const float2 *in, float *out, long n, cudaStream_t s);
cudaError_t bounded_wait_probe(int *err, int polls, int code, long long *cycles, cudaStream_t s);
cudaError_t median_stack(const float *ph, const float *am, int A, int R, float *ph_out, float *am_out,
                         cudaStream_t s);
cudaError_t set_carrier(int *carrier, int r, int c, int rad, cudaStream_t s);
}  // namespace ctdm

using namespace ctdm;

// ---------------------------------------------------------------- errors
static thread_local std::string g_err;

static void set_err(const char *fmt, ...)
{
    char b[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(b, sizeof b, fmt, ap);
    va_end(ap);
    g_err = b;
}

static ctdm_status cuda_fail(cudaError_t e, const char *what)
{
    set_err("%s: %s", what, cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? CTDM_ERR_NOMEM : CTDM_ERR_CUDA;
}

#define CK(x, what)                                    \
    do {                                               \
        cudaError_t e_ = (x);                          \
        if (e_ != cudaSuccess) return cuda_fail(e_, what); \
    } while (0)

static ctdm_status invalid(const char *fmt, ...)
{
    char b[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(b, sizeof b, fmt, ap);
    va_end(ap);
    g_err = b;
    return CTDM_ERR_INVALID;
}

extern "C" const char *ctdm_last_error(void) { return g_err.c_str(); }

namespace ctdm {
void set_error_message(const char *msg) { g_err = msg ? msg : ""; }
}  // namespace ctdm

static std::atomic<unsigned long long> g_launches{0};
namespace ctdm {
void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
void note_launches(unsigned long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
}  // namespace ctdm
extern "C" unsigned long long ctdm_launch_count(void) { return g_launches.load(); }
extern "C" const char *ctdm_version(void) { return "ctdm_gb300 0.1 (sm_103a)"; }

// ---------------------------------------------------------------- device tables
static const int kLengths[] = {16, 32, 64, 128, 256, 384, 512, 768, 1024, 1536, 2048};
static const int kCrops[] = {16, 32, 64, 128, 256, 384, 512, 768};
static const int kVolumes[] = {32, 64, 128, 256, 384, 512, 768};

static bool in_set(int v, const int *s, int n)
{
    for (int i = 0; i < n; i++)
        if (s[i] == v) return true;
    return false;
}
static bool ok_length(int L) { return in_set(L, kLengths, 11); }
static bool ok_crop(int M) { return in_set(M, kCrops, 8); }
static bool ok_volume(int R) { return in_set(R, kVolumes, 7); }

struct DevTables {
    std::map<int, float2 *> tw, dtw;
    std::map<int, float *> eig;
    bool complete = false;
};
static std::mutex g_tab_mu;
static std::map<int, DevTables> g_tables;

static cudaError_t build_tables(int dev, DevTables &t)
{
    for (int L : kLengths) {
        std::vector<float2> h(L);
        for (int e = 0; e < L; e++) {
            const double a = -2.0 * CTDM_PI_D * (double)e / (double)L;
            h[e] = make_float2((float)cos(a), (float)sin(a));
        }
        float2 *d = nullptr;
        cudaError_t err = cudaMalloc(&d, sizeof(float2) * L);
        if (err != cudaSuccess) return err;
        err = cudaMemcpy(d, h.data(), sizeof(float2) * L, cudaMemcpyHostToDevice);
        if (err != cudaSuccess) return err;
        t.tw[L] = d;
    }
    for (int M : kCrops) {
        std::vector<float2> h(2 * M + 1);
        for (int k = 0; k <= 2 * M; k++) {
            const double a = (double)k * CTDM_PI_D / (2.0 * M);
            h[k] = make_float2((float)cos(a), (float)sin(a));
        }
        std::vector<float> e(M);
        for (int k = 0; k < M; k++) {
            const double s = sin(2.0 * CTDM_PI_D * (double)k / (4.0 * M - 1.0));
            e[k] = (float)(4.0 * s * s);
        }
        float2 *d = nullptr;
        float *de = nullptr;
        cudaError_t err = cudaMalloc(&d, sizeof(float2) * (2 * M + 1));
        if (err == cudaSuccess) err = cudaMemcpy(d, h.data(), sizeof(float2) * (2 * M + 1), cudaMemcpyHostToDevice);
        if (err == cudaSuccess) err = cudaMalloc(&de, sizeof(float) * M);
        if (err == cudaSuccess) err = cudaMemcpy(de, e.data(), sizeof(float) * M, cudaMemcpyHostToDevice);
        if (err != cudaSuccess) return err;
        t.dtw[M] = d;
        t.eig[M] = de;
    }
    t.complete = true;
    (void)dev;
    return cudaSuccess;
}

static cudaError_t ensure_tables()
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lk(g_tab_mu);
    DevTables &t = g_tables[dev];
    if (t.complete) return cudaSuccess;
    return build_tables(dev, t);
}

static DevTables *tables_here()
{
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(g_tab_mu);
    auto it = g_tables.find(dev);
    return it == g_tables.end() ? nullptr : &it->second;
}

namespace ctdm {
cudaError_t device_tables() { return ensure_tables(); }

const float2 *twiddles(int L)
{
    DevTables *t = tables_here();
    if (!t) return nullptr;
    auto it = t->tw.find(L);
    return it == t->tw.end() ? nullptr : it->second;
}
const float2 *dct_twiddles(int M)
{
    DevTables *t = tables_here();
    if (!t) return nullptr;
    auto it = t->dtw.find(M);
    return it == t->dtw.end() ? nullptr : it->second;
}
const float *dct_eigen(int M)
{
    DevTables *t = tables_here();
    if (!t) return nullptr;
    auto it = t->eig.find(M);
    return it == t->eig.end() ? nullptr : it->second;
}
}  // namespace ctdm

// ---------------------------------------------------------------- context
enum BufId {
    B_PHASE, B_AMP, B_PHU, B_CHG, B_CUT, B_GOLD, B_U, B_F2, B_COUNTS, B_G, B_T1, B_S, B_BGF, B_DCT, B_MASK, B_GEOM,
    B_CARRIER, B_KEY, B_SCRATCH, B_HOLO, B_BG, B_RI, B_GSTATE, B_GLIST, B_GSTATUS, B_FASTW, B_FASTIN, B_TMP, B_GWORK,
    B_TMASK, B_TCOUNT, B_TVALS, B_QMAG, B_FIT, B_PV, B_PG, B_PV2, B_PG2, B_PVP, B_PPART, B_PCTL, B_PHIST, B_STAGE, B_STAGEBG, B_TPRE, B_RI2, B_XPREV, NBUF
};

// Stage boundaries recorded with CUDA events when timing is enabled.
enum StageTag { S_QPI, S_UNWRAP, S_GOLD, S_SPECTRA, S_EWALD, S_YINV, S_XPASS, S_YFWD, S_ZPASS, S_XFINAL, S_COUNT };

// Stage timing accumulates over every reconstruction between ctdm_ctx_set_timing(on)
// and the read, so a caller can time the stages of a whole timed loop.  Marks on the
// call's stream attribute the interval since the previous mark to a stage; work on
// the side stream is bracketed by its own event pairs.
struct StageTimer {
    static const int kMax = 16384, kSide = 1024;
    cudaEvent_t ev[kMax] = {};
    int tag[kMax] = {};
    int n = 0;
    cudaEvent_t side[2 * kSide] = {};
    int ns = 0;   // side events recorded (pairs: begin, end)
    bool on = false;
    void reset()
    {
        n = 0;
        ns = 0;
    }
    void start(cudaStream_t s) { mark(-1, s); }
    void mark(int t, cudaStream_t s)
    {
        if (!on || n >= kMax) return;
        if (!ev[n]) cudaEventCreate(&ev[n]);
        tag[n] = t;
        cudaEventRecord(ev[n], s);
        n++;
    }
    // begin (even ns) or end (odd ns) of a side-stream interval
    void side_mark(cudaStream_t s)
    {
        if (!on || ns >= 2 * kSide) return;
        if (!side[ns]) cudaEventCreate(&side[ns]);
        cudaEventRecord(side[ns], s);
        ns++;
    }
};

struct ctdm_ctx {
    int device = 0;
    void *buf[NBUF] = {};
    size_t cap[NBUF] = {};
    size_t used[NBUF] = {};
    int carrier[3] = {-1, -1, -1};
    StageTimer timer;
    // side stream for work whose result the reconstruction does not consume
    cudaStream_t side = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
    // pinned staging of the per-call angle geometry and the carrier readback, so that
    // neither copy blocks the calling thread behind copies in flight (a pageable copy
    // would); the events mark when the staging may be reused / read
    struct Pinned {
        AngleGeom geom[512];
        int carrier[4];
        int derr;
    } *pin = nullptr;
    cudaEvent_t geom_done = nullptr, carrier_done = nullptr;
    bool carrier_pending = false;
    // host-buffer uploads: a copy stream and one event per chunk of angles
    static const int kChunks = 16;
    cudaStream_t copy = nullptr;
    cudaEvent_t ready[kChunks + 1] = {};
    // host-buffer calls in flight (ctdm_submit): the input buffers are free again once
    // a call's front end has read them (inputs_free).  Consecutive calls write their
    // volumes into alternating buffers (slot 0: B_RI, 1: B_RI2); a call's volume is
    // downloaded on its own stream once the next call's front end is done (front_done),
    // so that the download runs beside that call's loop rather than its front end, and
    // a slot is written again after vol_free[slot].
    cudaStream_t d2h = nullptr;
    cudaEvent_t inputs_free = nullptr, front_done = nullptr, vol_ready[2] = {}, vol_free[2] = {};
    struct Download {
        ctdm_cfloat *host = nullptr;
        size_t bytes = 0;
        int slot = 0;
        bool pending = false;
    } dl;
    int slot = 0, in_flight = 0;
    // device status word (bounded device-side waits record a code here)
    int *d_err = nullptr;
};

// Angles [k per, (k + 1) per) of the hologram stack become valid on the device at
// event ready[k] (host-buffer calls upload them in chunks while the front end of the
// earlier chunks runs).
struct ChunkFeed {
    const cudaEvent_t *ready;
    int per;
    cudaEvent_t inputs_free;   // recorded once the front end has read the inputs
    cudaEvent_t out_free;      // the output volume may be written after it
    cudaEvent_t front_done;    // recorded after the Ewald mapping
    const void *counts;        // QPI Algorithm A reads the holograms from here when set:
    int bpc;                   // camera counts of bpc bytes, as uploaded
};

static cudaError_t ensure(ctdm_ctx *c, int id, size_t bytes)
{
    c->used[id] = bytes;
    if (c->cap[id] >= bytes && c->buf[id]) return cudaSuccess;
    if (c->buf[id]) {
        // calls in flight (submitted, or on the side and copy streams) may still use it
        cudaError_t e = cudaDeviceSynchronize();
        if (e != cudaSuccess) return e;
        cudaFree(c->buf[id]);
    }
    c->buf[id] = nullptr;
    c->cap[id] = 0;
    if (bytes == 0) return cudaSuccess;
    cudaError_t e = cudaMalloc(&c->buf[id], bytes);
    if (e == cudaSuccess) c->cap[id] = bytes;
    return e;
}

template <class T> static T *B(ctdm_ctx *c, int id) { return reinterpret_cast<T *>(c->buf[id]); }

extern "C" void ctdm_params_default(ctdm_params *p)
{
    std::memset(p, 0, sizeof *p);
    p->n_holo = 1024;
    p->m_crop = 0;
    p->r_vol = 256;
    p->iterations = 101;   // IterTime = 100 runs IterTime + 1 bodies (cTDM/HilbertTransform.cu:34,1957)
    p->unwrap_mode = CTDM_UNWRAP_REF;
    p->check_mode = CTDM_CHECK_REF;
    p->unwrap_method = CTDM_METHOD_DCT;
    p->carrier_r = p->carrier_c = p->carrier_radius = -1;
    p->n_med = 1.333;      // cTDM/HilbertTransform.cu:18
    p->wavelength = 532e-9;
    p->dx = 5.5e-6 / 85.0 * 1024.0 / 256.0;   // CameraPixelSize/Mag*1024/R (:1854) at the defaults
    p->qpi_method = CTDM_QPI_A;
}

extern "C" ctdm_status ctdm_ctx_create(int device, ctdm_ctx **out)
{
    if (!out) return invalid("ctdm_ctx_create: out is NULL");
    CK(cudaSetDevice(device), "cudaSetDevice");
    CK(ensure_tables(), "building twiddle tables");
    ctdm_ctx *c = new ctdm_ctx();
    c->device = device;
    // the side stream carries work the reconstruction does not wait for (Goldstein
    // beside the loop passes): lowest priority, so the block scheduler serves the
    // call's stream first
    int prio_lo = 0, prio_hi = 0;
    cudaError_t e = cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi);
    if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&c->side, cudaStreamNonBlocking, prio_lo);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->join, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->copy, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->d2h, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->inputs_free, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->front_done, cudaEventDisableTiming);
    for (int k = 0; k < 2 && e == cudaSuccess; k++) {
        e = cudaEventCreateWithFlags(&c->vol_ready[k], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->vol_free[k], cudaEventDisableTiming);
    }
    if (e == cudaSuccess) e = cudaMallocHost(&c->pin, sizeof(ctdm_ctx::Pinned));
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->geom_done, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->carrier_done, cudaEventDisableTiming);
    for (int k = 0; k <= ctdm_ctx::kChunks && e == cudaSuccess; k++)
        e = cudaEventCreateWithFlags(&c->ready[k], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaMalloc(&c->d_err, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(c->d_err, 0, sizeof(int));
    if (e != cudaSuccess) {
        ctdm_ctx_destroy(c);
        return cuda_fail(e, "creating the side stream");
    }
    *out = c;
    g_err.clear();
    return CTDM_OK;
}

extern "C" void ctdm_ctx_destroy(ctdm_ctx *c)
{
    if (!c) return;
    cudaSetDevice(c->device);
    // calls still in flight (ctdm_submit without ctdm_wait) finish before the buffers go
    for (cudaStream_t st : {c->copy, c->d2h, c->side})
        if (st) cudaStreamSynchronize(st);
    if (c->in_flight) cudaStreamSynchronize(0);
    for (int i = 0; i < NBUF; i++)
        if (c->buf[i]) cudaFree(c->buf[i]);
    for (int i = 0; i < StageTimer::kMax; i++)
        if (c->timer.ev[i]) cudaEventDestroy(c->timer.ev[i]);
    for (int i = 0; i < 2 * StageTimer::kSide; i++)
        if (c->timer.side[i]) cudaEventDestroy(c->timer.side[i]);
    if (c->side) cudaStreamDestroy(c->side);
    if (c->copy) cudaStreamDestroy(c->copy);
    if (c->d2h) cudaStreamDestroy(c->d2h);
    if (c->pin) cudaFreeHost(c->pin);
    for (cudaEvent_t e : {c->geom_done, c->carrier_done, c->inputs_free, c->front_done, c->vol_ready[0],
                          c->vol_ready[1], c->vol_free[0], c->vol_free[1]})
        if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : c->ready)
        if (e) cudaEventDestroy(e);
    if (c->d_err) cudaFree(c->d_err);
    for (cudaEvent_t e : {c->fork, c->join})
        if (e) cudaEventDestroy(e);
    delete c;
}

// Until ctdm_wait returns, a context serves ctdm_submit alone: the calls in flight
// still read and write its buffers, so every other entry point on it is refused.
static bool in_flight(const ctdm_ctx *c) { return c && c->in_flight > 0; }

extern "C" ctdm_status ctdm_ctx_set_timing(ctdm_ctx *c, int on)
{
    if (!c) return invalid("ctdm_ctx_set_timing: NULL context");
    c->timer.on = on != 0;
    c->timer.reset();
    return CTDM_OK;
}

// Per-stage device time (ms) and launch-group count summed over the pipeline calls
// made since timing was switched on.
extern "C" ctdm_status ctdm_ctx_stage_times(ctdm_ctx *c, double *ms, int *counts, int n)
{
    if (!c || !ms || n < 1) return invalid("ctdm_ctx_stage_times: bad argument");
    for (int i = 0; i < n; i++) {
        ms[i] = 0;
        if (counts) counts[i] = 0;
    }
    StageTimer &t = c->timer;
    if (t.n >= 2) CK(cudaEventSynchronize(t.ev[t.n - 1]), "stage timing");
    for (int i = 1; i < t.n; i++) {
        float dt = 0;
        CK(cudaEventElapsedTime(&dt, t.ev[i - 1], t.ev[i]), "stage timing");
        if (t.tag[i] >= 0 && t.tag[i] < n) {
            ms[t.tag[i]] += dt;
            if (counts) counts[t.tag[i]]++;
        }
    }
    for (int i = 0; i + 1 < t.ns && S_GOLD < n; i += 2) {
        float dt = 0;
        CK(cudaEventSynchronize(t.side[i + 1]), "stage timing");
        CK(cudaEventElapsedTime(&dt, t.side[i], t.side[i + 1]), "stage timing");
        ms[S_GOLD] += dt;
        if (counts) counts[S_GOLD]++;
    }
    return CTDM_OK;
}

// Status word of the context's bounded device-side waits: 0, or the code of the
// first wait that ran out since the last read (1: a TMA tile of the z pass).
// Synchronises the device; reading clears it.
extern "C" ctdm_status ctdm_ctx_device_status(ctdm_ctx *c, int *status)
{
    if (!c || !status) return invalid("ctdm_ctx_device_status: NULL argument");
    CK(cudaSetDevice(c->device), "cudaSetDevice");
    CK(cudaDeviceSynchronize(), "device status");
    CK(cudaMemcpy(status, c->d_err, sizeof(int), cudaMemcpyDeviceToHost), "device status");
    CK(cudaMemset(c->d_err, 0, sizeof(int)), "device status");
    g_err.clear();
    return CTDM_OK;
}

extern "C" ctdm_status ctdm_workspace_bytes(const ctdm_params *p, int n_angles, size_t *bytes)
{
    if (!p || !bytes) return invalid("ctdm_workspace_bytes: NULL argument");
    int M = 0;
    ctdm_status st = validate_params(p, n_angles, M);
    if (st != CTDM_OK) return st;
    *bytes = workspace_bytes(p, n_angles, M);
    g_err.clear();
    return CTDM_OK;
}

extern "C" ctdm_status ctdm_ctx_workspace(ctdm_ctx *c, size_t *bytes)
{
    if (!c || !bytes) return invalid("ctdm_ctx_workspace: NULL argument");
    *bytes = held_bytes(c);
    g_err.clear();
    return CTDM_OK;
}

// One bounded device-side wait that nothing completes, recorded as code 9 in the
// context's status word (see the header).
extern "C" ctdm_status ctdm_ctx_probe_wait(ctdm_ctx *c, int polls, double *ms)
{
    if (!c) return invalid("ctdm_ctx_probe_wait: NULL context");
    if (in_flight(c))
        return invalid("ctdm_ctx_probe_wait: calls submitted on this context are still in flight (ctdm_wait first)");
    CK(cudaSetDevice(c->device), "cudaSetDevice");
    long long *cycles = nullptr;
    CK(cudaMalloc(&cycles, sizeof(long long)), "alloc probe clock");
    cudaError_t e = bounded_wait_probe(c->d_err, polls, 9, cycles, 0);
    long long host = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&host, cycles, sizeof host, cudaMemcpyDeviceToHost);
    int khz = 0;
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&khz, cudaDevAttrClockRate, c->device);
    cudaFree(cycles);
    CK(e, "bounded wait probe");
    if (ms) *ms = khz > 0 ? (double)host / (double)khz : 0.0;
    g_err.clear();
    return CTDM_OK;
}

extern "C" ctdm_status ctdm_ctx_carrier(ctdm_ctx *c, int *carrier3)
{
    if (!c || !carrier3) return invalid("ctdm_ctx_carrier: NULL argument");
    if (c->carrier_pending) {
        CK(cudaEventSynchronize(c->carrier_done), "carrier readback");
        std::memcpy(c->carrier, c->pin->carrier, sizeof c->carrier);
        c->carrier_pending = false;
    }
    std::memcpy(carrier3, c->carrier, sizeof c->carrier);
    return CTDM_OK;
}

extern "C" ctdm_status ctdm_ctx_read_buffer(ctdm_ctx *c, int which, void *host, size_t bytes)
{
    if (in_flight(c))
        return invalid("ctdm_ctx_read_buffer: calls submitted on this context are still in flight (ctdm_wait first)");
    void *d = nullptr;
    size_t n = 0;
    ctdm_status st = ctdm_ctx_buffer(c, which, &d, &n);
    if (st != CTDM_OK) return st;
    if (!host || !d) return invalid("ctdm_ctx_read_buffer: buffer %d not allocated", which);
    CK(cudaSetDevice(c->device), "cudaSetDevice");
    CK(cudaDeviceSynchronize(), "synchronise");
    CK(cudaMemcpy(host, d, bytes < n ? bytes : n, cudaMemcpyDeviceToHost), "read buffer");
    return CTDM_OK;
}

extern "C" ctdm_status ctdm_ctx_buffer(ctdm_ctx *c, int which, void **dptr, size_t *bytes)
{
    if (in_flight(c))
        return invalid("ctdm_ctx_buffer: calls submitted on this context are still in flight (ctdm_wait first)");
    static const int map[] = {B_PHASE, B_AMP, B_PHU, B_CHG, B_CUT, B_GOLD, B_U, B_F2, B_COUNTS};
    if (!c || !dptr || which < 0 || which > 8) return invalid("ctdm_ctx_buffer: bad argument");
    *dptr = c->buf[map[which]];
    if (bytes) *bytes = c->used[map[which]];
    return CTDM_OK;
}

// ---------------------------------------------------------------- geometry
// Per-angle illumination for the voxel rule, computed like the FP64 oracle:
// fx0 = fm0 sin(AngY), fy0 = fm0 sin(AngX) (EdwardSphere, cTDM/Recon_kernel.cu:171-185).
static void angle_geometry(const float *angx, const float *angy, int A, double fm0, double df,
                           std::vector<AngleGeom> &g)
{
    g.resize(A);
    const double fm02 = fm0 * fm0;
    for (int a = 0; a < A; a++) {
        const double fx0 = fm0 * sin((double)angy[a]);
        const double fy0 = fm0 * sin((double)angx[a]);
        double rad0 = fm02 - fx0 * fx0;
        rad0 = rad0 - fy0 * fy0;
        AngleGeom &q = g[a];
        q.fx0 = fx0;
        q.fy0 = fy0;
        q.valid = rad0 >= 0.0;
        q.fz0 = q.valid ? sqrt(rad0) : 0.0;
        q.fx0s = (float)(fx0 / df);
        q.fy0s = (float)(fy0 / df);
        q.fz0s = (float)(q.fz0 / df);
    }
}

static ctdm_status upload_geometry(ctdm_ctx *c, const float *angx, const float *angy, int A, double fm0, double df,
                                   cudaStream_t s)
{
    std::vector<AngleGeom> g;
    angle_geometry(angx, angy, A, fm0, df, g);
    CK(ensure(c, B_GEOM, sizeof(AngleGeom) * A), "alloc geometry");
    if (A <= (int)(sizeof c->pin->geom / sizeof(AngleGeom))) {
        // pinned staging: the previous call's copy has left it once geom_done fired
        CK(cudaEventSynchronize(c->geom_done), "geometry staging");
        std::memcpy(c->pin->geom, g.data(), sizeof(AngleGeom) * A);
        CK(cudaMemcpyAsync(c->buf[B_GEOM], c->pin->geom, sizeof(AngleGeom) * A, cudaMemcpyHostToDevice, s),
           "upload geometry");
        CK(cudaEventRecord(c->geom_done, s), "geometry staging");
    } else {
        // pageable source: the copy is staged before the call returns
        CK(cudaMemcpyAsync(c->buf[B_GEOM], g.data(), sizeof(AngleGeom) * A, cudaMemcpyHostToDevice, s),
           "upload geometry");
    }
    return CTDM_OK;
}

// ---------------------------------------------------------------- stage helpers
static const int kMaxAngles = 512;

// QPI Algorithm A, first part: window side checks, the carrier (given or detected from
// the first background) and the background field(s).
// Holograms per QPI launch: the row pass's window output T1 (N x M complex per
// hologram) up to 256 MB.  Larger launches measured faster on 121 x 1024^2 (0.56 ms in
// chunks of 32, 0.53 in 64, 0.50 in one of 121), the smaller ones slower (0.68 in 16).
static long qpi_chunk(int N, int M, int A)
{
    long chunk = (256l << 20) / ((long)N * M * 8);
    if (chunk < 2) chunk = 2;
    return chunk > A ? A : chunk;
}

static ctdm_status qpi_setup(ctdm_ctx *c, int N, int M, int A, const float *bg, int bg_per_angle,
                             const int *carrier_in, cudaStream_t s)
{
    if (N < 64 || N > 2048 || (N & (N - 1))) return invalid("hologram side %d unsupported", N);
    if (!ok_length(M) || M > N) return invalid("window side %d unsupported", M);
    if (A < 1) return invalid("no angles");
    CK(ensure(c, B_CARRIER, sizeof(int) * 3), "alloc carrier");
    CK(ensure(c, B_KEY, sizeof(unsigned long long)), "alloc key");
    int *car = B<int>(c, B_CARRIER);
    if (carrier_in && carrier_in[0] >= 0 && carrier_in[1] >= 0 && carrier_in[2] >= 0) {
        if (carrier_in[1] - M / 2 < 0 || carrier_in[1] + M / 2 > N || carrier_in[0] - M / 2 < 0 ||
            carrier_in[0] + M / 2 > N)
            return invalid("window around carrier (%d, %d) leaves the spectrum", carrier_in[0], carrier_in[1]);
        CK(set_carrier(car, carrier_in[0], carrier_in[1], carrier_in[2], s), "set carrier");
    } else {
        CK(ensure(c, B_SCRATCH, sizeof(float2) * N * N), "alloc carrier scratch");
        CK(qpi_find_carrier(bg, N, B<float2>(c, B_SCRATCH), B<unsigned long long>(c, B_KEY), car, s),
           "carrier search");
    }
    const long chunk = qpi_chunk(N, M, A);
    const long mm = (long)M * M, nn = (long)N * N;
    CK(ensure(c, B_T1, sizeof(float2) * chunk * N * M), "alloc T1");
    CK(ensure(c, B_S, sizeof(float2) * chunk * mm), "alloc S");
    const int nbg = bg_per_angle ? A : 1;
    CK(ensure(c, B_BGF, sizeof(float2) * nbg * mm), "alloc BG field");
    for (long a0 = 0; a0 < nbg; a0 += chunk) {
        const int ac = (int)std::min<long>(chunk, nbg - a0);
        CK(qpi_forward_window(bg + a0 * nn, 4, ac, N, M, car, B<float2>(c, B_T1), B<float2>(c, B_S), s),
           "qpi bg fwd");
        CK(qpi_inverse_window(B<float2>(c, B_S), ac, M, car, B<float2>(c, B_BGF) + a0 * mm, nullptr, 0, nullptr,
                              nullptr, s),
           "qpi bg inv");
    }
    return CTDM_OK;
}

// Second part: phase and amplitude of angles [first, first + count) (holo: the whole
// stack; the background fields of qpi_setup).
// holo: the stack, bpc bytes per pixel (4 float, 2 / 1 camera counts)
static ctdm_status qpi_angles(ctdm_ctx *c, int N, int M, int A, int first, int count, const void *holo, int bpc,
                              int bg_per_angle, float *phase, float *amp, cudaStream_t s)
{
    const long chunk = qpi_chunk(N, M, A);
    const long mm = (long)M * M, nn = (long)N * N;
    const int *car = B<int>(c, B_CARRIER);
    for (long a0 = first; a0 < first + count; a0 += chunk) {
        const int ac = (int)std::min<long>(chunk, first + count - a0);
        CK(qpi_forward_window(static_cast<const char *>(holo) + (size_t)bpc * a0 * nn, bpc, ac, N, M, car,
                              B<float2>(c, B_T1), B<float2>(c, B_S), s),
           "qpi fwd");
        const float2 *bgf = B<float2>(c, B_BGF) + (bg_per_angle ? a0 * mm : 0);
        CK(qpi_inverse_window(B<float2>(c, B_S), ac, M, car, nullptr, bgf, bg_per_angle ? mm : 0, phase + a0 * mm,
                              amp + a0 * mm, s),
           "qpi inv");
    }
    return CTDM_OK;
}

static ctdm_status do_qpi(ctdm_ctx *c, int N, int M, int A, const float *holo, const float *bg, int bg_per_angle,
                          const int *carrier_in, float *phase, float *amp, cudaStream_t s)
{
    ctdm_status st = qpi_setup(c, N, M, A, bg, bg_per_angle, carrier_in, s);
    if (st != CTDM_OK) return st;
    return qpi_angles(c, N, M, A, 0, A, holo, 4, bg_per_angle, phase, amp, s);
}

// The positivity loop (BatchRecon, cTDM/HilbertTransform.cu:1943-2004), or with
// accelerated = 1 the same projection step with Nesterov momentum (projected FISTA
// with the data-replacement step, no regulariser): the pass that applies est_n and
// modify keeps the projected iterate x_k and sends x_k + beta_k (x_k - x_{k-1}) on,
// beta_k = (t_{k-1} - 1) / t_k, t_0 = 1, t_k = (1 + sqrt(1 + 4 t_{k-1}^2)) / 2.  It is
// the gradient form's projected iteration at lambda 0 and unit step, fused into the
// loop passes (one extra read and write of x per iteration).
static ctdm_status do_positivity(ctdm_ctx *c, int R, int iters, int check_mode, double k2, double n_med,
                                 const float2 *F2, const uint8_t *mask, float2 *G, float2 *ri, cudaStream_t s,
                                 int accelerated = 0)
{
    LoopArgs la = {};
    la.G = G;
    la.F2 = F2;
    la.mask = mask;
    la.out = ri;
    la.R = R;
    la.inv_n3 = (float)(1.0 / ((double)R * R * R));
    la.k2 = (float)k2;
    la.n_med = (float)n_med;
    la.n_med2 = (float)(n_med * n_med);
    la.s1 = (float)(-1.0 / ((double)R * R * R * k2));
    la.s2 = (float)(-k2 / (n_med * n_med));
    la.err = c->d_err;
    CK(ensure_tuned(R, check_mode, s), "autotune loop passes");
    // the z pass reads the measured samples packed per tile when its plan allows
    const int TB = loop_ztile(R);
    la.packed = 0;
    if (TB > 0) {
        const long r3 = (long)R * R * R, tiles = (long)R * R / TB;
        CK(ensure(c, B_TMASK, sizeof(uint32_t) * tiles * R), "alloc packed masks");
        CK(ensure(c, B_TCOUNT, sizeof(int) * tiles), "alloc packed counts");
        CK(ensure(c, B_TPRE, sizeof(int) * tiles * R), "alloc packed prefixes");
        CK(ensure(c, B_TVALS, sizeof(float2) * r3), "alloc packed values");
        CK(pack_measured(F2, check_mode == CTDM_CHECK_MASK ? mask : nullptr, R, TB, B<uint32_t>(c, B_TMASK),
                         B<int>(c, B_TCOUNT), B<int>(c, B_TPRE), B<float2>(c, B_TVALS), s),
           "pack measured samples");
        la.tmask = B<uint32_t>(c, B_TMASK);
        la.tcount = B<int>(c, B_TCOUNT);
        la.tprefix = B<int>(c, B_TPRE);
        la.tvals = B<float2>(c, B_TVALS);
        la.packed = 1;
    }
    la.xprev = nullptr;
    la.beta = 0.f;
    if (accelerated && iters > 0) {
        CK(ensure(c, B_XPREV, sizeof(float2) * (size_t)R * R * R), "alloc accelerated iterate");
        la.xprev = B<float2>(c, B_XPREV);
    }
    double t_k = 1.0;
    auto next_beta = [&]() {   // beta of this iteration (0 for the first: x_{-1} is not used)
        const double t_n = 0.5 * (1.0 + std::sqrt(1.0 + 4.0 * t_k * t_k));
        la.beta = (float)((t_k - 1.0) / t_n);
        t_k = t_n;
    };
    StageTimer &tm = c->timer;
    if (loop_scheme(R) >= 1) {
        // plane + z passes, 8- or 4-CTA clusters per plane (schemes 1, 2; the plane pass
        // records under the x-pass stage)
        for (int it = 0; it < iters; it++) {
            next_beta();
            CK(launch_plane(la, false, s), "plane pass");
            tm.mark(S_XPASS, s);
            CK(launch_zpass(la, check_mode, s), "z pass");
            tm.mark(S_ZPASS, s);
        }
        CK(launch_plane(la, true, s), "final plane pass");
        tm.mark(S_XFINAL, s);
        return CTDM_OK;
    }
    CK(launch_ypass(la, true, s), "y inverse pass");
    tm.mark(S_YINV, s);
    for (int it = 0; it < iters; it++) {
        next_beta();
        CK(launch_xpass(la, false, s), "x pass");
        tm.mark(S_XPASS, s);
        CK(launch_ypass(la, false, s), "y forward pass");
        tm.mark(S_YFWD, s);
        CK(launch_zpass(la, check_mode, s), "z pass");
        tm.mark(S_ZPASS, s);
        CK(launch_ypass(la, true, s), "y inverse pass");
        tm.mark(S_YINV, s);
    }
    CK(launch_xpass(la, true, s), "final x pass");
    tm.mark(S_XFINAL, s);
    return CTDM_OK;
}

// QPI Algorithm B for A holograms: carrier columns (frame 1 and background, or given),
// background field(s), window rows, inverse transforms with the phase/amp epilogue.
// car: {background column, frame-1 column, -1} on the device.
static ctdm_status do_qpi_b(ctdm_ctx *c, int N, int A, const float *holo, const float *bg, int bg_per_angle,
                            const int *center_in, float *phase, float *amp, cudaStream_t s)
{
    if (N < 64 || N > 2048 || (N & (N - 1))) return invalid("hologram side %d unsupported", N);
    if (A < 1) return invalid("no angles");
    const int M = N / 4;
    const long mm = (long)M * M, nn = (long)N * N;
    CK(ensure(c, B_CARRIER, sizeof(int) * 3), "alloc carrier");
    int *car = B<int>(c, B_CARRIER);
    if (center_in && center_in[0] >= 0 && center_in[1] >= 0) {
        if (center_in[0] >= N || center_in[1] >= N) return invalid("carrier column outside the spectrum");
        CK(set_carrier(car, center_in[0], center_in[1], -1, s), "set carrier");
    } else {
        CK(ensure(c, B_QMAG, sizeof(float) * (N / 4) * N), "alloc histogram scratch");
        CK(set_carrier(car, 0, 0, -1, s), "reset carrier");
        // frame 1 of sequence1DFFT: the SP frame's own column first, then the background's
        CK(qpib_spectrum_center(holo, N, B<float>(c, B_QMAG), car + 1, s), "carrier column (frame 1)");
        CK(qpib_spectrum_center(bg, N, B<float>(c, B_QMAG), car, s), "carrier column (background)");
    }
    const int nbg = bg_per_angle ? A : 1;
    const int rows = A > nbg ? A : nbg;
    CK(ensure(c, B_T1, sizeof(float2) * rows * mm), "alloc window rows");
    CK(ensure(c, B_BGF, sizeof(float2) * nbg * mm), "alloc BG field");
    float2 *T = B<float2>(c, B_T1), *bgf = B<float2>(c, B_BGF);
    CK(qpib_window(bg, nbg, N, car, T, s), "qpi B background window");
    CK(qpib_inverse(T, nbg, M, bgf, nullptr, 0, nullptr, nullptr, s), "qpi B background field");
    CK(qpib_window(holo, 1, N, car + 1, T, s), "qpi B window (frame 1)");
    if (A > 1) CK(qpib_window(holo + nn, A - 1, N, car, T + mm, s), "qpi B window");
    CK(qpib_inverse(T, A, M, nullptr, bgf, bg_per_angle ? mm : 0, phase, amp, s), "qpi B fields");
    return CTDM_OK;
}

extern "C" ctdm_status ctdm_qpi_b(ctdm_ctx *c, int N, int A, const float *d_holo, const float *d_bg, int bg_per_angle,
                                  int *center2, float *d_phase, float *d_amp, void *stream)
{
    if (!c || !d_holo || !d_bg || !d_phase || !d_amp) return invalid("ctdm_qpi_b: NULL argument");
    if (in_flight(c))
        return invalid("ctdm_qpi_b: calls submitted on this context are still in flight (ctdm_wait first)");
    CK(cudaSetDevice(c->device), "cudaSetDevice");
    cudaStream_t s = (cudaStream_t)stream;
    ctdm_status st = do_qpi_b(c, N, A, d_holo, d_bg, bg_per_angle, center2, d_phase, d_amp, s);
    if (st != CTDM_OK) return st;
    CK(cudaMemcpyAsync(c->carrier, c->buf[B_CARRIER], sizeof(int) * 3, cudaMemcpyDeviceToHost, s), "carrier");
    CK(cudaStreamSynchronize(s), "carrier");
    c->carrier_pending = false;
    if (center2) {
        center2[0] = c->carrier[0];
        center2[1] = c->carrier[1];
    }
    g_err.clear();
    return CTDM_OK;
}

static ctdm_status validate(const ctdm_params *p, int A, int &M)
{
    if (!p) return invalid("params is NULL");
    const int N = p->n_holo;
    M = p->m_crop ? p->m_crop : N / 4;
    if (p->qpi_method != CTDM_QPI_A && p->qpi_method != CTDM_QPI_B) return invalid("unknown QPI method %d", p->qpi_method);
    if (p->qpi_method == CTDM_QPI_B && M != N / 4) return invalid("QPI Algorithm B fixes the window side to N/4");
    if (N < 64 || N > 2048 || (N & (N - 1))) return invalid("hologram side %d unsupported", N);
    if (!ok_crop(M) || M > N) return invalid("window side %d unsupported", M);
    if (!ok_volume(p->r_vol) || p->r_vol > N) return invalid("volume side %d unsupported", p->r_vol);
    if (A < 1 || A > kMaxAngles) return invalid("angle count %d outside 1..%d", A, kMaxAngles);
    if (p->iterations < 0) return invalid("negative iteration count");
    if (p->n_med <= 0 || p->wavelength <= 0 || p->dx <= 0) return invalid("non-positive physical parameter");
    if (p->unwrap_method < 0 || p->unwrap_method > 2) return invalid("unknown unwrap method");
    if (p->unwrap_mode != CTDM_UNWRAP_REF && p->unwrap_mode != CTDM_UNWRAP_EXACT)
        return invalid("unknown unwrap mode %d", p->unwrap_mode);
    if (p->check_mode != CTDM_CHECK_REF && p->check_mode != CTDM_CHECK_MASK)
        return invalid("unknown check mode %d", p->check_mode);
    if (p->accelerated != 0 && p->accelerated != 1) return invalid("accelerated must be 0 or 1");
    return CTDM_OK;
}

// ---------------------------------------------------------------- pipeline
// The whole path on stream s with the angle geometry already on the device.  It
// makes no host-synchronous call once the context's workspace has grown to the
// call's sizes, so a warmed-up call can be captured into a CUDA graph.
static ctdm_status pipeline_core(ctdm_ctx *c, const ctdm_params *p, int A, int M, const float *d_holo,
                                 const float *d_bg, const AngleGeom *d_geom, ctdm_cfloat *d_ri, cudaStream_t s,
                                 const ChunkFeed *feed = nullptr)
{
    ctdm_status st;
    const int N = p->n_holo, R = p->r_vol;
    const long mm = (long)M * M, rr = (long)R * R, r3 = rr * R;
    CK(ensure(c, B_PHASE, sizeof(float) * A * mm), "alloc phase");
    CK(ensure(c, B_AMP, sizeof(float) * A * mm), "alloc amp");
    CK(ensure(c, B_PHU, sizeof(float) * A * mm), "alloc unwrapped");
    CK(ensure(c, B_DCT, sizeof(float) * A * mm), "alloc dct scratch");
    CK(ensure(c, B_U, sizeof(float2) * A * rr), "alloc spectra");
    CK(ensure(c, B_F2, sizeof(float2) * r3), "alloc F2");
    CK(ensure(c, B_G, sizeof(float2) * r3), "alloc G");
    const bool mask_mode = p->check_mode == CTDM_CHECK_MASK;
    CK(ensure(c, B_COUNTS, mask_mode ? sizeof(uint32_t) * r3 : 0), "alloc counts");
    CK(ensure(c, B_MASK, mask_mode ? r3 : 0), "alloc mask");

    StageTimer &tm = c->timer;
    tm.start(s);
    const int car_in[3] = {p->carrier_r, p->carrier_c, p->carrier_radius};
    const bool alg_b = p->qpi_method == CTDM_QPI_B;
    const int per = feed ? feed->per : A;
    const int nchunks = (A + per - 1) / per;
    if (alg_b) {
        // Algorithm B takes its carrier columns from frame 1 and the background and then
        // runs on the whole stack: it waits for every chunk
        for (int k = 0; feed && k < nchunks; k++) CK(cudaStreamWaitEvent(s, feed->ready[k], 0), "wait for holograms");
        const int cen_in[2] = {p->carrier_c, p->carrier_c};
        st = do_qpi_b(c, N, A, d_holo, d_bg, p->bg_per_angle, cen_in, B<float>(c, B_PHASE), B<float>(c, B_AMP), s);
        if (st != CTDM_OK) return st;
        tm.mark(S_QPI, s);
    } else {
        st = qpi_setup(c, N, M, A, d_bg, p->bg_per_angle, car_in, s);
        if (st != CTDM_OK) return st;
    }

    // Goldstein: when its phase does not feed the reconstruction it runs on the side
    // stream (latency-bound, one CTA per map) beside the loop passes, and the call's
    // stream joins it at the end.
    const bool run_gold = p->run_goldstein || p->unwrap_method == CTDM_METHOD_GOLDSTEIN;
    const bool gold_side = run_gold && p->unwrap_method != CTDM_METHOD_GOLDSTEIN;
    if (run_gold) {
        CK(ensure(c, B_CHG, A * mm), "alloc charges");
        CK(ensure(c, B_CUT, A * mm), "alloc cuts");
        CK(ensure(c, B_GOLD, sizeof(float) * A * mm), "alloc goldstein out");
        CK(ensure(c, B_GSTATE, A * mm), "alloc goldstein state");
        CK(ensure(c, B_GLIST, sizeof(int) * 5 * A * mm), "alloc goldstein lists");
        CK(ensure(c, B_GSTATUS, sizeof(int) * A), "alloc goldstein status");
        CK(ensure(c, B_GWORK, A * mm), "alloc goldstein work");
    }
    if (p->unwrap_method == CTDM_METHOD_FAST) {
        CK(ensure(c, B_FASTIN, sizeof(float) * A * mm), "alloc fast-unwrap input");
        CK(ensure(c, B_FASTW, sizeof(float2) * 3 * 4 * mm), "alloc fast-unwrap work");
    }
    const float *unwrapped =
        p->unwrap_method == CTDM_METHOD_GOLDSTEIN ? B<float>(c, B_GOLD) : B<float>(c, B_PHU);
    // Front end per chunk of angles (one chunk unless the holograms arrive in chunks):
    // QPI, unwrapping, spectra.  Goldstein runs once over all maps (its kernels are
    // latency-bound per map, so chunks would repeat that latency): after the last
    // chunk's QPI when its phase feeds the reconstruction (the spectra follow it), else
    // on the side stream after the Ewald mapping.
    const bool gold_feeds = p->unwrap_method == CTDM_METHOD_GOLDSTEIN;
    auto goldstein_all = [&](cudaStream_t gs) -> ctdm_status {
        const float *ph_all = B<float>(c, B_PHASE);
        CK(goldstein_residues(ph_all, A, M, M, B<int8_t>(c, B_CHG), gs), "goldstein residues");
        CK(goldstein_cuts(B<int8_t>(c, B_CHG), A, M, M, B<uint8_t>(c, B_CUT), B<int8_t>(c, B_GWORK), gs),
           "goldstein cuts");
        CK(goldstein_floodfill(B<uint8_t>(c, B_CUT), ph_all, A, M, M, B<float>(c, B_GOLD), B<uint8_t>(c, B_GSTATE),
                               B<int>(c, B_GLIST), B<int>(c, B_GSTATUS), gs),
           "goldstein flood fill");
        return CTDM_OK;
    };
    auto spectra = [&](int a0, int ac) -> ctdm_status {
        const long o = (long)a0 * mm;
        float2 *U = B<float2>(c, B_U) + (long)a0 * rr;
        CK(prep_rytov(unwrapped + o, B<float>(c, B_AMP) + o, ac, M, N, R, U, s), "prep");
        CK(fft_rows(U, R, (long)ac * R, false, s), "spectra rows");
        CK(fft_cols(U, R, (long)ac * R, R, rr, R, false, s), "spectra cols");
        tm.mark(S_SPECTRA, s);
        return CTDM_OK;
    };
    for (int k = 0; k < nchunks; k++) {
        const int a0 = k * per, ac = std::min(per, A - a0);
        const long o = (long)a0 * mm;
        float *phase = B<float>(c, B_PHASE) + o;
        if (!alg_b) {
            if (feed) CK(cudaStreamWaitEvent(s, feed->ready[k], 0), "wait for holograms");
            const bool cnt = feed && feed->counts;
            st = qpi_angles(c, N, M, A, a0, ac, cnt ? feed->counts : d_holo, cnt ? feed->bpc : 4, p->bg_per_angle,
                            B<float>(c, B_PHASE), B<float>(c, B_AMP),
                            s);
            if (st != CTDM_OK) return st;
            tm.mark(S_QPI, s);
        }
        if (run_gold && !gold_side && k == nchunks - 1) {
            if ((st = goldstein_all(s)) != CTDM_OK) return st;
            tm.mark(S_GOLD, s);
        }
        if (gold_feeds) continue;
        if (p->unwrap_method == CTDM_METHOD_DCT) {
            CK(dct_unwrap(phase, B<float>(c, B_PHU) + o, B<float>(c, B_DCT) + o, ac, M, p->unwrap_mode, s),
               "dct unwrap");
        } else {
            CK(cudaMemcpyAsync(B<float>(c, B_FASTIN) + o, phase, sizeof(float) * ac * mm, cudaMemcpyDeviceToDevice,
                               s),
               "copy phase");
            CK(fast_unwrap(B<float>(c, B_FASTIN) + o, B<float>(c, B_PHU) + o, B<float2>(c, B_FASTW), ac, M, s),
               "fast unwrap");
        }
        tm.mark(S_UNWRAP, s);
        if ((st = spectra(a0, ac)) != CTDM_OK) return st;
    }
    if (gold_feeds && (st = spectra(0, A)) != CTDM_OK) return st;
    if (feed && feed->inputs_free) CK(cudaEventRecord(feed->inputs_free, s), "inputs read");

    const double fm0 = p->n_med / p->wavelength;
    const double df = 1.0 / (R * p->dx);
    const double k = 2.0 * CTDM_PI_D * p->n_med / p->wavelength;
    EwaldArgs ea = {};
    ea.U = B<float2>(c, B_U);
    ea.geom = d_geom;
    ea.A = A;
    ea.R = R;
    ea.fm0 = fm0;
    ea.df = df;
    ea.fm02 = fm0 * fm0;
    ea.fm02s = (float)((fm0 / df) * (fm0 / df));
    ea.dx = (float)p->dx;
    ea.F2 = B<float2>(c, B_F2);
    ea.G = B<float2>(c, B_G);
    ea.counts = mask_mode ? B<uint32_t>(c, B_COUNTS) : nullptr;
    ea.mask = mask_mode ? B<uint8_t>(c, B_MASK) : nullptr;
    CK(launch_ewald(ea, s), "ewald mapping");
    tm.mark(S_EWALD, s);
    if (feed && feed->front_done) CK(cudaEventRecord(feed->front_done, s), "front end done");
    if (gold_side) {
        // forked after the mapping, whose CTAs lose room on an SM to a resident fill,
        // so that it runs beside the loop passes
        CK(cudaEventRecord(c->fork, s), "fork");
        CK(cudaStreamWaitEvent(c->side, c->fork, 0), "fork wait");
        tm.side_mark(c->side);
        if ((st = goldstein_all(c->side)) != CTDM_OK) return st;
        tm.side_mark(c->side);
        CK(cudaEventRecord(c->join, c->side), "join");
    }
    // the final pass writes the output volume: the previous call's download of it first
    if (feed && feed->out_free) CK(cudaStreamWaitEvent(s, feed->out_free, 0), "wait for the volume download");
    st = do_positivity(c, R, p->iterations, p->check_mode, k * k, p->n_med, B<float2>(c, B_F2),
                       mask_mode ? B<uint8_t>(c, B_MASK) : nullptr, B<float2>(c, B_G),
                       reinterpret_cast<float2 *>(d_ri), s, p->accelerated);
    if (st != CTDM_OK) return st;
    if (gold_side) CK(cudaStreamWaitEvent(s, c->join, 0), "join wait");
    return CTDM_OK;
}

// The whole path with host angles: geometry upload, pipeline, carrier readback.
static ctdm_status reconstruct_core(ctdm_ctx *c, const ctdm_params *p, int A, int M, const float *d_holo,
                                    const float *d_bg, const float *h_angx, const float *h_angy, ctdm_cfloat *d_ri,
                                    cudaStream_t s, const ChunkFeed *feed)
{
    ctdm_status st = upload_geometry(c, h_angx, h_angy, A, p->n_med / p->wavelength, 1.0 / (p->r_vol * p->dx), s);
    if (st != CTDM_OK) return st;
    st = pipeline_core(c, p, A, M, d_holo, d_bg, B<AngleGeom>(c, B_GEOM), d_ri, s, feed);
    if (st != CTDM_OK) return st;
    // the carrier comes back into pinned staging without blocking; ctdm_ctx_carrier waits for it
    CK(cudaMemcpyAsync(c->pin->carrier, c->buf[B_CARRIER], sizeof(int) * 3, cudaMemcpyDeviceToHost, s),
       "carrier readback");
    CK(cudaEventRecord(c->carrier_done, s), "carrier readback");
    c->carrier_pending = true;
    return CTDM_OK;
}

extern "C" ctdm_status ctdm_reconstruct_device(ctdm_ctx *c, const ctdm_params *p, int A, const float *d_holo,
                                               const float *d_bg, const float *h_angx, const float *h_angy,
                                               ctdm_cfloat *d_ri, void *stream)
{
    if (!c || !d_holo || !d_bg || !h_angx || !h_angy || !d_ri) return invalid("ctdm_reconstruct_device: NULL argument");
    int M = 0;
    ctdm_status st = validate(p, A, M);
    if (st != CTDM_OK) return st;
    if (in_flight(c))
        return invalid("ctdm_reconstruct_device: calls submitted on this context are still in flight (ctdm_wait first)");
    CK(cudaSetDevice(c->device), "cudaSetDevice");
    st = reconstruct_core(c, p, A, M, d_holo, d_bg, h_angx, h_angy, d_ri, (cudaStream_t)stream, nullptr);
    if (st != CTDM_OK) return st;
    g_err.clear();
    return CTDM_OK;
}

// ---------------------------------------------------------------- internal interface (batch scheduler)
namespace ctdm {
ctdm_status validate_params(const ctdm_params *p, int A, int &M) { return validate(p, A, M); }

// Device bytes a context holds after a device-buffer reconstruction of this job: an
// upper bound of what pipeline_core and do_positivity allocate (the buffers of the
// front end, the volumes of the loop, the packed measured samples at the finest tile,
// the accelerated iterate).  The reference sizes its single reconstruction the same
// way from free device memory (ReconMode, cTDM/HilbertTransform.cu:1932-1939).
size_t workspace_bytes(const ctdm_params *p, int A, int M)
{
    const size_t N = (size_t)p->n_holo, R = (size_t)p->r_vol, mm = (size_t)M * M, rr = R * R, r3 = rr * R;
    size_t b = 16 * (size_t)A * mm;                          // phase, amplitude, unwrapped, DCT scratch
    b += 8 * (size_t)A * rr;                                 // per-angle spectra
    b += 16 * r3;                                            // F2, G
    if (p->check_mode == CTDM_CHECK_MASK) b += 5 * r3;       // hit counts, hit mask
    if (p->run_goldstein || p->unwrap_method == CTDM_METHOD_GOLDSTEIN)
        b += (size_t)A * mm * (1 + 1 + 4 + 1 + 20 + 1) + 4 * (size_t)A;   // charges, cuts, out, state, lists, work
    if (p->unwrap_method == CTDM_METHOD_FAST) b += 4 * (size_t)A * mm + 96 * mm;
    const size_t chunk = (size_t)qpi_chunk((int)N, M, A);
    b += chunk * N * M * 8 + chunk * mm * 8 + (p->bg_per_angle ? (size_t)A : 1) * mm * 8 + N * N * 8 + 64;
    if (p->qpi_method == CTDM_QPI_B) b += N * N + N * N * 2;          // column histogram scratch, window rows
    b += 9 * r3 + 4 * rr;                                    // packed samples, masks, prefixes (tiles of >= 8)
    if (p->accelerated && p->iterations > 0) b += 8 * r3;    // the accelerated loop's iterate
    b += sizeof(AngleGeom) * (size_t)A + 4096;
    return b;
}

size_t held_bytes(const ctdm_ctx *c)
{
    size_t b = 0;
    for (int i = 0; i < NBUF; i++) b += c->cap[i];
    return b;
}

// Frees every workspace buffer of c once the device is idle (a lane left out of a plan).
void release_workspace(ctdm_ctx *c)
{
    cudaSetDevice(c->device);
    cudaDeviceSynchronize();
    for (int i = 0; i < NBUF; i++) ensure(c, i, 0);
}
ctdm_status run_pipeline(ctdm_ctx *c, const ctdm_params *p, int A, const float *d_holo, const float *d_bg,
                         const AngleGeom *d_geom, ctdm_cfloat *d_ri, cudaStream_t s)
{
    int M = 0;
    ctdm_status st = validate(p, A, M);
    if (st != CTDM_OK) return st;
    CK(cudaSetDevice(c->device), "cudaSetDevice");
    return pipeline_core(c, p, A, M, d_holo, d_bg, d_geom, d_ri, s);
}
void make_geometry(const float *angx, const float *angy, int A, double fm0, double df, std::vector<AngleGeom> &g)
{
    angle_geometry(angx, angy, A, fm0, df, g);
}
ctdm_status fail_invalid(const char *msg) { return invalid("%s", msg); }
ctdm_status fail_cuda(cudaError_t e, const char *what) { return cuda_fail(e, what); }
ctdm_status fail_io(const std::string &msg)
{
    g_err = msg;
    return CTDM_ERR_IO;
}
void clear_error() { g_err.clear(); }
int max_angles() { return kMaxAngles; }
}  // namespace ctdm

// Host-buffer reconstruction.  bpc: bytes per hologram value, 4 (float) or 1 / 2 (integer
// camera counts, uploaded as they are: QPI Algorithm A reads them so, the background
// and Algorithm B's holograms are widened to float on the copy stream).
// The pending volume download on the download stream (once its volume is ready and
// after whatever that stream already waits for), then the device status word; the
// volume's slot is free again at vol_free.
static cudaError_t start_download(ctdm_ctx *c)
{
    ctdm_ctx::Download &d = c->dl;
    cudaError_t e = cudaStreamWaitEvent(c->d2h, c->vol_ready[d.slot], 0);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d.host, c->buf[d.slot ? B_RI2 : B_RI], d.bytes, cudaMemcpyDeviceToHost, c->d2h);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&c->pin->derr, c->d_err, sizeof(int), cudaMemcpyDeviceToHost, c->d2h);
    if (e == cudaSuccess) e = cudaEventRecord(c->vol_free[d.slot], c->d2h);
    d.pending = false;
    return e;
}

// Host-buffer call, enqueued only: the backgrounds, then the holograms in chunks of
// angles go up on the copy stream (the front end of a chunk runs while the later chunks
// are in flight), the pipeline runs on the legacy default stream and the volume comes
// back on the download stream.  Consecutive calls overlap: a call's uploads wait only
// until the previous call's front end has read the input buffers (so they run beside
// its loop), and its final pass waits for the previous call's download (which runs
// beside this call's front end).  With pageable host buffers the copies are staged by
// the driver and the overlap is lost, the result is the same.
static ctdm_status submit_enqueue(ctdm_ctx *c, const ctdm_params *p, int A, const void *h_holo, const void *h_bg,
                                  int bpc, const float *h_angx, const float *h_angy, ctdm_cfloat *h_ri)
{
    if (!c || !p || !h_holo || !h_bg || !h_ri) return invalid("ctdm_reconstruct: NULL argument");
    if (bpc != 1 && bpc != 2 && bpc != 4) return invalid("ctdm_submit: bytes per count must be 1, 2 or 4");
    int M = 0;
    ctdm_status st = validate(p, A, M);
    if (st != CTDM_OK) return st;
    CK(cudaSetDevice(c->device), "cudaSetDevice");
    const long nn = (long)p->n_holo * p->n_holo, r3 = (long)p->r_vol * p->r_vol * p->r_vol;
    const int nbg = p->bg_per_angle ? A : 1;
    const bool counts = bpc != 4;
    // QPI Algorithm A reads camera counts as they were uploaded; Algorithm B and the
    // background path take floats, widened on the copy stream
    const bool direct = counts && p->qpi_method == CTDM_QPI_A;
    const int slot = c->slot, vol = slot ? B_RI2 : B_RI;
    // a volume of another size: the pending download goes first (a buffer may move)
    if (c->dl.pending && c->dl.bytes != sizeof(float2) * r3) CK(start_download(c), "volume download");
    if (!direct) CK(ensure(c, B_HOLO, sizeof(float) * A * nn), "alloc holograms");
    CK(ensure(c, B_BG, sizeof(float) * nbg * nn), "alloc background");
    CK(ensure(c, vol, sizeof(float2) * r3), "alloc volume");
    if (counts) {
        CK(ensure(c, B_STAGE, (size_t)bpc * A * nn), "alloc hologram staging");
        CK(ensure(c, B_STAGEBG, (size_t)bpc * nbg * nn), "alloc background staging");
    }
    auto upload = [&](void *dst_stage, float *dst, const void *src, long count, bool widen) -> cudaError_t {
        if (!counts) return cudaMemcpyAsync(dst, src, sizeof(float) * count, cudaMemcpyHostToDevice, c->copy);
        cudaError_t e = cudaMemcpyAsync(dst_stage, src, (size_t)bpc * count, cudaMemcpyHostToDevice, c->copy);
        return e == cudaSuccess && widen ? widen_counts(dst_stage, bpc, count, dst, c->copy) : e;
    };
    cudaStream_t s = 0;
    // chunks of at least 32 angles keep each stage's grid full (8-angle chunks measured
    // 2.5x slower front ends); the first chunk's upload is the one not overlapped.  With
    // an earlier call still in flight the uploads finish beside its loop, before this
    // call starts, and one chunk runs the front end on full grids.
    const int per = c->in_flight > 0 ? A : std::max(32, (A + ctdm_ctx::kChunks - 1) / ctdm_ctx::kChunks);
    const int nchunks = (A + per - 1) / per;
    // the staging and input buffers: free once every earlier call's front end has read
    // them (a device-buffer or stage call in between ran on the default stream too)
    CK(cudaStreamWaitEvent(c->copy, c->inputs_free, 0), "copy start");
    CK(upload(c->buf[B_STAGEBG], B<float>(c, B_BG), h_bg, nbg * nn, true), "upload background");
    CK(cudaEventRecord(c->ready[ctdm_ctx::kChunks], c->copy), "background uploaded");
    const char *hsrc = static_cast<const char *>(h_holo);
    char *stage = static_cast<char *>(c->buf[B_STAGE]);
    for (int k = 0; k < nchunks; k++) {
        const long a0 = (long)k * per, ac = std::min<long>(per, A - a0);
        CK(upload(counts ? stage + (size_t)bpc * a0 * nn : nullptr, direct ? nullptr : B<float>(c, B_HOLO) + a0 * nn,
                  hsrc + (size_t)bpc * a0 * nn, ac * nn, !direct),
           "upload holograms");
        CK(cudaEventRecord(c->ready[k], c->copy), "holograms uploaded");
    }
    CK(cudaStreamWaitEvent(s, c->ready[ctdm_ctx::kChunks], 0), "wait for the background");
    const ChunkFeed feed = {c->ready, per, c->inputs_free, c->vol_free[slot], c->front_done,
                            direct ? c->buf[B_STAGE] : nullptr, bpc};
    st = reconstruct_core(c, p, A, M, B<float>(c, B_HOLO), B<float>(c, B_BG), h_angx, h_angy, B<ctdm_cfloat>(c, vol),
                          s, &feed);
    if (st != CTDM_OK) return st;
    // the previous call's volume: downloaded beside this call's loop
    if (c->dl.pending) {
        CK(cudaStreamWaitEvent(c->d2h, c->front_done, 0), "front end done");
        CK(start_download(c), "volume download");
    }
    CK(cudaEventRecord(c->vol_ready[slot], s), "volume ready");
    c->dl.host = h_ri;
    c->dl.bytes = sizeof(float2) * r3;
    c->dl.slot = slot;
    c->dl.pending = true;
    c->slot ^= 1;
    c->in_flight++;
    g_err.clear();
    return CTDM_OK;
}

static ctdm_status submit_host(ctdm_ctx *c, const ctdm_params *p, int A, const void *h_holo, const void *h_bg, int bpc,
                               const float *h_angx, const float *h_angy, ctdm_cfloat *h_ri)
{
    const ctdm_status st = submit_enqueue(c, p, A, h_holo, h_bg, bpc, h_angx, h_angy, h_ri);
    if (st != CTDM_OK && c) {
        // a call that failed part way may have copies in flight from the caller's buffers:
        // they finish before the error returns (their own errors are not reported)
        for (cudaStream_t q : {c->copy, c->d2h, (cudaStream_t)0}) cudaStreamSynchronize(q);
    }
    return st;
}

// Waits for every submitted call; reports a bounded device-side wait that ran out in
// any of them.
static ctdm_status wait_host(ctdm_ctx *c)
{
    if (!c) return invalid("ctdm_wait: NULL context");
    CK(cudaSetDevice(c->device), "cudaSetDevice");
    if (c->in_flight == 0) return CTDM_OK;
    if (c->dl.pending) CK(start_download(c), "volume download");
    CK(cudaStreamSynchronize(c->d2h), "synchronise");
    CK(cudaStreamSynchronize(0), "synchronise");
    c->in_flight = 0;
    // the device is idle: the next call starts again from the first volume buffer, so
    // a context that never has two calls in flight keeps only that one
    c->slot = 0;
    const int derr = c->pin->derr;
    if (derr != 0) {
        c->pin->derr = 0;
        cudaMemset(c->d_err, 0, sizeof(int));
        g_err = "a bounded device-side wait ran out (code " + std::to_string(derr) + ")";
        return CTDM_ERR_TIMEOUT;
    }
    g_err.clear();
    return CTDM_OK;
}

static ctdm_status reconstruct_host(ctdm_ctx *c, const ctdm_params *p, int A, const void *h_holo, const void *h_bg,
                                    int bpc, const float *h_angx, const float *h_angy, ctdm_cfloat *h_ri)
{
    ctdm_status st = submit_host(c, p, A, h_holo, h_bg, bpc, h_angx, h_angy, h_ri);
    if (st != CTDM_OK) return st;
    return wait_host(c);
}

extern "C" ctdm_status ctdm_submit(ctdm_ctx *c, const ctdm_params *p, int A, const void *h_holo, const void *h_bg,
                                   int bytes_per_count, const float *h_angx, const float *h_angy, ctdm_cfloat *h_ri)
{
    return submit_host(c, p, A, h_holo, h_bg, bytes_per_count, h_angx, h_angy, h_ri);
}

extern "C" ctdm_status ctdm_wait(ctdm_ctx *c)
{
    return wait_host(c);
}

extern "C" ctdm_status ctdm_reconstruct(ctdm_ctx *c, const ctdm_params *p, int A, const float *h_holo,
                                        const float *h_bg, const float *h_angx, const float *h_angy,
                                        ctdm_cfloat *h_ri)
{
    return reconstruct_host(c, p, A, h_holo, h_bg, 4, h_angx, h_angy, h_ri);
}

extern "C" ctdm_status ctdm_reconstruct_u16(ctdm_ctx *c, const ctdm_params *p, int A, const uint16_t *h_holo,
                                            const uint16_t *h_bg, const float *h_angx, const float *h_angy,
                                            ctdm_cfloat *h_ri)
{
    return reconstruct_host(c, p, A, h_holo, h_bg, 2, h_angx, h_angy, h_ri);
}

extern "C" ctdm_status ctdm_reconstruct_u8(ctdm_ctx *c, const ctdm_params *p, int A, const uint8_t *h_holo,
                                           const uint8_t *h_bg, const float *h_angx, const float *h_angy,
                                           ctdm_cfloat *h_ri)
{
    return reconstruct_host(c, p, A, h_holo, h_bg, 1, h_angx, h_angy, h_ri);
}

// ---------------------------------------------------------------- stage API
extern "C" ctdm_status ctdm_qpi(ctdm_ctx *c, int N, int M, int A, const float *d_holo, const float *d_bg,
                                int bg_per_angle, int *carrier3, float *d_phase, float *d_amp, void *stream)
{
    if (!c || !d_holo || !d_bg || !d_phase || !d_amp) return invalid("ctdm_qpi: NULL argument");
    if (in_flight(c))
        return invalid("ctdm_qpi: calls submitted on this context are still in flight (ctdm_wait first)");
    CK(cudaSetDevice(c->device), "cudaSetDevice");
    cudaStream_t s = (cudaStream_t)stream;
    ctdm_status st = do_qpi(c, N, M, A, d_holo, d_bg, bg_per_angle, carrier3, d_phase, d_amp, s);
    if (st != CTDM_OK) return st;
    CK(cudaMemcpyAsync(c->carrier, c->buf[B_CARRIER], sizeof(int) * 3, cudaMemcpyDeviceToHost, s), "carrier");
    CK(cudaStreamSynchronize(s), "synchronise");
    c->carrier_pending = false;
    if (carrier3) std::memcpy(carrier3, c->carrier, sizeof c->carrier);
    return CTDM_OK;
}

extern "C" ctdm_status ctdm_unwrap_dct(ctdm_ctx *c, int A, int M, int mode, const float *d_phi, float *d_out,
                                       void *stream)
{
    if (!c || !d_phi || !d_out) return invalid("ctdm_unwrap_dct: NULL argument");
    if (in_flight(c))
        return invalid("ctdm_unwrap_dct: calls submitted on this context are still in flight (ctdm_wait first)");
    if (!ok_crop(M) || A < 1) return invalid("ctdm_unwrap_dct: size %d unsupported", M);
    if (mode != CTDM_UNWRAP_REF && mode != CTDM_UNWRAP_EXACT) return invalid("ctdm_unwrap_dct: unknown mode %d", mode);
    CK(cudaSetDevice(c->device), "cudaSetDevice");
    CK(ensure(c, B_TMP, sizeof(float) * A * M * M), "alloc scratch");
    CK(dct_unwrap(d_phi, d_out, B<float>(c, B_TMP), A, M, mode, (cudaStream_t)stream), "dct unwrap");
    return CTDM_OK;
}

extern "C" ctdm_status ctdm_unwrap_fast(ctdm_ctx *c, int A, int M, float *d_phi, float *d_out, void *stream)
{
    if (!c || !d_phi || !d_out) return invalid("ctdm_unwrap_fast: NULL argument");
    if (in_flight(c))
        return invalid("ctdm_unwrap_fast: calls submitted on this context are still in flight (ctdm_wait first)");
    if (!ok_crop(M) || A < 1) return invalid("ctdm_unwrap_fast: size %d unsupported", M);
    CK(cudaSetDevice(c->device), "cudaSetDevice");
    CK(ensure(c, B_FASTW, sizeof(float2) * 3 * 4 * M * M), "alloc scratch");
    CK(fast_unwrap(d_phi, d_out, B<float2>(c, B_FASTW), A, M, (cudaStream_t)stream), "fast unwrap");
    return CTDM_OK;
}

extern "C" ctdm_status ctdm_goldstein(ctdm_ctx *c, int A, int W, int H, const float *d_phi, int8_t *d_charges,
                                      uint8_t *d_cuts, float *d_out, int *h_status, void *stream)
{
    if (!c || !d_phi || !d_charges || !d_cuts || !d_out) return invalid("ctdm_goldstein: NULL argument");
    if (in_flight(c))
        return invalid("ctdm_goldstein: calls submitted on this context are still in flight (ctdm_wait first)");
    if (W < 4 || H < 4 || W > 1024 || H > 1024 || A < 1) return invalid("ctdm_goldstein: size unsupported");
    CK(cudaSetDevice(c->device), "cudaSetDevice");
    cudaStream_t s = (cudaStream_t)stream;
    const long n = (long)W * H;
    CK(ensure(c, B_GSTATE, A * n), "alloc state");
    CK(ensure(c, B_GLIST, sizeof(int) * 5 * A * n), "alloc lists");
    CK(ensure(c, B_GSTATUS, sizeof(int) * A), "alloc status");
    CK(ensure(c, B_TMP, A * n), "alloc work");
    CK(goldstein_residues(d_phi, A, W, H, d_charges, s), "residues");
    CK(goldstein_cuts(d_charges, A, W, H, d_cuts, B<int8_t>(c, B_TMP), s), "branch cuts");
    CK(goldstein_floodfill(d_cuts, d_phi, A, W, H, d_out, B<uint8_t>(c, B_GSTATE), B<int>(c, B_GLIST),
                           B<int>(c, B_GSTATUS), s),
       "flood fill");
    std::vector<int> stv(A);
    CK(cudaMemcpyAsync(stv.data(), c->buf[B_GSTATUS], sizeof(int) * A, cudaMemcpyDeviceToHost, s), "status");
    CK(cudaStreamSynchronize(s), "synchronise");
    bool stalled = false;
    for (int a = 0; a < A; a++) stalled |= stv[a] != 0;
    if (h_status) std::memcpy(h_status, stv.data(), sizeof(int) * A);
    if (stalled) {
        set_err("ctdm_goldstein: flood fill stopped early on at least one map");
        return CTDM_ERR_STALLED;
    }
    return CTDM_OK;
}

extern "C" ctdm_status ctdm_goldstein_fill(ctdm_ctx *c, int A, int W, int H, const uint8_t *d_cuts,
                                           const float *d_phi, float *d_out, int *h_status, void *stream)
{
    if (!c || !d_cuts || !d_phi || !d_out) return invalid("ctdm_goldstein_fill: NULL argument");
    if (in_flight(c))
        return invalid("ctdm_goldstein_fill: calls submitted on this context are still in flight (ctdm_wait first)");
    if (W < 4 || H < 4 || W > 1024 || H > 1024 || A < 1) return invalid("ctdm_goldstein_fill: size unsupported");
    CK(cudaSetDevice(c->device), "cudaSetDevice");
    cudaStream_t s = (cudaStream_t)stream;
    const long n = (long)W * H;
    CK(ensure(c, B_GSTATE, A * n), "alloc state");
    CK(ensure(c, B_GLIST, sizeof(int) * 5 * A * n), "alloc lists");
    CK(ensure(c, B_GSTATUS, sizeof(int) * A), "alloc status");
    CK(goldstein_floodfill(d_cuts, d_phi, A, W, H, d_out, B<uint8_t>(c, B_GSTATE), B<int>(c, B_GLIST),
                           B<int>(c, B_GSTATUS), s),
       "flood fill");
    std::vector<int> stv(A);
    CK(cudaMemcpyAsync(stv.data(), c->buf[B_GSTATUS], sizeof(int) * A, cudaMemcpyDeviceToHost, s), "status");
    CK(cudaStreamSynchronize(s), "synchronise");
    if (h_status) std::memcpy(h_status, stv.data(), sizeof(int) * A);
    return CTDM_OK;
}

extern "C" ctdm_status ctdm_prepare_spectra(ctdm_ctx *c, int A, int M, int N, int R, const float *d_phase,
                                            const float *d_amp, ctdm_cfloat *d_U, void *stream)
{
    if (!c || !d_phase || !d_amp || !d_U) return invalid("ctdm_prepare_spectra: NULL argument");
    if (in_flight(c))
        return invalid("ctdm_prepare_spectra: calls submitted on this context are still in flight (ctdm_wait first)");
    if (!ok_volume(R) || R > N || M < 2 || A < 1) return invalid("ctdm_prepare_spectra: size unsupported");
    CK(cudaSetDevice(c->device), "cudaSetDevice");
    cudaStream_t s = (cudaStream_t)stream;
    float2 *U = reinterpret_cast<float2 *>(d_U);
    CK(prep_rytov(d_phase, d_amp, A, M, N, R, U, s), "prep");
    CK(fft_rows(U, R, (long)A * R, false, s), "rows");
    CK(fft_cols(U, R, (long)A * R, R, (long)R * R, R, false, s), "cols");
    return CTDM_OK;
}

extern "C" ctdm_status ctdm_stack_spectra(ctdm_ctx *c, int A, int R, const float *d_ph, const float *d_am,
                                          ctdm_cfloat *d_U, void *stream)
{
    if (!c || !d_ph || !d_am || !d_U) return invalid("ctdm_stack_spectra: NULL argument");
    if (in_flight(c))
        return invalid("ctdm_stack_spectra: calls submitted on this context are still in flight (ctdm_wait first)");
    if (!ok_volume(R) || A < 1) return invalid("ctdm_stack_spectra: size unsupported");
    CK(cudaSetDevice(c->device), "cudaSetDevice");
    cudaStream_t s = (cudaStream_t)stream;
    float2 *U = reinterpret_cast<float2 *>(d_U);
    CK(stack_to_rytov(d_ph, d_am, A, R, U, s), "stack prep");
    CK(fft_rows(U, R, (long)A * R, false, s), "rows");
    CK(fft_cols(U, R, (long)A * R, R, (long)R * R, R, false, s), "cols");
    return CTDM_OK;
}

extern "C" ctdm_status ctdm_prepare_stack(ctdm_ctx *c, int A, int M, int N, int R, const float *d_phase,
                                          const float *d_amp, float *d_ph_out, float *d_am_out, void *stream)
{
    if (!c || !d_phase || !d_amp || !d_ph_out || !d_am_out) return invalid("ctdm_prepare_stack: NULL argument");
    if (in_flight(c))
        return invalid("ctdm_prepare_stack: calls submitted on this context are still in flight (ctdm_wait first)");
    if (R > N || R < 1 || M < 2 || A < 1) return invalid("ctdm_prepare_stack: size unsupported");
    CK(cudaSetDevice(c->device), "cudaSetDevice");
    CK(prep_stack(d_phase, d_amp, A, M, N, R, d_ph_out, d_am_out, (cudaStream_t)stream), "prep stack");
    return CTDM_OK;
}

extern "C" ctdm_status ctdm_map_ewald(ctdm_ctx *c, int A, int R, const ctdm_cfloat *d_U, const float *h_angx,
                                      const float *h_angy, double fm0, double df, double dx, ctdm_cfloat *d_F2,
                                      uint32_t *d_counts, void *stream)
{
    if (!c || !d_U || !h_angx || !h_angy || !d_F2) return invalid("ctdm_map_ewald: NULL argument");
    if (in_flight(c))
        return invalid("ctdm_map_ewald: calls submitted on this context are still in flight (ctdm_wait first)");
    if (!ok_volume(R) || A < 1 || A > kMaxAngles) return invalid("ctdm_map_ewald: size unsupported");
    CK(cudaSetDevice(c->device), "cudaSetDevice");
    cudaStream_t s = (cudaStream_t)stream;
    const long r3 = (long)R * R * R;
    ctdm_status st = upload_geometry(c, h_angx, h_angy, A, fm0, df, s);
    if (st != CTDM_OK) return st;
    CK(ensure(c, B_TMP, sizeof(float2) * r3), "alloc G");
    EwaldArgs ea = {};
    ea.U = reinterpret_cast<const float2 *>(d_U);
    ea.geom = B<AngleGeom>(c, B_GEOM);
    ea.A = A;
    ea.R = R;
    ea.fm0 = fm0;
    ea.df = df;
    ea.fm02 = fm0 * fm0;
    ea.fm02s = (float)((fm0 / df) * (fm0 / df));
    ea.dx = (float)dx;
    ea.F2 = reinterpret_cast<float2 *>(d_F2);
    ea.G = B<float2>(c, B_TMP);
    ea.counts = d_counts;
    ea.mask = nullptr;
    CK(launch_ewald(ea, s), "ewald mapping");
    return CTDM_OK;
}

extern "C" ctdm_status ctdm_map_fi(ctdm_ctx *c, int A, int R, const ctdm_cfloat *d_U, const float *h_angx,
                                   double fm0, double df, double dx, ctdm_cfloat *d_F2, uint32_t *d_counts,
                                   void *stream)
{
    if (!c || !d_U || !h_angx || !d_F2) return invalid("ctdm_map_fi: NULL argument");
    if (in_flight(c))
        return invalid("ctdm_map_fi: calls submitted on this context are still in flight (ctdm_wait first)");
    if (!ok_volume(R) || A < 1 || A > kMaxAngles) return invalid("ctdm_map_fi: size unsupported");
    for (int a = 0; a < A; a++)
        if (!std::isfinite(h_angx[a]) || std::fabs(h_angx[a]) >= 0.5 * CTDM_PI_D)
            return invalid("ctdm_map_fi: scan angle %d outside (-pi/2, pi/2)", a);
    CK(cudaSetDevice(c->device), "cudaSetDevice");
    cudaStream_t s = (cudaStream_t)stream;
    const long r3 = (long)R * R * R;
    // one scan axis: the tilt AngX, AngY taken as zero (FrquencyInterpolation uses AngleX only)
    std::vector<float> zeros(A, 0.f);
    ctdm_status st = upload_geometry(c, h_angx, zeros.data(), A, fm0, df, s);
    if (st != CTDM_OK) return st;
    // scan angles ascending (ties in frame order) and their frames
    std::vector<int> order(A);
    for (int a = 0; a < A; a++) order[a] = a;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return h_angx[x] < h_angx[y]; });
    std::vector<unsigned char> tab(A * (sizeof(double) + sizeof(int)));
    double *th = reinterpret_cast<double *>(tab.data());
    int *fr = reinterpret_cast<int *>(th + A);
    for (int k = 0; k < A; k++) {
        th[k] = (double)h_angx[order[k]];
        fr[k] = order[k];
    }
    CK(ensure(c, B_FIT, tab.size()), "alloc FI tables");
    CK(cudaMemcpyAsync(c->buf[B_FIT], tab.data(), tab.size(), cudaMemcpyHostToDevice, s), "upload FI tables");
    CK(ensure(c, B_TMP, sizeof(float2) * r3), "alloc G");
    EwaldArgs ea = {};
    ea.U = reinterpret_cast<const float2 *>(d_U);
    ea.geom = B<AngleGeom>(c, B_GEOM);
    ea.A = A;
    ea.R = R;
    ea.fm0 = fm0;
    ea.df = df;
    ea.fm02 = fm0 * fm0;
    ea.fm02s = (float)((fm0 / df) * (fm0 / df));
    ea.dx = (float)dx;
    ea.F2 = reinterpret_cast<float2 *>(d_F2);
    ea.G = B<float2>(c, B_TMP);
    ea.counts = d_counts;
    ea.fi_theta = B<double>(c, B_FIT);
    ea.fi_frame = reinterpret_cast<const int *>(B<double>(c, B_FIT) + A);
    CK(launch_ewald(ea, s), "frequency-interpolation mapping");
    return CTDM_OK;
}

extern "C" void ctdm_pocs_defaults(ctdm_pocs_params *p)
{
    if (!p) return;
    // BatchReconPOCS (cTDM/HilbertTransform.cu:2133-2141, 2208): 100 iterations of 20 TV steps
    p->iterations = 100;
    p->tv_steps = 20;
    p->beta = 1.0;
    p->beta_red = 0.995;
    p->alpha = 0.2;
    p->alpha_red = 0.95;
    p->r_max = 0.95;
    p->eps_data = 0.0;
    p->tv_eps = 1e-8;
}

extern "C" ctdm_status ctdm_pocs(ctdm_ctx *c, int R, const ctdm_pocs_params *p, double k2, double n_med,
                                 const ctdm_cfloat *d_F2, ctdm_cfloat *d_ri, double *h_hist, void *stream)
{
    if (!c || !p || !d_F2 || !d_ri) return invalid("ctdm_pocs: NULL argument");
    if (in_flight(c))
        return invalid("ctdm_pocs: calls submitted on this context are still in flight (ctdm_wait first)");
    if (!ok_volume(R)) return invalid("ctdm_pocs: volume side %d unsupported", R);
    if (p->iterations < 0 || p->iterations > 100000 || p->tv_steps < 1 || p->tv_steps > 1000)
        return invalid("ctdm_pocs: iterations or tv_steps out of range");
    if (!(k2 > 0) || !(n_med > 0) || !(p->tv_eps >= 0)) return invalid("ctdm_pocs: k2, n_med and tv_eps");
    CK(cudaSetDevice(c->device), "cudaSetDevice");
    cudaStream_t s = (cudaStream_t)stream;
    const long r3 = (long)R * R * R;
    const int nh = p->iterations > 0 ? p->iterations : 1;
    const int vol[] = {B_PV, B_PG, B_PV2, B_PG2, B_PVP};
    for (int id : vol) CK(ensure(c, id, sizeof(float) * r3), "alloc POCS volumes");
    CK(ensure(c, B_G, sizeof(float2) * r3), "alloc G");
    CK(ensure(c, B_PPART, sizeof(double) * pocs_partials(R)), "alloc partial sums");
    CK(ensure(c, B_PCTL, sizeof(PocsCtl)), "alloc controller");
    CK(ensure(c, B_PHIST, sizeof(double) * 4 * nh), "alloc history");
    const bool want_dd = h_hist != nullptr || p->eps_data > 0;
    PocsCtl ctl = {};
    ctl.beta = p->beta;
    ctl.beta_red = p->beta_red;
    ctl.alpha = p->alpha;
    ctl.alpha_red = p->alpha_red;
    ctl.r_max = p->r_max;
    ctl.eps_data = p->eps_data;
    ctl.dd = want_dd ? 0.0 : HUGE_VAL;   // not measured: the data condition holds
    ctl.first = 1;
    ctl.n_hist = p->iterations;
    PocsBufs b;
    b.V = B<float>(c, B_PV);
    b.g = B<float>(c, B_PG);
    b.V2 = B<float>(c, B_PV2);
    b.g2 = B<float>(c, B_PG2);
    b.Vp = B<float>(c, B_PVP);
    b.G = B<float2>(c, B_G);
    b.F2 = reinterpret_cast<const float2 *>(d_F2);
    b.part = B<double>(c, B_PPART);
    b.ctl = B<PocsCtl>(c, B_PCTL);
    b.hist = B<double>(c, B_PHIST);
    b.R = R;
    b.y_scale = (float)(-1.0 / k2);
    b.tv_eps = (float)p->tv_eps;
    CK(cudaMemcpyAsync(b.ctl, &ctl, sizeof ctl, cudaMemcpyHostToDevice, s), "upload controller");
    CK(cudaMemsetAsync(b.V, 0, sizeof(float) * r3, s), "zero V");
    CK(cudaMemsetAsync(b.G, 0, sizeof(float2) * r3, s), "zero G");
    for (int it = 0; it < p->iterations; it++) CK(pocs_iteration(b, p->tv_steps, want_dd, s), "POCS iteration");
    CK(pocs_finish(b, (float)n_med, reinterpret_cast<float2 *>(d_ri), s), "POCS output");
    if (h_hist && p->iterations > 0) {
        CK(cudaMemcpyAsync(h_hist, b.hist, sizeof(double) * 4 * p->iterations, cudaMemcpyDeviceToHost, s),
           "history");
        CK(cudaStreamSynchronize(s), "history");
    }
    g_err.clear();
    return CTDM_OK;
}

extern "C" ctdm_status ctdm_positivity_ex(ctdm_ctx *c, int R, int iterations, int check_mode, int accelerated,
                                          double k2, double n_med, const ctdm_cfloat *d_F2, const uint32_t *d_counts,
                                          ctdm_cfloat *d_ri, void *stream);

extern "C" ctdm_status ctdm_positivity(ctdm_ctx *c, int R, int iterations, int check_mode, double k2, double n_med,
                                       const ctdm_cfloat *d_F2, const uint32_t *d_counts, ctdm_cfloat *d_ri,
                                       void *stream)
{
    return ctdm_positivity_ex(c, R, iterations, check_mode, 0, k2, n_med, d_F2, d_counts, d_ri, stream);
}

extern "C" ctdm_status ctdm_positivity_ex(ctdm_ctx *c, int R, int iterations, int check_mode, int accelerated,
                                          double k2, double n_med, const ctdm_cfloat *d_F2, const uint32_t *d_counts,
                                          ctdm_cfloat *d_ri, void *stream)
{
    if (!c || !d_F2 || !d_ri) return invalid("ctdm_positivity: NULL argument");
    if (in_flight(c))
        return invalid("ctdm_positivity: calls submitted on this context are still in flight (ctdm_wait first)");
    if (!ok_volume(R) || iterations < 0) return invalid("ctdm_positivity: size unsupported");
    if (accelerated != 0 && accelerated != 1) return invalid("ctdm_positivity: accelerated must be 0 or 1");
    if (check_mode == CTDM_CHECK_MASK && !d_counts) return invalid("ctdm_positivity: mask mode needs counts");
    CK(cudaSetDevice(c->device), "cudaSetDevice");
    cudaStream_t s = (cudaStream_t)stream;
    const long rr = (long)R * R, r3 = rr * R;
    CK(ensure(c, B_G, sizeof(float2) * r3), "alloc G");
    float2 *G = B<float2>(c, B_G);
    CK(cudaMemcpyAsync(G, d_F2, sizeof(float2) * r3, cudaMemcpyDeviceToDevice, s), "copy F2");
    CK(fft_cols(G, R, rr, (int)rr, 0, rr, true, s), "z inverse");
    const uint8_t *mask = nullptr;
    if (check_mode == CTDM_CHECK_MASK) {
        CK(ensure(c, B_MASK, r3), "alloc mask");
        CK(counts_to_mask(d_counts, B<uint8_t>(c, B_MASK), r3, s), "mask");
        mask = B<uint8_t>(c, B_MASK);
    }
    c->timer.start(s);
    return do_positivity(c, R, iterations, check_mode, k2, n_med, reinterpret_cast<const float2 *>(d_F2), mask, G,
                         reinterpret_cast<float2 *>(d_ri), s, accelerated);
}

extern "C" ctdm_status ctdm_fft(ctdm_cfloat *d_data, int rank, const int *dims, int batch, int inverse, void *stream)
{
    if (!d_data || !dims || rank < 1 || rank > 3 || batch < 1) return invalid("ctdm_fft: bad argument");
    for (int r = 0; r < rank; r++)
        if (!ok_length(dims[r])) return invalid("ctdm_fft: length %d unsupported", dims[r]);
    if (reinterpret_cast<uintptr_t>(d_data) & 15) return invalid("ctdm_fft: data must be 16-byte aligned");
    CK(ensure_tables(), "tables");
    cudaStream_t s = (cudaStream_t)stream;
    float2 *d = reinterpret_cast<float2 *>(d_data);
    const long nx = dims[0], ny = rank > 1 ? dims[1] : 1, nz = rank > 2 ? dims[2] : 1;
    const long per = nx * ny * nz;
    CK(fft_rows(d, (int)nx, per / nx * batch, inverse != 0, s), "fft x");
    if (rank > 1) CK(fft_cols(d, (int)ny, nx * nz * batch, (int)nx, nx * ny, nx, inverse != 0, s), "fft y");
    if (rank > 2) CK(fft_cols(d, (int)nz, nx * ny * batch, (int)(nx * ny), per, nx * ny, inverse != 0, s), "fft z");
    return CTDM_OK;
}

// ---------------------------------------------------------------- reference-named entry points
static std::mutex g_def_mu;
static std::map<int, ctdm_ctx *> g_default;

static ctdm_ctx *default_ctx()
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
    std::lock_guard<std::mutex> lk(g_def_mu);
    auto it = g_default.find(dev);
    if (it != g_default.end()) return it->second;
    ctdm_ctx *c = nullptr;
    if (ctdm_ctx_create(dev, &c) != CTDM_OK) return nullptr;
    g_default[dev] = c;
    return c;
}

static bool finish(const char *what)
{
    cudaError_t e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) {
        cuda_fail(e, what);
        return false;
    }
    g_err.clear();
    return true;
}

// Reference globals for BatchRecon (cTDM/HilbertTransform.cu:11-35).
static int g_recon = 256, g_iter_time = 100, g_recon_save = 0;
static double g_nmed = 1.333, g_wavelength_nm = 532, g_pixel_um = 5.5, g_mag = 85.0;
static std::string g_save_dir = ".";

extern "C" void ctdm_set_recon_globals(int recon_size, double n_med, double wavelength_nm, double camera_pixel_um,
                                       double mag, int iter_time, int recon_save, const char *save_dir)
{
    g_recon = recon_size;
    g_nmed = n_med;
    g_wavelength_nm = wavelength_nm;
    g_pixel_um = camera_pixel_um;
    g_mag = mag;
    g_iter_time = iter_time;
    g_recon_save = recon_save;
    g_save_dir = save_dir ? save_dir : ".";
}

// Carrier {row, column, radius} of Algorithm A per device, set by frame 1 (the reference
// keeps rCircle, cCircle and radiusCircle as globals that obtainRadius sets when
// frame == 1, cTDM/HilbertTransform.cu:1572).
static std::map<int, std::array<int, 3>> g_qpia_carrier;

// extractQPI_AlgorithmA (cTDM/HilbertTransform.cu:1546-1585): host holograms as
// cufftComplex with zero imaginary parts (the job loop fills them that way,
// :711-716,879-883); the M x M fields (M = N / 4) after the inverse transform, 1/M^2 and
// the conjugation of scaleFFT2D go to cuSP_FFT / cuBG_FFT on the device.  The reference
// writes them into its globals cuSP2 / cuBG2, which its call sites pass as these two
// arguments (:969,972), so the caller sees the same arrays.
extern "C" void extractQPI_AlgorithmA(ctdm_cfloat *SP, ctdm_cfloat *BG, ctdm_cfloat *cuSP_FFT, ctdm_cfloat *cuBG_FFT,
                                      int Nx, int Ny, int frame)
{
    ctdm_ctx *c = default_ctx();
    if (!c) return;
    if (!SP || !BG || !cuSP_FFT || !cuBG_FFT) { invalid("extractQPI_AlgorithmA: NULL argument"); return; }
    if (Nx != Ny || Nx < 64 || Nx > 2048 || (Nx & (Nx - 1))) {
        invalid("extractQPI_AlgorithmA: square power-of-two holograms of 64..2048 only");
        return;
    }
    const int N = Nx, M = N / 4;
    const long nn = (long)N * N, mm = (long)M * M;
    const int *known = nullptr;
    std::array<int, 3> kept{};
    if (frame != 1) {
        auto it = g_qpia_carrier.find(c->device);
        if (it == g_qpia_carrier.end()) { invalid("extractQPI_AlgorithmA: frame 1 has not run on this device"); return; }
        kept = it->second;
        known = kept.data();
    }
    if (wait_host(c) != CTDM_OK) return;   // host-buffer calls in flight still own B_HOLO / B_BG
    if (ensure(c, B_HOLO, sizeof(float) * nn) != cudaSuccess || ensure(c, B_BG, sizeof(float) * nn) != cudaSuccess ||
        ensure(c, B_TMP, sizeof(float2) * nn) != cudaSuccess) {
        cuda_fail(cudaErrorMemoryAllocation, "extractQPI_AlgorithmA");
        return;
    }
    float2 *stage = B<float2>(c, B_TMP);
    cudaError_t e = cudaMemcpy(stage, BG, sizeof(float2) * nn, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = real_parts(stage, B<float>(c, B_BG), nn, 0);
    if (e == cudaSuccess) e = cudaMemcpy(stage, SP, sizeof(float2) * nn, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = real_parts(stage, B<float>(c, B_HOLO), nn, 0);
    if (e != cudaSuccess) { cuda_fail(e, "extractQPI_AlgorithmA upload"); return; }
    // carrier (detected from the background on frame 1) and the background field
    if (qpi_setup(c, N, M, 1, B<float>(c, B_BG), 0, known, 0) != CTDM_OK) return;
    if (frame == 1) {
        int host[3] = {0, 0, 0};
        e = cudaMemcpy(host, c->buf[B_CARRIER], sizeof host, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) { cuda_fail(e, "extractQPI_AlgorithmA carrier"); return; }
        g_qpia_carrier[c->device] = {host[0], host[1], host[2]};
    }
    e = cudaMemcpyAsync(cuBG_FFT, c->buf[B_BGF], sizeof(float2) * mm, cudaMemcpyDeviceToDevice, 0);
    if (e == cudaSuccess)
        e = qpi_forward_window(B<float>(c, B_HOLO), 4, 1, N, M, B<int>(c, B_CARRIER), B<float2>(c, B_T1),
                               B<float2>(c, B_S), 0);
    if (e == cudaSuccess)
        e = qpi_inverse_window(B<float2>(c, B_S), 1, M, B<int>(c, B_CARRIER), reinterpret_cast<float2 *>(cuSP_FFT),
                               nullptr, 0, nullptr, nullptr, 0);
    if (e != cudaSuccess) { cuda_fail(e, "extractQPI_AlgorithmA"); return; }
    finish("extractQPI_AlgorithmA");
}

// Carrier column of Algorithm B per device, set by frame 1 (the reference keeps it in
// the global max_idx_seq1D, cTDM/HilbertTransform.cu:1636-1640).
static std::map<int, int> g_qpib_column;

extern "C" void extractQPI_AlgorithmB(float *SP, float *BG, ctdm_cfloat *cuSP_FFT, ctdm_cfloat *cuBG_FFT, int Nx, int Ny,
                                      int frame)
{
    ctdm_ctx *c = default_ctx();
    if (!c) return;
    if (!SP || !BG || !cuSP_FFT || !cuBG_FFT) { invalid("extractQPI_AlgorithmB: NULL argument"); return; }
    if (Nx != Ny || Nx < 64 || Nx > 2048 || (Nx & (Nx - 1))) {
        invalid("extractQPI_AlgorithmB: square power-of-two holograms of 64..2048 only");
        return;
    }
    const int N = Nx, M = N / 4;
    const long nn = (long)N * N;
    if (wait_host(c) != CTDM_OK) return;   // host-buffer calls in flight still own B_HOLO / B_BG
    if (ensure(c, B_HOLO, sizeof(float) * nn) != cudaSuccess || ensure(c, B_BG, sizeof(float) * nn) != cudaSuccess ||
        ensure(c, B_T1, sizeof(float2) * M * M) != cudaSuccess || ensure(c, B_QMAG, sizeof(float) * M * N) != cudaSuccess ||
        ensure(c, B_CARRIER, sizeof(int) * 3) != cudaSuccess) {
        cuda_fail(cudaErrorMemoryAllocation, "extractQPI_AlgorithmB");
        return;
    }
    if (cudaMemcpy(c->buf[B_HOLO], SP, sizeof(float) * nn, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(c->buf[B_BG], BG, sizeof(float) * nn, cudaMemcpyHostToDevice) != cudaSuccess) {
        cuda_fail(cudaGetLastError(), "extractQPI_AlgorithmB upload");
        return;
    }
    int *car = B<int>(c, B_CARRIER);
    cudaError_t e = cudaSuccess;
    if (frame == 1) {
        // the SP frame's own column, then the background's, which later frames keep
        e = qpib_spectrum_center(B<float>(c, B_HOLO), N, B<float>(c, B_QMAG), car + 1, 0);
        if (e == cudaSuccess) e = qpib_spectrum_center(B<float>(c, B_BG), N, B<float>(c, B_QMAG), car, 0);
        int host[2] = {0, 0};
        if (e == cudaSuccess) e = cudaMemcpy(host, car, sizeof(int) * 2, cudaMemcpyDeviceToHost);
        if (e == cudaSuccess) g_qpib_column[c->device] = host[0];
    } else {
        auto it = g_qpib_column.find(c->device);
        if (it == g_qpib_column.end()) { invalid("extractQPI_AlgorithmB: frame 1 has not run on this device"); return; }
        e = set_carrier(car, it->second, it->second, -1, 0);
    }
    float2 *T = B<float2>(c, B_T1);
    if (e == cudaSuccess) e = qpib_window(B<float>(c, B_HOLO), 1, N, car + 1, T, 0);
    if (e == cudaSuccess) e = qpib_inverse(T, 1, M, reinterpret_cast<float2 *>(cuSP_FFT), nullptr, 0, nullptr, nullptr, 0);
    if (e == cudaSuccess) e = qpib_window(B<float>(c, B_BG), 1, N, car, T, 0);
    if (e == cudaSuccess) e = qpib_inverse(T, 1, M, reinterpret_cast<float2 *>(cuBG_FFT), nullptr, 0, nullptr, nullptr, 0);
    if (e != cudaSuccess) { cuda_fail(e, "extractQPI_AlgorithmB"); return; }
    finish("extractQPI_AlgorithmB");
}

extern "C" void DCT_UWLS_Unwrapped(float *ImgDst, float *ImgSrc, int sizeX, int sizeY)
{
    ctdm_ctx *c = default_ctx();
    if (!c) return;
    if (sizeX != sizeY) { invalid("DCT_UWLS_Unwrapped: square maps only"); return; }
    if (ctdm_unwrap_dct(c, 1, sizeX, CTDM_UNWRAP_REF, ImgSrc, ImgDst, 0) != CTDM_OK) return;
    finish("DCT_UWLS_Unwrapped");
}

extern "C" void FastUnwrapping(float *ImgSrc, float *ImgDst, int sizeX, int sizeY)
{
    ctdm_ctx *c = default_ctx();
    if (!c) return;
    if (sizeX != sizeY) { invalid("FastUnwrapping: square maps only"); return; }
    if (ctdm_unwrap_fast(c, 1, sizeX, ImgSrc, ImgDst, 0) != CTDM_OK) return;
    finish("FastUnwrapping");
}

extern "C" void cudaGoldsteinUnwrap2D(float *cu_phi, float *cu_UnWrapPhase, int sizeX, int sizeY, int frameNumber)
{
    (void)frameNumber;
    ctdm_ctx *c = default_ctx();
    if (!c) return;
    const long n = (long)sizeX * sizeY;
    int8_t *chg = nullptr;
    uint8_t *cut = nullptr;
    if (cudaMalloc(&chg, n) != cudaSuccess || cudaMalloc(&cut, n) != cudaSuccess) {
        cudaFree(chg);
        set_err("cudaGoldsteinUnwrap2D: allocation failed");
        return;
    }
    ctdm_goldstein(c, 1, sizeX, sizeY, cu_phi, chg, cut, cu_UnWrapPhase, nullptr, 0);
    cudaFree(chg);
    cudaFree(cut);
}

extern "C" void MedianFilter(float *PhaseData, float *AmpData, float *Phase_img, float *Amp_img, int nx, int ny,
                             int nz)
{
    ctdm_ctx *c = default_ctx();
    if (!c) return;
    if (nx != ny) { invalid("MedianFilter: square slices only"); return; }
    const long n = (long)nx * ny * nz;
    if (ensure(c, B_TMP, sizeof(float) * 2 * n) != cudaSuccess) { set_err("MedianFilter: allocation failed"); return; }
    float *tp = B<float>(c, B_TMP), *ta = tp + n;
    if (cudaMemcpy(tp, Phase_img, sizeof(float) * n, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(ta, Amp_img, sizeof(float) * n, cudaMemcpyHostToDevice) != cudaSuccess) {
        set_err("MedianFilter: upload failed");
        return;
    }
    cudaError_t e = median_stack(tp, ta, nz, nx, PhaseData, AmpData, 0);
    if (e != cudaSuccess) { cuda_fail(e, "MedianFilter"); return; }
    finish("MedianFilter");
}

extern "C" void CopyDataArray(ctdm_cfloat *u_sp, float *phase, float *amp, int sizeX, int sizeY, int sizeZ, int numZ)
{
    (void)sizeZ;
    cudaError_t e = compat_copy_data_array(reinterpret_cast<float2 *>(u_sp), phase, amp, sizeX, sizeY, numZ, 0);
    if (e != cudaSuccess) { cuda_fail(e, "CopyDataArray"); return; }
    finish("CopyDataArray");
}

extern "C" void EdwardSphere(ctdm_cfloat *u_sp, ctdm_cfloat *F, float *C, float fm0, float df, float AngX, float AngY,
                             int sizeX, int sizeY, int sizeZ)
{
    std::vector<AngleGeom> g;
    angle_geometry(&AngX, &AngY, 1, (double)fm0, (double)df, g);
    const double fm02 = (double)fm0 * (double)fm0;
    const float fm02s = (float)(((double)fm0 / df) * ((double)fm0 / df));
    cudaError_t e = compat_edward_sphere(reinterpret_cast<const float2 *>(u_sp), reinterpret_cast<float2 *>(F), C, g[0],
                                         (double)df, fm02, fm02s, sizeX, sizeY, sizeZ, 0);
    if (e != cudaSuccess) { cuda_fail(e, "EdwardSphere"); return; }
    finish("EdwardSphere");
}

extern "C" void initial_F_and_F2(float *C, ctdm_cfloat *cuF, ctdm_cfloat *cuF2, float recon_dx, int W, int H, int S)
{
    cudaError_t e = compat_initial_f(C, reinterpret_cast<float2 *>(cuF), reinterpret_cast<float2 *>(cuF2), recon_dx,
                                     (long)W * H * S, 0);
    if (e != cudaSuccess) { cuda_fail(e, "initial_F_and_F2"); return; }
    finish("initial_F_and_F2");
}

extern "C" void est_n_3D(ctdm_cfloat *n, ctdm_cfloat *F, float recon_k2, float recon_med, int W, int H, int S)
{
    cudaError_t e = compat_est_n(reinterpret_cast<float2 *>(n), reinterpret_cast<const float2 *>(F), recon_k2,
                                 recon_med, (long)W * H * S, 0);
    if (e != cudaSuccess) { cuda_fail(e, "est_n_3D"); return; }
    finish("est_n_3D");
}

extern "C" void modify_F_3D(ctdm_cfloat *n, ctdm_cfloat *F, float recon_k2, float recon_med, int W, int H, int S)
{
    cudaError_t e = compat_modify(reinterpret_cast<const float2 *>(n), reinterpret_cast<float2 *>(F), recon_k2,
                                  recon_med, (long)W * H * S, 0);
    if (e != cudaSuccess) { cuda_fail(e, "modify_F_3D"); return; }
    finish("modify_F_3D");
}

extern "C" void check_F_3D(ctdm_cfloat *F, ctdm_cfloat *F2, int W, int H, int S)
{
    cudaError_t e = compat_check(reinterpret_cast<float2 *>(F), reinterpret_cast<const float2 *>(F2), (long)W * H * S, 0);
    if (e != cudaSuccess) { cuda_fail(e, "check_F_3D"); return; }
    finish("check_F_3D");
}

extern "C" void cuFFT3D(ctdm_cfloat *ImgArray, int sizeX, int sizeY, int sizeZ, int dir)
{
    const int dims[3] = {sizeX, sizeY, sizeZ};
    if (ctdm_fft(ImgArray, 3, dims, 1, dir > 0, 0) != CTDM_OK) return;
    if (dir > 0) {
        const long n = (long)sizeX * sizeY * sizeZ;
        cudaError_t e = scale_complex(reinterpret_cast<float2 *>(ImgArray), n, 1.0f / (float)n, false, 0);
        if (e != cudaSuccess) { cuda_fail(e, "cuFFT3D"); return; }
    }
    finish("cuFFT3D");
}

extern "C" void cuFFT2D(ctdm_cfloat *ImgArray, int sizeX, int sizeY, int dir)
{
    const int dims[2] = {sizeX, sizeY};
    if (ctdm_fft(ImgArray, 2, dims, 1, dir > 0, 0) != CTDM_OK) return;
    if (dir > 0) {
        const long n = (long)sizeX * sizeY;
        cudaError_t e = scale_complex(reinterpret_cast<float2 *>(ImgArray), n, 1.0f / (float)n, true, 0);
        if (e != cudaSuccess) { cuda_fail(e, "cuFFT2D"); return; }
    }
    finish("cuFFT2D");
}

namespace ctdm {
// BatchRecon with the globals above (cTDM/HilbertTransform.cu:1825-2047): host R x R
// stacks and angles in, 3D-RI-*.rimap written into SaveDir.
ctdm_status batch_recon(const float *PhaseStack, const float *AmpStack, const float *sampleAngleRadX,
                        const float *sampleAngleRadY, int ReconFrame)
{
    ctdm_ctx *c = default_ctx();
    if (!c) return invalid("BatchRecon: no CUDA device");
    const int R = g_recon;
    if (!ok_volume(R) || ReconFrame < 1 || ReconFrame > kMaxAngles) return invalid("BatchRecon: size unsupported");
    const long rr = (long)R * R, r3 = rr * R;
    // constants of BatchRecon (cTDM/HilbertTransform.cu:1839-1862)
    const double lambda = g_wavelength_nm * 1e-9;
    const double fm0 = g_nmed / lambda;
    const double dx = (g_pixel_um * 1e-6) / g_mag * 1024.0 / R;
    const double k = 2.0 * CTDM_PI_D * g_nmed / lambda;
    const double df = 1.0 / (R * dx);
    float *ph = nullptr, *am = nullptr;
    float2 *U = nullptr, *F2 = nullptr, *ri = nullptr;
    auto cleanup = [&]() { cudaFree(ph); cudaFree(am); cudaFree(U); cudaFree(F2); cudaFree(ri); };
    if (cudaMalloc(&ph, sizeof(float) * ReconFrame * rr) != cudaSuccess ||
        cudaMalloc(&am, sizeof(float) * ReconFrame * rr) != cudaSuccess ||
        cudaMalloc(&U, sizeof(float2) * ReconFrame * rr) != cudaSuccess ||
        cudaMalloc(&F2, sizeof(float2) * r3) != cudaSuccess || cudaMalloc(&ri, sizeof(float2) * r3) != cudaSuccess) {
        cleanup();
        cudaGetLastError();
        set_err("BatchRecon: device allocation failed");
        return CTDM_ERR_NOMEM;
    }
    cudaError_t e = cudaMemcpy(ph, PhaseStack, sizeof(float) * ReconFrame * rr, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(am, AmpStack, sizeof(float) * ReconFrame * rr, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cleanup();
        return cuda_fail(e, "BatchRecon upload");
    }
    ctdm_status st = ctdm_stack_spectra(c, ReconFrame, R, ph, am, reinterpret_cast<ctdm_cfloat *>(U), 0);
    if (st == CTDM_OK)
        st = ctdm_map_ewald(c, ReconFrame, R, reinterpret_cast<ctdm_cfloat *>(U), sampleAngleRadX, sampleAngleRadY, fm0,
                            df, dx, reinterpret_cast<ctdm_cfloat *>(F2), nullptr, 0);
    if (st == CTDM_OK)
        st = ctdm_positivity(c, R, g_iter_time + 1, CTDM_CHECK_REF, k * k, g_nmed, reinterpret_cast<ctdm_cfloat *>(F2),
                             nullptr, reinterpret_cast<ctdm_cfloat *>(ri), 0);
    if (st != CTDM_OK) {
        cleanup();
        return st;
    }
    std::vector<ctdm_cfloat> host(r3);
    e = cudaMemcpy(host.data(), ri, sizeof(float2) * r3, cudaMemcpyDeviceToHost);
    cleanup();
    if (e != cudaSuccess) return cuda_fail(e, "BatchRecon download");
    return ctdm_write_rimap(g_save_dir.c_str(), R, g_recon_save, host.data());
}
}  // namespace ctdm

extern "C" void BatchRecon(float *PhaseStack, float *AmpStack, float *sampleAngleRadX, float *sampleAngleRadY,
                           int ReconFrame)
{
    batch_recon(PhaseStack, AmpStack, sampleAngleRadX, sampleAngleRadY, ReconFrame);
}

// BatchReconPOCS (cTDM/HilbertTransform.cu:2049-2402): the same spectra, the
// frequency-interpolation mapping over the AngX scan and ASD-POCS with the reference's
// constants; writes 3D-RI-{Complex,Real,Imag}_RxRxR.raw into SaveDir like the reference.
extern "C" void BatchReconPOCS(float *PhaseStack, float *AmpStack, float *sampleAngleRadX, float *sampleAngleRadY,
                               int ReconFrame)
{
    (void)sampleAngleRadY;
    ctdm_ctx *c = default_ctx();
    if (!c) { invalid("BatchReconPOCS: no CUDA device"); return; }
    const int R = g_recon;
    if (!ok_volume(R) || ReconFrame < 1 || ReconFrame > kMaxAngles) { invalid("BatchReconPOCS: size unsupported"); return; }
    const long rr = (long)R * R, r3 = rr * R;
    const double lambda = g_wavelength_nm * 1e-9;
    const double fm0 = g_nmed / lambda;
    const double dx = (g_pixel_um * 1e-6) / g_mag * 1024.0 / R;
    const double k = 2.0 * CTDM_PI_D * g_nmed / lambda;
    const double df = 1.0 / (R * dx);
    float *ph = nullptr, *am = nullptr;
    float2 *U = nullptr, *F2 = nullptr, *ri = nullptr;
    auto cleanup = [&]() { cudaFree(ph); cudaFree(am); cudaFree(U); cudaFree(F2); cudaFree(ri); };
    if (cudaMalloc(&ph, sizeof(float) * ReconFrame * rr) != cudaSuccess ||
        cudaMalloc(&am, sizeof(float) * ReconFrame * rr) != cudaSuccess ||
        cudaMalloc(&U, sizeof(float2) * ReconFrame * rr) != cudaSuccess ||
        cudaMalloc(&F2, sizeof(float2) * r3) != cudaSuccess || cudaMalloc(&ri, sizeof(float2) * r3) != cudaSuccess) {
        cleanup();
        cudaGetLastError();
        set_err("BatchReconPOCS: device allocation failed");
        return;
    }
    cudaError_t e = cudaMemcpy(ph, PhaseStack, sizeof(float) * ReconFrame * rr, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(am, AmpStack, sizeof(float) * ReconFrame * rr, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) { cleanup(); cuda_fail(e, "BatchReconPOCS upload"); return; }
    ctdm_pocs_params pp;
    ctdm_pocs_defaults(&pp);
    ctdm_status st = ctdm_stack_spectra(c, ReconFrame, R, ph, am, reinterpret_cast<ctdm_cfloat *>(U), 0);
    if (st == CTDM_OK)
        st = ctdm_map_fi(c, ReconFrame, R, reinterpret_cast<ctdm_cfloat *>(U), sampleAngleRadX, fm0, df, dx,
                         reinterpret_cast<ctdm_cfloat *>(F2), nullptr, 0);
    if (st == CTDM_OK)
        st = ctdm_pocs(c, R, &pp, k * k, g_nmed, reinterpret_cast<ctdm_cfloat *>(F2), reinterpret_cast<ctdm_cfloat *>(ri),
                       nullptr, 0);
    if (st != CTDM_OK) { cleanup(); return; }
    std::vector<ctdm_cfloat> host(r3);
    e = cudaMemcpy(host.data(), ri, sizeof(float2) * r3, cudaMemcpyDeviceToHost);
    cleanup();
    if (e != cudaSuccess) { cuda_fail(e, "BatchReconPOCS download"); return; }
    if (write_ri_volume(g_save_dir, R, g_recon_save, host.data(), "raw") == CTDM_OK) g_err.clear();
}
