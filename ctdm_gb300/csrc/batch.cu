// Batched reconstruction: many independent tomograms (uneven angle counts,
// hologram and volume sizes) scheduled over a few concurrent lanes and captured
// into one CUDA graph, so a whole batch is a single cudaGraphLaunch.
//
// No reference counterpart: the reference reconstructs one tomogram per
// BatchRecon call (cTDM/HilbertTransform.cu:1825-2047) on the legacy stream.
//
// Scheduling.  Each lane owns a workspace (a ctdm_ctx with its own Goldstein side
// stream) and a stream.  Jobs go to lanes longest-first onto the least-loaded lane
// (LPT), by the algorithmic HBM bytes of the whole path.  The memory-bound volume
// passes of one lane overlap the latency-bound per-angle stages (QPI, unwrapping,
// Goldstein, Ewald mapping) of the others, and the graph removes the per-kernel
// launch gaps of the ~5 R^3-sized passes per iteration.
//
// Admission by free HBM.  Before planning, each job's workspace is bounded
// (workspace_bytes), and the batch uses only as many lanes as fit beside each other in
// the device memory that is free plus what the lanes already hold (capped by
// ctdm_batch_set_memory_limit), keeping back room for the autotuner's scratch volumes.
// A batch whose largest job does not fit alone is refused before anything is
// allocated.  The reference makes the same decision for its one volume from free device
// memory (ReconMode, cTDM/HilbertTransform.cu:1932-1939).
//
// Planning runs every job once eagerly (growing each lane's workspace to its
// largest job and validating everything), then captures the same launch sequence.
// The graph keeps the job pointers it was planned with: to reconstruct new data,
// write it into the same input buffers and launch again.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <vector>

#include "api_internal.h"

using namespace ctdm;

struct ctdm_batch {
    int device = 0;
    int lanes = 1;
    std::vector<ctdm_ctx *> ctx;
    std::vector<cudaStream_t> streams;
    std::vector<cudaEvent_t> joins;
    cudaEvent_t fork = nullptr;
    cudaStream_t origin = nullptr;   // capture origin
    std::vector<ctdm_job> jobs;
    std::vector<AngleGeom *> geom;   // per job, device
    std::vector<std::vector<int>> order;
    std::vector<int> lane_of;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    unsigned long long graph_kernels = 0;   // kernel launches captured into the graph
    size_t mem_limit = 0;                   // 0: free device memory decides alone
    int active = 0;                         // lanes admitted by the last plan
    size_t lane_bytes = 0, avail_bytes = 0; // largest job's workspace; memory the plan could use
};

#define BK(x, what)                                          \
    do {                                                     \
        cudaError_t e_ = (x);                                \
        if (e_ != cudaSuccess) return fail_cuda(e_, what);   \
    } while (0)

// Algorithmic HBM bytes of one tomogram (the per-stage model of the path).
static double job_bytes(const ctdm_job &j)
{
    const ctdm_params &p = j.params;
    const double A = j.n_angles, N = p.n_holo, M = p.m_crop ? p.m_crop : p.n_holo / 4, R = p.r_vol;
    const double r3 = R * R * R;
    double b = (A + 1) * (4 * N * N + 8 * M * M) + A * 8 * M * M + A * (8 * M * M + 8 * R * R) + A * 24 * R * R;
    if (p.run_goldstein || p.unwrap_method == CTDM_METHOD_GOLDSTEIN) b += A * 6 * M * M;
    b += 60 * r3 + p.iterations * 72 * r3 + 16 * r3;
    return b;
}

static void free_plan(ctdm_batch *b)
{
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
    for (AngleGeom *g : b->geom)
        if (g) cudaFree(g);
    b->geom.clear();
    b->jobs.clear();
    b->order.assign(b->lanes, {});
    b->lane_of.clear();
}

extern "C" ctdm_status ctdm_batch_create(int device, int lanes, ctdm_batch **out)
{
    if (!out) return fail_invalid("ctdm_batch_create: out is NULL");
    if (lanes < 1 || lanes > 16) return fail_invalid("ctdm_batch_create: lanes outside 1..16");
    BK(cudaSetDevice(device), "cudaSetDevice");
    ctdm_batch *b = new ctdm_batch();
    b->device = device;
    b->lanes = lanes;
    b->order.assign(lanes, {});
    cudaError_t e = cudaStreamCreateWithFlags(&b->origin, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
    for (int l = 0; l < lanes && e == cudaSuccess; l++) {
        cudaStream_t s = nullptr;
        cudaEvent_t j = nullptr;
        e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&j, cudaEventDisableTiming);
        b->streams.push_back(s);
        b->joins.push_back(j);
    }
    if (e != cudaSuccess) {
        ctdm_batch_destroy(b);
        return fail_cuda(e, "creating batch lanes");
    }
    for (int l = 0; l < lanes; l++) {
        ctdm_ctx *c = nullptr;
        ctdm_status st = ctdm_ctx_create(device, &c);
        if (st != CTDM_OK) {
            ctdm_batch_destroy(b);
            return st;
        }
        b->ctx.push_back(c);
    }
    *out = b;
    clear_error();
    return CTDM_OK;
}

extern "C" void ctdm_batch_destroy(ctdm_batch *b)
{
    if (!b) return;
    cudaSetDevice(b->device);
    free_plan(b);
    for (ctdm_ctx *c : b->ctx) ctdm_ctx_destroy(c);
    for (cudaStream_t s : b->streams)
        if (s) cudaStreamDestroy(s);
    for (cudaEvent_t e : b->joins)
        if (e) cudaEventDestroy(e);
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->origin) cudaStreamDestroy(b->origin);
    delete b;
}

// Every lane's jobs in order on the lane streams, forked from and joined back into s.
static ctdm_status issue(ctdm_batch *b, cudaStream_t s)
{
    BK(cudaEventRecord(b->fork, s), "batch fork");
    for (int l = 0; l < b->lanes; l++) {
        cudaStream_t ls = b->streams[l];
        BK(cudaStreamWaitEvent(ls, b->fork, 0), "batch fork wait");
        for (int j : b->order[l]) {
            const ctdm_job &jb = b->jobs[j];
            ctdm_status st = run_pipeline(b->ctx[l], &jb.params, jb.n_angles, jb.d_holo, jb.d_bg, b->geom[j],
                                          jb.d_ri, ls);
            if (st != CTDM_OK) return st;
        }
        BK(cudaEventRecord(b->joins[l], ls), "batch join");
        BK(cudaStreamWaitEvent(s, b->joins[l], 0), "batch join wait");
    }
    return CTDM_OK;
}

extern "C" ctdm_status ctdm_batch_plan(ctdm_batch *b, const ctdm_job *jobs, int n_jobs)
{
    if (!b || !jobs || n_jobs < 1) return fail_invalid("ctdm_batch_plan: bad argument");
    BK(cudaSetDevice(b->device), "cudaSetDevice");
    BK(cudaDeviceSynchronize(), "batch plan");
    free_plan(b);
    for (int j = 0; j < n_jobs; j++) {
        const ctdm_job &jb = jobs[j];
        int M;
        ctdm_status st = validate_params(&jb.params, jb.n_angles, M);
        if (st != CTDM_OK) return st;
        if (!jb.d_holo || !jb.d_bg || !jb.h_angx || !jb.h_angy || !jb.d_ri)
            return fail_invalid("ctdm_batch_plan: a job has a NULL pointer");
    }
    // admission: lanes whose workspaces fit beside each other in the available memory
    size_t w_max = 0, r_max = 0;
    for (int j = 0; j < n_jobs; j++) {
        int M;
        validate_params(&jobs[j].params, jobs[j].n_angles, M);
        w_max = std::max(w_max, workspace_bytes(&jobs[j].params, jobs[j].n_angles, M));
        r_max = std::max(r_max, (size_t)jobs[j].params.r_vol);
    }
    size_t held = 0;
    for (ctdm_ctx *c : b->ctx) held += held_bytes(c);
    size_t free_b = 0, total_b = 0;
    BK(cudaMemGetInfo(&free_b, &total_b), "free device memory");
    size_t avail = free_b + held;
    if (b->mem_limit && b->mem_limit < avail) avail = b->mem_limit;
    const size_t margin = 24 * r_max * r_max * r_max + (256ull << 20);   // tuner scratch volumes, plan state
    const size_t fit = avail > margin ? (avail - margin) / w_max : 0;
    b->lane_bytes = w_max;
    b->avail_bytes = avail;
    b->active = (int)std::min<size_t>((size_t)b->lanes, fit);
    if (b->active < 1) {
        char msg[256];
        snprintf(msg, sizeof msg,
                 "ctdm_batch_plan: the largest job needs %.2f GB of workspace (+ %.2f GB reserve), %.2f GB available",
                 w_max / 1e9, margin / 1e9, avail / 1e9);
        ctdm_status st = fail_invalid(msg);
        (void)st;
        return CTDM_ERR_NOMEM;
    }
    for (int l = b->active; l < b->lanes; l++) release_workspace(b->ctx[l]);
    b->jobs.assign(jobs, jobs + n_jobs);
    // geometry per job (device, owned by the plan)
    for (int j = 0; j < n_jobs; j++) {
        const ctdm_job &jb = b->jobs[j];
        std::vector<AngleGeom> g;
        make_geometry(jb.h_angx, jb.h_angy, jb.n_angles, jb.params.n_med / jb.params.wavelength,
                      1.0 / (jb.params.r_vol * jb.params.dx), g);
        AngleGeom *d = nullptr;
        BK(cudaMalloc(&d, sizeof(AngleGeom) * g.size()), "alloc job geometry");
        b->geom.push_back(d);
        BK(cudaMemcpy(d, g.data(), sizeof(AngleGeom) * g.size(), cudaMemcpyHostToDevice), "upload job geometry");
    }
    // longest job first onto the least-loaded lane
    std::vector<int> idx(n_jobs);
    for (int j = 0; j < n_jobs; j++) idx[j] = j;
    std::stable_sort(idx.begin(), idx.end(),
                     [&](int x, int y) { return job_bytes(b->jobs[x]) > job_bytes(b->jobs[y]); });
    std::vector<double> load(b->active, 0.0);
    b->lane_of.assign(n_jobs, 0);
    for (int j : idx) {
        const int l = (int)(std::min_element(load.begin(), load.end()) - load.begin());
        load[l] += job_bytes(b->jobs[j]);
        b->order[l].push_back(j);
        b->lane_of[j] = l;
    }
    // eager run: grows each lane's workspace and validates the launches
    ctdm_status st = issue(b, b->origin);
    if (st != CTDM_OK) return st;
    BK(cudaStreamSynchronize(b->origin), "batch warm-up");
    // capture the same sequence
    BK(cudaStreamBeginCapture(b->origin, cudaStreamCaptureModeRelaxed), "begin capture");
    const unsigned long long k0 = ctdm_launch_count();
    st = issue(b, b->origin);
    b->graph_kernels = ctdm_launch_count() - k0;
    cudaGraph_t g = nullptr;
    cudaError_t ce = cudaStreamEndCapture(b->origin, &g);
    if (st != CTDM_OK) {
        if (g) cudaGraphDestroy(g);
        return st;
    }
    BK(ce, "end capture");
    b->graph = g;
    BK(cudaGraphInstantiate(&b->exec, g, 0), "instantiate batch graph");
    BK(cudaGraphUpload(b->exec, b->origin), "upload batch graph");
    BK(cudaStreamSynchronize(b->origin), "batch plan");
    clear_error();
    return CTDM_OK;
}

extern "C" ctdm_status ctdm_batch_run(ctdm_batch *b, void *stream)
{
    if (!b || !b->exec) return fail_invalid("ctdm_batch_run: no plan");
    BK(cudaSetDevice(b->device), "cudaSetDevice");
    BK(cudaGraphLaunch(b->exec, (cudaStream_t)stream), "batch graph launch");
    note_launches(b->graph_kernels);
    clear_error();
    return CTDM_OK;
}

extern "C" ctdm_status ctdm_batch_run_eager(ctdm_batch *b, void *stream)
{
    if (!b || b->jobs.empty()) return fail_invalid("ctdm_batch_run_eager: no plan");
    BK(cudaSetDevice(b->device), "cudaSetDevice");
    ctdm_status st = issue(b, (cudaStream_t)stream);
    if (st == CTDM_OK) clear_error();
    return st;
}

extern "C" ctdm_status ctdm_batch_set_memory_limit(ctdm_batch *b, size_t bytes)
{
    if (!b) return fail_invalid("ctdm_batch_set_memory_limit: NULL batch");
    b->mem_limit = bytes;
    clear_error();
    return CTDM_OK;
}

extern "C" ctdm_status ctdm_batch_admission(const ctdm_batch *b, int *lanes_used, size_t *bytes_per_lane,
                                            size_t *bytes_available)
{
    if (!b || b->active < 1) return fail_invalid("ctdm_batch_admission: no plan");
    if (lanes_used) *lanes_used = b->active;
    if (bytes_per_lane) *bytes_per_lane = b->lane_bytes;
    if (bytes_available) *bytes_available = b->avail_bytes;
    clear_error();
    return CTDM_OK;
}

extern "C" ctdm_status ctdm_batch_lanes(const ctdm_batch *b, int *lane_of_job, int n_jobs)
{
    if (!b || !lane_of_job || n_jobs != (int)b->lane_of.size()) return fail_invalid("ctdm_batch_lanes: bad argument");
    for (int j = 0; j < n_jobs; j++) lane_of_job[j] = b->lane_of[j];
    clear_error();
    return CTDM_OK;
}
