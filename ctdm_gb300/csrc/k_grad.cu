// Differentiable form of the Fourier-domain ODT: the measurement operator
// A = P F~ (unitary 3-D FFT F~ = F / R^{3/2} followed by sampling P at the measured
// voxels of the Ewald caps), its hand-written adjoint A^H = F~^H P^T (scatter then
// inverse transform), a smoothed isotropic total variation and an accelerated
// gradient (FISTA) driver for
//     min_V  1/2 || P F~ V - y ||^2 + lambda TV(V),
// with V the dimensionless scattering contrast f / (-k^2) (n = n_med sqrt(1 + V)).
// No reference counterpart: the reference only has the positivity loop.
//
// The tape (ctdm_tape) holds the sorted measured-voxel indices and their data; the
// forward keeps no 3-D intermediates -- the backward recomputes its transform.
// Complex gradients follow the conjugate-Wirtinger convention of torch autograd:
// dL/dV = dL/dRe V + i dL/dIm V.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "ctdm.h"
#include "kernels.cuh"

namespace ctdm {
void set_error_message(const char *msg);
}

using namespace ctdm;

struct ctdm_tape {
    int device = 0, R = 0;
    long S = 0;
    uint32_t *idx = nullptr;   // S voxel indices, ascending
    float2 *y = nullptr;       // S data values (scaled by 1 / (-k^2 R^{3/2}))
    float2 *work = nullptr;    // R^3 transform buffer
    float2 *resid = nullptr, *wmom = nullptr, *grad = nullptr;   // driver state (allocated on demand)
    double *red = nullptr;     // reduction scratch
    int *flags = nullptr;
};

namespace {

thread_local char g_msg[256];

ctdm_status fail(ctdm_status st, const char *fmt, const char *detail = "")
{
    snprintf(g_msg, sizeof g_msg, fmt, detail);
    set_error_message(g_msg);
    return st;
}

ctdm_status cuda_fail(cudaError_t e, const char *what)
{
    snprintf(g_msg, sizeof g_msg, "%s: %s", what, cudaGetErrorString(e));
    set_error_message(g_msg);
    return e == cudaErrorMemoryAllocation ? CTDM_ERR_NOMEM : CTDM_ERR_CUDA;
}

#define GCK(x, what)                                        \
    do {                                                    \
        cudaError_t e_ = (x);                               \
        if (e_ != cudaSuccess) return cuda_fail(e_, what);  \
    } while (0)

unsigned grid_for(long n)
{
    long b = (n + 255) / 256;
    return (unsigned)(b > 16384 ? 16384 : (b < 1 ? 1 : b));
}

// ------------------------------------------------------------ tape construction
// Measured voxels: the reference's data-replacement predicate (F2.re != 0 and
// F2.im != 0) or, with counts, the hit mask.  Flags then an ordered compaction.
__global__ void measured_flags(const float2 *__restrict__ F2, const uint32_t *__restrict__ counts, long n, int *flags)
{
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const float2 v = F2[i];
        flags[i] = counts ? (counts[i] != 0u) : (v.x != 0.0f && v.y != 0.0f);
    }
}

constexpr int kScanBlock = 1024;

// per-block counts of flagged voxels (block b covers [b*chunk, (b+1)*chunk))
__global__ void block_counts(const int *__restrict__ flags, long n, long chunk, int *bc)
{
    __shared__ int s[32];
    const long b0 = blockIdx.x * chunk, b1 = min(n, b0 + chunk);
    int c = 0;
    for (long i = b0 + threadIdx.x; i < b1; i += blockDim.x) c += flags[i];
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += s[w];
        bc[blockIdx.x] = t;
    }
}

// ordered write: each block scans its range in order (warp-cooperative prefix)
__global__ void block_write(const int *__restrict__ flags, const int *__restrict__ boff, long n, long chunk,
                            const float2 *__restrict__ F2, float scale, uint32_t *idx, float2 *y)
{
    __shared__ int warp_tot[32];
    __shared__ int base;
    const long b0 = blockIdx.x * chunk, b1 = min(n, b0 + chunk);
    if (threadIdx.x == 0) base = boff[blockIdx.x];
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (long s0 = b0; s0 < b1; s0 += blockDim.x) {
        const long i = s0 + threadIdx.x;
        const int f = (i < b1) ? flags[i] : 0;
        const unsigned bal = __ballot_sync(0xffffffffu, f);
        const int before = __popc(bal & ((1u << lane) - 1u));
        if (lane == 0) warp_tot[wid] = __popc(bal);
        __syncthreads();
        int woff = 0, tot = 0;
        for (int w = 0; w < nw; w++) {
            if (w < wid) woff += warp_tot[w];
            tot += warp_tot[w];
        }
        if (f) {
            const int pos = base + woff + before;
            idx[pos] = (uint32_t)i;
            const float2 v = F2[i];
            y[pos] = make_float2(v.x * scale, v.y * scale);
        }
        __syncthreads();
        if (threadIdx.x == 0) base += tot;
        __syncthreads();
    }
}

// ------------------------------------------------------------ operators
__global__ void gather_kernel(const float2 *__restrict__ vol, const uint32_t *__restrict__ idx, long S, float scale,
                              float2 *y)
{
    for (long s = blockIdx.x * (long)blockDim.x + threadIdx.x; s < S; s += (long)gridDim.x * blockDim.x) {
        const float2 v = vol[idx[s]];
        y[s] = make_float2(v.x * scale, v.y * scale);
    }
}

__global__ void scatter_kernel(const float2 *__restrict__ y, const uint32_t *__restrict__ idx, long S, float scale,
                               float2 *vol)
{
    for (long s = blockIdx.x * (long)blockDim.x + threadIdx.x; s < S; s += (long)gridDim.x * blockDim.x) {
        const float2 v = y[s];
        vol[idx[s]] = make_float2(v.x * scale, v.y * scale);
    }
}

// residual in place of the prediction, and its squared norm (block partials)
__global__ void residual_kernel(float2 *yp, const float2 *__restrict__ y, long S, double *partial)
{
    double acc = 0.0;
    for (long s = blockIdx.x * (long)blockDim.x + threadIdx.x; s < S; s += (long)gridDim.x * blockDim.x) {
        const float2 a = yp[s], b = y[s];
        const float2 r = make_float2(a.x - b.x, a.y - b.y);
        yp[s] = r;
        acc += (double)r.x * r.x + (double)r.y * r.y;
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    __shared__ double sh[32];
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += sh[w];
        partial[blockIdx.x] = t;
    }
}

__device__ __forceinline__ float2 ld(const float2 *V, int x, int y, int z, int R)
{
    return V[x + (long)R * y + (long)R * R * z];
}

// Smoothed isotropic TV with forward differences (zero past the last index):
// TV = sum sqrt(|Dx V|^2 + |Dy V|^2 + |Dz V|^2 + eps^2).  Its gradient is
// -div(grad V / |grad V|_eps) with the adjoint (backward) differences; the kernel
// adds lambda times it to g and accumulates TV itself.
__device__ __forceinline__ float2 tv_flux(const float2 *V, int x, int y, int z, int R, float eps2, int comp,
                                          float &mag)
{
    const float2 c = ld(V, x, y, z, R);
    const float2 dx = x + 1 < R ? csub(ld(V, x + 1, y, z, R), c) : make_float2(0.f, 0.f);
    const float2 dy = y + 1 < R ? csub(ld(V, x, y + 1, z, R), c) : make_float2(0.f, 0.f);
    const float2 dz = z + 1 < R ? csub(ld(V, x, y, z + 1, R), c) : make_float2(0.f, 0.f);
    mag = sqrtf(dx.x * dx.x + dx.y * dx.y + dy.x * dy.x + dy.y * dy.y + dz.x * dz.x + dz.y * dz.y + eps2);
    const float2 d = comp == 0 ? dx : (comp == 1 ? dy : dz);
    return make_float2(d.x / mag, d.y / mag);
}

__global__ void tv_grad_kernel(const float2 *__restrict__ V, int R, float lambda, float eps, float2 *g, double *partial)
{
    const long n = (long)R * R * R;
    const float eps2 = eps * eps;
    double acc = 0.0;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const int x = (int)(i % R), y = (int)((i / R) % R), z = (int)(i / ((long)R * R));
        float mag;
        // flux out of this voxel (the three forward differences share one magnitude)
        const float2 c = ld(V, x, y, z, R);
        const float2 dx = x + 1 < R ? csub(ld(V, x + 1, y, z, R), c) : make_float2(0.f, 0.f);
        const float2 dy = y + 1 < R ? csub(ld(V, x, y + 1, z, R), c) : make_float2(0.f, 0.f);
        const float2 dz = z + 1 < R ? csub(ld(V, x, y, z + 1, R), c) : make_float2(0.f, 0.f);
        mag = sqrtf(dx.x * dx.x + dx.y * dx.y + dy.x * dy.x + dy.y * dy.y + dz.x * dz.x + dz.y * dz.y + eps2);
        acc += (double)mag;
        float2 div = make_float2(-(dx.x + dy.x + dz.x) / mag, -(dx.y + dy.y + dz.y) / mag);
        // flux into it from the lower neighbours
        float m2;
        if (x > 0) { const float2 q = tv_flux(V, x - 1, y, z, R, eps2, 0, m2); div.x += q.x; div.y += q.y; }
        if (y > 0) { const float2 q = tv_flux(V, x, y - 1, z, R, eps2, 1, m2); div.x += q.x; div.y += q.y; }
        if (z > 0) { const float2 q = tv_flux(V, x, y, z - 1, R, eps2, 2, m2); div.x += q.x; div.y += q.y; }
        float2 gv = g[i];
        g[i] = make_float2(gv.x + lambda * div.x, gv.y + lambda * div.y);
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    __shared__ double sh[32];
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += sh[w];
        partial[blockIdx.x] = t;
    }
}

// FISTA: V+ = W - tau g;  W = V+ + beta (V+ - V)
// Projection of a contrast V onto the positivity set of the reference's est_n clamp
// (cTDM/Recon_kernel.cu:305-342: Re n >= n_med, Im n >= 0 for n = n_med sqrt(1 + V)):
// s = sqrt(1 + V) (principal root), s' = (max(Re s, 1), max(Im s, 0)), V' = s'^2 - 1.
__device__ __forceinline__ float2 project_contrast(float2 v)
{
    const float c = 1.0f + v.x, d = v.y;
    const float mod = hypotf(c, d);
    float a, b;
    if (d == 0.0f) {
        a = sqrtf(fmaxf(c, 0.0f));
        b = 0.0f;
    } else if (c >= 0.0f) {
        a = sqrtf((mod + c) * 0.5f);
        b = d / (2.0f * a);
    } else {
        b = sqrtf((mod - c) * 0.5f);
        a = fabsf(d) / (2.0f * b);
        if (d < 0.0f) b = -b;
    }
    a = fmaxf(a, 1.0f);
    b = fmaxf(b, 0.0f);
    return make_float2(a * a - b * b - 1.0f, 2.0f * a * b);
}

template <bool PROJECT>
__global__ void fista_kernel(float2 *V, float2 *W, const float2 *__restrict__ g, long n, float tau, float beta)
{
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const float2 w = W[i], gg = g[i], v = V[i];
        float2 vn = make_float2(w.x - tau * gg.x, w.y - tau * gg.y);
        if (PROJECT) vn = project_contrast(vn);
        V[i] = vn;
        W[i] = make_float2(vn.x + beta * (vn.x - v.x), vn.y + beta * (vn.y - v.y));
    }
}

// n = n_med sqrt(1 + V) (principal root), optional positivity clamp, octant shift.
__global__ void contrast_to_ri(const float2 *__restrict__ V, int R, float nm, int clamp, float2 *out)
{
    const long n = (long)R * R * R;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const int x = (int)(i % R), y = (int)((i / R) % R), z = (int)(i / ((long)R * R));
        const float2 v = V[i];
        const float c = 1.0f + v.x, d = 0.0f + v.y;   // complex 1 + V: a -0 imaginary part becomes +0
        const float mod = hypotf(c, d);
        float a, b;
        if (c >= 0.f) {
            a = sqrtf((mod + c) * 0.5f);
            b = a > 0.f ? d / (2.f * a) : 0.f;
        } else {   // mod - c > 0: no cancellation, b != 0
            b = copysignf(sqrtf((mod - c) * 0.5f), d);
            a = fabsf(d) / (2.f * fabsf(b));
        }
        float nr = a * nm, ni = b * nm;
        if (clamp) { nr = fmaxf(nr, nm); ni = fmaxf(ni, 0.f); }
        const long o = (long)((x + R / 2) % R) + (long)R * ((y + R / 2) % R) + (long)R * R * ((z + R / 2) % R);
        out[o] = make_float2(nr, ni);
    }
}

double sum_partials(const double *d, int n)
{
    std::vector<double> h(n);
    if (cudaMemcpy(h.data(), d, sizeof(double) * n, cudaMemcpyDeviceToHost) != cudaSuccess) return NAN;
    double s = 0;
    for (double v : h) s += v;
    return s;
}

constexpr int kRedBlocks = 1024;

// Unitary 3-D transform of the tape's working volume.
cudaError_t unitary_fft3(float2 *d, int R, bool inverse, cudaStream_t s)
{
    const long r2 = (long)R * R;
    cudaError_t e = fft_rows(d, R, r2, inverse, s);
    if (e == cudaSuccess) e = fft_cols(d, R, r2, R, r2, R, inverse, s);
    if (e == cudaSuccess) e = fft_cols(d, R, r2, R, R, r2, inverse, s);
    if (e == cudaSuccess) e = scale_complex(d, r2 * R, (float)(1.0 / std::pow((double)R, 1.5)), false, s);
    return e;
}

// forward: y_pred = P F~ V  (recomputes the transform in tape->work)
cudaError_t op_forward(ctdm_tape *t, const float2 *V, float2 *y, cudaStream_t s)
{
    const long n = (long)t->R * t->R * t->R;
    cudaError_t e = cudaMemcpyAsync(t->work, V, sizeof(float2) * n, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess) e = unitary_fft3(t->work, t->R, false, s);
    if (e != cudaSuccess) return e;
    gather_kernel<<<grid_for(t->S), 256, 0, s>>>(t->work, t->idx, t->S, 1.0f, y); note_launch();
    return cudaGetLastError();
}

// adjoint: g = F~^H P^T r
cudaError_t op_adjoint(ctdm_tape *t, const float2 *r, float2 *g, cudaStream_t s)
{
    const long n = (long)t->R * t->R * t->R;
    cudaError_t e = cudaMemsetAsync(g, 0, sizeof(float2) * n, s);
    if (e != cudaSuccess) return e;
    scatter_kernel<<<grid_for(t->S), 256, 0, s>>>(r, t->idx, t->S, 1.0f, g); note_launch();
    e = cudaGetLastError();
    if (e == cudaSuccess) e = unitary_fft3(g, t->R, true, s);
    return e;
}

bool ok_volume(int R)
{
    return R == 32 || R == 64 || R == 128 || R == 256 || R == 384 || R == 512 || R == 768;
}

}  // namespace

extern "C" ctdm_status ctdm_tape_create(int device, int R, const ctdm_cfloat *d_F2, const uint32_t *d_counts,
                                        double k2, ctdm_tape **out)
{
    if (!d_F2 || !out || k2 <= 0) return fail(CTDM_ERR_INVALID, "ctdm_tape_create: bad argument%s");
    if (!ok_volume(R)) return fail(CTDM_ERR_INVALID, "ctdm_tape_create: volume side unsupported%s");
    GCK(cudaSetDevice(device), "cudaSetDevice");
    GCK(device_tables(), "building twiddle tables");
    cudaError_t e = cudaSuccess;
    const long n = (long)R * R * R;
    const long chunk = 65536;
    const int nb = (int)((n + chunk - 1) / chunk);
    ctdm_tape *t = new ctdm_tape();
    t->device = device;
    t->R = R;
    auto cleanup = [&](ctdm_status st) {
        ctdm_tape_destroy(t);
        return st;
    };
    if ((e = cudaMalloc(&t->flags, sizeof(int) * (n + 2 * nb + 1))) != cudaSuccess) return cleanup(cuda_fail(e, "alloc"));
    int *bc = t->flags + n;
    measured_flags<<<grid_for(n), 256>>>(reinterpret_cast<const float2 *>(d_F2), d_counts, n, t->flags); note_launch();
    block_counts<<<nb, kScanBlock>>>(t->flags, n, chunk, bc); note_launch();
    std::vector<int> hc(nb), ho(nb);
    if ((e = cudaMemcpy(hc.data(), bc, sizeof(int) * nb, cudaMemcpyDeviceToHost)) != cudaSuccess)
        return cleanup(cuda_fail(e, "tape counts"));
    long S = 0;
    for (int b = 0; b < nb; b++) {
        ho[b] = (int)S;
        S += hc[b];
    }
    t->S = S;
    if (S == 0) return cleanup(fail(CTDM_ERR_INVALID, "ctdm_tape_create: no measured voxels%s"));
    if ((e = cudaMemcpy(bc + nb, ho.data(), sizeof(int) * nb, cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMalloc(&t->idx, sizeof(uint32_t) * S)) != cudaSuccess ||
        (e = cudaMalloc(&t->y, sizeof(float2) * S)) != cudaSuccess ||
        (e = cudaMalloc(&t->work, sizeof(float2) * n)) != cudaSuccess ||
        (e = cudaMalloc(&t->red, sizeof(double) * kRedBlocks)) != cudaSuccess)
        return cleanup(cuda_fail(e, "alloc"));
    const float scale = (float)(1.0 / (-k2 * std::pow((double)R, 1.5)));
    block_write<<<nb, kScanBlock>>>(t->flags, bc + nb, n, chunk, reinterpret_cast<const float2 *>(d_F2), scale, t->idx,
                                    t->y); note_launch();
    if ((e = cudaDeviceSynchronize()) != cudaSuccess) return cleanup(cuda_fail(e, "tape build"));
    *out = t;
    set_error_message("");
    return CTDM_OK;
}

extern "C" void ctdm_tape_destroy(ctdm_tape *t)
{
    if (!t) return;
    cudaSetDevice(t->device);
    for (void *p : {(void *)t->idx, (void *)t->y, (void *)t->work, (void *)t->resid, (void *)t->wmom,
                    (void *)t->grad, (void *)t->red, (void *)t->flags})
        if (p) cudaFree(p);
    delete t;
}

extern "C" long ctdm_tape_samples(const ctdm_tape *t) { return t ? t->S : 0; }

extern "C" ctdm_status ctdm_tape_data(const ctdm_tape *t, ctdm_cfloat *h_y, uint32_t *h_idx)
{
    if (!t) return fail(CTDM_ERR_INVALID, "ctdm_tape_data: NULL tape%s");
    GCK(cudaSetDevice(t->device), "cudaSetDevice");
    if (h_y) GCK(cudaMemcpy(h_y, t->y, sizeof(float2) * t->S, cudaMemcpyDeviceToHost), "tape data");
    if (h_idx) GCK(cudaMemcpy(h_idx, t->idx, sizeof(uint32_t) * t->S, cudaMemcpyDeviceToHost), "tape indices");
    return CTDM_OK;
}

extern "C" ctdm_status ctdm_forward(ctdm_tape *t, const ctdm_cfloat *d_V, ctdm_cfloat *d_y, void *stream)
{
    if (!t || !d_V || !d_y) return fail(CTDM_ERR_INVALID, "ctdm_forward: NULL argument%s");
    GCK(cudaSetDevice(t->device), "cudaSetDevice");
    GCK(op_forward(t, reinterpret_cast<const float2 *>(d_V), reinterpret_cast<float2 *>(d_y), (cudaStream_t)stream),
        "forward");
    return CTDM_OK;
}

extern "C" ctdm_status ctdm_backward(ctdm_tape *t, const ctdm_cfloat *d_gy, ctdm_cfloat *d_gV, void *stream)
{
    if (!t || !d_gy || !d_gV) return fail(CTDM_ERR_INVALID, "ctdm_backward: NULL argument%s");
    GCK(cudaSetDevice(t->device), "cudaSetDevice");
    GCK(op_adjoint(t, reinterpret_cast<const float2 *>(d_gy), reinterpret_cast<float2 *>(d_gV), (cudaStream_t)stream),
        "backward");
    return CTDM_OK;
}

extern "C" ctdm_status ctdm_loss_grad(ctdm_tape *t, const ctdm_cfloat *d_V, double lambda, double eps,
                                      ctdm_cfloat *d_grad, double *loss)
{
    if (!t || !d_V || !d_grad) return fail(CTDM_ERR_INVALID, "ctdm_loss_grad: NULL argument%s");
    GCK(cudaSetDevice(t->device), "cudaSetDevice");
    const long n = (long)t->R * t->R * t->R;
    float2 *r = nullptr;
    GCK(cudaMalloc(&r, sizeof(float2) * t->S), "alloc residual");
    cudaError_t e = op_forward(t, reinterpret_cast<const float2 *>(d_V), r, 0);
    if (e == cudaSuccess) {
        residual_kernel<<<kRedBlocks, 256>>>(r, t->y, t->S, t->red); note_launch();
        e = cudaGetLastError();
    }
    double data = 0, tv = 0;
    if (e == cudaSuccess) data = 0.5 * sum_partials(t->red, kRedBlocks);
    if (e == cudaSuccess) e = op_adjoint(t, r, reinterpret_cast<float2 *>(d_grad), 0);
    if (e == cudaSuccess && lambda != 0.0) {
        tv_grad_kernel<<<kRedBlocks, 256>>>(reinterpret_cast<const float2 *>(d_V), t->R, (float)lambda, (float)eps,
                                            reinterpret_cast<float2 *>(d_grad), t->red); note_launch();
        e = cudaGetLastError();
        if (e == cudaSuccess) tv = sum_partials(t->red, kRedBlocks);
    }
    cudaFree(r);
    if (e != cudaSuccess) return cuda_fail(e, "loss and gradient");
    if (loss) *loss = data + lambda * tv;
    (void)n;
    return CTDM_OK;
}

extern "C" ctdm_status ctdm_reconstruct_gradient_ex(ctdm_tape *t, int iterations, double lambda, double eps,
                                                    double step, int positivity, ctdm_cfloat *d_V, double *h_loss,
                                                    void *stream)
{
    if (!t || !d_V || iterations < 0) return fail(CTDM_ERR_INVALID, "ctdm_reconstruct_gradient: bad argument%s");
    GCK(cudaSetDevice(t->device), "cudaSetDevice");
    cudaStream_t s = (cudaStream_t)stream;
    const long n = (long)t->R * t->R * t->R;
    if (!t->wmom) GCK(cudaMalloc(&t->wmom, sizeof(float2) * n), "alloc momentum");
    if (!t->grad) GCK(cudaMalloc(&t->grad, sizeof(float2) * n), "alloc gradient");
    if (!t->resid) GCK(cudaMalloc(&t->resid, sizeof(float2) * t->S), "alloc residual");
    float2 *V = reinterpret_cast<float2 *>(d_V);
    GCK(cudaMemcpyAsync(t->wmom, V, sizeof(float2) * n, cudaMemcpyDeviceToDevice, s), "momentum init");
    // the data term's Lipschitz constant is 1 (unitary transform, 0/1 sampling);
    // the smoothed TV adds at most 12 lambda / eps
    const double tau = step > 0 ? step : 1.0 / (1.0 + 12.0 * lambda / eps);
    double tk = 1.0;
    for (int it = 0; it < iterations; it++) {
        GCK(op_forward(t, t->wmom, t->resid, s), "forward");
        residual_kernel<<<kRedBlocks, 256, 0, s>>>(t->resid, t->y, t->S, t->red); note_launch();
        GCK(cudaGetLastError(), "residual");
        double loss = 0;
        if (h_loss) {
            GCK(cudaStreamSynchronize(s), "loss");
            loss = 0.5 * sum_partials(t->red, kRedBlocks);
        }
        GCK(op_adjoint(t, t->resid, t->grad, s), "adjoint");
        if (lambda != 0.0) {
            tv_grad_kernel<<<kRedBlocks, 256, 0, s>>>(t->wmom, t->R, (float)lambda, (float)eps, t->grad, t->red); note_launch();
            GCK(cudaGetLastError(), "tv");
            if (h_loss) {
                GCK(cudaStreamSynchronize(s), "loss");
                loss += lambda * sum_partials(t->red, kRedBlocks);
            }
        }
        if (h_loss) h_loss[it] = loss;   // objective at the extrapolated point
        const double tn = 0.5 * (1.0 + std::sqrt(1.0 + 4.0 * tk * tk));
        const float beta = (float)((tk - 1.0) / tn);
        if (positivity)
            fista_kernel<true><<<grid_for(n), 256, 0, s>>>(V, t->wmom, t->grad, n, (float)tau, beta);
        else
            fista_kernel<false><<<grid_for(n), 256, 0, s>>>(V, t->wmom, t->grad, n, (float)tau, beta);
        note_launch();
        GCK(cudaGetLastError(), "update");
        tk = tn;
    }
    return CTDM_OK;
}

extern "C" ctdm_status ctdm_reconstruct_gradient(ctdm_tape *t, int iterations, double lambda, double eps,
                                                 double step, ctdm_cfloat *d_V, double *h_loss, void *stream)
{
    return ctdm_reconstruct_gradient_ex(t, iterations, lambda, eps, step, 0, d_V, h_loss, stream);
}

extern "C" ctdm_status ctdm_contrast_to_ri(int R, const ctdm_cfloat *d_V, double n_med, int clamp, ctdm_cfloat *d_ri,
                                           void *stream)
{
    if (!d_V || !d_ri || !ok_volume(R)) return fail(CTDM_ERR_INVALID, "ctdm_contrast_to_ri: bad argument%s");
    const long n = (long)R * R * R;
    contrast_to_ri<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(reinterpret_cast<const float2 *>(d_V), R,
                                                                   (float)n_med, clamp,
                                                                   reinterpret_cast<float2 *>(d_ri)); note_launch();
    GCK(cudaGetLastError(), "contrast to RI");
    return CTDM_OK;
}
