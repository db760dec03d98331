// Single-stage kernels behind the reference-named entry points (one call = one
// reference stage, same arguments and semantics), used when a reference driver
// calls the stages one by one instead of the fused pipeline.
#include <cmath>

#include "kernels_front.cuh"
#include "point_ops.cuh"
#include "tma.cuh"

namespace ctdm {

// cuCopyArray (cTDM/Recon_kernel.cu:154-169): u[j + i*H] = (log amp, phase) of
// slice numZ (transposed).
__global__ void copy_data_array_kernel(float2 *u, const float *__restrict__ phase, const float *__restrict__ amp,
                                       int W, int H, int numZ)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= W || j >= H) return;
    const long idx = i + (long)W * j + (long)numZ * W * H;
    u[j + (long)i * H] = make_float2(logf(amp[idx]), phase[idx]);
}

// fillEdwardSphere (cTDM/Recon_kernel.cu:187-229) for one angle with the voxel
// rule of ewald_nz; (Nx, Ny) is unique per thread so the adds do not race.
__global__ void edward_sphere_kernel(const float2 *__restrict__ u, float2 *F, float *C, AngleGeom g, double df,
                                     double fm02, float fm02s, int W, int H, int Z)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= W || j >= H || !g.valid) return;
    const int ii = i - W / 2, jj = j - H / 2;
    float fz;
    const int nz = ewald_nz(ii, jj, g, df, fm02, fm02s, Z, fz);
    if (nz < 0) return;
    const int nx = imod(ii, W), ny = imod(jj, H);
    const long idx = nx + (long)ny * W + (long)nz * W * H;
    const float2 v = u[nx + (long)ny * W];
    const float s = fz * 4.0f * CTDM_PI_F;
    F[idx] = make_float2(F[idx].x - s * v.y, F[idx].y + s * v.x);
    C[idx] += 1.0f;
}

// Initial_F_F2 (cTDM/Recon_kernel.cu:253-276).
__global__ void initial_f_kernel(const float *__restrict__ C, float2 *F, float2 *F2, float dx, long n)
{
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        float2 f = F[i];
        const float c = C[i];
        if (c != 0.f) f = make_float2(f.x / c, f.y / c);
        const float2 f2 = make_float2(f.x / dx, f.y / dx);
        F2[i] = f2;
        F[i] = f2;
    }
}

__global__ void est_n_kernel(float2 *n, const float2 *__restrict__ F, float k2, float nm, long cnt)
{
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < cnt; i += (long)gridDim.x * blockDim.x)
        n[i] = est_n(F[i], k2, nm);
}

__global__ void modify_kernel(const float2 *__restrict__ n, float2 *F, float k2, float nm2, long cnt)
{
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < cnt; i += (long)gridDim.x * blockDim.x)
        F[i] = modify_f(n[i], k2, nm2);
}

__global__ void check_kernel(float2 *F, const float2 *__restrict__ F2, long cnt)
{
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < cnt; i += (long)gridDim.x * blockDim.x) {
        const float2 f2 = F2[i];
        if (f2.x != 0.0f && f2.y != 0.0f) F[i] = f2;
    }
}

// Real parts of complex holograms: the reference passes camera frames to
// extractQPI_AlgorithmA as cufftComplex with zero imaginary parts
// (cTDM/HilbertTransform.cu:711-716,879-883).
__global__ void real_parts_kernel(const float2 *__restrict__ in, float *out, long n)
{
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        out[i] = in[i].x;
}

// A bounded device-side wait that nothing completes: thread 0 initialises an
// mbarrier for one arrival that never comes and waits on its first phase with the
// wait the z pass uses for its TMA tiles (polls <= 0: its production bound).  The
// wait runs out and records `code` in *err; no copy was issued, so nothing is in
// flight when the kernel returns.  cycles[0] receives the wait's length in SM clocks.
__global__ void bounded_wait_probe_kernel(int *err, int polls, int code, long long *cycles)
{
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x != 0) return;
    tma::mbar_init(&bar, 1);
    tma::fence_barrier_init();
    const long long t0 = clock64();
    if (polls > 0) tma::mbar_wait(&bar, 0, err, code, polls);
    else tma::mbar_wait(&bar, 0, err, code);
    cycles[0] = clock64() - t0;
}

__global__ void counts_to_mask_kernel(const uint32_t *__restrict__ c, uint8_t *m, long n)
{
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        m[i] = c[i] != 0u;
}

static unsigned grid_for(long n)
{
    long b = (n + 255) / 256;
    return (unsigned)(b > 8192 ? 8192 : (b < 1 ? 1 : b));
}

cudaError_t compat_copy_data_array(float2 *u, const float *ph, const float *am, int W, int H, int numZ,
                                   cudaStream_t s)
{
    dim3 block(32, 8), grid((W + 31) / 32, (H + 7) / 8);
    copy_data_array_kernel<<<grid, block, 0, s>>>(u, ph, am, W, H, numZ); note_launch();
    return cudaGetLastError();
}

cudaError_t compat_edward_sphere(const float2 *u, float2 *F, float *C, const AngleGeom &g, double df, double fm02,
                                 float fm02s, int W, int H, int Z, cudaStream_t s)
{
    dim3 block(32, 8), grid((W + 31) / 32, (H + 7) / 8);
    edward_sphere_kernel<<<grid, block, 0, s>>>(u, F, C, g, df, fm02, fm02s, W, H, Z); note_launch();
    return cudaGetLastError();
}

cudaError_t compat_initial_f(const float *C, float2 *F, float2 *F2, float dx, long n, cudaStream_t s)
{
    initial_f_kernel<<<grid_for(n), 256, 0, s>>>(C, F, F2, dx, n); note_launch();
    return cudaGetLastError();
}

cudaError_t compat_est_n(float2 *n, const float2 *F, float k2, float nm, long cnt, cudaStream_t s)
{
    est_n_kernel<<<grid_for(cnt), 256, 0, s>>>(n, F, k2, nm, cnt); note_launch();
    return cudaGetLastError();
}

cudaError_t compat_modify(const float2 *n, float2 *F, float k2, float nm2, long cnt, cudaStream_t s)
{
    modify_kernel<<<grid_for(cnt), 256, 0, s>>>(n, F, k2, nm2, cnt); note_launch();
    return cudaGetLastError();
}

cudaError_t compat_check(float2 *F, const float2 *F2, long cnt, cudaStream_t s)
{
    check_kernel<<<grid_for(cnt), 256, 0, s>>>(F, F2, cnt); note_launch();
    return cudaGetLastError();
}

cudaError_t real_parts(const float2 *in, float *out, long n, cudaStream_t s)
{
    real_parts_kernel<<<grid_for(n), 256, 0, s>>>(in, out, n); note_launch();
    return cudaGetLastError();
}

cudaError_t bounded_wait_probe(int *err, int polls, int code, long long *cycles, cudaStream_t s)
{
    bounded_wait_probe_kernel<<<1, 32, 0, s>>>(err, polls, code, cycles); note_launch();
    return cudaGetLastError();
}

cudaError_t counts_to_mask(const uint32_t *c, uint8_t *m, long n, cudaStream_t s)
{
    counts_to_mask_kernel<<<grid_for(n), 256, 0, s>>>(c, m, n); note_launch();
    return cudaGetLastError();
}

}  // namespace ctdm
