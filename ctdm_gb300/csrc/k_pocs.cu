// ASD-POCS reconstruction: data consistency and positivity projections alternated with
// total-variation steepest descent, with the step adapted from the distances each
// part moves the volume (Sidky and Pan, Phys. Med. Biol. 53 (2008) 4777, the
// algorithm the reference's BatchReconPOCS follows, cTDM/HilbertTransform.cu:
// 2049-2402, kernels cTDM/Recon_kernel.cu:834-1106).  The reference's version is not
// usable as written (complex square root with the wrong precedence, a data step that
// copies the measured data onto itself, the fourth TV term on the x neighbour,
// numerator minus denominator instead of their quotient, the TV result discarded by
// the next iteration, an uninitialised data tolerance); this is the algorithm with
// those parts written from the mathematics.
//
// The volume is the contrast V = n^2 / n_med^2 - 1 (the scattering potential is
// -k^2 V), real after the positivity projection.  One iteration:
//   F = FFT3(V); F = beta Y + (1 - beta) F where measured (Y = F2 / -k^2); V = IFFT3(F)
//   V+ = (max(Re sqrt(1 + V), 1))^2 - 1        (n real and n >= n_med)
//   Dp = |V+ - V_start|, Dd = |FFT3(V+) - Y| over the measured samples (optional)
//   first iteration: dtvg = alpha Dp
//   tv_steps times: g = grad TV(V); V -= dtvg g / |g|
//   Dg = |V - V+|; if Dg > r_max Dp and Dd > eps: dtvg *= alpha_red; beta *= beta_red
// TV is the isotropic total variation with backward differences and periodic
// boundaries, sum_q sqrt(eps + |V(q) - V(q - x)|^2 + |V(q) - V(q - y)|^2 + |V(q) - V(q - z)|^2).
//
// Device side: every sum is a per-block partial in double followed by a last-block sum
// in fixed order (deterministic), and the controller (PocsCtl) lives in device memory:
// the TV step reads its size from there, the reductions' last blocks update it.  An
// iteration is therefore a fixed launch sequence that a CUDA graph can replay.
#include "kernels.cuh"
#include "point_ops.cuh"

namespace ctdm {

namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ double warp_sum(double v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block sum of v in a fixed order; the result is valid in thread 0.
__device__ double block_sum(double v)
{
    __shared__ double sw[kThreads / 32];
    v = warp_sum(v);
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) sw[w] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x == 0)
        for (int i = 0; i < kThreads / 32; i++) t += sw[i];
    __syncthreads();
    return t;
}

// Writes this block's partial; the last block to finish sums all partials in index
// order and returns true in its thread 0 with *total set.
__device__ bool grid_sum(double v, double *part, unsigned *ticket, double *total)
{
    __shared__ bool last;
    const double b = block_sum(v);
    if (threadIdx.x == 0) {
        part[blockIdx.x] = b;
        __threadfence();
        last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;   // four chains: the loads overlap
    const int n = (int)gridDim.x;
    int i = threadIdx.x;
    for (; i + 3 * kThreads < n; i += 4 * kThreads) {
        s0 += __ldcg(&part[i]);
        s1 += __ldcg(&part[i + kThreads]);
        s2 += __ldcg(&part[i + 2 * kThreads]);
        s3 += __ldcg(&part[i + 3 * kThreads]);
    }
    for (; i < n; i += kThreads) s0 += __ldcg(&part[i]);
    double s = block_sum((s0 + s1) + (s2 + s3));
    if (threadIdx.x == 0) {
        *total = s;
        *ticket = 0u;
        return true;
    }
    return false;
}

// Re sqrt(1 + v) - 1 without cancellation for small v.
__device__ __forceinline__ float re_sqrt1p_m1(float2 v)
{
    const float zr = 1.0f + v.x;
    const float mod = sqrtf(zr * zr + v.y * v.y);
    const float mod_m1 = (2.0f * v.x + v.x * v.x + v.y * v.y) / (mod + 1.0f);   // |1 + v| - 1
    const float h = 0.5f * (mod_m1 + v.x);                                      // (|z| + Re z)/2 - 1
    return h / (sqrtf(1.0f + h) + 1.0f);
}

// Elementwise kernels: each CTA owns kPer * kThreads consecutive elements and each
// thread issues its kPer loads before it uses any of them (R^3 is a multiple of 1024).
constexpr int kPer = 4;

__global__ void __launch_bounds__(kThreads) dc_kernel(float2 *G, const float2 *__restrict__ F2, long n,
                                                      const PocsCtl *__restrict__ ctl, float y_scale)
{
    const float beta = (float)ctl->beta, keep = (float)(1.0 - ctl->beta);
    const long i0 = (long)blockIdx.x * (kPer * kThreads) + threadIdx.x;
    float2 f[kPer];
#pragma unroll
    for (int k = 0; k < kPer; k++) f[k] = i0 + k * kThreads < n ? F2[i0 + k * kThreads] : make_float2(0.f, 0.f);
#pragma unroll
    for (int k = 0; k < kPer; k++) {
        if (f[k].x != 0.f || f[k].y != 0.f) {
            const long i = i0 + k * kThreads;
            const float2 g = G[i];
            G[i] = make_float2(beta * (f[k].x * y_scale) + keep * g.x, beta * (f[k].y * y_scale) + keep * g.y);
        }
    }
}

__global__ void __launch_bounds__(kThreads) project_kernel(float2 *G, float *V, float *Vp, long n, float inv_n3,
                                                           PocsCtl *ctl, double *part, bool write_g)
{
    float acc = 0.f;
    for (long c = blockIdx.x; c * (kPer * kThreads) < n; c += gridDim.x) {
        const long i0 = c * (kPer * kThreads) + threadIdx.x;
        float2 g[kPer];
        float v0[kPer];
#pragma unroll
        for (int k = 0; k < kPer; k++) {
            const long i = i0 + k * kThreads;
            g[k] = i < n ? G[i] : make_float2(0.f, 0.f);
            v0[k] = i < n ? V[i] : 0.f;
        }
#pragma unroll
        for (int k = 0; k < kPer; k++) {
            const long i = i0 + k * kThreads;
            if (i >= n) continue;
            const float u = re_sqrt1p_m1(make_float2(g[k].x * inv_n3, g[k].y * inv_n3));
            const float vn = u > 0.f ? u * (2.0f + u) : 0.f;
            const float d = vn - v0[k];
            acc = fmaf(d, d, acc);
            V[i] = vn;
            Vp[i] = vn;
            if (write_g) G[i] = make_float2(vn, 0.f);
        }
    }
    double t;
    if (grid_sum(acc, part, &ctl->ticket, &t)) ctl->dp = sqrt(t);
}

__global__ void __launch_bounds__(kThreads) dd_kernel(const float2 *__restrict__ G, const float2 *__restrict__ F2,
                                                      long n, float y_scale, PocsCtl *ctl, double *part)
{
    float acc = 0.f;
    for (long c = blockIdx.x; c * (kPer * kThreads) < n; c += gridDim.x) {
        const long i0 = c * (kPer * kThreads) + threadIdx.x;
        float2 f[kPer];
#pragma unroll
        for (int k = 0; k < kPer; k++) f[k] = i0 + k * kThreads < n ? F2[i0 + k * kThreads] : make_float2(0.f, 0.f);
#pragma unroll
        for (int k = 0; k < kPer; k++) {
            if (f[k].x != 0.f || f[k].y != 0.f) {
                const float2 g = G[i0 + k * kThreads];
                const float dx = g.x - f[k].x * y_scale, dy = g.y - f[k].y * y_scale;
                acc = fmaf(dx, dx, fmaf(dy, dy, acc));
            }
        }
    }
    double t;
    if (grid_sum(acc, part, &ctl->ticket, &t)) ctl->dd = sqrt(t);
}

// 1 / sqrt(x) by the hardware approximation (rsqrt.approx.ftz; x >= eps > 0 here, so
// flushing subnormal inputs changes nothing).
__device__ __forceinline__ float rsqrt_approx(float x)
{
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// Gradient of TV at a voxel from the 13 values of its stencil (c: the voxel, xm / xp
// the x neighbours, and so on; "xp_ym" the voxel at (+1, -1, 0)).  Each term is a
// difference over the local gradient magnitude, taken with the reciprocal square root.
__device__ __forceinline__ float tv_grad(float v, float vxm, float vym, float vzm, float vxp, float vyp, float vzp,
                                         float xp_ym, float xp_zm, float xm_yp, float yp_zm, float xm_zp, float ym_zp,
                                         float eps)
{
    const float a0 = v - vxm, b0 = v - vym, c0 = v - vzm;
    const float r0 = rsqrt_approx(eps + a0 * a0 + b0 * b0 + c0 * c0);
    const float ax = vxp - v, bx = vxp - xp_ym, cx = vxp - xp_zm;
    const float rx = rsqrt_approx(eps + ax * ax + bx * bx + cx * cx);
    const float ay = vyp - xm_yp, by = vyp - v, cy = vyp - yp_zm;
    const float ry = rsqrt_approx(eps + ay * ay + by * by + cy * cy);
    const float az = vzp - xm_zp, bz = vzp - ym_zp, cz = vzp - v;
    const float rz = rsqrt_approx(eps + az * az + bz * bz + cz * cz);
    return (a0 + b0 + c0) * r0 - ax * rx - by * ry - cz * rz;
}

// TV tile: 32 x 16 voxels of a plane per CTA (two rows per thread, eight apart),
// marching through kZc planes along z with the planes z - 1, z, z + 1 (each with a
// one-voxel periodic halo) in shared memory; the next plane's loads are issued before
// the current plane is computed.  Every input element is read about 1.3 times.
constexpr int kTx = 32, kTy = 16, kZc = 32;
constexpr int kPw = kTx + 2, kPh = kTy + 2, kPlane = kPw * kPh, kLoads = (kPlane + kThreads - 1) / kThreads;

int tv_blocks(int R) { return (R / kTx) * (R / kTy) * (R / kZc); }

template <bool STEP>
struct TvTile {
    const float *__restrict__ Vin;
    const float *__restrict__ gin;
    float s;
    int off[kLoads];    // plane offsets of this thread's tile elements (periodic halo)
    int sidx[kLoads];   // their shared-memory index, -1 when unused

    __device__ __forceinline__ void fetch(int base, float *r) const
    {
#pragma unroll
        for (int j = 0; j < kLoads; j++) {
            if (sidx[j] < 0) continue;
            float v = __ldg(&Vin[base + off[j]]);
            if constexpr (STEP) v = v - s * __ldg(&gin[base + off[j]]);
            r[j] = v;
        }
    }
    __device__ __forceinline__ void put(float *plane, const float *r) const
    {
#pragma unroll
        for (int j = 0; j < kLoads; j++)
            if (sidx[j] >= 0) plane[sidx[j]] = r[j];
    }
};

// The two voxels of this thread on plane pc (rows ly and ly + 8).
__device__ __forceinline__ void tv_two(const float (*pm)[kPw], const float (*pc)[kPw], const float (*pp)[kPw], int lx,
                                       int ly, float eps, float *v, float *g)
{
#pragma unroll
    for (int h = 0; h < 2; h++) {
        const int y = ly + 8 * h;
        v[h] = pc[y][lx];
        g[h] = tv_grad(v[h], pc[y][lx - 1], pc[y - 1][lx], pm[y][lx], pc[y][lx + 1], pc[y + 1][lx], pp[y][lx],
                       pc[y - 1][lx + 1], pm[y][lx + 1], pc[y + 1][lx - 1], pm[y + 1][lx], pp[y][lx - 1],
                       pp[y - 1][lx], eps);
    }
}

// STEP = false: g = grad TV(Vin).  STEP = true: the volume is Vin - s gin with
// s = dtvg / |gin| (the previous descent step, applied while the planes are loaded),
// written to Vout, and gout = grad TV of it.  The last block stores |gout| and, on the
// first iteration, sets dtvg = alpha Dp.  Offsets are 32-bit (R^3 < 2^31 for R <= 768).
template <bool STEP>
__global__ void __launch_bounds__(kThreads) tv_kernel(const float *__restrict__ Vin, const float *__restrict__ gin,
                                                      float *Vout, float *gout, int R, float eps, PocsCtl *ctl,
                                                      double *part)
{
    static_assert(kTx * kTy == 2 * kThreads, "two voxels of the tile per thread");
    __shared__ float pl[3][kPh][kPw];
    TvTile<STEP> t;
    t.Vin = Vin;
    t.gin = gin;
    t.s = 0.f;
    if constexpr (STEP) t.s = ctl->gnorm > 0.0 ? (float)(ctl->dtvg / ctl->gnorm) : 0.f;
    const int nbx = R / kTx, nby = R / kTy;
    int bi = blockIdx.x;
    const int x0 = (bi % nbx) * kTx;
    bi /= nbx;
    const int y0 = (bi % nby) * kTy, z0 = (bi / nby) * kZc;
    const int rr = R * R;
#pragma unroll
    for (int j = 0; j < kLoads; j++) {
        const int e = threadIdx.x + j * kThreads;
        const int lx = e % kPw, ly = e / kPw;
        int gx = x0 - 1 + lx, gy = y0 - 1 + ly;
        gx = gx < 0 ? gx + R : (gx >= R ? gx - R : gx);
        gy = gy < 0 ? gy + R : (gy >= R ? gy - R : gy);
        t.sidx[j] = e < kPlane ? e : -1;
        t.off[j] = e < kPlane ? gx + R * gy : 0;
    }
    auto zbase = [&](int z) { return rr * (z < 0 ? z + R : (z >= R ? z - R : z)); };
    const int tx = threadIdx.x % kTx, ty = threadIdx.x / kTx, lx = tx + 1, ly = ty + 1;
    const int out0 = (x0 + tx) + R * (y0 + ty);
    float nxt[kLoads];
    t.fetch(zbase(z0 - 1), nxt);
    t.put(&pl[0][0][0], nxt);
    t.fetch(zbase(z0), nxt);
    t.put(&pl[1][0][0], nxt);
    t.fetch(zbase(z0 + 1), nxt);
    float acc = 0.f;
    auto plane_step = [&](int k, float *pnew, const float (*pm)[kPw], const float (*pc)[kPw],
                          const float (*pp)[kPw]) {
        t.put(pnew, nxt);   // plane z0 + k + 1
        __syncthreads();
        if (k + 1 < kZc) t.fetch(zbase(z0 + k + 2), nxt);   // in flight while this plane is computed
        float v[2], g[2];
        tv_two(pm, pc, pp, lx, ly, eps, v, g);
        const int q = out0 + rr * (z0 + k);
#pragma unroll
        for (int h = 0; h < 2; h++) {
            if constexpr (STEP) Vout[q + 8 * R * h] = v[h];
            gout[q + 8 * R * h] = g[h];
            acc = fmaf(g[h], g[h], acc);
        }
        __syncthreads();
    };
    for (int k = 0; k < kZc; k++) {
        switch (k % 3) {   // plane slots as constants: z - 1, z, z + 1
        case 0: plane_step(k, &pl[2][0][0], pl[0], pl[1], pl[2]); break;
        case 1: plane_step(k, &pl[0][0][0], pl[1], pl[2], pl[0]); break;
        default: plane_step(k, &pl[1][0][0], pl[2], pl[0], pl[1]); break;
        }
    }
    double tot;
    if (grid_sum(acc, part, &ctl->ticket, &tot)) {
        ctl->gnorm = sqrt(tot);
        if (!STEP && ctl->first) {
            ctl->dtvg = ctl->alpha * ctl->dp;
            ctl->first = 0;
        }
    }
}

// The last descent step, Dg, the step-size rule and the history entry; G = V for the
// next iteration's transform.
__global__ void __launch_bounds__(kThreads) tv_final_kernel(const float *Vin, const float *gin, float *V,
                                                            const float *__restrict__ Vp, float2 *G, long n,
                                                            PocsCtl *ctl, double *part, double *hist)
{
    const float s = ctl->gnorm > 0.0 ? (float)(ctl->dtvg / ctl->gnorm) : 0.f;
    float acc = 0.f;
    for (long c = blockIdx.x; c * (kPer * kThreads) < n; c += gridDim.x) {
        const long i0 = c * (kPer * kThreads) + threadIdx.x;
        float vi[kPer], gi[kPer], pi[kPer];
#pragma unroll
        for (int k = 0; k < kPer; k++) {
            const long i = i0 + k * kThreads;
            vi[k] = i < n ? Vin[i] : 0.f;
            gi[k] = i < n ? gin[i] : 0.f;
            pi[k] = i < n ? Vp[i] : 0.f;
        }
#pragma unroll
        for (int k = 0; k < kPer; k++) {
            const long i = i0 + k * kThreads;
            if (i >= n) continue;
            const float v = vi[k] - s * gi[k];
            const float d = v - pi[k];
            acc = fmaf(d, d, acc);
            V[i] = v;
            G[i] = make_float2(v, 0.f);
        }
    }
    double t;
    if (grid_sum(acc, part, &ctl->ticket, &t)) {
        ctl->dg = sqrt(t);
        if (ctl->it < ctl->n_hist) {
            double *h = hist + 4 * ctl->it;
            h[0] = ctl->dp;
            h[1] = ctl->dd;
            h[2] = ctl->dg;
            h[3] = ctl->dtvg;
        }
        if (ctl->dg > ctl->r_max * ctl->dp && ctl->dd > ctl->eps_data) ctl->dtvg *= ctl->alpha_red;
        ctl->beta *= ctl->beta_red;
        ctl->it++;
    }
}

// n = n_med sqrt(1 + V) (principal root, Re n >= n_med, Im n >= 0, as calculate_n3D),
// octant shifted like cuFFT3Dshift.
__global__ void __launch_bounds__(kThreads) pocs_n_kernel(const float2 *__restrict__ G, int R, float inv_n3,
                                                          float n_med, float2 *ri)
{
    // 32-bit index arithmetic: R^3 < 2^31 for R <= 768
    const unsigned ur = (unsigned)R, rr = ur * ur, n = rr * ur, h = ur / 2;
    const unsigned i0 = blockIdx.x * (kPer * kThreads) + threadIdx.x;
    float2 g[kPer];
#pragma unroll
    for (int k = 0; k < kPer; k++) g[k] = i0 + k * kThreads < n ? G[i0 + k * kThreads] : make_float2(0.f, 0.f);
#pragma unroll
    for (int k = 0; k < kPer; k++) {
        const unsigned i = i0 + k * kThreads;
        if (i >= n) continue;
        const unsigned x = i % ur, yz = i / ur, y = yz % ur, z = yz / ur;
        const unsigned xs = x + h >= ur ? x + h - ur : x + h, ys = y + h >= ur ? y + h - ur : y + h,
                       zs = z + h >= ur ? z + h - ur : z + h;
        ri[xs + ur * ys + rr * zs] = est_n_scaled(g[k], inv_n3, n_med);
    }
}

unsigned grid_for(long n) { return (unsigned)((n + kPer * kThreads - 1) / (kPer * kThreads)); }

// Reducing elementwise kernels: at most 8 CTAs per SM of 152, each looping over chunks
// (one ticket atomic per CTA).
constexpr unsigned kReduceGrid = 8 * 152;
unsigned grid_reduce(long n)
{
    const unsigned g = grid_for(n);
    return g < kReduceGrid ? g : kReduceGrid;
}

cudaError_t fft3_unscaled(float2 *G, int R, bool inverse, cudaStream_t s)
{
    const long rr = (long)R * R;
    cudaError_t e = fft_rows(G, R, rr, inverse, s);
    if (e == cudaSuccess) e = fft_cols(G, R, rr, R, rr, R, inverse, s);
    if (e == cudaSuccess) e = fft_cols(G, R, rr, R, R, rr, inverse, s);
    return e;
}

// FFT3(G) -> data step -> IFFT3 (unscaled; the 1/R^3 is applied by the consumer).
cudaError_t data_step(const PocsBufs &b, cudaStream_t s)
{
    const long n = (long)b.R * b.R * b.R;
    cudaError_t e = fft3_unscaled(b.G, b.R, false, s);
    if (e != cudaSuccess) return e;
    dc_kernel<<<grid_for(n), kThreads, 0, s>>>(b.G, b.F2, n, b.ctl, b.y_scale);
    note_launch();
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    return fft3_unscaled(b.G, b.R, true, s);
}

}  // namespace

int pocs_partials(int R)
{
    const int t = tv_blocks(R), e = (int)grid_for((long)R * R * R);
    return t > e ? t : e;
}

cudaError_t pocs_iteration(const PocsBufs &b, int tv_steps, bool want_dd, cudaStream_t s)
{
    const int R = b.R;
    const long n = (long)R * R * R;
    const float inv_n3 = 1.0f / (float)n;
    cudaError_t e = data_step(b, s);
    if (e != cudaSuccess) return e;
    project_kernel<<<grid_reduce(n), kThreads, 0, s>>>(b.G, b.V, b.Vp, n, inv_n3, b.ctl, b.part, want_dd);
    note_launch();
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if (want_dd) {
        if ((e = fft3_unscaled(b.G, R, false, s)) != cudaSuccess) return e;
        dd_kernel<<<grid_reduce(n), kThreads, 0, s>>>(b.G, b.F2, n, b.y_scale, b.ctl, b.part);
        note_launch();
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    // TV steepest descent: gradient at the POCS result, then tv_steps - 1 fused
    // (step, gradient) passes between two buffer pairs, then the last step
    const unsigned tvg = (unsigned)tv_blocks(R);
    tv_kernel<false><<<tvg, kThreads, 0, s>>>(b.V, nullptr, nullptr, b.g, R, b.tv_eps, b.ctl, b.part);
    note_launch();
    const float *vin = b.V, *gin = b.g;
    float *vout = b.V2, *gout = b.g2;
    for (int t = 1; t < tv_steps; t++) {
        tv_kernel<true><<<tvg, kThreads, 0, s>>>(vin, gin, vout, gout, R, b.tv_eps, b.ctl, b.part);
        note_launch();
        const float *nv = vout, *ng = gout;
        vout = const_cast<float *>(vin);
        gout = const_cast<float *>(gin);
        vin = nv;
        gin = ng;
    }
    tv_final_kernel<<<grid_reduce(n), kThreads, 0, s>>>(vin, gin, b.V, b.Vp, b.G, n, b.ctl, b.part, b.hist);
    note_launch();
    return cudaGetLastError();
}

cudaError_t pocs_finish(const PocsBufs &b, float n_med, float2 *ri, cudaStream_t s)
{
    const long n = (long)b.R * b.R * b.R;
    cudaError_t e = data_step(b, s);
    if (e != cudaSuccess) return e;
    pocs_n_kernel<<<grid_for(n), kThreads, 0, s>>>(b.G, b.R, 1.0f / (float)n, n_med, ri);
    note_launch();
    return cudaGetLastError();
}

}  // namespace ctdm
