// Plane pass of the positivity loop: the x and y transforms of one z plane, and the
// real-space operators between them, in one pass over HBM.
//
// A thread-block cluster of C CTAs owns one plane (R x R complex64, 512 KiB at
// R = 256).  CTA r transforms rows y in [r R/C, (r+1) R/C) along x and writes them
// back in place; the plane stays resident in L2, so after a cluster barrier (release
// / acquire at cluster scope) the CTA reads columns x in [r R/C, (r+1) R/C) through
// L2, runs IFFT_y -> est_n -> modify -> FFT_y in registers and writes them back;
// after a second barrier the rows get FFT_x and stream back to HBM.  A plane thus
// crosses HBM once each way, the exchanges between the phases stay in L2.
// With the z pass this makes the loop body two passes (40 R^3 bytes of HBM
// traffic per iteration instead of the 72 R^3 of the x / y / z / y sequence).
//
// The reference runs this part of BatchRecon's loop (cTDM/HilbertTransform.cu:
// 1943-2004) as cuFFT3D calls (cTDM/FFT.cu:807-838) around calculate_n3D and
// Modify_F3D (cTDM/Recon_kernel.cu:305-383).
#pragma once
#include <cooperative_groups.h>

#include "fft_line.cuh"
#include "kernels.cuh"
#include "point_ops.cuh"
#include "tma.cuh"

namespace ctdm {

// PP: the line plan (lines per CTA, threads per line, radices) of the rows and columns.
template <int L, int C, class PP = fftl::Plan<L>>
struct PlaneCfg {
    using P = PP;
    static constexpr int RL = L / C;   // rows (and columns) per CTA
    static constexpr int SB = RL / P::B;
    static constexpr size_t SMEM = fftl::plan_smem_row<P>() > fftl::plan_smem<P>() ? fftl::plan_smem_row<P>()
                                                                                   : fftl::plan_smem<P>();
    static_assert(RL % P::B == 0, "rows per CTA must be a multiple of the plan's lines per CTA");
};

// MINB: resident CTAs per SM the register allocation aims for (3: no spills at
// R = 256; 4: more latency hiding for some spill traffic).  C: CTAs per plane.
// MOM: the accelerated loop (momentum on the projected iterate, LoopArgs::xprev).
template <int L, int C, int MINB, bool FINAL, bool MOM = false, class PP = fftl::Plan<L>>
__global__ void __launch_bounds__(PP::THREADS, MINB) plane_kernel(LoopArgs a, const float2 *__restrict__ tw)
{
    namespace cg = cooperative_groups;
    using Cfg = PlaneCfg<L, C, PP>;
    using P = typename Cfg::P;
    constexpr int RL = Cfg::RL;
    cg::cluster_group cluster = cg::this_cluster();
    const int rank = (int)cluster.block_rank();
    const int z = (int)(blockIdx.x / C);
    extern __shared__ float4 smem4[];
    float2 *scr = reinterpret_cast<float2 *>(smem4);
    float2 *plane = a.G + (long)z * L * L;
    const int tid = threadIdx.x;

    // ---- phase A: IFFT_x of this CTA's rows, in place (the plane stays in L2)
    {
        const int t = tid % P::T, b = tid / P::T;
#pragma unroll 1
        for (int sb = 0; sb < Cfg::SB; sb++) {
            float2 *row = plane + (long)(rank * RL + sb * P::B + b) * L;
            float2 v[P::E];
#pragma unroll
            for (int i = 0; i < P::E; i++) v[i] = __ldcs(&row[fftl::slot_pos<L, P::T, P::F0>(i, t)]);
            P::template seq_row<true>(scr, v, tw);
#pragma unroll
            for (int i = 0; i < P::E; i++) __stcg(&row[fftl::slot_pos<L, P::T, P::RV0>(i, t)], v[i]);
        }
    }
    cluster.sync();   // release / acquire at cluster scope: the rows are visible to the peers

    // ---- phase B: columns (read through L2), y transforms and point operators
    {
        const int b = tid % P::B, t = tid / P::B;
#pragma unroll 1
        for (int sb = 0; sb < Cfg::SB; sb++) {
            const int x = rank * RL + sb * P::B + b;
            float2 *col = plane + x;
            if constexpr (MOM && !FINAL) {
                // the previous iterate of these columns comes from HBM during the transform
                const float2 *xp = a.xprev + (long)z * L * L + x;
#pragma unroll
                for (int i = 0; i < P::E; i++) prefetch_l2(xp + (long)L * fftl::slot_pos<L, P::T, P::RV0>(i, t));
            }
            float2 v[P::E];
#pragma unroll
            for (int i = 0; i < P::E; i++) v[i] = __ldcg(&col[(long)fftl::slot_pos<L, P::T, P::F0>(i, t) * L]);
            P::template seq<true, false, false>(scr, v, tw);
            if constexpr (FINAL) {
                // est_n then the octant shift (cuFFT3Dshift, cTDM/FFT.cu:324-350) on the write
                float2 *dst = a.out + (long)((x + L / 2) % L) + (long)L * L * ((z + L / 2) % L);
#pragma unroll
                for (int i = 0; i < P::E; i++) {
                    const int y = fftl::slot_pos<L, P::T, P::RV0>(i, t);
                    dst[(long)L * ((y + L / 2) % L)] = est_n_scaled(v[i], a.s1, a.n_med);
                }
            } else {
#pragma unroll
                for (int i = 0; i < P::E; i++) v[i] = modify_f_scaled(est_n_scaled(v[i], a.s1, a.n_med), a.s2, a.k2);
                if constexpr (MOM) {
                    float2 *xp = a.xprev + (long)z * L * L + x;
#pragma unroll
                    for (int i = 0; i < P::E; i++) {
                        const long o = (long)L * fftl::slot_pos<L, P::T, P::RV0>(i, t);
                        const float2 prev = xp[o];
                        xp[o] = v[i];
                        v[i] = momentum_step(v[i], prev, a.beta);
                    }
                }
                P::template seqr<false, false, false>(scr, v, tw);
#pragma unroll
                for (int i = 0; i < P::E; i++) __stcg(&col[(long)fftl::slot_pos<L, P::T, P::F0>(i, t) * L], v[i]);
            }
        }
    }
    if constexpr (FINAL) return;
    cluster.sync();

    // ---- phase C: FFT_x of the rows, back to HBM
    {
        const int t = tid % P::T, b = tid / P::T;
#pragma unroll 1
        for (int sb = 0; sb < Cfg::SB; sb++) {
            float2 *row = plane + (long)(rank * RL + sb * P::B + b) * L;
            float2 v[P::E];
#pragma unroll
            for (int i = 0; i < P::E; i++) v[i] = __ldcg(&row[fftl::slot_pos<L, P::T, P::F0>(i, t)]);
            P::template seq_row<false>(scr, v, tw);
#pragma unroll
            for (int i = 0; i < P::E; i++) __stcs(&row[fftl::slot_pos<L, P::T, P::RV0>(i, t)], v[i]);
        }
    }
}

// Launches the plane pass of side L with C-CTA clusters over all L planes.
template <int L, int C, int MINB, class PP = fftl::Plan<L>>
static cudaError_t run_plane_pass(const LoopArgs &a, bool final_pass, cudaStream_t s)
{
    using Cfg = PlaneCfg<L, C, PP>;
    auto k = final_pass ? plane_kernel<L, C, MINB, true, false, PP>
                        : (a.xprev ? plane_kernel<L, C, MINB, false, true, PP> : plane_kernel<L, C, MINB, false, false, PP>);
    if (!twiddles(L)) return cudaErrorInitializationError;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const void *fn = reinterpret_cast<const void *>(k);
    if (!kernel_configured(fn, dev)) {
        e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Cfg::SMEM);
        if (e == cudaSuccess && C > 8) e = cudaFuncSetAttribute(k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        if (e != cudaSuccess) return e;
        mark_kernel_configured(fn, dev);
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(L * C), 1, 1);
    cfg.blockDim = dim3(PP::THREADS, 1, 1);
    cfg.dynamicSmemBytes = Cfg::SMEM;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    e = cudaLaunchKernelEx(&cfg, k, a, twiddles(L));
    note_launch();
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
}

// Number of clusters of the plane pass that fit on the device at once (0: none).
template <int L, int C, int MINB, class PP = fftl::Plan<L>>
static int plane_pass_clusters()
{
    using Cfg = PlaneCfg<L, C, PP>;
    auto k = plane_kernel<L, C, MINB, false, false, PP>;
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Cfg::SMEM) != cudaSuccess) return 0;
    if (C > 8 && cudaFuncSetAttribute(k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) return 0;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(L * C), 1, 1);
    cfg.blockDim = dim3(PP::THREADS, 1, 1);
    cfg.dynamicSmemBytes = Cfg::SMEM;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, k, &cfg) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

}  // namespace ctdm
