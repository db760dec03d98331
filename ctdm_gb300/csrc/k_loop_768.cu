// Positivity-loop passes for 768^3 volumes: all plan variants (fft_line.cuh PV<768, v>)
// and the plane pass.  A 768^2 plane is 4.5 MiB, so only 16-CTA clusters keep the
// resident planes within L2 between the phases (48 rows per CTA): variant 1 with the
// 8-line plan at 2 CTAs per SM (19 planes, 86 MiB in flight), variant 2 with the
// 16-line plan at 1 CTA per SM (9 planes); both at 128 registers (at 3 CTAs per SM the
// 24-point register tiles spilled 284-572 bytes per thread).  The autotuner picks.  One
// iteration on synthetic data at 768^3: x / y / z / y 10.62 ms, variant 1 + z 9.86 ms,
// variant 2 + z 10.40 ms.
#include "loop_passes.cuh"
#include "plane_pass.cuh"

CTDM_LOOP_SIZE_3(768)

namespace ctdm {
cudaError_t plane_pass_768(const LoopArgs &a, bool final_pass, int variant, cudaStream_t s)
{
    return variant == 2 ? run_plane_pass<768, 16, 1, fftl::PV<768, 2>>(a, final_pass, s)
                        : run_plane_pass<768, 16, 2, fftl::PV<768, 1>>(a, final_pass, s);
}
int plane_clusters_768() { return plane_pass_clusters<768, 16, 2, fftl::PV<768, 1>>(); }
}  // namespace ctdm
