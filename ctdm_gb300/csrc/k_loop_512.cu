// Positivity-loop passes for 512^3 volumes: all plan variants (fft_line.cuh PV<512, v>)
// and the plane pass.  A 512^2 plane is 2 MiB, and the planes of the clusters resident
// at once must stay in L2 between the phases: 16-CTA clusters (variant 1, 32 rows per
// CTA, 19 planes = 38 MiB in flight at 2 CTAs per SM) or 8-CTA clusters (variant 2, 64
// rows per CTA, 38 planes = 76 MiB); the autotuner picks per device.  The three radix-8
// stages keep more values live than the 256-point plan: 2 CTAs per SM (128 registers)
// run without spills, 3 spilled 256-540 bytes per thread.
#include "loop_passes.cuh"
#include "plane_pass.cuh"

CTDM_LOOP_SIZE_3(512)

namespace ctdm {
using Plane512 = fftl::PV<512, 2>;   // 8 lines x 32 threads, 16 points per thread

cudaError_t plane_pass_512(const LoopArgs &a, bool final_pass, int variant, cudaStream_t s)
{
    return variant == 2 ? run_plane_pass<512, 8, 2, Plane512>(a, final_pass, s)
                        : run_plane_pass<512, 16, 2, Plane512>(a, final_pass, s);
}
int plane_clusters_512() { return plane_pass_clusters<512, 16, 2, Plane512>(); }
}  // namespace ctdm
