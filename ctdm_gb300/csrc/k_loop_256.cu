// Positivity-loop passes for 256^3 volumes: all plan variants (fft_line.cuh PV<256, v>)
// and the plane pass with 8-CTA (variant 1) or 4-CTA (variant 2) clusters per plane.
// One loop iteration (plane + packed z pass) measured 0.199 ms with 8-CTA clusters,
// 0.183-0.187 with 4 (64 rows per CTA: twice the work between the cluster barriers),
// 0.238 with 16, and 0.192 with 4 at 4 CTAs per SM; the autotuner picks per device.
#include "loop_passes.cuh"
#include "plane_pass.cuh"

CTDM_LOOP_SIZE_3(256)

namespace ctdm {
cudaError_t plane_pass_256(const LoopArgs &a, bool final_pass, int variant, cudaStream_t s)
{
    return variant == 2 ? run_plane_pass<256, 4, 3>(a, final_pass, s) : run_plane_pass<256, 8, 3>(a, final_pass, s);
}
int plane_clusters_256() { return plane_pass_clusters<256, 8, 3>(); }
}  // namespace ctdm
