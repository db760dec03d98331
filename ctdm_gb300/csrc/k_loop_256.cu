// Positivity-loop passes for 256^3 volumes: all plan variants (fft_line.cuh PV<256, v>)
// and the plane pass with 8-CTA clusters.
#include "loop_passes.cuh"
#include "plane_pass.cuh"

CTDM_LOOP_SIZE_3(256)

namespace ctdm {
cudaError_t plane_pass_256(const LoopArgs &a, bool final_pass, int variant, cudaStream_t s)
{
    return variant == 2 ? run_plane_pass<256, 8, 4>(a, final_pass, s) : run_plane_pass<256, 8, 3>(a, final_pass, s);
}
int plane_clusters_256() { return plane_pass_clusters<256, 8, 3>(); }
}  // namespace ctdm
