// Goldstein branch-cut unwrapping -- placeholder launchers until the kernels land.
#include "kernels_front.cuh"

namespace ctdm {
cudaError_t goldstein_residues(const float *, int, int, int, int8_t *, cudaStream_t) { return cudaErrorNotSupported; }
cudaError_t goldstein_cuts(const int8_t *, int, int, int, uint8_t *, int8_t *, cudaStream_t)
{
    return cudaErrorNotSupported;
}
cudaError_t goldstein_floodfill(const uint8_t *, const float *, int, int, int, float *, uint8_t *, int *, int *,
                                cudaStream_t)
{
    return cudaErrorNotSupported;
}
}  // namespace ctdm
