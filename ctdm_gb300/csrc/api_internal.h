// Internal interface between the C-ABI runtime (ctdm_api.cu) and the batch
// scheduler (batch.cu).  Not part of the public header.
#pragma once
#include <vector>

#include "ctdm.h"
#include "kernels.cuh"

namespace ctdm {
// Parameter checks of the whole path; M receives the window side.
ctdm_status validate_params(const ctdm_params *p, int A, int &M);
// The whole path on stream s with device-resident angle geometry (A entries).
// Capture-safe once the context's workspace has grown to the call's sizes.
ctdm_status run_pipeline(ctdm_ctx *c, const ctdm_params *p, int A, const float *d_holo, const float *d_bg,
                         const AngleGeom *d_geom, ctdm_cfloat *d_ri, cudaStream_t s);
// Per-angle illumination geometry (host, FP64).
void make_geometry(const float *angx, const float *angy, int A, double fm0, double df, std::vector<AngleGeom> &g);
ctdm_status fail_invalid(const char *msg);
ctdm_status fail_cuda(cudaError_t e, const char *what);
void clear_error();
int max_angles();
// Counts kernels a graph replay launches (the launch counter of ctdm_launch_count).
void note_launches(unsigned long long n);
}  // namespace ctdm
