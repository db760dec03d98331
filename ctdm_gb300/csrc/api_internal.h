// Internal interface between the C-ABI runtime (ctdm_api.cu), the batch scheduler
// (batch.cu) and the job driver (driver.cu).  Not part of the public header.
#pragma once
#include <string>
#include <vector>

#include "ctdm.h"
#include "kernels.cuh"

namespace ctdm {
// Parameter checks of the whole path; M receives the window side.
ctdm_status validate_params(const ctdm_params *p, int A, int &M);
// Upper bound of the device bytes a context holds for one device-buffer reconstruction.
size_t workspace_bytes(const ctdm_params *p, int A, int M);
// Device bytes a context holds now; release_workspace frees them (device idle first).
size_t held_bytes(const ctdm_ctx *c);
void release_workspace(ctdm_ctx *c);
// The whole path on stream s with device-resident angle geometry (A entries).
// Capture-safe once the context's workspace has grown to the call's sizes.
ctdm_status run_pipeline(ctdm_ctx *c, const ctdm_params *p, int A, const float *d_holo, const float *d_bg,
                         const AngleGeom *d_geom, ctdm_cfloat *d_ri, cudaStream_t s);
// Per-angle illumination geometry (host, FP64).
void make_geometry(const float *angx, const float *angy, int A, double fm0, double df, std::vector<AngleGeom> &g);
ctdm_status fail_invalid(const char *msg);
ctdm_status fail_cuda(cudaError_t e, const char *what);
ctdm_status fail_io(const std::string &msg);
void clear_error();
int max_angles();
// Counts kernels a graph replay launches (the launch counter of ctdm_launch_count).
void note_launches(unsigned long long n);
// BatchRecon on host R x R stacks with the globals of ctdm_set_recon_globals; writes
// the .rimap file (the status-returning form of the reference-named BatchRecon).
ctdm_status batch_recon(const float *PhaseStack, const float *AmpStack, const float *sampleAngleRadX,
                        const float *sampleAngleRadY, int ReconFrame);
// dir/3D-RI-{Complex,Real,Imag}_RxRxR.<ext> from a host R^3 volume (save_mode 0, 1, 2).
ctdm_status write_ri_volume(const std::string &dir, int R, int save_mode, const ctdm_cfloat *h_ri, const char *ext);
}  // namespace ctdm
