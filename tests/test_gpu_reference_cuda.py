"""The FP64 oracle pinned against the reference's own CUDA code (cuFFT, IEEE build),
run on the GPU on the same seeded holograms (oracle/refcuda: the reference's kernels
and cuFFT calls, unmodified, driven in its job-loop and BatchRecon order).  Skipped
where the comparison sources were not assembled (oracle/refcuda/assemble.py needs the
reference checkout) or nvcc is missing.

Stage by stage: the wrapped phase and amplitude of calcWrapPhase, the DCT unwrap, the
Ewald hit counts (the reference decides the voxel index in float, the oracle in FP64:
a few boundary voxels may differ) and F2; then the RI volumes of the reference, of the
oracle and of this library.  Beside them, one stage each: QPI Algorithm B, FastUnwrapping
and the Goldstein residues (bit-exact)."""
import os
import shutil
import sys
import tempfile

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "oracle", "_ref", "refcuda", "src")


@pytest.fixture(scope="module")
def compare():
    if not os.path.isdir(SRC) or shutil.which("nvcc") is None:
        pytest.skip("reference comparison sources not assembled, or no nvcc")
    sys.path.insert(0, os.path.join(ROOT, "oracle", "refcuda"))
    import compare as CMP
    return CMP


def test_reference_stages_and_volume(compare, oracle, ctx, dev):
    import torch
    import ctdm_gb300 as C
    from ctdm_gb300 import phantom
    exes = compare.build()
    acq = phantom.acquisition(256, 128, 8, seed=77, pixel=0.2e-6)
    iters = 3
    car = oracle.qpi_carrier(acq.background)
    r = acq.r_vol
    with tempfile.TemporaryDirectory() as tmp:
        fin, dump = os.path.join(tmp, "in.bin"), os.path.join(tmp, "dump")
        os.makedirs(dump)
        compare.write_input(fin, acq, iters, car)
        _, ref_vol = compare.run_reference(exes["ieee"], fin, 1, r, dump=dump)
        st = compare.stage_parity(oracle, acq, car, dump)
    assert st["wrapped_phase_rms_rad_max"] < 1e-6, st
    assert st["amplitude_rmse_max"] < 1e-6, st
    assert st["dct_unwrapped_rmse_rad_max"] < 1e-4, st
    assert st["hit_voxels_differing"] <= 1e-5 * r ** 3, st
    assert st["f2_rel_l2_on_equal_hit_voxels"] < 1e-4, st
    par = oracle.make_params(acq.n_holo, acq.m_crop, r, iters, acq.fm0, acq.df, acq.dx, acq.k2, acq.n_med)
    fp64, _ = oracle.pipeline(par, acq.holograms, acq.background, acq.ang_x, acq.ang_y)
    out = torch.empty((r, r, r), dtype=torch.complex64, device=dev)
    ctx.reconstruct_device(C.params_for(acq, iters), torch.from_numpy(acq.holograms).to(dev),
                           torch.from_numpy(acq.background).to(dev), acq.ang_x, acq.ang_y, out)
    torch.cuda.synchronize()
    ours = out.cpu().numpy()
    ref_err = compare.rmse(ref_vol, fp64)
    our_err = compare.rmse(ours, fp64)
    print(f"reference CUDA vs FP64 RI RMSE {ref_err:.2e}, this library {our_err:.2e}; stages {st}")
    assert np.isfinite(ref_vol).all()
    assert ref_err < 1e-3          # the reference's own float error (median race, float est_n, voxel rule)
    assert our_err < 1e-5


def test_reference_qpi_b(compare, oracle, ctx):
    """QPI Algorithm B (the reference's default method): the reference's own
    extractQPI_AlgorithmB and calcWrapPhase (IEEE build) and this library's, each against
    the FP64 oracle on the same holograms with the carrier along x."""
    exes = compare.build()
    acq = compare.qpib_workload(n=512, angles=4, seed=91)
    res = compare.qpib_parity(oracle, {"ieee": exes["ieee"]}, acq, ctx)
    ref, mine = res["reference_ieee"], res["this_library"]
    print(res)
    assert ref["non_finite"] == 0
    assert ref["carrier_column"] == res["carrier_column_oracle"], res
    assert mine["carrier_column"] == res["carrier_column_oracle"], res
    assert mine["carrier_column_frame1"] == res["carrier_column_frame1_oracle"], res
    assert ref["wrapped_phase_rms_rad_max"] < 1e-4, res   # the reference's float transforms
    assert ref["amplitude_rmse_max"] < 1e-4, res
    assert mine["wrapped_phase_rms_rad_max"] < 1e-4, res
    assert mine["amplitude_rmse_max"] < 1e-5, res


def test_reference_fast_unwrapping(compare, oracle, ctx):
    """FastUnwrapping: the reference's own function (with FTUP plans of the (2M)^2 size its
    code transforms; the reference's driver creates them at (M/2)^2) and this library's,
    each against the FP64 oracle: the in-place normalisation, and the unwrapped maps."""
    exes = compare.build()
    maps = compare.fastuw_maps(m=256, count=3, seed=71)
    res = compare.fastuw_parity(oracle, {"ieee": exes["ieee"]}, maps, ctx)
    ref, mine = res["reference_ieee"], res["this_library"]
    print(res)
    assert ref["normalised_rmse_max"] < 1e-6, res
    assert mine["normalised_rmse_max"] < 1e-6, res
    assert ref["agree_fraction_min"] > 0.999, res
    assert mine["agree_fraction_min"] > 0.999, res


def test_reference_goldstein_residues(compare, oracle, ctx):
    """Goldstein residues: the reference's own cudaPhaseResidues (IEEE and Release builds)
    and this library's charges, bit-exact against the oracle, on noisy maps, a ragged one
    and a map whose phase differences land on the remainder's boundaries."""
    exes = compare.build()
    res = compare.residues_parity(oracle, exes, compare.residue_maps(seed=73), ctx)
    print(res)
    assert min(res["residues_oracle"]) > 100, res
    assert res["reference_ieee"]["pixels_differing"] == [0] * len(res["maps"]), res
    assert res["this_library"]["pixels_differing"] == [0] * len(res["maps"]), res
