"""The benchmark workloads end to end against the FP64 oracle, at their own sizes.

* wrap_heavy, exactly as bench.py runs it (121 x 1024^2 holograms -> 256^2 windows
  -> 256^3, DCT + Goldstein, 20 iterations, seed 1000): the carrier equal, every
  angle's wrapped phase within 1e-4 rad RMS, every residue-charge map and branch-cut
  mask bit-exact (on the wrapped phase the path computed, the definition of
  bit-exactness for Goldstein), the flood-filled phase within 1e-4 rad RMS, and the
  RI volume within 1e-5 RMS.
* 384^3 and 512^3 volumes from 1024^2 holograms (the batched and differentiable
  configurations' hologram size; fewer angles and iterations to bound the oracle's
  time): RI within 1e-5 RMS.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
PHASE_TOL = 1e-4
RI_TOL = 1e-5


def wrap(x):
    return np.angle(np.exp(1j * x))


def run_path(ctx, dev, acq, p):
    import torch
    r = acq.r_vol
    out = torch.empty((r, r, r), dtype=torch.complex64, device=dev)
    ctx.reconstruct_device(p, torch.from_numpy(acq.holograms).to(dev), torch.from_numpy(acq.background).to(dev),
                           acq.ang_x, acq.ang_y, out)
    torch.cuda.synchronize()
    return out.cpu().numpy()


def oracle_volume(oracle, acq, iters):
    par = oracle.make_params(acq.n_holo, acq.m_crop, acq.r_vol, iters, acq.fm0, acq.df, acq.dx, acq.k2, acq.n_med)
    return oracle.pipeline(par, acq.holograms, acq.background, acq.ang_x, acq.ang_y)


def ri_rmse(got, ref):
    return float(np.sqrt(np.mean(np.abs(got.astype(np.complex128) - ref) ** 2)))


def test_wrap_heavy_full_size(ctx, dev, oracle):
    import ctdm_gb300 as C
    from ctdm_gb300 import phantom
    acq = phantom.config_wrap_heavy(seed=1000)
    iters = 20
    A, m = len(acq.ang_x), acq.m_crop
    assert (A, acq.n_holo, m, acq.r_vol) == (121, 1024, 256, 256)
    got = run_path(ctx, dev, acq, C.params_for(acq, iters, run_goldstein=1))
    assert ctx.device_status() == 0
    car = oracle.qpi_carrier(acq.background)
    assert ctx.carrier() == car
    phase = ctx.read_buffer(0, np.float32).reshape(A, m, m)
    charges = ctx.read_buffer(3, np.int8).reshape(A, m, m)
    cuts = ctx.read_buffer(4, np.uint8).reshape(A, m, m)
    gold = ctx.read_buffer(5, np.float32).reshape(A, m, m)
    bgf = oracle.qpi_field(acq.background, m, *car)
    residues = 0
    for a in range(A):
        oph, _ = oracle.wrap_phase(oracle.qpi_field(acq.holograms[a], m, *car), bgf)
        assert np.sqrt(np.mean(wrap(phase[a] - oph) ** 2)) < PHASE_TOL, a
        oq = oracle.goldstein_residues(phase[a])
        assert np.array_equal(charges[a], oq), a
        oc = oracle.goldstein_cuts(oq)
        assert np.array_equal(cuts[a], oc), a
        oo, _, st = oracle.goldstein_floodfill(oc, phase[a])
        assert np.sqrt(np.mean((gold[a] - oo) ** 2)) < PHASE_TOL, a
        residues += int(np.count_nonzero(oq))
    assert residues > 0          # the workload does exercise the branch cuts
    ref, ocar = oracle_volume(oracle, acq, iters)
    assert ocar == car
    assert ri_rmse(got, ref) < RI_TOL


@pytest.mark.parametrize("r,angles,na,iters", [(384, 16, 0.9, 3), (512, 12, 1.2, 2)])
def test_large_volumes_from_1024_holograms(ctx, dev, oracle, r, angles, na, iters):
    import ctdm_gb300 as C
    from ctdm_gb300 import phantom
    acq = phantom.acquisition(1024, r, angles, na=na, seed=4000 + r)
    got = run_path(ctx, dev, acq, C.params_for(acq, iters))
    assert ctx.device_status() == 0
    ref, car = oracle_volume(oracle, acq, iters)
    assert ctx.carrier() == car
    assert ri_rmse(got, ref) < RI_TOL
