"""The large configuration's sizes and the admission of tomograms by free device memory.

* 2048^2 holograms with 768^2 windows reconstructed into 768^3 (a few angles and
  iterations to bound the FP64 oracle's time and memory): carrier equal, RI RMSE
  <= 1e-5 against the oracle, and the context's workspace within the bound that
  ctdm_workspace_bytes gives callers for their own admission.
* A batch planned under a memory limit that admits one lane only: the plan uses one
  lane, every volume still equals its single call bit for bit; a limit below the
  largest job's workspace refuses the plan before anything is allocated.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_768_from_2048_holograms_matches_oracle(dev, oracle):
    import torch
    import ctdm_gb300 as C
    from ctdm_gb300 import phantom
    acq = phantom.acquisition(2048, 768, 4, na=0.9, seed=7680, pixel=0.1e-6)
    acq.m_crop = 768
    iters = 2
    p = C.params_for(acq, iters)
    ctx = C.Context(0)                     # a fresh workspace, to compare with the bound
    r = acq.r_vol
    out = torch.empty((r, r, r), dtype=torch.complex64, device=dev)
    ctx.reconstruct_device(p, torch.from_numpy(acq.holograms).to(dev), torch.from_numpy(acq.background).to(dev),
                           acq.ang_x, acq.ang_y, out)
    torch.cuda.synchronize()
    assert ctx.device_status() == 0
    held, bound = ctx.workspace(), C.workspace_bytes(p, len(acq.ang_x))
    assert 0.5 * bound <= held <= bound, (held, bound)
    got = out.cpu().numpy()
    del out
    torch.cuda.empty_cache()
    par = oracle.make_params(acq.n_holo, 768, r, iters, acq.fm0, acq.df, acq.dx, acq.k2, acq.n_med)
    ref, car = oracle.pipeline(par, acq.holograms, acq.background, acq.ang_x, acq.ang_y)
    assert ctx.carrier() == car
    err = float(np.sqrt(np.mean(np.abs(got.astype(np.complex128) - ref) ** 2)))
    assert err < 1e-5, err


def test_batch_admission_by_memory(ctx, dev):
    import torch
    import ctdm_gb300 as C
    from ctdm_gb300 import phantom
    specs = [(256, 256, 6, 2, 1), (512, 256, 5, 3, 2), (256, 128, 7, 2, 3)]
    jobs, refs = [], []
    for n, r, a, it, seed in specs:
        acq = phantom.acquisition(n, r, a, seed=seed, pixel=0.1e-6 * 512 / n)
        p = C.params_for(acq, it)
        holo = torch.from_numpy(acq.holograms).to(dev)
        bg = torch.from_numpy(acq.background).to(dev)
        ref = torch.empty((r, r, r), dtype=torch.complex64, device=dev)
        ctx.reconstruct_device(p, holo, bg, acq.ang_x, acq.ang_y, ref)
        jobs.append((p, holo, bg, acq.ang_x, acq.ang_y, torch.zeros_like(ref)))
        refs.append(ref)
    torch.cuda.synchronize()
    w_max = max(C.workspace_bytes(j[0], len(j[3])) for j in jobs)
    reserve = 24 * 256 ** 3 + (256 << 20)
    b = C.Batch(lanes=3)
    b.set_memory_limit(reserve + w_max + w_max // 2)     # room for one lane only
    b.plan(jobs)
    used, per_lane, avail = b.admission()
    assert used == 1 and per_lane == w_max and avail == reserve + w_max + w_max // 2
    assert set(b.lanes()) == {0}
    for job in jobs:
        job[5].zero_()
    b.run()
    torch.cuda.synchronize()
    for job, ref in zip(jobs, refs):
        assert torch.equal(job[5], ref)
    b.set_memory_limit(0)                                  # free memory decides: all three lanes
    b.plan(jobs)
    assert b.admission()[0] == 3
    b.set_memory_limit(reserve + w_max // 2)               # the largest job cannot fit
    with pytest.raises(C.CtdmError) as e:
        b.plan(jobs)
    assert e.value.status == 3 and "largest job" in str(e.value)   # CTDM_ERR_NOMEM
    b.close()
