"""Batched reconstruction through the C ABI: every job of a mixed batch (uneven
angle counts, hologram, window and volume sizes, with and without Goldstein) gives
bit-for-bit the volume of its own single ctdm_reconstruct_device call, both when the
batch runs as one CUDA graph launch and when it runs eagerly."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def jobs_and_refs(ctx):
    import torch
    import ctdm_gb300 as C
    from ctdm_gb300 import phantom
    dev = torch.device("cuda:0")
    specs = [  # (n, r, angles, iterations, goldstein, seed)
        (64, 64, 7, 3, 0, 1),
        (128, 64, 5, 2, 1, 2),
        (64, 32, 9, 4, 0, 3),
        (128, 128, 6, 2, 0, 4),
        (64, 64, 4, 5, 1, 5),
    ]
    jobs, refs = [], []
    for n, r, a, it, gold, seed in specs:
        acq = phantom.acquisition(n, r, a, seed=seed, pixel=0.4e-6 * 64 / n)
        p = C.params_for(acq, it, run_goldstein=gold)
        holo = torch.from_numpy(acq.holograms).to(dev)
        bg = torch.from_numpy(acq.background).to(dev)
        ref = torch.empty((r, r, r), dtype=torch.complex64, device=dev)
        ctx.reconstruct_device(p, holo, bg, acq.ang_x, acq.ang_y, ref)
        out = torch.zeros((r, r, r), dtype=torch.complex64, device=dev)
        jobs.append((p, holo, bg, acq.ang_x, acq.ang_y, out))
        refs.append(ref)
    torch.cuda.synchronize()
    return jobs, refs


def _check(jobs, refs):
    import torch
    torch.cuda.synchronize()
    for j, (job, ref) in enumerate(zip(jobs, refs)):
        assert torch.equal(job[5], ref), f"job {j} differs from its single-call result"


def _clear(jobs):
    for job in jobs:
        job[5].zero_()


def test_batch_plan_graph_and_eager_match_single_calls(jobs_and_refs):
    import ctdm_gb300 as C
    import torch
    jobs, refs = jobs_and_refs
    b = C.Batch(lanes=3)
    b.plan(jobs)                 # the eager warm-up run already produces the results
    _check(jobs, refs)
    for _ in range(2):           # the graph, twice (it keeps the job pointers)
        _clear(jobs)
        b.run()
        _check(jobs, refs)
    _clear(jobs)
    b.run_eager()
    _check(jobs, refs)
    lanes = b.lanes()
    assert sorted(set(lanes)) == [0, 1, 2]
    b.close()
    torch.cuda.synchronize()


def test_batch_single_lane(jobs_and_refs):
    import ctdm_gb300 as C
    jobs, refs = jobs_and_refs
    b = C.Batch(lanes=1)
    b.plan(jobs[:2])
    _clear(jobs[:2])
    b.run()
    _check(jobs[:2], refs[:2])
    assert b.lanes() == [0, 0]
    b.close()


def test_batch_rejects_invalid_job(jobs_and_refs):
    import ctdm_gb300 as C
    jobs, _ = jobs_and_refs
    bad = list(jobs[0])
    p = C.Params()
    ctypes_copy = type(jobs[0][0]).from_buffer_copy(jobs[0][0])
    ctypes_copy.r_vol = 100          # not a supported volume side
    bad[0] = ctypes_copy
    b = C.Batch(lanes=2)
    with pytest.raises(C.CtdmError):
        b.plan([jobs[1], tuple(bad)])
    b.close()
    del p


def test_batch_of_256_and_384_volumes_matches_single_calls(ctx):
    """A batch at the batched configuration's sizes (512^2 and 1024^2 holograms, 256^3
    and 384^3 volumes; few angles to bound the test's time), one job with Goldstein:
    each volume equals its own single call bit for bit, from the graph and eagerly."""
    import torch
    import ctdm_gb300 as C
    from ctdm_gb300 import phantom
    dev = torch.device("cuda:0")
    specs = [(512, 384, 6, 2, 0, 11), (1024, 256, 5, 2, 1, 12), (512, 256, 7, 3, 0, 13), (1024, 384, 4, 2, 0, 14)]
    jobs, refs = [], []
    for n, r, a, it, gold, seed in specs:
        acq = phantom.acquisition(n, r, a, seed=seed, pixel=0.1e-6 * 1024 / n)
        p = C.params_for(acq, it, run_goldstein=gold)
        holo = torch.from_numpy(acq.holograms).to(dev)
        bg = torch.from_numpy(acq.background).to(dev)
        ref = torch.empty((r, r, r), dtype=torch.complex64, device=dev)
        ctx.reconstruct_device(p, holo, bg, acq.ang_x, acq.ang_y, ref)
        jobs.append((p, holo, bg, acq.ang_x, acq.ang_y, torch.zeros_like(ref)))
        refs.append(ref)
    torch.cuda.synchronize()
    b = C.Batch(lanes=2)
    b.plan(jobs)
    _check(jobs, refs)
    _clear(jobs)
    b.run()
    _check(jobs, refs)
    _clear(jobs)
    b.run_eager()
    _check(jobs, refs)
    b.close()
    del jobs, refs
    torch.cuda.empty_cache()
