"""The host-buffer entry (ctdm_reconstruct) uploads the holograms in chunks of angles on
a copy stream and runs each chunk's front end while later chunks are in flight; every
stage works per map, so its volume must equal the device-buffer entry's bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("method,gold,qpi", [(0, 1, 1), (1, 0, 1), (2, 0, 1), (0, 0, 0)])
def test_host_chunks_equal_device_path(ctx, dev, method, gold, qpi):
    import torch
    import ctdm_gb300 as C
    from ctdm_gb300 import phantom
    carrier = (0.25, 0.0) if qpi == 0 else (0.125, 0.125)
    acq = phantom.acquisition(128, 64, 37, seed=21, pixel=0.2e-6, photons=1e4, carrier=carrier)
    p = C.params_for(acq, 3, unwrap_method=method, run_goldstein=gold, qpi_method=qpi)
    r = acq.r_vol
    out = torch.empty((r, r, r), dtype=torch.complex64, device=dev)
    ctx.reconstruct_device(p, torch.from_numpy(acq.holograms).to(dev), torch.from_numpy(acq.background).to(dev),
                           acq.ang_x, acq.ang_y, out)
    torch.cuda.synchronize()
    want = out.cpu().numpy()
    got = ctx.reconstruct(p, acq.holograms, acq.background, acq.ang_x, acq.ang_y)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("kind", ["u16", "u8"])
def test_integer_counts_equal_float_path(ctx, dev, kind):
    """16- and 8-bit camera frames (uploaded as integers, widened on the GPU) give the
    float path's volume bit for bit."""
    import ctdm_gb300 as C
    from ctdm_gb300 import phantom
    acq = phantom.acquisition(128, 64, 19, seed=23, pixel=0.2e-6, photons=1e4)
    if kind == "u16":
        holo, bg = acq.holograms.astype(np.uint16), acq.background.astype(np.uint16)
    else:
        scale = 250.0 / max(acq.holograms.max(), acq.background.max())
        holo = np.rint(acq.holograms * scale).astype(np.uint8)
        bg = np.rint(acq.background * scale).astype(np.uint8)
    p = C.params_for(acq, 2, run_goldstein=1)
    want = ctx.reconstruct(p, holo.astype(np.float32), bg.astype(np.float32), acq.ang_x, acq.ang_y)
    got = ctx.reconstruct(p, holo, bg, acq.ang_x, acq.ang_y)
    assert np.array_equal(got, want)


def test_submitted_calls_overlap_and_match(ctx, dev):
    """ctdm_submit: three different tomograms in flight at once (pinned buffers, so each
    call's uploads run beside the previous call's loop and its download beside the next
    call's front end) give the synchronous call's volumes bit for bit, in any order and
    with pageable buffers too."""
    import torch
    import ctdm_gb300 as C
    from ctdm_gb300 import phantom
    acqs = [phantom.acquisition(128, 64, 70, seed=31 + k, pixel=0.2e-6, photons=1e4) for k in range(3)]
    ps = [C.params_for(a, 3, run_goldstein=k % 2) for k, a in enumerate(acqs)]
    r = acqs[0].r_vol
    want = [ctx.reconstruct(p, a.holograms.astype(np.uint16), a.background.astype(np.uint16), a.ang_x, a.ang_y)
            for p, a in zip(ps, acqs)]
    pinned = [(torch.from_numpy(a.holograms.astype(np.uint16)).pin_memory(),
               torch.from_numpy(a.background.astype(np.uint16)).pin_memory()) for a in acqs]
    for order in ([0, 1, 2], [2, 0, 1, 0]):
        outs = [torch.empty((r, r, r), dtype=torch.complex64).pin_memory() for _ in order]
        for o, k in zip(outs, order):
            ctx.submit(ps[k], pinned[k][0], pinned[k][1], acqs[k].ang_x, acqs[k].ang_y, o)
        ctx.wait()
        for o, k in zip(outs, order):
            assert np.array_equal(o.numpy(), want[k]), (order, k)
    outs = [np.empty((r, r, r), np.complex64) for _ in range(2)]
    hs = [(a.holograms.astype(np.uint16), a.background.astype(np.uint16)) for a in acqs[:2]]
    for k in range(2):
        ctx.submit(ps[k], hs[k][0], hs[k][1], acqs[k].ang_x, acqs[k].ang_y, outs[k])
    ctx.wait()
    for k in range(2):
        assert np.array_equal(outs[k], want[k])
    ctx.wait()   # nothing in flight: returns at once


def test_submit_rejects_bad_arguments_and_recovers(ctx, dev):
    """A refused submission leaves nothing in flight: the next call runs normally."""
    import ctypes
    import ctdm_gb300 as C
    from ctdm_gb300 import _lib, phantom
    acq = phantom.acquisition(128, 64, 19, seed=29, pixel=0.2e-6, photons=1e4)
    p = C.params_for(acq, 2)
    r = acq.r_vol
    h = np.ascontiguousarray(acq.holograms.astype(np.uint16))
    b = np.ascontiguousarray(acq.background.astype(np.uint16))
    ax, ay = np.ascontiguousarray(acq.ang_x, np.float32), np.ascontiguousarray(acq.ang_y, np.float32)
    out = np.empty((r, r, r), np.complex64)
    lib = _lib.load()
    rc = lib.ctdm_submit(ctx.handle, ctypes.byref(p), len(ax), h.ctypes.data, b.ctypes.data, 3, ax.ctypes.data,
                         ay.ctypes.data, out.ctypes.data)
    assert rc != 0 and "bytes per count" in _lib.last_error()
    assert lib.ctdm_wait(ctx.handle) == 0
    want = ctx.reconstruct(p, h, b, acq.ang_x, acq.ang_y)
    ctx.submit(p, h, b, acq.ang_x, acq.ang_y, out)
    ctx.wait()
    assert np.array_equal(out, want)


def test_context_refuses_other_calls_while_submissions_are_in_flight(ctx, dev):
    """Between ctdm_submit and ctdm_wait the context's buffers belong to the calls in
    flight: any other entry point on that context is refused with a message (and
    nothing is enqueued), and after ctdm_wait the context serves every call again."""
    import torch
    import ctdm_gb300 as C
    from ctdm_gb300 import _lib, phantom
    acq = phantom.acquisition(128, 64, 19, seed=41, pixel=0.2e-6, photons=1e4)
    p = C.params_for(acq, 2)
    r = acq.r_vol
    h, b = acq.holograms.astype(np.uint16), acq.background.astype(np.uint16)
    want = ctx.reconstruct(p, h, b, acq.ang_x, acq.ang_y)
    out = np.empty((r, r, r), np.complex64)
    phi = torch.zeros((1, 64, 64), dtype=torch.float32, device=dev)
    dst = torch.zeros_like(phi)
    ctx.submit(p, h, b, acq.ang_x, acq.ang_y, out)
    with pytest.raises(C.CtdmError):
        ctx.unwrap_dct(phi, dst, 1, 64)
    assert "in flight" in _lib.last_error()
    vol = torch.empty((r, r, r), dtype=torch.complex64, device=dev)
    with pytest.raises(C.CtdmError):
        ctx.reconstruct_device(p, torch.from_numpy(acq.holograms).to(dev), torch.from_numpy(acq.background).to(dev),
                               acq.ang_x, acq.ang_y, vol)
    ctx.wait()
    assert np.array_equal(out, want)
    ctx.unwrap_dct(phi, dst, 1, 64)
    torch.cuda.synchronize()
