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
