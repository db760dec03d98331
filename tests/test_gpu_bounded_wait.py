"""Failure detection without a GPU fault: a bounded device-side wait that nothing
completes (an mbarrier whose phase never ends, waited on with the z pass's own
bounded wait) runs out, the kernel returns, the code reaches the host through the
context's status word and through ctdm_wait of the next submitted call
(CTDM_ERR_TIMEOUT), and the context keeps working afterwards."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_wait_that_runs_out_is_reported(ctx, dev):
    ms_small = ctx.probe_wait(1 << 12)
    assert ctx.device_status() == 9
    assert ctx.device_status() == 0            # reading clears it
    ms_large = ctx.probe_wait(1 << 16)
    assert ctx.device_status() == 9
    per_poll = (ms_large - ms_small) / ((1 << 16) - (1 << 12))
    print(f"bounded wait: {ms_small:.3f} ms for 4096 polls, {ms_large:.3f} ms for 65536; "
          f"production bound of 2^22 polls ~ {per_poll * (1 << 22):.1f} ms")
    assert ms_large > ms_small > 0


def test_timeout_reaches_ctdm_wait_and_context_recovers(ctx, dev):
    import ctdm_gb300 as C
    from ctdm_gb300 import _lib, phantom
    acq = phantom.acquisition(128, 64, 19, seed=43, pixel=0.2e-6, photons=1e4)
    p = C.params_for(acq, 2)
    r = acq.r_vol
    h, b = acq.holograms.astype(np.uint16), acq.background.astype(np.uint16)
    want = ctx.reconstruct(p, h, b, acq.ang_x, acq.ang_y)
    ctx.probe_wait(1 << 12)                    # the code is pending when the next call runs
    out = np.empty((r, r, r), np.complex64)
    ctx.submit(p, h, b, acq.ang_x, acq.ang_y, out)
    with pytest.raises(C.CtdmError):
        ctx.wait()
    assert "ran out" in _lib.last_error()
    assert ctx.device_status() == 0            # ctdm_wait cleared it
    got = ctx.reconstruct(p, h, b, acq.ang_x, acq.ang_y)
    assert np.array_equal(got, want)
