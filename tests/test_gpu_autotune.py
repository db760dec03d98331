"""Autotuned FFT plan variants of the positivity-loop passes: every variant of every
pass gives the FP64 oracle's volume (RI RMSE <= 1e-5), and the autotuner reports a
time for each variant and keeps one of them."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
RI_TOL = 1e-5
K2 = (2 * np.pi * 1.337 / 532e-9) ** 2
N_MED = 1.337


def synthetic_f2(r, seed, fill=0.15, contrast=1e-2):
    """Measured k-space data on a random subset of voxels, scaled to a ~1e-2 contrast."""
    rng = np.random.default_rng(seed)
    keep = rng.random((r, r, r)) < fill
    amp = contrast * K2 * np.sqrt(r ** 3 / fill)
    f2 = (rng.standard_normal((r, r, r)) + 1j * rng.standard_normal((r, r, r))) * amp
    return np.where(keep, f2, 0).astype(np.complex64)


@pytest.mark.parametrize("r", [256, 384])
def test_every_variant_matches_oracle(ctx, dev, oracle, r):
    import ctdm_gb300 as C
    import torch
    f2 = synthetic_f2(r, seed=r)
    counts = ((f2.real != 0) & (f2.imag != 0)).astype(np.uint32)
    iters = 2
    ref = oracle.positivity(f2, counts, iters, K2, N_MED, 0)
    d_f2 = torch.from_numpy(f2).to(dev)
    out = torch.empty_like(d_f2)
    saved, _ = C.plans(r)
    try:
        for v in range(C.plan_count(r)):
            C.set_plans(r, (v, v, v))
            ctx.positivity(d_f2, r, iters, K2, N_MED, out)
            torch.cuda.synchronize()
            g = out.cpu().numpy().astype(np.complex128)
            err = float(np.sqrt(np.mean(np.abs(g - ref) ** 2)))
            assert err < RI_TOL, (r, v, err)
    finally:
        C.set_plans(r, saved)


def test_autotune_reports_all_variants(ctx):
    import ctdm_gb300 as C
    r = 256
    chosen, ms = C.autotune(r)
    n = C.plan_count(r)
    assert n == 3
    assert all(0 <= v < n for v in chosen)
    for p in range(3):
        times = [ms[(p, v)] for v in range(n)]
        assert all(t > 0 for t in times)
        assert ms[(p, chosen[p])] == min(times)
    got, tuned = C.plans(r)
    assert got == chosen and tuned
