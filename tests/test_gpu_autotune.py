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


@pytest.mark.parametrize("r", [256, 512])
def test_loop_schemes_agree(ctx, dev, oracle, r):
    """The plane + z schemes (two cluster sizes of plane pass: 8 and 4 CTAs per plane at
    256^3, 16 and 8 at 512^3) and the x / y / z / y scheme give the oracle's volume, with
    and without the hit-mask predicate, and each scheme runs its own passes (the stage
    timer sees y passes only in scheme 0)."""
    import ctdm_gb300 as C
    import torch
    iters = 3 if r == 256 else 2
    f2 = synthetic_f2(r, seed=7)
    counts = ((f2.real != 0) & (f2.imag != 0)).astype(np.uint32)
    d_f2 = torch.from_numpy(f2).to(dev)
    d_counts = torch.from_numpy(counts.view(np.int32)).to(dev)
    out = torch.empty_like(d_f2)
    saved = C.loop_scheme(r)
    try:
        for mode in (0, 1):
            ref = oracle.positivity(f2, counts, iters, K2, N_MED, mode)
            for scheme in (0, 1, 2):
                C.set_loop_scheme(r, scheme)
                ctx.set_timing(True)
                ctx.positivity(d_f2, r, iters, K2, N_MED, out, check_mode=mode, counts=d_counts)
                torch.cuda.synchronize()
                st = ctx.stage_times()
                ctx.set_timing(False)
                y_launches = st["y_inverse"][1] + st["y_forward"][1]
                assert (y_launches == 0) == (scheme >= 1), (scheme, st)
                if scheme >= 1:
                    assert st["x_pass"][1] == iters and st["z_pass"][1] == iters, (scheme, st)
                g = out.cpu().numpy().astype(np.complex128)
                err = float(np.sqrt(np.mean(np.abs(g - ref) ** 2)))
                assert err < RI_TOL, (mode, scheme, err)
                assert ctx.device_status() == 0
    finally:
        C.set_loop_scheme(r, saved)


def test_pipeline_full_size_plain(ctx, dev, oracle):
    """The plain-method workload at its full size (49 x 256^2 holograms -> 256^3,
    10 iterations) against the FP64 oracle."""
    import ctdm_gb300 as C
    import torch
    from ctdm_gb300 import phantom
    acq = phantom.config_plain_small(seed=1000)
    iters = 10
    p = C.params_for(acq, iters)
    out = torch.empty((acq.r_vol,) * 3, dtype=torch.complex64, device=dev)
    ctx.reconstruct_device(p, torch.from_numpy(acq.holograms).to(dev), torch.from_numpy(acq.background).to(dev),
                           acq.ang_x, acq.ang_y, out)
    torch.cuda.synchronize()
    par = oracle.make_params(acq.n_holo, acq.m_crop, acq.r_vol, iters, acq.fm0, acq.df, acq.dx, acq.k2, acq.n_med)
    ref, car = oracle.pipeline(par, acq.holograms, acq.background, acq.ang_x, acq.ang_y)
    assert ctx.carrier() == car
    err = float(np.sqrt(np.mean(np.abs(out.cpu().numpy().astype(np.complex128) - ref) ** 2)))
    assert err < RI_TOL, err


@pytest.mark.parametrize("r", [64, 256])
def test_packed_measured_samples_bit_identical(ctx, dev, r):
    """The z pass on packed measured samples replaces exactly the voxels the dense
    pass replaces, with the same values: volumes are bit-identical (both predicates)."""
    import os
    import torch
    f2 = synthetic_f2(r, seed=11 + r)
    counts = ((f2.real != 0) & (f2.imag != 0)).astype(np.uint32)
    counts[: r // 2] = 0                        # hit mask differs from the value predicate
    d_f2 = torch.from_numpy(f2).to(dev)
    d_counts = torch.from_numpy(counts.view(np.int32)).to(dev)
    outs = {}
    for packed in ("1", "0"):
        os.environ["CTDM_PACKED_Z"] = packed
        try:
            for mode in (0, 1):
                out = torch.empty_like(d_f2)
                ctx.positivity(d_f2, r, 3, K2, N_MED, out, check_mode=mode, counts=d_counts)
                torch.cuda.synchronize()
                outs[(packed, mode)] = out.cpu().numpy()
        finally:
            os.environ.pop("CTDM_PACKED_Z", None)
    for mode in (0, 1):
        assert np.array_equal(outs[("1", mode)], outs[("0", mode)]), mode
    assert not np.array_equal(outs[("1", 0)], outs[("1", 1)])


@pytest.mark.parametrize("r,variant", [(384, 2), (768, 1)])
def test_packed_z_pass_at_large_sides_bit_identical(ctx, dev, r, variant):
    """The z-pass plans with 8 or 16 lines per tile read packed measured samples at
    384^3 and 768^3 too: the volume equals the dense pass's bit for bit (F2 drawn on the
    device, 5% of the voxels measured)."""
    import os
    import torch
    import ctdm_gb300 as C
    gen = torch.Generator(device=dev).manual_seed(r)
    keep = torch.rand((r, r, r), generator=gen, device=dev) < 0.05
    f2 = torch.randn((r, r, r), dtype=torch.complex64, generator=gen, device=dev) * (1e-2 * K2 * 100)
    f2 = torch.where(keep, f2, torch.zeros_like(f2))
    del keep
    saved, _ = C.plans(r)
    outs = {}
    try:
        C.set_plans(r, (saved[0], saved[1], variant))
        for packed in ("1", "0"):
            os.environ["CTDM_PACKED_Z"] = packed
            try:
                out = torch.empty_like(f2)
                ctx.positivity(f2, r, 2, K2, N_MED, out)
                torch.cuda.synchronize()
                outs[packed] = out
            finally:
                os.environ.pop("CTDM_PACKED_Z", None)
        assert torch.equal(outs["1"], outs["0"])
        assert ctx.device_status() == 0
    finally:
        C.set_plans(r, saved)
    del outs, f2
    torch.cuda.empty_cache()
