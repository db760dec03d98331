"""ASD-POCS with total variation and the frequency-interpolation mapping (the
reference's BatchReconPOCS with its mathematics fixed) through the C ABI against the
FP64 oracle.

Tolerances: hit counts bit-exact; F2 RMSE <= 1e-6 of its peak (the Ewald mapping's
bar); every step-size decision identical; after up to 4 iterations of 5 TV steps the
per-iteration distances Dp, Dd, Dg and the TV step within 1e-3 relative and RI RMSE
<= 1e-5; after 8 iterations of 20, 5e-3 and 5e-5 (the TV gradient's slope near zero
differences is 1/sqrt(eps) = 1e4, so float32 rounding grows over 160 steps)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
RI_TOL = 1e-5


def T(a, dev):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


def rmse(a, b):
    return float(np.sqrt(np.mean(np.abs(np.asarray(a, np.complex128) - np.asarray(b, np.complex128)) ** 2)))


@pytest.fixture(scope="module")
def line_scan():
    from ctdm_gb300 import phantom
    return phantom.acquisition(64, 64, 31, na=0.9, seed=5, pixel=0.4e-6, photons=1e6, scan="line")


@pytest.fixture(scope="module")
def line_data(oracle, line_scan):
    acq = line_scan
    par = oracle.make_params(acq.n_holo, acq.m_crop, acq.r_vol, 0, acq.fm0, acq.df, acq.dx, acq.k2, acq.n_med)
    ph, am, _ = oracle.front_end(par, acq.holograms, acq.background)
    U = np.stack([oracle.rytov_spectrum(ph[a], am[a]) for a in range(len(ph))]).astype(np.complex64)
    F2, C = oracle.fi_map(U.astype(np.complex128), acq.ang_x, acq.fm0, acq.df, acq.dx)
    return U, F2, C, ph, am


def test_fi_map_matches_oracle(ctx, dev, oracle, line_scan, line_data):
    import torch
    acq = line_scan
    U, oF2, oC = line_data[:3]
    r = acq.r_vol
    F2 = torch.zeros((r, r, r), dtype=torch.complex64, device=dev)
    cnt = torch.zeros((r, r, r), dtype=torch.int32, device=dev)
    ctx.map_fi(T(U, dev), acq.ang_x, acq.fm0, acq.df, acq.dx, F2, cnt)
    torch.cuda.synchronize()
    assert np.array_equal(cnt.cpu().numpy().astype(np.uint32), oC)
    g = F2.cpu().numpy()
    assert rmse(g, oF2) / np.abs(oF2).max() < 1e-6
    # the interpolation changes the values but not the sampled voxels of the Ewald mapping
    _, eC = oracle.ewald_map(U.astype(np.complex128), acq.ang_x, acq.ang_y, acq.fm0, acq.df, acq.dx)
    assert np.array_equal(eC > 0, oC > 0)
    assert rmse(g, oracle.ewald_map(U.astype(np.complex128), acq.ang_x, acq.ang_y, acq.fm0, acq.df, acq.dx)[0]) > 0


def test_fi_map_unsorted_scan_at_256(ctx, dev, oracle):
    """A scan given out of order (the mapping sorts it) on the 256-point kernel."""
    import torch
    r, A = 256, 24
    rng = np.random.default_rng(3)
    ang = rng.permutation(np.linspace(-0.6, 0.6, A)).astype(np.float32)
    U = (rng.normal(size=(A, r, r)) + 1j * rng.normal(size=(A, r, r))).astype(np.complex64)
    fm0, dx = 1.337 / 532e-9, 0.1e-6
    df = 1.0 / (r * dx)
    F2 = torch.zeros((r, r, r), dtype=torch.complex64, device=dev)
    cnt = torch.zeros((r, r, r), dtype=torch.int32, device=dev)
    ctx.map_fi(T(U, dev), ang, fm0, df, dx, F2, cnt)
    torch.cuda.synchronize()
    oF2, oC = oracle.fi_map(U.astype(np.complex128), ang, fm0, df, dx)
    assert np.array_equal(cnt.cpu().numpy().astype(np.uint32), oC)
    assert rmse(F2.cpu().numpy(), oF2) / np.abs(oF2).max() < 1e-6


@pytest.mark.parametrize("iters,steps,rtol,tol", [(0, 1, 1e-3, RI_TOL), (4, 5, 1e-3, RI_TOL), (8, 20, 5e-3, 5e-5)])
def test_pocs_matches_oracle(ctx, dev, oracle, line_scan, line_data, iters, steps, rtol, tol):
    import torch
    import ctdm_gb300 as C
    acq = line_scan
    oF2 = line_data[1]
    r = acq.r_vol
    op = oracle.pocs_params(iterations=iters, tv_steps=steps)
    ref, oh = oracle.pocs(oF2, op, acq.k2, acq.n_med)
    out = torch.zeros((r, r, r), dtype=torch.complex64, device=dev)
    h = ctx.pocs(T(oF2.astype(np.complex64), dev), r, acq.k2, acq.n_med, out,
                 params=C.pocs_params(iterations=iters, tv_steps=steps), history=True)
    torch.cuda.synchronize()
    if iters:
        np.testing.assert_allclose(h, oh, rtol=rtol, atol=1e-9)
        # the step-size rule took the same branch every iteration
        assert np.array_equal(h[1:, 3] < h[:-1, 3], oh[1:, 3] < oh[:-1, 3])
    assert rmse(out.cpu().numpy(), ref) < tol


def test_pocs_improves_on_the_zero_filled_estimate(ctx, dev, oracle, line_scan, line_data):
    """Against the phantom: 20 ASD-POCS iterations beat the zero-filled inverse (the
    positivity path with no loop body) and the positivity loop at 20 iterations."""
    import torch
    import ctdm_gb300 as C
    from ctdm_gb300 import phantom
    acq = line_scan
    r = acq.r_vol
    U, oF2 = line_data[0], line_data[1]
    truth = oracle.positivity(phantom.f2_truth(acq).astype(np.complex128), np.ones((r, r, r), np.uint32), 0,
                              acq.k2, acq.n_med)
    F2 = T(oF2.astype(np.complex64), dev)
    out = torch.zeros((r, r, r), dtype=torch.complex64, device=dev)
    ctx.pocs(F2, r, acq.k2, acq.n_med, out, params=C.pocs_params(iterations=20))
    e_pocs = rmse(out.cpu().numpy(), truth)
    eF2, _ = oracle.ewald_map(U.astype(np.complex128), acq.ang_x, acq.ang_y, acq.fm0, acq.df, acq.dx)
    ctx.positivity(T(eF2.astype(np.complex64), dev), r, 0, acq.k2, acq.n_med, out)
    e0 = rmse(out.cpu().numpy(), truth)
    ctx.positivity(T(eF2.astype(np.complex64), dev), r, 20, acq.k2, acq.n_med, out)
    e20 = rmse(out.cpu().numpy(), truth)
    assert e_pocs < e0 and e_pocs < e20, (e_pocs, e0, e20)


def test_batchreconpocs_dropin(ctx, dev, oracle, line_scan, line_data, tmp_path):
    """The reference-named entry: stacks in, 3D-RI-Complex_RxRxR.raw out, equal to the
    stage calls with the reference's constants."""
    import torch
    import ctdm_gb300 as C
    from ctdm_gb300 import _lib
    acq = line_scan
    r = acq.r_vol
    ph, am = line_data[3].astype(np.float32), line_data[4].astype(np.float32)
    A = ph.shape[0]
    lib = _lib.load()
    # BatchRecon's optics: dx = pixel / Mag * 1024 / R with the phantom's voxel
    mag = 85.0
    pixel_um = acq.dx * mag * r / 1024 * 1e6
    lib.ctdm_set_recon_globals(r, acq.n_med, acq.wavelength * 1e9, pixel_um, mag, 100, 0, str(tmp_path).encode())
    angx = np.ascontiguousarray(acq.ang_x, np.float32)
    angy = np.ascontiguousarray(acq.ang_y, np.float32)
    lib.BatchReconPOCS(ph.ctypes.data, am.ctypes.data, angx.ctypes.data, angy.ctypes.data, A)
    assert _lib.last_error() == ""
    got = np.fromfile(tmp_path / f"3D-RI-Complex_{r}x{r}x{r}.raw", np.complex64).reshape(r, r, r)
    dx = pixel_um * 1e-6 / mag * 1024 / r
    fm0 = acq.n_med / acq.wavelength
    k2 = (2 * np.pi * acq.n_med / acq.wavelength) ** 2
    U = torch.zeros((A, r, r), dtype=torch.complex64, device=dev)
    ctx.stack_spectra(T(ph, dev), T(am, dev), U, A, r)
    F2 = torch.zeros((r, r, r), dtype=torch.complex64, device=dev)
    ctx.map_fi(U, acq.ang_x, fm0, 1.0 / (r * dx), dx, F2)
    out = torch.zeros((r, r, r), dtype=torch.complex64, device=dev)
    ctx.pocs(F2, r, k2, acq.n_med, out, params=C.pocs_params())
    torch.cuda.synchronize()
    assert np.isfinite(got).all()
    assert rmse(got, out.cpu().numpy()) < 1e-6
