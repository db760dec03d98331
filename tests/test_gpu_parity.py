"""GPU parity: every stage of the CUDA path against the FP64 oracle on the same
seeded inputs, through the C ABI.

Tolerances: integer outputs bit-exact (carrier, hit counts); phase RMSE <= 1e-4
rad; RI RMSE <= 1e-5 (float32 path vs FP64)."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
PHASE_TOL = 1e-4
RI_TOL = 1e-5


def T(a, dev):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


def zeros(shape, dtype, dev):
    import torch
    return torch.zeros(shape, dtype=dtype, device=dev)


def rmse(a, b):
    return float(np.sqrt(np.mean(np.abs(np.asarray(a, np.complex128) - np.asarray(b, np.complex128)) ** 2)))


def wrap(x):
    return np.angle(np.exp(1j * x))


@pytest.fixture(scope="module")
def small():
    from ctdm_gb300 import phantom
    return phantom.small_case(seed=5, n=64, r=64, angles=8)


# ---------------------------------------------------------------- FFT
@pytest.mark.parametrize("L", [16, 32, 64, 128, 256, 384, 512, 768, 1024, 1536, 2048])
def test_fft1d_all_lengths(ctx, dev, L):
    import ctdm_gb300 as C
    import torch
    rng = np.random.default_rng(L)
    batch = max(1, 8192 // L)
    a = (rng.standard_normal((batch, L)) + 1j * rng.standard_normal((batch, L))).astype(np.complex64)
    for inv in (False, True):
        t = T(a, dev)
        C.fft(t, [L], batch=batch, inverse=inv)
        torch.cuda.synchronize()
        ref = np.fft.ifft(a.astype(np.complex128), axis=1) * L if inv else np.fft.fft(a.astype(np.complex128), axis=1)
        err = np.abs(t.cpu().numpy() - ref).max() / np.abs(ref).max()
        assert err < 2e-6, (L, inv, err)


@pytest.mark.parametrize("dims", [(64, 64, 64), (256, 32, 16), (384, 384, 1), (32, 768, 1)])
def test_fft_multidim(ctx, dev, dims):
    import ctdm_gb300 as C
    import torch
    nx, ny, nz = dims
    rng = np.random.default_rng(nx + ny)
    a = (rng.standard_normal((nz, ny, nx)) + 1j * rng.standard_normal((nz, ny, nx))).astype(np.complex64)
    t = T(a, dev)
    rank = 3 if nz > 1 else 2
    C.fft(t, list(dims[:rank]))
    torch.cuda.synchronize()
    ref = np.fft.fftn(a.astype(np.complex128), axes=(0, 1, 2) if rank == 3 else (1, 2))
    assert np.abs(t.cpu().numpy() - ref).max() / np.abs(ref).max() < 2e-6


# ---------------------------------------------------------------- QPI
@pytest.mark.parametrize("n,angles", [(64, 4), (256, 3), (512, 3), (1024, 2), (2048, 1)])
def test_qpi_matches_oracle(ctx, dev, oracle, n, angles):
    from ctdm_gb300 import phantom
    acq = phantom.acquisition(n, n, angles, seed=n, pixel=0.1e-6 * 256 / n)
    m = n // 4
    ph = zeros((angles, m, m), __import__("torch").float32, dev)
    am = zeros((angles, m, m), __import__("torch").float32, dev)
    car = ctx.qpi(n, m, T(acq.holograms, dev), T(acq.background, dev), ph, am, angles)
    ocar = oracle.qpi_carrier(acq.background)
    assert car == ocar
    bgf = oracle.qpi_field(acq.background, m, *ocar)
    for a in range(angles):
        spf = oracle.qpi_field(acq.holograms[a], m, *ocar)
        oph, oam = oracle.wrap_phase(spf, bgf)
        gph = ph[a].cpu().numpy()
        assert np.sqrt(np.mean(wrap(gph - oph) ** 2)) < PHASE_TOL
        assert rmse(am[a].cpu().numpy(), oam) < 1e-5


@pytest.mark.parametrize("n", [256, 1024])
def test_extract_qpi_algorithm_a_drop_in(ctx, dev, oracle, n):
    """The reference-named symbol (cTDM/HilbertTransform.cu:1546-1585): host complex
    holograms with zero imaginary parts in, the conjugated 1/M^2-scaled window fields
    out on the device; frame 1 detects the carrier from the background and frame 2
    reuses it."""
    import ctdm_gb300 as C
    import torch
    from ctdm_gb300 import phantom
    acq = phantom.acquisition(n, n, 2, seed=n + 7, pixel=0.1e-6 * 256 / n)
    L = C.load()
    m = n // 4
    sp_f = torch.zeros((m, m), dtype=torch.complex64, device=dev)
    bg_f = torch.zeros_like(sp_f)
    car = oracle.qpi_carrier(acq.background)
    bg = np.ascontiguousarray(acq.background.astype(np.complex64))
    for frame in (1, 2):
        sp = np.ascontiguousarray(acq.holograms[frame - 1].astype(np.complex64))
        L.extractQPI_AlgorithmA(sp.ctypes.data, bg.ctypes.data, sp_f.data_ptr(), bg_f.data_ptr(), n, n, frame)
        assert L.ctdm_last_error() == b""
        osp = oracle.qpi_field(acq.holograms[frame - 1], m, *car)
        obg = oracle.qpi_field(acq.background, m, *car)
        scale = np.abs(obg).max()
        assert rmse(sp_f.cpu().numpy(), osp) / scale < 1e-5
        assert rmse(bg_f.cpu().numpy(), obg) / scale < 1e-5
        oph, _ = oracle.wrap_phase(osp, obg)
        gph, _ = oracle.wrap_phase(sp_f.cpu().numpy(), bg_f.cpu().numpy())
        assert np.sqrt(np.mean(wrap(gph - oph) ** 2)) < PHASE_TOL


def test_qpi_explicit_carrier_and_bg_per_angle(ctx, dev, oracle, small):
    import torch
    acq = small
    n, m, A = acq.n_holo, acq.m_crop, 3
    bgs = np.stack([acq.background, acq.holograms[5], acq.holograms[6]])
    car = oracle.qpi_carrier(acq.background)
    ph = zeros((A, m, m), torch.float32, dev)
    am = zeros((A, m, m), torch.float32, dev)
    got = ctx.qpi(n, m, T(acq.holograms[:A], dev), T(bgs, dev), ph, am, A, bg_per_angle=True, carrier=car)
    assert got == car
    for a in range(A):
        oph, oam = oracle.wrap_phase(oracle.qpi_field(acq.holograms[a], m, *car), oracle.qpi_field(bgs[a], m, *car))
        assert np.sqrt(np.mean(wrap(ph[a].cpu().numpy() - oph) ** 2)) < PHASE_TOL


# ---------------------------------------------------------------- DCT unwrap
@pytest.mark.parametrize("mode", [0, 1])
def test_dct_unwrap_golden_input(ctx, dev, oracle, mode):
    import torch
    src = np.load(os.path.join(GOLD, "dct_chain_src.npy"))
    out = zeros((256, 256), torch.float32, dev)
    ctx.unwrap_dct(T(src, dev), out, 1, 256, mode=mode)
    torch.cuda.synchronize()
    ref = oracle.dct_unwrap(src.astype(np.float64), mode)
    assert rmse(out.cpu().numpy(), ref) < PHASE_TOL
    if mode == 0:
        ref_dump = np.load(os.path.join(GOLD, "dct_chain_IDCT.npy"))
        assert rmse(out.cpu().numpy(), ref_dump) < 1e-3   # the reference's float denominator


@pytest.mark.parametrize("m", [16, 32, 64, 128, 256, 384, 512, 768])
def test_dct_unwrap_sizes(ctx, dev, oracle, m):
    import torch
    rng = np.random.default_rng(m)
    y, x = np.mgrid[0:m, 0:m] / m
    true = 9.0 * np.sin(2.1 * x + 0.4) * np.cos(1.7 * y) + 4 * x * y + 0.05 * rng.standard_normal((m, m))
    phi = wrap(true).astype(np.float32)
    A = 2
    stack = np.stack([phi, wrap(-true).astype(np.float32)])
    out = zeros((A, m, m), torch.float32, dev)
    ctx.unwrap_dct(T(stack, dev), out, A, m, mode=0)
    torch.cuda.synchronize()
    for a in range(A):
        ref = oracle.dct_unwrap(stack[a].astype(np.float64), 0)
        assert rmse(out[a].cpu().numpy(), ref) < PHASE_TOL


def test_dct_drop_in(ctx, dev, oracle):
    import ctdm_gb300 as C
    import torch
    src = np.load(os.path.join(GOLD, "dct_chain_src.npy"))
    s = T(src, dev)
    d = zeros((256, 256), torch.float32, dev)
    C.load().DCT_UWLS_Unwrapped(d.data_ptr(), s.data_ptr(), 256, 256)
    assert C._lib.last_error() == ""
    assert rmse(d.cpu().numpy(), oracle.dct_unwrap(src.astype(np.float64), 0)) < PHASE_TOL


# ---------------------------------------------------------------- FastUnwrapping
@pytest.mark.parametrize("m", [32, 64, 128, 256])
def test_fast_unwrap(ctx, dev, oracle, m):
    import torch
    y, x = np.mgrid[0:m, 0:m] / m
    true = 6.0 * np.sin(2.3 * x) * np.cos(1.9 * y) + 3 * x
    phi = wrap(true).astype(np.float32)
    t = T(phi, dev)
    out = zeros((m, m), torch.float32, dev)
    ctx.unwrap_fast(t, out, 1, m)
    torch.cuda.synchronize()
    ref, norm = oracle.fast_unwrap(phi.astype(np.float64))
    assert rmse(t.cpu().numpy(), norm) < 1e-5            # the input is normalised in place
    g = out.cpu().numpy()
    # the result is the normalised phase moved by multiples of 2 pi, minus its minimum
    # (subtractMin, cTDM/FastUnwrapping.cu:347-359)
    d = wrap(g - norm)
    assert (np.abs(wrap(d - d[0, 0])) < 1e-4).all()
    assert abs(g.min()) < 1e-6
    agree = np.mean(np.abs(g - ref) < 1e-3)
    assert agree > 0.999, agree


# ---------------------------------------------------------------- stack / spectra
def test_prepare_stack_and_spectra(ctx, dev, oracle, small):
    import torch
    acq = small
    n, m, r, A = acq.n_holo, acq.m_crop, acq.r_vol, 4
    rng = np.random.default_rng(2)
    ph = (rng.standard_normal((A, m, m)) * 2).astype(np.float32)
    am = (0.5 + rng.random((A, m, m))).astype(np.float32)
    phs = zeros((A, r, r), torch.float32, dev)
    ams = zeros((A, r, r), torch.float32, dev)
    ctx.prepare_stack(T(ph, dev), T(am, dev), phs, ams, A, m, n, r)
    U = zeros((A, r, r), torch.complex64, dev)
    ctx.prepare_spectra(T(ph, dev), T(am, dev), U, A, m, n, r)
    torch.cuda.synchronize()
    for a in range(A):
        p1, a1 = oracle.resize_crop(ph[a], am[a], n, r)
        p2, a2 = oracle.median_check(p1, a1)
        assert rmse(phs[a].cpu().numpy(), p2) < 1e-5
        assert rmse(ams[a].cpu().numpy(), a2) < 1e-5
        u = oracle.rytov_spectrum(p2, a2)
        assert rmse(U[a].cpu().numpy(), u) / np.abs(u).max() < 1e-6


# ---------------------------------------------------------------- mapping + loop
def _spectra(oracle, acq, A):
    rng = np.random.default_rng(9)
    r = acq.r_vol
    U = (rng.standard_normal((A, r, r)) + 1j * rng.standard_normal((A, r, r))) * 50
    return U


def test_ewald_counts_bit_exact(ctx, dev, oracle, small):
    import torch
    acq = small
    A, r = len(acq.ang_x), acq.r_vol
    U = _spectra(oracle, acq, A)
    F2 = zeros((r, r, r), torch.complex64, dev)
    cnt = zeros((r, r, r), torch.int32, dev)
    ctx.map_ewald(T(U.astype(np.complex64), dev), acq.ang_x, acq.ang_y, acq.fm0, acq.df, acq.dx, F2, cnt)
    torch.cuda.synchronize()
    oF2, oC = oracle.ewald_map(U.astype(np.complex64).astype(np.complex128), acq.ang_x, acq.ang_y, acq.fm0, acq.df,
                               acq.dx)
    assert np.array_equal(cnt.cpu().numpy().astype(np.uint32), oC)
    assert oC.sum() > 0
    g = F2.cpu().numpy()
    assert rmse(g, oF2) / np.abs(oF2).max() < 1e-6
    # zero pattern (the reference's data-replacement predicate) identical
    assert np.array_equal((g.real != 0) & (g.imag != 0), (oF2.real != 0) & (oF2.imag != 0))


@pytest.mark.parametrize("check_mode", [0, 1])
def test_positivity_matches_oracle(ctx, dev, oracle, small, check_mode):
    import torch
    acq = small
    r = acq.r_vol
    ph, am, _ = oracle.front_end(oracle.make_params(acq.n_holo, acq.m_crop, r, 0, acq.fm0, acq.df, acq.dx, acq.k2,
                                                    acq.n_med), acq.holograms, acq.background)
    U = np.stack([oracle.rytov_spectrum(ph[a], am[a]) for a in range(len(ph))])
    oF2, oC = oracle.ewald_map(U, acq.ang_x, acq.ang_y, acq.fm0, acq.df, acq.dx)
    iters = 4
    ref = oracle.positivity(oF2, oC, iters, acq.k2, acq.n_med, check_mode)
    out = zeros((r, r, r), torch.complex64, dev)
    cnt = T(oC.astype(np.int32), dev)
    ctx.positivity(T(oF2.astype(np.complex64), dev), r, iters, acq.k2, acq.n_med, out, check_mode=check_mode,
                   counts=cnt)
    torch.cuda.synchronize()
    assert rmse(out.cpu().numpy(), ref) < RI_TOL


# ---------------------------------------------------------------- whole path
@pytest.mark.parametrize("unwrap_mode", [0, 1])
def test_pipeline_matches_oracle(ctx, dev, oracle, small, unwrap_mode):
    import ctdm_gb300 as C
    import torch
    acq = small
    iters = 5
    p = C.params_for(acq, iters, unwrap_mode=unwrap_mode)
    out = zeros((acq.r_vol,) * 3, torch.complex64, dev)
    ctx.reconstruct_device(p, T(acq.holograms, dev), T(acq.background, dev), acq.ang_x, acq.ang_y, out)
    torch.cuda.synchronize()
    par = oracle.make_params(acq.n_holo, acq.m_crop, acq.r_vol, iters, acq.fm0, acq.df, acq.dx, acq.k2, acq.n_med,
                             unwrap_mode=unwrap_mode)
    ref, car = oracle.pipeline(par, acq.holograms, acq.background, acq.ang_x, acq.ang_y)
    assert ctx.carrier() == car
    g = out.cpu().numpy()
    assert rmse(g, ref) < RI_TOL
    assert g.real.max() > acq.n_med + 1e-3   # the object is reconstructed


def test_pipeline_host_buffers_match_device(ctx, dev, small):
    import ctdm_gb300 as C
    import torch
    acq = small
    p = C.params_for(acq, 3)
    host = ctx.reconstruct(p, acq.holograms, acq.background, acq.ang_x, acq.ang_y)
    out = zeros((acq.r_vol,) * 3, torch.complex64, dev)
    ctx.reconstruct_device(p, T(acq.holograms, dev), T(acq.background, dev), acq.ang_x, acq.ang_y, out)
    torch.cuda.synchronize()
    assert np.array_equal(host, out.cpu().numpy())   # deterministic


def test_pipeline_256_case(ctx, dev, oracle):
    """49-angle-shaped case at 128^2 holograms (-> 32 crop) into a 128^3 volume."""
    import ctdm_gb300 as C
    import torch
    from ctdm_gb300 import phantom
    acq = phantom.acquisition(128, 128, 12, seed=3, pixel=0.2e-6)
    iters = 3
    p = C.params_for(acq, iters)
    out = zeros((128,) * 3, torch.complex64, dev)
    ctx.reconstruct_device(p, T(acq.holograms, dev), T(acq.background, dev), acq.ang_x, acq.ang_y, out)
    torch.cuda.synchronize()
    par = oracle.make_params(128, 32, 128, iters, acq.fm0, acq.df, acq.dx, acq.k2, acq.n_med)
    ref, car = oracle.pipeline(par, acq.holograms, acq.background, acq.ang_x, acq.ang_y)
    assert rmse(out.cpu().numpy(), ref) < RI_TOL


# ---------------------------------------------------------------- reference-named stage calls
def test_reference_stage_sequence(ctx, dev, oracle, small):
    """BatchRecon's call sequence through the drop-in symbols (cTDM/HilbertTransform.cu:1943-1975)."""
    import ctdm_gb300 as C
    import torch
    L = C.load()
    acq = small
    r = acq.r_vol
    ph, am, _ = oracle.front_end(oracle.make_params(acq.n_holo, acq.m_crop, r, 0, acq.fm0, acq.df, acq.dx, acq.k2,
                                                    acq.n_med), acq.holograms, acq.background)
    U = np.stack([oracle.rytov_spectrum(ph[a], am[a]) for a in range(len(ph))]).astype(np.complex64)
    F = zeros((r, r, r), torch.complex64, dev)
    Cn = zeros((r, r, r), torch.float32, dev)
    for a in range(len(U)):
        u = T(U[a], dev)
        L.EdwardSphere(u.data_ptr(), F.data_ptr(), Cn.data_ptr(), float(np.float32(acq.fm0)), float(np.float32(acq.df)),
                       float(acq.ang_x[a]), float(acq.ang_y[a]), r, r, r)
    F2 = zeros((r, r, r), torch.complex64, dev)
    L.initial_F_and_F2(Cn.data_ptr(), F.data_ptr(), F2.data_ptr(), float(acq.dx), r, r, r)
    L.cuFFT3D(F.data_ptr(), r, r, r, 1)
    n = zeros((r, r, r), torch.complex64, dev)
    k2, nm = float(acq.k2), float(acq.n_med)
    L.est_n_3D(n.data_ptr(), F.data_ptr(), k2, nm, r, r, r)
    for _ in range(3):
        L.modify_F_3D(n.data_ptr(), F.data_ptr(), k2, nm * nm, r, r, r)
        L.cuFFT3D(F.data_ptr(), r, r, r, -1)
        L.check_F_3D(F.data_ptr(), F2.data_ptr(), r, r, r)
        L.cuFFT3D(F.data_ptr(), r, r, r, 1)
        L.est_n_3D(n.data_ptr(), F.data_ptr(), k2, nm, r, r, r)
    assert C._lib.last_error() == ""
    got = np.fft.fftshift(n.cpu().numpy())
    fm0f, dff = float(np.float32(acq.fm0)), float(np.float32(acq.df))
    oF2, oC = oracle.ewald_map(U.astype(np.complex128), acq.ang_x, acq.ang_y, fm0f, dff, float(np.float32(acq.dx)))
    ref = oracle.positivity(oF2, oC, 3, k2, nm, 0)
    assert rmse(got, ref) < RI_TOL
