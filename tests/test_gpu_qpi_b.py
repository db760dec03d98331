"""QPI Algorithm B (the reference's default QPI_Method = 0) against the FP64 oracle,
through the C ABI: carrier columns bit-exact, phase RMSE <= 1e-4 rad, amplitude
RMSE <= 1e-5, and the whole path with Algorithm B at RI RMSE <= 1e-5."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
PHASE_TOL = 1e-4
RI_TOL = 1e-5
XCARRIER = (0.25, 0.0)   # Algorithm B filters along x only


def T(a, dev):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


def wrap(x):
    return np.angle(np.exp(1j * x))


def rmse(a, b):
    return float(np.sqrt(np.mean(np.abs(np.asarray(a, np.complex128) - np.asarray(b, np.complex128)) ** 2)))


@pytest.mark.parametrize("n,angles", [(64, 3), (256, 3), (1024, 2)])
def test_qpi_b_matches_oracle(ctx, dev, oracle, n, angles):
    import torch
    from ctdm_gb300 import phantom
    acq = phantom.acquisition(n, n, angles, seed=n + 1, pixel=0.1e-6 * 256 / n, carrier=XCARRIER)
    m = n // 4
    ph = torch.zeros((angles, m, m), dtype=torch.float32, device=dev)
    am = torch.zeros_like(ph)
    cb, cs = ctx.qpi_b(n, T(acq.holograms, dev), T(acq.background, dev), ph, am, angles)
    ocb, ocs = oracle.qpib_center(acq.background), oracle.qpib_center(acq.holograms[0])
    assert (cb, cs) == (ocb, ocs)
    bgf = oracle.qpib_field(acq.background, ocb)
    for a in range(angles):
        spf = oracle.qpib_field(acq.holograms[a], ocs if a == 0 else ocb)
        oph, oam = oracle.wrap_phase(spf, bgf)
        assert np.sqrt(np.mean(wrap(ph[a].cpu().numpy() - oph) ** 2)) < PHASE_TOL
        assert rmse(am[a].cpu().numpy(), oam) < 1e-5


def test_qpi_b_given_column_and_bg_per_angle(ctx, dev, oracle):
    import torch
    from ctdm_gb300 import phantom
    n, A = 128, 3
    acq = phantom.acquisition(n, n, 5, seed=9, pixel=0.2e-6, carrier=XCARRIER)
    bgs = np.stack([acq.background, acq.holograms[3], acq.holograms[4]])
    c = oracle.qpib_center(acq.background)
    m = n // 4
    ph = torch.zeros((A, m, m), dtype=torch.float32, device=dev)
    am = torch.zeros_like(ph)
    got = ctx.qpi_b(n, T(acq.holograms[:A], dev), T(bgs, dev), ph, am, A, bg_per_angle=True, center=(c, c))
    assert got == (c, c)
    for a in range(A):
        oph, _ = oracle.wrap_phase(oracle.qpib_field(acq.holograms[a], c), oracle.qpib_field(bgs[a], c))
        assert np.sqrt(np.mean(wrap(ph[a].cpu().numpy() - oph) ** 2)) < PHASE_TOL


def test_qpi_b_recovers_the_object_phase(ctx, dev):
    """On an x-carrier hologram the method returns the Rytov phase Im u (transposed,
    as the reference's copySharedMem stores it), up to the downsampling."""
    import torch
    from ctdm_gb300 import phantom
    n = 256
    rng = np.random.default_rng(1)
    ells = phantom.cell_phantom(rng)
    ax, ay = phantom.cone_angles(3, 0.9, 1.337)
    u = phantom.rytov_field(ells, 1.337, 532e-9, n, 0.1e-6, ax[0], ay[0])
    holo = phantom.holograms_from_fields(u[None], 1e6, rng, XCARRIER)
    bg = phantom.holograms_from_fields(np.zeros((1, n, n), np.complex128), 1e6, rng, XCARRIER)[0]
    m = n // 4
    ph = torch.zeros((1, m, m), dtype=torch.float32, device=dev)
    am = torch.zeros_like(ph)
    ctx.qpi_b(n, T(holo, dev), T(bg, dev), ph, am, 1)
    got = wrap(ph[0].cpu().numpy())
    truth = u.imag[::4, ::4].T
    assert np.corrcoef(got.ravel(), truth.ravel())[0, 1] > 0.99


def test_pipeline_with_qpi_b_matches_oracle(ctx, dev, oracle):
    import ctdm_gb300 as C
    import torch
    from ctdm_gb300 import phantom
    acq = phantom.acquisition(64, 64, 8, seed=5, pixel=0.4e-6, carrier=XCARRIER)
    iters = 4
    p = C.params_for(acq, iters, qpi_method=C.CTDM_QPI_B)
    out = torch.zeros((acq.r_vol,) * 3, dtype=torch.complex64, device=dev)
    ctx.reconstruct_device(p, T(acq.holograms, dev), T(acq.background, dev), acq.ang_x, acq.ang_y, out)
    torch.cuda.synchronize()
    par = oracle.make_params(acq.n_holo, acq.m_crop, acq.r_vol, iters, acq.fm0, acq.df, acq.dx, acq.k2, acq.n_med,
                             qpi_method=0)
    ref, car = oracle.pipeline(par, acq.holograms, acq.background, acq.ang_x, acq.ang_y)
    assert ctx.carrier()[:2] == car[:2]
    assert rmse(out.cpu().numpy(), ref) < RI_TOL


def test_extract_qpi_algorithm_b_drop_in(ctx, dev, oracle):
    """The reference-named symbol: host holograms in, device fields out; frame 1 sets
    the carrier columns that frame 2 reuses."""
    import ctdm_gb300 as C
    import torch
    from ctdm_gb300 import phantom
    n = 256
    acq = phantom.acquisition(n, n, 2, seed=3, pixel=0.1e-6, carrier=XCARRIER)
    L = C.load()
    m = n // 4
    sp_f = torch.zeros((m, m), dtype=torch.complex64, device=dev)
    bg_f = torch.zeros_like(sp_f)
    cb, cs = oracle.qpib_center(acq.background), oracle.qpib_center(acq.holograms[0])
    for frame in (1, 2):
        sp = np.ascontiguousarray(acq.holograms[frame - 1], np.float32)
        bg = np.ascontiguousarray(acq.background, np.float32)
        L.extractQPI_AlgorithmB(sp.ctypes.data, bg.ctypes.data, sp_f.data_ptr(), bg_f.data_ptr(), n, n, frame)
        assert L.ctdm_last_error() == b""
        osp = oracle.qpib_field(sp, cs if frame == 1 else cb)
        obg = oracle.qpib_field(bg, cb)
        scale = np.abs(obg).max()
        assert rmse(sp_f.cpu().numpy(), osp) / scale < 1e-5
        assert rmse(bg_f.cpu().numpy(), obg) / scale < 1e-5
