"""GPU checks of the differentiable form (ctdm_tape, ctdm_forward/ctdm_backward,
ctdm_loss_grad, ctdm_reconstruct_gradient, ctdm_contrast_to_ri) through the C ABI
against the FP64 oracle (oracle/adjoint.py), finite differences and the
positivity path.

Tolerances (float32 transforms vs FP64): forward / backward / gradient relative
L2 error <= 1e-5; loss relative error <= 1e-5; central differences of the GPU loss
(h = 1e-3, 64 voxels, real and imaginary perturbations) within 5e-3 of the
largest gradient component; RI RMSE <= 1e-5."""
import numpy as np
import pytest

import adjoint as AD

pytestmark = pytest.mark.gpu

REL = 1e-5


def T(a, dev):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


def rel(a, b):
    a = np.asarray(a, np.complex128).ravel()
    b = np.asarray(b, np.complex128).ravel()
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _random_tape(ctx, dev, r, frac=0.3, seed=0, with_counts=True, k2=4.0, scale=1.0):
    import ctdm_gb300 as C
    rng = np.random.default_rng(seed)
    F2 = (rng.standard_normal((r, r, r)) + 1j * rng.standard_normal((r, r, r))).astype(np.complex64)
    hit = rng.random((r, r, r)) < frac
    F2[~hit] = 0
    counts = (hit * rng.integers(1, 4, (r, r, r))).astype(np.int32)
    F2 *= np.float32(-k2 * r ** 1.5 * scale)   # data y of the given scale
    tape = C.Tape(T(F2, dev), r, k2, T(counts, dev) if with_counts else None)
    return tape, F2, counts, rng


@pytest.mark.parametrize("with_counts", [True, False])
def test_tape_indices_and_data(ctx, dev, with_counts):
    r, k2 = 32, 4.0
    tape, F2, counts, _ = _random_tape(ctx, dev, r, with_counts=with_counts, k2=k2)
    y, idx = tape.data()
    ref_idx = AD.measured_indices(F2, counts if with_counts else None)
    assert np.array_equal(idx, ref_idx)
    np.testing.assert_allclose(y, AD.tape_data(F2, ref_idx, r, k2), rtol=1e-6)
    tape.close()


@pytest.mark.parametrize("r", [32, 64, 128])
def test_forward_backward_match_fp64(ctx, dev, r):
    import torch
    tape, _, _, rng = _random_tape(ctx, dev, r, seed=r)
    _, idx = tape.data()
    V = (rng.standard_normal((r, r, r)) + 1j * rng.standard_normal((r, r, r))).astype(np.complex64)
    g = (rng.standard_normal(idx.size) + 1j * rng.standard_normal(idx.size)).astype(np.complex64)
    y = torch.zeros(idx.size, dtype=torch.complex64, device=dev)
    gV = torch.zeros((r, r, r), dtype=torch.complex64, device=dev)
    tape.forward(T(V, dev), y)
    tape.backward(T(g, dev), gV)
    torch.cuda.synchronize()
    yh, gVh = y.cpu().numpy(), gV.cpu().numpy()
    assert rel(yh, AD.forward(V, idx)) < REL
    assert rel(gVh, AD.adjoint(g, idx, r)) < REL
    # adjoint identity <A V, g> = <V, A^H g> on the GPU results themselves
    lhs = np.vdot(g.astype(np.complex128), yh.astype(np.complex128))
    rhs = np.vdot(gVh.astype(np.complex128), V.astype(np.complex128))
    assert abs(lhs - rhs) <= 1e-5 * np.linalg.norm(g) * np.linalg.norm(V)
    tape.close()


def test_adjoint_identity_512(ctx, dev):
    """Size-independent property at the full 512^3 volume (transform recomputed in
    the backward): <A V, g> = <V, A^H g> and A A^H = I on the samples."""
    import torch
    r = 512
    gen = torch.Generator(device=dev).manual_seed(3)
    F2 = torch.zeros((r, r, r), dtype=torch.complex64, device=dev)
    hit = torch.rand((r, r, r), generator=gen, device=dev) < 0.02
    F2[hit] = torch.complex(torch.ones((), device=dev), torch.ones((), device=dev))
    import ctdm_gb300 as C
    tape = C.Tape(F2, r, 1.0)
    S = tape.samples
    assert S == int(hit.sum().item())
    del F2, hit
    V = torch.randn((r, r, r), dtype=torch.complex64, device=dev, generator=gen)
    g = torch.randn(S, dtype=torch.complex64, device=dev, generator=gen)
    y = torch.empty(S, dtype=torch.complex64, device=dev)
    gV = torch.empty((r, r, r), dtype=torch.complex64, device=dev)
    tape.forward(V, y)
    tape.backward(g, gV)
    y2 = torch.empty(S, dtype=torch.complex64, device=dev)
    tape.forward(gV, y2)
    torch.cuda.synchronize()
    lhs = torch.vdot(g.to(torch.complex128), y.to(torch.complex128)).item()
    rhs = torch.vdot(gV.to(torch.complex128).ravel(), V.to(torch.complex128).ravel()).item()
    scale = (torch.linalg.vector_norm(g) * torch.linalg.vector_norm(V)).item()
    assert abs(lhs - rhs) <= 1e-5 * scale
    assert (torch.linalg.vector_norm(y2 - g) / torch.linalg.vector_norm(g)).item() < 1e-5
    tape.close()


@pytest.mark.parametrize("lam", [0.0, 0.05])
def test_loss_grad_matches_fp64(ctx, dev, lam):
    import torch
    r, eps = 32, 1e-2
    tape, _, _, rng = _random_tape(ctx, dev, r, seed=7)
    y, idx = tape.data()
    V = (0.1 * (rng.standard_normal((r, r, r)) + 1j * rng.standard_normal((r, r, r)))).astype(np.complex64)
    grad = torch.zeros((r, r, r), dtype=torch.complex64, device=dev)
    L = tape.loss_grad(T(V, dev), grad, lam, eps)
    Lr, gr = AD.loss_grad(V, idx, y.astype(np.complex128), lam, eps)
    assert abs(L - Lr) <= REL * Lr
    assert rel(grad.cpu().numpy(), gr) < REL
    tape.close()


@pytest.mark.parametrize("lam", [0.0, 0.05])
def test_gradient_finite_differences(ctx, dev, lam):
    """Central differences of the GPU loss itself, h = 1e-3, on 64 voxels, against
    the GPU gradient (real part <- Re perturbation, imaginary <- Im perturbation).
    Contrast and data of physical scale (~0.02) keep the float32 loss noise / 2h
    small against the gradient."""
    import torch
    r, eps, h = 32, 1e-2, 1e-3
    tape, F2, _, rng = _random_tape(ctx, dev, r, seed=11, scale=0.02)
    V = (0.02 * (rng.standard_normal((r, r, r)) + 1j * rng.standard_normal((r, r, r)))).astype(np.complex64)
    grad = torch.zeros((r, r, r), dtype=torch.complex64, device=dev)
    Vd = T(V, dev)
    tape.loss_grad(Vd, grad, lam, eps)
    g = grad.cpu().numpy().ravel()
    picks = rng.choice(r ** 3, 64, replace=False)
    err = []
    for p in picks:
        z, yy, x = np.unravel_index(p, (r, r, r))
        for unit, comp in ((1.0, g[p].real), (1j, g[p].imag)):
            base = Vd[z, yy, x].item()
            Vd[z, yy, x] = base + h * unit
            Lp = tape.loss_grad(Vd, grad, lam, eps)
            Vd[z, yy, x] = base - h * unit
            Lm = tape.loss_grad(Vd, grad, lam, eps)
            Vd[z, yy, x] = base
            err.append((Lp - Lm) / (2 * h) - comp)
    err = np.abs(np.array(err))
    assert err.max() <= 5e-3 * np.abs(g).max()
    tape.close()


def test_fista_matches_fp64(ctx, dev):
    import torch
    r, lam, eps, iters = 32, 1e-3, 1e-2, 10
    tape, _, _, rng = _random_tape(ctx, dev, r, seed=5)
    y, idx = tape.data()
    V0 = np.zeros((r, r, r), np.complex64)
    V = T(V0, dev)
    hist = tape.reconstruct(V, iters, lam, eps, record_loss=True)
    torch.cuda.synchronize()
    Vr, hr = AD.fista(V0, idx, y.astype(np.complex128), iters, lam, eps)
    assert rel(V.cpu().numpy(), Vr) < 1e-4
    np.testing.assert_allclose(hist, hr, rtol=1e-4)
    assert hist[-1] < 0.2 * hist[0]
    tape.close()


def test_projected_fista_matches_fp64(ctx, dev):
    """FISTA with the positivity constraint as a proximal step, against FP64."""
    import torch
    r, iters = 32, 8
    tape, _, _, rng = _random_tape(ctx, dev, r, seed=9)
    y, idx = tape.data()
    V0 = np.zeros((r, r, r), np.complex64)
    V = T(V0, dev)
    tape.reconstruct(V, iters, 0.0, 1e-2, step=1.0, positivity=True)
    torch.cuda.synchronize()
    Vr, _ = AD.fista(V0, idx, y.astype(np.complex128), iters, 0.0, 1e-2, step=1.0, positivity=True)
    assert rel(V.cpu().numpy(), Vr) < 1e-4
    s = np.sqrt(1.0 + V.cpu().numpy().astype(np.complex128))
    assert s.real.min() >= 1.0 - 1e-5 and s.imag.min() >= -1e-5    # every iterate is feasible
    tape.close()


def test_contrast_to_ri(ctx, dev):
    import torch
    import ctdm_gb300 as C
    r, nm = 32, 1.337
    rng = np.random.default_rng(9)
    V = (0.05 * rng.standard_normal((r, r, r)) + 0.01j * rng.standard_normal((r, r, r))).astype(np.complex64)
    V[0, 0, :4] = [-2.0, -2.0 - 0.0j, 0.0, -1.0]
    for clamp in (False, True):
        out = torch.zeros((r, r, r), dtype=torch.complex64, device=dev)
        C.contrast_to_ri(T(V, dev), r, nm, out, clamp=clamp)
        torch.cuda.synchronize()
        ref = AD.contrast_to_ri(V, nm, clamp)
        assert np.sqrt(np.mean(np.abs(out.cpu().numpy() - ref) ** 2)) < 1e-6


def test_gradient_recon_ties_to_positivity_path(ctx, dev, oracle):
    """One plain gradient step from V = 0 (lambda 0, step 1) is A^H y, the
    zero-filled inverse -- the RI the positivity path returns with no loop bodies.
    Then TV-regularised FISTA on the same phantom data lowers the objective."""
    import torch
    import ctdm_gb300 as C
    from ctdm_gb300 import phantom
    acq = phantom.small_case(seed=5, n=64, r=64, angles=8)
    r = acq.r_vol
    ph, am, _ = oracle.front_end(oracle.make_params(acq.n_holo, acq.m_crop, r, 0, acq.fm0, acq.df, acq.dx, acq.k2,
                                                    acq.n_med), acq.holograms, acq.background)
    U = np.stack([oracle.rytov_spectrum(ph[a], am[a]) for a in range(len(ph))])
    oF2, oC = oracle.ewald_map(U, acq.ang_x, acq.ang_y, acq.fm0, acq.df, acq.dx)
    ref = oracle.positivity(oF2, oC, 0, acq.k2, acq.n_med, 0)
    F2 = T(oF2.astype(np.complex64), dev)
    tape = C.Tape(F2, r, acq.k2, T(oC.astype(np.int32), dev))
    V = torch.zeros((r, r, r), dtype=torch.complex64, device=dev)
    tape.reconstruct(V, 1, 0.0, 1.0, step=1.0)
    n = torch.zeros_like(V)
    C.contrast_to_ri(V, r, acq.n_med, n, clamp=True)   # est_n clamps (cTDM/Recon_kernel.cu:est_n_3D)
    torch.cuda.synchronize()
    assert np.sqrt(np.mean(np.abs(n.cpu().numpy() - ref) ** 2)) < 1e-5
    V.zero_()
    hist = tape.reconstruct(V, 30, 1e-4, 1e-3, record_loss=True)
    assert np.all(np.isfinite(hist)) and hist[-1] < hist[0]
    tape.close()


def test_tape_rejects_bad_arguments(ctx, dev):
    import torch
    import ctdm_gb300 as C
    F2 = torch.zeros((32, 32, 32), dtype=torch.complex64, device=dev)
    with pytest.raises(RuntimeError, match="no measured voxels"):
        C.Tape(F2, 32, 1.0)
    with pytest.raises(RuntimeError, match="unsupported"):
        C.Tape(F2, 48, 1.0)


def test_gradient_checks_at_512_on_the_differentiable_configuration(ctx, dev):
    """The differentiable configuration's own checks at its size: 181 x 1024^2
    holograms on a cone at NA 1.2 reconstructed into 512^3; the measurement operator
    built from that tomogram's mapped data; V from 5 TV-regularised FISTA steps
    (lambda 1e-3).  At that V:
    * the GPU gradient of 1/2 ||A V - y||^2 + 1e-3 TV(V) equals the FP64 host gradient
      (relative L2 over the whole volume, and at 64 random voxels);
    * central differences of the GPU loss (h = 1e-3, real and imaginary parts) at the
      64 voxels agree with the GPU gradient within 5e-3 of its largest component."""
    import torch
    import ctdm_gb300 as C
    from ctdm_gb300 import phantom
    r, lam, eps, h = 512, 1e-3, 1e-3, 1e-3
    acq = phantom.acquisition(1024, r, 181, na=1.2, seed=4000)
    p = C.params_for(acq, 2)
    out = torch.empty((r, r, r), dtype=torch.complex64, device=dev)
    ctx.reconstruct_device(p, T(acq.holograms, dev), T(acq.background, dev), acq.ang_x, acq.ang_y, out)
    torch.cuda.synchronize()
    del out
    f2_ptr, _ = ctx.buffer(7)                     # the mapped data F2 of that call
    tape = C.Tape(f2_ptr, r, acq.k2)
    y, idx = tape.data()
    V = torch.zeros((r, r, r), dtype=torch.complex64, device=dev)
    tape.reconstruct(V, 5, lam, eps)
    grad = torch.zeros_like(V)
    tape.loss_grad(V, grad, lam, eps)
    torch.cuda.synchronize()
    g = grad.cpu().numpy()
    Vh = V.cpu().numpy()
    # FP64 host gradient at the same V
    Lr, gr = AD.loss_grad(Vh, idx, y.astype(np.complex128), lam, eps)
    assert rel(g, gr) < 1e-5
    rng = np.random.default_rng(512)
    picks = rng.choice(r ** 3, 64, replace=False)
    gflat, grflat = g.ravel(), gr.ravel()
    assert rel(gflat[picks], grflat[picks]) < 1e-4
    del gr, grflat
    # central differences of the GPU loss
    gmax = np.abs(gflat).max()
    err = []
    for pk in picks:
        z, yy, x = np.unravel_index(pk, (r, r, r))
        for unit, comp in ((1.0, gflat[pk].real), (1j, gflat[pk].imag)):
            base = V[z, yy, x].item()
            V[z, yy, x] = base + h * unit
            Lp = tape.loss_grad(V, grad, lam, eps)
            V[z, yy, x] = base - h * unit
            Lm = tape.loss_grad(V, grad, lam, eps)
            V[z, yy, x] = base
            err.append((Lp - Lm) / (2 * h) - comp)
    err = np.abs(np.array(err))
    print(f"512^3: {idx.size} samples, FD max error {err.max():.3e} of max |g| {gmax:.3e}")
    assert err.max() <= 5e-3 * gmax
    tape.close()


@pytest.mark.parametrize("r,iters", [(64, 6), (256, 4)])
def test_accelerated_loop_is_projected_fista(ctx, dev, r, iters):
    """The accelerated positivity loop (momentum fused into the loop passes; 256^3 runs
    the plane scheme, 64^3 the line passes) equals projected FISTA at lambda 0 and unit
    step with one more step (FP64 restatement, and the library's own gradient driver),
    RI RMSE <= 1e-5; and differs from the plain loop."""
    import torch
    import ctdm_gb300 as C
    k2 = float((2 * np.pi * 1.337 / 532e-9) ** 2)
    n_med = 1.337
    rng = np.random.default_rng(r + iters)
    keep = rng.random((r, r, r)) < 0.15
    amp = 1e-2 * k2 * np.sqrt(r ** 3 / 0.15)
    F2 = np.where(keep, (rng.standard_normal((r, r, r)) + 1j * rng.standard_normal((r, r, r))) * amp, 0)
    F2 = F2.astype(np.complex64)
    dF2 = T(F2, dev)
    out = torch.empty_like(dF2)
    ctx.positivity(dF2, r, iters, k2, n_med, out, accelerated=True)
    plain = torch.empty_like(dF2)
    ctx.positivity(dF2, r, iters, k2, n_med, plain)
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    idx = AD.measured_indices(F2)
    y = AD.tape_data(F2, idx, r, k2)
    V, _ = AD.fista(np.zeros((r, r, r), np.complex64), idx, y, iters + 1, 0.0, 1.0, step=1.0, positivity=True)
    ref = AD.contrast_to_ri(V, n_med, clamp=True)
    err = np.sqrt(np.mean(np.abs(got.astype(np.complex128) - ref) ** 2))
    assert err < 1e-5, err
    tape = C.Tape(dF2, r, k2)
    Vg = torch.zeros((r, r, r), dtype=torch.complex64, device=dev)
    tape.reconstruct(Vg, iters + 1, 0.0, 1.0, step=1.0, positivity=True)
    ng = torch.empty_like(Vg)
    C.contrast_to_ri(Vg, r, n_med, ng, clamp=True)
    torch.cuda.synchronize()
    assert np.sqrt(np.mean(np.abs(ng.cpu().numpy().astype(np.complex128) - ref) ** 2)) < 1e-5
    diff = np.sqrt(np.mean(np.abs(plain.cpu().numpy().astype(np.complex128) - ref) ** 2))
    assert diff > 10 * err        # momentum changes the iterates
    tape.close()


def test_accelerated_loop_at_512_across_schemes(ctx, dev):
    """At 512^3 the accelerated loop carries its momentum through the 16- or 8-CTA plane
    pass or through the x pass of the line scheme; every scheme gives the library's own
    projected FISTA (the gradient driver, an independent set of passes) to RI RMSE <= 1e-5."""
    import torch
    import ctdm_gb300 as C
    r, iters = 512, 3
    k2 = float((2 * np.pi * 1.337 / 532e-9) ** 2)
    n_med = 1.337
    rng = np.random.default_rng(512)
    keep = rng.random((r, r, r), dtype=np.float32) < 0.05
    amp = np.float32(1e-2 * k2 * np.sqrt(r ** 3 / 0.05))
    F2 = np.zeros((r, r, r), np.complex64)
    n = int(keep.sum())
    F2[keep] = (rng.standard_normal(n, dtype=np.float32) + 1j * rng.standard_normal(n, dtype=np.float32)) * amp
    dF2 = T(F2, dev)
    del F2, keep
    tape = C.Tape(dF2, r, k2)
    Vg = torch.zeros((r, r, r), dtype=torch.complex64, device=dev)
    tape.reconstruct(Vg, iters + 1, 0.0, 1.0, step=1.0, positivity=True)
    ref = torch.empty_like(Vg)
    C.contrast_to_ri(Vg, r, n_med, ref, clamp=True)
    tape.close()
    del Vg
    out = torch.empty_like(dF2)
    saved = C.loop_scheme(r)
    try:
        for scheme in (0, 1, 2):
            C.set_loop_scheme(r, scheme)
            ctx.positivity(dF2, r, iters, k2, n_med, out, accelerated=True)
            torch.cuda.synchronize()
            err = float(torch.sqrt(torch.mean(torch.abs(out - ref) ** 2)).item())
            assert err < 1e-5, (scheme, err)
            assert ctx.device_status() == 0
    finally:
        C.set_loop_scheme(r, saved)
