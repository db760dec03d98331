"""Goldstein on the GPU against the oracle: residue charges and branch-cut masks
bit-exact, flood-filled phase within 1e-4 rad RMSE (the only float stage)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
PHASE_TOL = 1e-4


def T(a, dev):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


def noisy_phase(m, seed, noise, slope=0.6):
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:m, 0:m]
    true = slope * x + 0.25 * slope * y + 3 * np.sin(x / 9.0) + rng.standard_normal((m, m)) * noise
    return np.angle(np.exp(1j * true)).astype(np.float32)


def run_gpu(ctx, dev, maps):
    import torch
    A, h, w = maps.shape
    q = torch.zeros((A, h, w), dtype=torch.int8, device=dev)
    c = torch.zeros((A, h, w), dtype=torch.uint8, device=dev)
    o = torch.zeros((A, h, w), dtype=torch.float32, device=dev)
    st = ctx.goldstein(T(maps, dev), q, c, o, A, w, h)
    torch.cuda.synchronize()
    return q.cpu().numpy(), c.cpu().numpy(), o.cpu().numpy(), st


@pytest.mark.parametrize("m,noise", [(64, 0.9), (128, 0.6), (256, 0.3), (256, 1.2)])
def test_goldstein_bit_exact(ctx, dev, oracle, m, noise):
    maps = np.stack([noisy_phase(m, s, noise) for s in range(3)])
    q, c, o, st = run_gpu(ctx, dev, maps)
    for a in range(len(maps)):
        oq = oracle.goldstein_residues(maps[a])
        assert np.array_equal(q[a], oq)
        oc = oracle.goldstein_cuts(oq)
        assert np.array_equal(c[a], oc), np.argwhere(c[a] != oc)[:5]
        oo, ub, ost = oracle.goldstein_floodfill(oc, maps[a])
        assert st[a] == ost
        assert np.sqrt(np.mean((o[a] - oo) ** 2)) < PHASE_TOL
    if noise >= 0.6:
        assert np.count_nonzero(q) > 10   # the case exercises the branch cuts


@pytest.mark.parametrize("m,x1,x2", [(64, 32, 40), (96, 48, 60)])
def test_goldstein_walk_start_on_cut(ctx, dev, oracle, m, x1, x2):
    """A residue at (W/2, 2) puts the start of the reference's diagonal seed walk on a
    cut; the seed stays at (2, W/2) (FloodFill, cTDM/Goldstein.cu:656-663)."""
    yy, xx = np.mgrid[0:m, 0:m].astype(np.float64)
    th = np.arctan2(yy - 2.5, xx - (x1 + 0.5)) - np.arctan2(yy - 2.5, xx - (x2 + 0.5))
    phi = np.angle(np.exp(1j * (th + 0.3 * xx + 0.1 * yy))).astype(np.float32)
    q, c, o, st = run_gpu(ctx, dev, phi[None])
    oq = oracle.goldstein_residues(phi)
    oc = oracle.goldstein_cuts(oq)
    assert oc[2, m // 2] == 1
    assert np.array_equal(q[0], oq) and np.array_equal(c[0], oc)
    oo, ub, ost = oracle.goldstein_floodfill(oc, phi)
    assert st[0] == ost == 0
    assert o[0, m // 2, 2] == phi[m // 2, 2]   # the seed keeps its wrapped value
    assert np.sqrt(np.mean((o[0] - oo) ** 2)) < PHASE_TOL


def test_goldstein_global_state_path(ctx, dev, oracle):
    m = 512   # above the shared-memory limit: state in global memory
    maps = noisy_phase(m, 7, 0.5)[None]
    q, c, o, st = run_gpu(ctx, dev, maps)
    oq = oracle.goldstein_residues(maps[0])
    oc = oracle.goldstein_cuts(oq)
    assert np.array_equal(q[0], oq) and np.array_equal(c[0], oc)
    oo, ub, ost = oracle.goldstein_floodfill(oc, maps[0])
    assert st[0] == ost and np.sqrt(np.mean((o[0] - oo) ** 2)) < PHASE_TOL


@pytest.mark.parametrize("cap", [16, 200])
def test_goldstein_list_overflow_restart(ctx, dev, oracle, cap):
    """A fill whose list outgrows the shared-memory capacity starts over on the global
    lists: the same result, bit for bit, as with room to spare."""
    import ctdm_gb300 as C
    maps = np.stack([noisy_phase(256, s, 0.6) for s in range(2)])
    ref = run_gpu(ctx, dev, maps)
    try:
        C.set_fill_list_capacity(cap)
        got = run_gpu(ctx, dev, maps)
    finally:
        C.set_fill_list_capacity(0)
    assert np.array_equal(got[2], ref[2]) and np.array_equal(got[3], ref[3])
    oo, _, ost = oracle.goldstein_floodfill(oracle.goldstein_cuts(oracle.goldstein_residues(maps[0])), maps[0])
    assert ref[3][0] == ost and np.sqrt(np.mean((ref[2][0] - oo) ** 2)) < PHASE_TOL
    with pytest.raises(Exception):
        C.set_fill_list_capacity(8)
    with pytest.raises(Exception):
        C.set_fill_list_capacity(4096)


def test_goldstein_enclosed_regions(ctx, dev, oracle):
    """Planted cut pixels enclose regions the fill cannot reach; status, reached set
    and values still match the serial specification."""
    import torch
    m = 64
    rng = np.random.default_rng(1)
    for trial in range(3):
        phi = noisy_phase(m, 3 + trial, 0.4)
        q = oracle.goldstein_residues(phi)
        cuts = (oracle.goldstein_cuts(q) | (rng.random((m, m)) < 0.12)).astype(np.uint8)
        out = torch.zeros((m, m), dtype=torch.float32, device=dev)
        st = ctx.goldstein_fill(T(cuts, dev), T(phi, dev), out, 1, m, m)
        torch.cuda.synchronize()
        oo, ub, ost = oracle.goldstein_floodfill(cuts, phi)
        assert st[0] == ost
        assert ub.sum() < m * m
        assert np.sqrt(np.mean((out.cpu().numpy() - oo) ** 2)) < PHASE_TOL


def test_goldstein_smooth_no_residues(ctx, dev, oracle):
    m = 128
    y, x = np.mgrid[0:m, 0:m]
    true = 0.4 * x + 0.3 * y + 5 * np.sin(x / 17.0) * np.cos(y / 23.0)
    phi = np.angle(np.exp(1j * true)).astype(np.float32)
    q, c, o, st = run_gpu(ctx, dev, phi[None])
    assert not q.any() and not c.any() and st[0] == 0
    d = o[0] - true
    assert np.abs(d - d[2, m // 2]).max() < 1e-3   # unwrapped up to a constant


def test_goldstein_drop_in(ctx, dev, oracle):
    import ctdm_gb300 as C
    import torch
    m = 128
    phi = noisy_phase(m, 11, 0.7)
    src = T(phi, dev)
    dst = torch.zeros((m, m), dtype=torch.float32, device=dev)
    C.load().cudaGoldsteinUnwrap2D(src.data_ptr(), dst.data_ptr(), m, m, 1)
    torch.cuda.synchronize()
    oq = oracle.goldstein_residues(phi)
    oo, ub, st = oracle.goldstein_floodfill(oracle.goldstein_cuts(oq), phi)
    assert np.sqrt(np.mean((dst.cpu().numpy() - oo) ** 2)) < PHASE_TOL


def test_pipeline_with_goldstein(ctx, dev, oracle):
    """Wrap-heavy-shaped small case: the pipeline runs Goldstein on every angle's
    wrapped phase; charges and cuts are bit-exact to the oracle on that phase."""
    import ctdm_gb300 as C
    import torch
    from ctdm_gb300 import phantom
    acq = phantom.acquisition(256, 64, 4, seed=21, pixel=0.1e-6, n_cell=1.40, n_nuc=1.40,
                              semi=(7e-6, 5e-6, 5e-6))
    p = C.params_for(acq, 2, run_goldstein=1)
    out = torch.zeros((64,) * 3, dtype=torch.complex64, device=dev)
    ctx.reconstruct_device(p, T(acq.holograms, dev), T(acq.background, dev), acq.ang_x, acq.ang_y, out)
    torch.cuda.synchronize()
    A, m = 4, acq.m_crop
    phase = ctx.read_buffer(0, np.float32).reshape(A, m, m)
    charges = ctx.read_buffer(3, np.int8).reshape(A, m, m)
    cuts = ctx.read_buffer(4, np.uint8).reshape(A, m, m)
    gold = ctx.read_buffer(5, np.float32).reshape(A, m, m)
    for a in range(A):
        oq = oracle.goldstein_residues(phase[a])
        assert np.array_equal(charges[a], oq)
        oc = oracle.goldstein_cuts(oq)
        assert np.array_equal(cuts[a], oc)
        oo, ub, st = oracle.goldstein_floodfill(oc, phase[a])
        assert np.sqrt(np.mean((gold[a] - oo) ** 2)) < PHASE_TOL


def test_goldstein_deterministic(ctx, dev):
    """Repeated runs give identical bits (no ordering races in the parallel fill)."""
    maps = np.stack([noisy_phase(256, s, 1.2) for s in range(4)])
    first = run_gpu(ctx, dev, maps)
    for _ in range(3):
        again = run_gpu(ctx, dev, maps)
        for x, y in zip(first[:3], again[:3]):
            assert np.array_equal(x, y)
