"""The allocation-free DCT unwrap entry point (ctdm_unwrap_dct_noalloc).

It exists for callers that cannot allocate device memory -- an acquisition loop
that must not allocate once it runs, or a host that hands out all GPU memory from
its own pool -- and keeps its scratch in file-scope device arrays.  It must return
what ctdm_unwrap_dct returns for the same maps, call after call, for every map side
and both unwrap modes, up to exactly its fixed capacity, and refuse anything beyond
it.  This file is collected last on purpose."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
PHASE_TOL = 1e-4
CAPACITY = 4194304          # points of the fixed scratch


def wrapped_maps(a, m, seed):
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:m, 0:m] / m
    maps = []
    for k in range(a):
        true = (6 + 3 * k) * np.sin(2.1 * x + 0.3 * k) * np.cos(1.7 * y) + 5 * x * y + 0.05 * rng.standard_normal((m, m))
        maps.append(np.angle(np.exp(1j * true)))
    return np.ascontiguousarray(np.stack(maps), dtype=np.float32)


def both_entry_points(ctx, dev, a, m, mode, seed):
    import torch
    import ctdm_gb300 as C
    lib = C.load()
    phi = torch.from_numpy(wrapped_maps(a, m, seed)).to(dev)
    ref = torch.zeros_like(phi)
    ctx.unwrap_dct(phi, ref, a, m, mode=mode)
    out = torch.full_like(phi, float("nan"))
    rc = lib.ctdm_unwrap_dct_noalloc(a, m, mode, phi.data_ptr(), out.data_ptr(), None)
    assert rc == 0, C._lib.last_error()
    torch.cuda.synchronize()
    return phi.cpu().numpy(), ref.cpu().numpy(), out.cpu().numpy()


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("m,a", [(16, 7), (32, 6), (64, 5), (128, 4), (256, 3)])
def test_noalloc_matches_allocating_entry_point(ctx, dev, m, a, mode):
    for call, seed in enumerate((1, 2)):            # two calls in a row
        _, r, o = both_entry_points(ctx, dev, a, m, mode, seed + 10 * mode)
        assert np.isfinite(o).all()
        assert np.sqrt(np.mean((o - r) ** 2)) < PHASE_TOL, call
        assert np.abs(o - r).max() < 1e-5


def test_noalloc_matches_oracle(ctx, dev, oracle):
    """The same maps against the FP64 oracle's DCT unwrap, both modes."""
    for mode in (0, 1):
        phi, _, o = both_entry_points(ctx, dev, 2, 128, mode, 5)
        for k in range(2):
            want = oracle.dct_unwrap(phi[k], mode)
            assert np.sqrt(np.mean((o[k] - want) ** 2)) < PHASE_TOL, mode


def test_noalloc_at_exact_capacity(ctx, dev):
    """64 maps of 256 x 256 fill the scratch exactly: accepted, and equal to the
    allocating entry point."""
    a, m = CAPACITY // (256 * 256), 256
    assert a * m * m == CAPACITY
    _, r, o = both_entry_points(ctx, dev, a, m, 0, 3)
    assert np.sqrt(np.mean((o - r) ** 2)) < PHASE_TOL
    assert np.abs(o - r).max() < 1e-5


def test_noalloc_rejects_sizes_beyond_its_scratch(ctx, dev):
    import torch
    import ctdm_gb300 as C
    lib = C.load()
    phi = torch.zeros((2, 512, 512), dtype=torch.float32, device=dev)
    out = torch.zeros_like(phi)
    assert lib.ctdm_unwrap_dct_noalloc(2, 512, 0, phi.data_ptr(), out.data_ptr(), None) == 1
    assert "not in" in C._lib.last_error()
    big = torch.zeros((65, 256, 256), dtype=torch.float32, device=dev)
    assert lib.ctdm_unwrap_dct_noalloc(65, 256, 0, big.data_ptr(), big.data_ptr(), None) == 1
    assert "scratch" in C._lib.last_error()
    assert lib.ctdm_unwrap_dct_noalloc(1, 64, 2, phi.data_ptr(), out.data_ptr(), None) == 1
    assert "mode" in C._lib.last_error()
    # the allocating entry point refuses an unknown mode the same way
    with pytest.raises(C.CtdmError):
        ctx.unwrap_dct(phi, out, 1, 64, mode=2)
