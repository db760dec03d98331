"""The oracle against the reference's own host functions, compiled from its sources.

oracle/refcpu/assemble.py cuts FloodFill and sumAdjoin (cTDM/Goldstein.cu:643-1105),
bilinear (cTDM/HilbertTransform.cu:2404-2435) and FFT, Powerof2, FFT2D, FFT3D and
FFT3Dshift (cTDM/FFT.cu:29-543) into oracle/_ref/refcpu/src (build() does it where the
reference checkout is present); oracle/refcpu/Makefile compiles them with g++ and
oracle/refcpu/driver.cpp into oracle/_ref/refcpu/ref_cpu.  The tests run that binary
in a child process with a time limit: FloodFill spins forever on maps whose sweeps
stall.  Skipped where the assembled sources are absent.

Bars: the flood fill and the resize bit-exact (the oracle evaluates the same float
expressions); the transforms within float rounding (the reference stores float between
the axes, the oracle keeps FP64 throughout); the octant swap exact.
"""
import os
import subprocess
import tempfile

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
REFCPU = os.path.join(os.path.dirname(HERE), "oracle", "refcpu")
SRC = os.path.join(os.path.dirname(HERE), "oracle", "_ref", "refcpu", "src", "ref_cpu.cpp")
EXE = os.path.join(os.path.dirname(HERE), "oracle", "_ref", "refcpu", "ref_cpu")


@pytest.fixture(scope="module")
def ref_cpu():
    if not os.path.exists(SRC):
        pytest.skip("oracle/_ref/refcpu/src is missing: the reference checkout was not present at build time")
    subprocess.check_call(["make", "-s", "-C", REFCPU], timeout=300)
    return EXE


def run(exe, op, header, payload, dtype, count, timeout=120):
    with tempfile.TemporaryDirectory() as d:
        fi, fo = os.path.join(d, "in"), os.path.join(d, "out")
        with open(fi, "wb") as f:
            np.asarray(header, np.int32).tofile(f)
            for a in payload:
                np.ascontiguousarray(a).tofile(f)
        r = subprocess.run([exe, op, fi, fo], timeout=timeout, capture_output=True)
        assert r.returncode == 0, (op, r.returncode, r.stderr[-400:])
        return np.fromfile(fo, dtype, count)


def noisy_phase(m, seed, noise, slope=0.6):
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:m, 0:m]
    true = slope * x + 0.25 * slope * y + 3 * np.sin(x / 9.0) + rng.standard_normal((m, m)) * noise
    return np.angle(np.exp(1j * true)).astype(np.float32)


def dipole_phase(m, x1, x2, y):
    """Two opposite vortices at (x1 + 0.5, y + 0.5) and (x2 + 0.5, y + 0.5) over a tilt:
    residues at (x1, y) and (x2, y), each cut to the nearer border when y is small."""
    yy, xx = np.mgrid[0:m, 0:m].astype(np.float64)
    th = np.arctan2(yy - (y + 0.5), xx - (x1 + 0.5)) - np.arctan2(yy - (y + 0.5), xx - (x2 + 0.5))
    return np.angle(np.exp(1j * (th + 0.3 * xx + 0.1 * yy))).astype(np.float32)


def ref_floodfill(exe, cut, phi):
    h, w = phi.shape
    out = run(exe, "floodfill", [w, h], [cut.astype(np.float32), phi.astype(np.float32)], np.float32, w * h)
    return out.reshape(h, w)


MAPS = [("noisy", 64, 0.9, 0), ("noisy", 64, 0.9, 1), ("noisy", 128, 0.6, 0), ("noisy", 128, 0.6, 2),
        ("noisy", 256, 0.3, 0), ("noisy", 256, 1.2, 0), ("noisy", 256, 1.2, 1), ("noisy", 64, 0.0, 0),
        ("dipole", 64, 32, 40), ("dipole", 96, 48, 60)]


@pytest.mark.parametrize("kind,m,a,b", MAPS)
def test_floodfill_matches_reference(ref_cpu, oracle, kind, m, a, b):
    phi = noisy_phase(m, b, a) if kind == "noisy" else dipole_phase(m, a, b, 2)
    cut = oracle.goldstein_cuts(oracle.goldstein_residues(phi))
    out, ub, st = oracle.goldstein_floodfill(cut, phi)
    assert st == 0
    ref = ref_floodfill(ref_cpu, cut, phi)
    assert np.array_equal(ref, out), int((ref != out).sum())


def test_floodfill_walk_start_on_cut_is_covered(oracle):
    """The reference fixes the seed at (row 2, column W/2) before its diagonal walk off
    the cuts, so the walk changes nothing: the maps above include walk starts
    (x = W/2, y = 2) on a cut, where a walked seed would differ."""
    hits = 0
    for kind, m, a, b in MAPS:
        phi = noisy_phase(m, b, a) if kind == "noisy" else dipole_phase(m, a, b, 2)
        cut = oracle.goldstein_cuts(oracle.goldstein_residues(phi))
        hits += int(cut[2, m // 2] == 1)
    assert hits >= 2


@pytest.mark.parametrize("n1,m1,n2,m2", [(64, 64, 256, 256), (100, 80, 37, 53), (1024, 1024, 256, 256)])
def test_bilinear_matches_reference(ref_cpu, oracle, n1, m1, n2, m2):
    img = np.random.default_rng(n1 + m2).standard_normal((n1, m1)).astype(np.float32)
    ref = run(ref_cpu, "bilinear", [m1, n1, m2, n2], [img], np.float32, n2 * m2).reshape(n2, m2)
    assert np.array_equal(ref, oracle.bilinear(img, m2, n2))


def cnoise(shape, seed):
    rng = np.random.default_rng(seed)
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)


@pytest.mark.parametrize("nx,ny", [(8, 8), (64, 32), (256, 256)])
@pytest.mark.parametrize("d", [1, -1])
def test_fft2d_matches_reference(ref_cpu, oracle, nx, ny, d):
    """The host FFT2D: dir 1 is the forward transform scaled by 1 / (nx ny), dir -1 the
    unscaled inverse (the opposite of cuFFT3D's dir, which the GPU path follows)."""
    c = cnoise((nx, ny), nx * ny)
    ref = run(ref_cpu, "fft2d", [nx, ny, d], [c], np.complex64, c.size).reshape(c.shape)
    o = oracle.fft2(c, sign=-1 if d == 1 else 1)
    if d == 1:
        o = o / c.size
    assert np.abs(ref - o).max() <= 2e-7 * np.abs(o).max()


@pytest.mark.parametrize("nx,ny,nz", [(8, 8, 8), (32, 16, 8), (64, 64, 64)])
@pytest.mark.parametrize("d", [1, -1])
def test_fft3d_matches_reference(ref_cpu, oracle, nx, ny, nz, d):
    c = cnoise((nz, nx, ny), nx + ny + nz)
    ref = run(ref_cpu, "fft3d", [nx, ny, nz, d], [c], np.complex64, c.size).reshape(c.shape)
    o = oracle.fft3(c, -1 if d == 1 else 1)
    o = o / c.size if d == 1 else o * c.size
    assert np.abs(ref - o).max() <= 2e-7 * np.abs(o).max()


@pytest.mark.parametrize("w,h,s", [(8, 8, 8), (16, 8, 4), (64, 64, 64)])
def test_octant_shift_matches_reference(ref_cpu, oracle, w, h, s):
    c = cnoise((s, h, w), w * h * s)
    ref = run(ref_cpu, "shift3d", [w, h, s], [c], np.complex64, c.size).reshape(c.shape)
    assert np.array_equal(ref, oracle.shift3d(c).astype(np.complex64))
