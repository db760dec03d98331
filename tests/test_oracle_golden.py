"""Pins the FP64 oracle: the reference's own DCT-unwrap dumps (tests/golden) and
closed-form known answers for the stages that have no reference vectors."""
import json
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def gold(name):
    return np.load(os.path.join(GOLD, f"dct_chain_{name}.npy")).astype(np.float64)


def test_golden_manifest():
    man = json.load(open(os.path.join(GOLD, "dct_chain_manifest.json")))
    assert set(man) == {"src", "Laplace", "DCT", "DCT2", "IDCT"}
    for name in man:
        assert gold(name).shape == (256, 256)


def test_laplacian_matches_reference_dump(oracle):
    # NumericDerivative1 + SumDerivative on the reference input (cTDM/DCT_Unwrapping.cu:336-417)
    lap = oracle.wrapped_laplacian(gold("src"))
    assert np.abs(lap - gold("Laplace")).max() < 2e-5


def test_dct_matches_reference_dump(oracle):
    d = oracle.dct2d(gold("Laplace"))
    assert np.abs(d - gold("DCT")).max() < 1e-5


def test_poisson_divide_matches_reference_dump(oracle):
    d2 = oracle.poisson_divide(gold("DCT"))
    ref = gold("DCT2")
    rel = np.abs(d2 - ref) / np.maximum(np.abs(ref), 1e-30)
    # the reference evaluates 2cos+2cos-4 in float: relative error up to ~2e-4 at low (i, j)
    assert np.median(rel) < 1e-6 and rel.max() < 5e-4


def test_idct_reference_twiddle_matches_reference_dump(oracle):
    out = oracle.idct2d(gold("DCT2"), mode=0)
    assert np.abs(out - gold("IDCT")).max() < 2e-6


def test_idct_exact_differs_like_survey(oracle):
    exact = oracle.idct2d(gold("DCT2"), mode=1)
    rmse = np.sqrt(np.mean((exact - gold("IDCT")) ** 2))
    assert 5e-4 < rmse < 2e-3   # the reference twiddle quirk: RMSE ~8.6e-4 rad


def test_full_chain_end_to_end(oracle):
    out = oracle.dct_unwrap(gold("src"), mode=0)
    ref = gold("IDCT")
    # float cancellation in the reference's Poisson denominator dominates
    assert np.sqrt(np.mean((out - ref) ** 2)) < 1e-3
    # the unwrapped phase stays congruent to the wrapped input mod 2 pi up to the LS residual
    k = np.round((out - gold("src")) / (2 * np.pi))
    assert np.std(out - gold("src") - 2 * np.pi * k) < 0.05


def test_dct_matches_textbook(oracle):
    sf = pytest.importorskip("scipy.fft")
    rng = np.random.default_rng(0)
    a = rng.standard_normal((32, 32))
    assert np.allclose(oracle.dct2d(a), sf.dctn(a, norm="ortho"), atol=1e-12)
    assert np.allclose(oracle.idct2d(sf.dctn(a, norm="ortho"), mode=1), a, atol=1e-12)


@pytest.mark.parametrize("n", [16, 48, 64, 96, 384])
def test_fft_known_answers(oracle, n):
    rng = np.random.default_rng(n)
    a = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    assert np.allclose(oracle.fft2(a, -1), np.fft.fft2(a), atol=1e-9 * n * n)
    assert np.allclose(oracle.fft2(a, +1), np.fft.ifft2(a) * n * n, atol=1e-9 * n * n)
    imp = np.zeros((n, n), complex)
    imp[0, 0] = 1
    assert np.allclose(oracle.fft2(imp, -1), 1.0)


def test_fft3_roundtrip(oracle):
    rng = np.random.default_rng(3)
    a = rng.standard_normal((24, 24, 24)) + 1j * rng.standard_normal((24, 24, 24))
    f = oracle.fft3(a, -1)
    assert np.allclose(f, np.fft.fftn(a), atol=1e-8)
    assert np.allclose(oracle.fft3(f, +1), a, atol=1e-12)


def test_residue_known_answer(oracle):
    # a single phase vortex at (20.5, 12.5): one residue at the loop (20, 12).  The
    # reference sums (phi_here - phi_next) around (r,c)->(r+1,c)->(r+1,c+1)->(r,c+1),
    # so a vortex whose phase grows with atan2(y, x) has charge -1.
    w = h = 40
    y, x = np.mgrid[0:h, 0:w]
    phi = np.angle(np.exp(1j * np.arctan2(y - 12.5, x - 20.5))).astype(np.float32)
    q = oracle.goldstein_residues(phi)
    assert q[12, 20] == -1 and np.count_nonzero(q) == 1
    q2 = oracle.goldstein_residues(-phi)
    assert q2[12, 20] == 1 and np.count_nonzero(q2) == 1


def test_branch_cut_pairs_dipole(oracle):
    w = h = 40
    y, x = np.mgrid[0:h, 0:w]
    phi = np.arctan2(y - 20.5, x - 15.5) - np.arctan2(y - 20.5, x - 22.5)
    phi = np.angle(np.exp(1j * phi)).astype(np.float32)
    q = oracle.goldstein_residues(phi)
    assert np.count_nonzero(q) == 2
    cuts = oracle.goldstein_cuts(q)
    # the two residues are joined by a horizontal cut along row 20
    assert cuts[20, 15:23].all()
    out, ub, st = oracle.goldstein_floodfill(cuts, phi)
    assert st == 0 and ub.sum() == w * h


def test_floodfill_smooth_phase(oracle):
    w = h = 32
    y, x = np.mgrid[0:h, 0:w]
    true = 0.35 * x + 0.2 * y
    phi = np.angle(np.exp(1j * true)).astype(np.float32)
    q = oracle.goldstein_residues(phi)
    assert not q.any()
    out, ub, st = oracle.goldstein_floodfill(np.zeros((h, w), np.uint8), phi)
    assert st == 0
    d = out - true
    assert np.abs(d - d[0, 0]).max() < 1e-4


def test_ewald_index_normal_incidence(oracle):
    r = 32
    fm0 = 1.337 / 532e-9
    df = 1.0 / (r * 0.4e-6)
    vox, fz = oracle.ewald_index(r, fm0, df, 0.0, 0.0)
    # DC bin maps to voxel 0 with fz = fm0
    assert vox[0] == 0 and abs(fz[0] - fm0) < 1e-6 * fm0
    # every sample of an axial illumination lies on the cap below kz = 0
    nz = vox[vox >= 0] // (r * r)
    assert ((nz == 0) | (nz > r // 2)).all()


def test_positivity_clamps(oracle):
    r = 16
    F2 = np.zeros((r, r, r), complex)
    n = oracle.positivity(F2, np.zeros((r, r, r), np.uint32), 2, 1e14, 1.33)
    assert np.allclose(n.real, 1.33) and np.allclose(n.imag, 0)
