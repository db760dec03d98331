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

The same binary runs the reference's job-list and parameter-file reading
(scriptFileRead, obtainParameter; a stand-in HilbertTransform records each job), its
frame reader (bmp_header, read_bmp), its .phimap writer (outputImg) and its frame check
(checkArray), against this library's host functions through the C ABI: parsed fields,
stored bytes, written bytes and check results equal.
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


@pytest.fixture(scope="module")
def lib():
    from ctdm_gb300 import _lib
    return _lib.load()


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


# ---------------------------------------------------------------- job files and frame formats
def run_paths(exe, op, src, out, timeout=60):
    r = subprocess.run([exe, op, str(src), str(out)], timeout=timeout, capture_output=True)
    assert r.returncode == 0, (op, r.returncode, r.stderr[-400:])


JOB3 = """# parameter file with notes before the keys
sample folder   SPDir={d}/SP
background BGDir={d}/BG
AngDir={d}/Ang
SaveDir={d}/out=run7
rowPts0=12abc
rowPts1=1035
colPts0=0
colPts1=1023
ReconFlag=2.9
ReconSave=1
SizeType=1
ResizeFlag=0
Nmed=1.333e0
Mag=62.5
CameraPixelSize=6.5
wavelength=0.532e3
SavePhaseStack=1.7
SaveAmpStack=0
criteriaRange=9.42477796076938
criteriaSTD=0.25
"""


def test_job_list_matches_reference(ref_cpu, tmp_path):
    """scriptFileRead (cTDM/HilbertTransform.cu:70-175) with obtainParameter, on a job
    list of four parameter files, against ctdm_parse_job_file: the 20 fields in order,
    including notes before the keys, integers read by atoi from decimals and trailing
    text, exponents, and a value with '=' in it (the reference keeps its last piece).
    The reference ignores the optional fields after the 20th.  No value here has a space
    after its '=': the reference then reads a token of '=' alone and returns an unset
    pointer, where this library skips the spaces."""
    from ctdm_gb300 import jobs
    d = str(tmp_path)
    p1 = jobs.write_job_file(tmp_path / "job1.txt", optional=False, sp_dir=d + "/SP", bg_dir=d + "/BG",
                             ang_dir=d + "/Ang", save_dir=d + "/Save", row_pts=(0, 511), col_pts=(10, 521),
                             recon_flag=2, n_med=1.337, mag=62.5, camera_pixel_um=6.5, wavelength_nm=532.5,
                             criteria_range=7.25, criteria_std=0.75)
    p2 = jobs.write_job_file(tmp_path / "job2.txt", optional=True, sp_dir=d + "/a", bg_dir=d + "/b",
                             ang_dir=d + "/c", save_dir=d + "/e", recon_flag=0, recon_save=2, qpi_method=1,
                             iter_time=19, n_med=1.3371234567890123)
    p3 = tmp_path / "job3.txt"
    p3.write_text(JOB3.format(d=d))
    # a trailing '=' and doubled '=' signs: the last non-empty piece is kept
    p4 = tmp_path / "job4.txt"
    p4.write_text(JOB3.format(d=d).replace("SaveDir={d}/out=run7".format(d=d), "SaveDir={d}/keep=".format(d=d))
                  .replace("Mag=62.5", "Mag==62.5").replace("ReconSave=1", "ReconSave=2==="))
    lst = tmp_path / "JobList.txt"
    lst.write_text(f"{p1}\n{p2}\n{p3}\n{p4}\n")
    out = tmp_path / "jobs.json"
    run_paths(ref_cpu, "joblist", lst, out)
    import json
    ref = [json.loads(x) for x in out.read_text().splitlines()]
    assert len(ref) == 4
    keys = ["sp_dir", "bg_dir", "ang_dir", "save_dir", "row_pts", "col_pts", "recon_flag", "recon_save",
            "size_type", "resize_flag", "n_med", "mag", "camera_pixel_um", "wavelength_nm", "save_phase_stack",
            "save_amp_stack", "criteria_range", "criteria_std"]
    for path, r in zip((p1, p2, p3, p4), ref):
        mine = jobs.job_dict(jobs.parse_job_file(path))
        assert {k: mine[k] for k in keys} == {k: r[k] for k in keys}, path
    assert ref[2]["save_dir"] == "run7" and ref[2]["recon_flag"] == 2 and ref[2]["row_pts"] == [12, 1035]
    assert ref[3]["save_dir"] == d + "/keep" and ref[3]["mag"] == 62.5 and ref[3]["recon_save"] == 2


@pytest.mark.parametrize("h,w", [(8, 8), (30, 30), (64, 64), (8, 30)])
def test_bmp_reader_matches_reference(ref_cpu, tmp_path, h, w):
    """bmp_header + read_bmp (cTDM/HilbertTransform.cu:2680-2731) against ctdm_read_bmp:
    the same header fields and storage bytes, padded lines included (the reference reads
    width as its row count, so a wide picture is stored the same odd way by both)."""
    from ctdm_gb300 import dataset, jobs
    pic = np.random.default_rng(h * 100 + w).integers(0, 256, (h, w), dtype=np.uint8)
    path, out = tmp_path / "Buffer1.bmp", tmp_path / "ref.bin"
    dataset.write_bmp(path, pic)
    run_paths(ref_cpu, "bmp", path, out)
    raw = out.read_bytes()
    nr, nc = np.frombuffer(raw[:8], np.int32)
    assert (nr, nc) == jobs.bmp_size(path)
    assert np.array_equal(np.frombuffer(raw[8:], np.uint8), jobs.read_bmp(path).ravel())


@pytest.mark.parametrize("sx,sy,status", [(64, 64, 1), (37, 53, 0)])
def test_phimap_writer_matches_reference(ref_cpu, tmp_path, sx, sy, status):
    """outputImg (cTDM/HilbertTransform.cu:2437-2455) against ctdm_write_phimap: the same
    bytes; ctdm_read_phimap reads the reference's file back exactly."""
    from ctdm_gb300 import jobs
    rng = np.random.default_rng(sx * sy)
    ph = rng.standard_normal((sy, sx)).astype(np.float32)
    am = rng.random((sy, sx)).astype(np.float32)
    ax, ay = float(rng.standard_normal()), float(rng.standard_normal())
    src, ref_file, mine = tmp_path / "in.bin", tmp_path / "ref.phimap", tmp_path / "mine.phimap"
    with open(src, "wb") as f:
        np.array([status, sx, sy], np.int32).tofile(f)
        np.array([ax, ay], np.float64).tofile(f)
        ph.tofile(f)
        am.tofile(f)
    run_paths(ref_cpu, "phimap", src, ref_file)
    jobs.write_phimap(mine, status, ax, ay, ph, am)
    assert ref_file.read_bytes() == mine.read_bytes()
    back = jobs.read_phimap(ref_file)
    assert back["status"] == bool(status) and back["angle_x"] == ax and back["angle_y"] == ay
    assert np.array_equal(back["phase"], ph) and np.array_equal(back["amp"], am)


def test_check_array_matches_reference(ref_cpu, lib, tmp_path):
    """checkArray (cTDM/HilbertTransform.cu:3056-3092) against this library's drop-in with
    the limits at the float nearest to each statistic and one float either side."""
    import ctypes
    rng = np.random.default_rng(11)
    for seed in range(6):
        n = int(rng.integers(16, 5000))
        v = (rng.standard_normal(n) * rng.uniform(0.1, 3) + rng.uniform(-2, 2)).astype(np.float32)
        s = np.float32(np.sqrt(np.mean((v.astype(np.float64) - v.astype(np.float64).mean()) ** 2)))
        r = np.float32(abs(float(v.max()) - float(v.min())))
        for ls in (s, np.nextafter(s, np.float32(np.inf)), np.nextafter(s, np.float32(-np.inf))):
            for lr in (r, np.nextafter(r, np.float32(np.inf)), np.nextafter(r, np.float32(-np.inf)),
                       np.float32(1e9)):
                src = tmp_path / "chk.bin"
                with open(src, "wb") as f:
                    np.array([n], np.int32).tofile(f)
                    np.array([ls, lr], np.float32).tofile(f)
                    v.tofile(f)
                run_paths(ref_cpu, "check", src, tmp_path / "chk.out")
                ref = bool(np.fromfile(tmp_path / "chk.out", np.int32)[0])
                mine = lib.checkArray(v.ctypes.data, ctypes.c_float(ls), ctypes.c_float(lr), n)
                assert mine == ref, (seed, float(ls), float(lr))
