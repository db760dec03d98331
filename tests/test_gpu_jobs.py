"""The JobList driver end to end on synthetic BMP datasets, and AngCal_GPU, through the
C ABI against the oracle.

* AngCal_GPU: the spectrum peak index bit-exact against the numpy restatement, and the
  known answer of a drawn fringe; the angle within 1e-6 rad.
* Maps: each buffer%03d.phimap (Algorithm B and A, batched per frame on the GPU) against
  the FP64 oracle's QPI -> DCT unwrap -> bilinear resize chain, phase RMSE <= 1e-3 rad
  (two float32 stages chained) and amplitude RMSE <= 1e-4; the frame check bit-exact
  against the oracle's checkArray; batching over several GPU batches changes nothing.
* Reconstruction: RefreshStack keeps the frames that pass; the .rimap equals BatchRecon
  on the stacks and angles read back from the .phimap files (RI RMSE <= 1e-5), and the
  ReconFlag 2 resume through scriptFileRead reproduces it.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
PHASE_TOL = 1e-3
AMP_TOL = 1e-4
RI_TOL = 1e-5
OPTICS = dict(n_med=1.333, wavelength_nm=532.0, mag=85.0, camera_pixel_um=5.5)


def rmse(a, b):
    return float(np.sqrt(np.mean(np.abs(np.asarray(a, np.complex128) - np.asarray(b, np.complex128)) ** 2)))


@pytest.mark.parametrize("n", [256, 1024])
def test_angcal_known_answer(ctx, oracle, n):
    from ctdm_gb300 import _lib, dataset, jobs
    lib = _lib.load()
    for kx in (-40, -7, 0, 3, 25):
        pic = dataset.angle_picture(n, kx)
        ang, peak = jobs.angle_from_image(pic, **OPTICS)
        assert peak == (n // 2 + n // 8) * n + n // 2 + kx
        assert peak == oracle.angcal_peak(pic)
        want = oracle.angcal_angle(peak, n, **OPTICS)
        assert abs(ang - want) <= 1e-6
        img = np.ascontiguousarray(pic, np.float32)
        assert abs(lib.AngCal_GPU(img.ctypes.data, n, n, 1, 1) - want) <= 1e-6   # the defaults' optics
    # a noisy picture: the first maximum against the restatement
    rng = np.random.default_rng(n)
    pic = dataset.angle_picture(n, 11).astype(np.float32) + rng.normal(0, 20, (n, n)).astype(np.float32)
    assert jobs.angle_from_image(pic, **OPTICS)[1] == oracle.angcal_peak(pic)


def expected_maps_b(oracle, ds):
    """Oracle chain of the job loop for Algorithm B: frame 1 uses its own carrier column,
    later frames and every background the first background's."""
    n, hs, bs = ds["n"], ds["holograms"], ds["backgrounds"]
    cb, c1 = oracle.qpib_center(bs[0]), oracle.qpib_center(hs[0])
    out = []
    for k in range(ds["frames"]):
        spf = oracle.qpib_field(hs[k], c1 if k == 0 else cb)
        ph, am = oracle.wrap_phase(spf, oracle.qpib_field(bs[k], cb))
        out.append(oracle.resize_crop(oracle.dct_unwrap(ph, 0), am, n, n))
    return out


def expected_maps_a(oracle, ds):
    """Algorithm A sees the picture (read_bmp storage transposed); the carrier comes from
    the first background."""
    from ctdm_gb300 import dataset
    n = ds["n"]
    m = n // 4
    hs = [dataset.storage_picture(h) for h in ds["holograms"]]
    bs = [dataset.storage_picture(b) for b in ds["backgrounds"]]
    car = oracle.qpi_carrier(bs[0])
    out = []
    for k in range(ds["frames"]):
        ph, am = oracle.wrap_phase(oracle.qpi_field(hs[k], m, *car), oracle.qpi_field(bs[k], m, *car))
        out.append(oracle.resize_crop(oracle.dct_unwrap(ph, 0), am, n, n))
    return out


def check_maps(oracle, ds, want, criteria=(1e3, 1e3)):
    from ctdm_gb300 import jobs
    n = ds["n"]
    for k in range(ds["frames"]):
        got = jobs.read_phimap(os.path.join(ds["save_dir"], f"buffer{k + 1:03d}.phimap"))
        assert got["phase"].shape == (n, n)
        assert rmse(got["phase"], want[k][0]) < PHASE_TOL, k
        assert rmse(got["amp"], want[k][1]) < AMP_TOL, k
        assert got["status"] == (not oracle.check_frame(got["phase"], 1, criteria[1], criteria[0]))
        # angles: AngCal of the drawn fringes, within a fringe step of the true angles
        for axis in ("x", "y"):
            peak = (n // 2 + n // 8) * n + n // 2 + ds["fringe_" + axis][k]
            assert abs(got["angle_" + axis] - oracle.angcal_angle(peak, n, **OPTICS)) <= 1e-6
            assert abs(got["angle_" + axis] - ds["ang_" + axis][k]) < 0.05


@pytest.fixture(scope="module")
def job_b(tmp_path_factory, ctx):
    from ctdm_gb300 import dataset
    return dataset.make_dataset(tmp_path_factory.mktemp("job_b"), n=256, frames=6, seed=3, recon_flag=0)


def test_job_maps_algorithm_b(ctx, oracle, job_b):
    from ctdm_gb300 import jobs
    r = jobs.run_job(jobs.parse_job_file(job_b["job_file"]))
    assert (r.frames, r.rejected, r.recon_frames, r.n_holo, r.recon_size) == (6, 0, 0, 256, 256)
    check_maps(oracle, job_b, expected_maps_b(oracle, job_b))
    assert not os.path.exists(os.path.join(job_b["save_dir"], "3D-RI-Complex_256x256x256.rimap"))


def test_job_batches_agree(ctx, job_b):
    """Three GPU batches of two frames give the maps of one batch of six."""
    from ctdm_gb300 import jobs
    ref = [jobs.read_phimap(os.path.join(job_b["save_dir"], f"buffer{k:03d}.phimap")) for k in range(1, 7)]
    j = jobs.parse_job_file(job_b["job_file"])
    j.save_dir = os.fsencode(os.path.join(job_b["root"], "Save2"))
    os.environ["CTDM_JOB_BATCH_FRAMES"] = "2"
    try:
        jobs.run_job(j)
    finally:
        del os.environ["CTDM_JOB_BATCH_FRAMES"]
    for k in range(1, 7):
        got = jobs.read_phimap(os.path.join(job_b["root"], "Save2", f"buffer{k:03d}.phimap"))
        np.testing.assert_array_equal(got["phase"], ref[k - 1]["phase"])
        np.testing.assert_array_equal(got["amp"], ref[k - 1]["amp"])
        assert got["angle_x"] == ref[k - 1]["angle_x"] and got["status"] == ref[k - 1]["status"]


def stacks_from_maps(save_dir, frames):
    from ctdm_gb300 import jobs
    maps = [jobs.read_phimap(os.path.join(save_dir, f"buffer{k:03d}.phimap")) for k in range(1, frames + 1)]
    keep = [m for m in maps if m["status"]]
    ph = np.stack([np.nan_to_num(m["phase"], nan=0.0, posinf=0.0, neginf=0.0) for m in keep]).astype(np.float32)
    am = np.stack([np.nan_to_num(m["amp"], nan=1.0, posinf=1.0, neginf=1.0) for m in keep]).astype(np.float32)
    ax = np.array([m["angle_x"] for m in keep], np.float32)
    ay = np.array([m["angle_y"] for m in keep], np.float32)
    return [m["status"] for m in maps], ph, am, ax, ay


def test_job_rejects_and_reconstructs(ctx, oracle, job_b, tmp_path):
    """ReconFlag 1 with a criteriaSTD between the frames' standard deviations: the frames
    above it are rejected and the volume is BatchRecon of the others."""
    from ctdm_gb300 import _lib, jobs
    n, F = job_b["n"], job_b["frames"]
    stds = []
    for k in range(1, F + 1):
        ph = jobs.read_phimap(os.path.join(job_b["save_dir"], f"buffer{k:03d}.phimap"))["phase"]
        stds.append(float(np.std(ph[n // 4:3 * n // 4, n // 4:3 * n // 4].astype(np.float64))))
    s = sorted(stds)
    limit = 0.5 * (s[3] + s[4])
    j = jobs.parse_job_file(job_b["job_file"])
    j.recon_flag, j.criteria_std, j.criteria_range = 1, limit, 1e3
    jobs.write_job_file(os.path.join(job_b["root"], "job_recon.txt"), j)
    r = jobs.run_job(j)
    assert (r.frames, r.rejected, r.recon_frames) == (F, 2, F - 2)
    status, ph, am, ax, ay = stacks_from_maps(job_b["save_dir"], F)
    assert status == [sd <= limit for sd in stds]
    got = jobs.read_rimap(os.path.join(job_b["save_dir"], jobs.rimap_name(256)), 256)
    # BatchRecon (reference-named entry) on the same stacks into another folder
    lib = _lib.load()
    lib.ctdm_set_recon_globals(256, OPTICS["n_med"], OPTICS["wavelength_nm"], OPTICS["camera_pixel_um"],
                               OPTICS["mag"], 2, 0, os.fsencode(str(tmp_path)))
    lib.BatchRecon(ph.ctypes.data, am.ctypes.data, ax.ctypes.data, ay.ctypes.data, len(ax))
    assert _lib.last_error() == ""
    want = jobs.read_rimap(os.path.join(str(tmp_path), jobs.rimap_name(256)), 256)
    assert np.isfinite(got).all()
    assert rmse(got, want) < RI_TOL


def test_job_resume_from_saved_maps(ctx, job_b):
    """ReconFlag 2 through scriptFileRead: the volume from the saved .phimap files equals
    the ReconFlag 1 volume, y angles included."""
    from ctdm_gb300 import _lib, jobs
    path = os.path.join(job_b["save_dir"], jobs.rimap_name(256))
    first = jobs.read_rimap(path, 256).copy()
    os.remove(path)
    j = jobs.parse_job_file(os.path.join(job_b["root"], "job_recon.txt"))
    j.recon_flag = 2
    jf = jobs.write_job_file(os.path.join(job_b["root"], "job_resume.txt"), j)
    lst = os.path.join(job_b["root"], "JobList_resume.txt")
    with open(lst, "w") as f:
        f.write(jf + "\n")
    assert jobs.script_file_read(lst) == 1
    assert _lib.last_error() == ""
    again = jobs.read_rimap(path, 256)
    assert rmse(again, first) < RI_TOL


def test_job_maps_algorithm_a_and_raw_files(ctx, oracle, tmp_path):
    from ctdm_gb300 import dataset, jobs
    ds = dataset.make_dataset(tmp_path, n=256, frames=3, seed=5, qpi_method=1, recon_flag=0, separate_xy=True,
                              save_phase=1, save_amp=1)
    r = jobs.run_job(jobs.parse_job_file(ds["job_file"]))
    assert (r.frames, r.rejected) == (3, 0)
    check_maps(oracle, ds, expected_maps_a(oracle, ds))
    for k in range(1, 4):
        m = jobs.read_phimap(os.path.join(ds["save_dir"], f"buffer{k:03d}.phimap"))
        raw = np.fromfile(os.path.join(ds["save_dir"], f"Phase{k:03d}_256x256.raw"), np.float32).reshape(256, 256)
        np.testing.assert_array_equal(raw, m["phase"])
        raw = np.fromfile(os.path.join(ds["save_dir"], f"Amp{k:03d}_256x256.raw"), np.float32).reshape(256, 256)
        np.testing.assert_array_equal(raw, m["amp"])


def test_job_resize_flag_0(ctx, oracle, tmp_path):
    """ResizeFlag 0: the frame check runs on the whole map with 0.5 and 5 pi, and the
    stacks are the bilinear resize N -> R of each map (Combine2Stack's first branch);
    the volume equals BatchRecon on those stacks."""
    from ctdm_gb300 import _lib, jobs
    from ctdm_gb300 import dataset
    ds = dataset.make_dataset(tmp_path, n=512, frames=4, seed=8, recon_flag=1, resize_flag=0, photons=1e5, na=0.3)
    r = jobs.run_job(jobs.parse_job_file(ds["job_file"]))
    maps = [jobs.read_phimap(os.path.join(ds["save_dir"], f"buffer{k:03d}.phimap")) for k in range(1, 5)]
    want_status = [not oracle.check_frame(m["phase"], 0, 0.5, 5 * np.pi) for m in maps]
    assert [m["status"] for m in maps] == want_status
    assert (r.frames, r.rejected, r.n_holo, r.recon_size) == (4, 4 - sum(want_status), 512, 256)
    keep = [m for m in maps if m["status"]]
    if len(keep) < 2:
        assert r.recon_frames == 0
        return
    assert r.recon_frames == len(keep)
    ph = np.stack([oracle.bilinear(m["phase"], 256, 256) for m in keep]).astype(np.float32)
    am = np.stack([oracle.bilinear(m["amp"], 256, 256) for m in keep]).astype(np.float32)
    ax = np.array([m["angle_x"] for m in keep], np.float32)
    ay = np.array([m["angle_y"] for m in keep], np.float32)
    out = tmp_path / "ref"
    out.mkdir()
    lib = _lib.load()
    lib.ctdm_set_recon_globals(256, OPTICS["n_med"], OPTICS["wavelength_nm"], OPTICS["camera_pixel_um"],
                               OPTICS["mag"], 2, 0, os.fsencode(str(out)))
    lib.BatchRecon(ph.ctypes.data, am.ctypes.data, ax.ctypes.data, ay.ctypes.data, len(ax))
    assert _lib.last_error() == ""
    got = jobs.read_rimap(os.path.join(ds["save_dir"], jobs.rimap_name(256)), 256)
    want = jobs.read_rimap(os.path.join(str(out), jobs.rimap_name(256)), 256)
    assert rmse(got, want) < RI_TOL
