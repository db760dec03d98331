"""On-disk formats and the JobList parser through the C ABI, host side only (no GPU):
BMP ingest with read_bmp's transposed storage and line padding, the .phimap and .rimap
byte layouts, the frame check against the oracle's checkArray, parameter files in the
reference's field order, and the driver's error paths that stop before any device work."""
import os
import struct

import numpy as np
import pytest

from ctdm_gb300 import dataset, jobs
from ctdm_gb300._lib import CtdmError

CTDM_ERR_INVALID, CTDM_ERR_IO = 1, 4


@pytest.fixture(scope="module")
def lib():
    from ctdm_gb300 import _lib
    return _lib.load()


@pytest.mark.parametrize("n", [8, 30, 64])
def test_bmp_storage_is_the_transposed_picture(lib, tmp_path, n):
    rng = np.random.default_rng(n)
    pic = rng.integers(0, 256, (n, n), dtype=np.uint8)
    path = tmp_path / "Buffer1.bmp"
    dataset.write_bmp(path, pic)
    assert os.path.getsize(path) == 54 + 1024 + ((n + 3) & ~3) * n   # lines padded to 4 bytes
    assert jobs.bmp_size(path) == (n, n)
    s = jobs.read_bmp(path)
    np.testing.assert_array_equal(s, pic.T)
    np.testing.assert_array_equal(dataset.storage_picture(s), pic)


def test_bmp_errors(lib, tmp_path):
    with pytest.raises(CtdmError) as e:
        jobs.read_bmp(tmp_path / "missing.bmp")
    assert e.value.status == CTDM_ERR_IO
    bad = tmp_path / "bad.bmp"
    bad.write_bytes(b"XX" + bytes(100))
    with pytest.raises(CtdmError) as e:
        jobs.read_bmp(bad)
    assert e.value.status == CTDM_ERR_IO
    # a 24-bit header is refused (read_bmp reads one byte per pixel)
    pic = tmp_path / "rgb.bmp"
    dataset.write_bmp(pic, np.zeros((4, 4), np.uint8))
    raw = bytearray(pic.read_bytes())
    raw[28] = 24
    pic.write_bytes(bytes(raw))
    with pytest.raises(CtdmError) as e:
        jobs.read_bmp(pic)
    assert e.value.status == CTDM_ERR_INVALID
    # truncated pixel data
    short = tmp_path / "short.bmp"
    dataset.write_bmp(short, np.zeros((16, 16), np.uint8))
    short.write_bytes(short.read_bytes()[:-40])
    with pytest.raises(CtdmError) as e:
        jobs.read_bmp(short)
    assert e.value.status == CTDM_ERR_IO


def test_phimap_layout_and_round_trip(lib, tmp_path):
    rng = np.random.default_rng(1)
    ph = rng.normal(size=(6, 5)).astype(np.float32)
    am = rng.random((6, 5)).astype(np.float32)
    path = tmp_path / "buffer001.phimap"
    jobs.write_phimap(path, True, -0.25, 0.125, ph, am)
    raw = path.read_bytes()
    # outputImg: bool, two doubles, two ints (size x, size y), then (phase, amp) pairs
    assert len(raw) == 1 + 8 + 8 + 4 + 4 + 8 * ph.size
    st, ax, ay, sx, sy = struct.unpack("<?ddii", raw[:25])
    assert (st, ax, ay, sx, sy) == (True, -0.25, 0.125, 5, 6)
    pairs = np.frombuffer(raw[25:], np.float32).reshape(-1, 2)
    np.testing.assert_array_equal(pairs[:, 0], ph.ravel())
    np.testing.assert_array_equal(pairs[:, 1], am.ravel())
    got = jobs.read_phimap(path)
    assert got["status"] is True and got["angle_x"] == -0.25 and got["angle_y"] == 0.125
    np.testing.assert_array_equal(got["phase"], ph)
    np.testing.assert_array_equal(got["amp"], am)
    jobs.write_phimap(path, False, 0, 0, ph, am)
    assert jobs.read_phimap(path)["status"] is False
    path.write_bytes(raw[:30])
    with pytest.raises(CtdmError):
        jobs.read_phimap(path)


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_rimap_files(lib, tmp_path, mode):
    rng = np.random.default_rng(mode)
    r = 8
    ri = (rng.normal(size=(r, r, r)) + 1j * rng.normal(size=(r, r, r))).astype(np.complex64)
    path = jobs.write_rimap(tmp_path, ri, mode)
    assert os.path.basename(path) == ("3D-RI-Complex_8x8x8.rimap", "3D-RI-Real_8x8x8.rimap",
                                      "3D-RI-Imag_8x8x8.rimap")[mode]
    got = jobs.read_rimap(path, r, mode)
    want = (ri, ri.real, ri.imag)[mode]
    np.testing.assert_array_equal(got, want)


@pytest.mark.parametrize("resize_flag", [0, 1])
def test_frame_check_matches_oracle(lib, oracle, resize_flag):
    rng = np.random.default_rng(5 + resize_flag)
    n = 64
    for scale in (0.05, 0.3, 0.6, 2.0, 5.0):
        ph = (rng.normal(size=(n, n)) * scale).astype(np.float32)
        for lim_std, lim_rng in ((0.5, 3 * np.pi), (1.0, 10.0), (0.2, 100.0)):
            want = oracle.check_frame(ph, resize_flag, lim_std, lim_rng)
            assert jobs.check_frame(ph, resize_flag, lim_std, lim_rng) == want
    # the reference-named entry on a plain array
    v = np.array([0, 0, 0, 4], np.float32)
    assert lib.checkArray(v.ctypes.data, 1.0, 100.0, 4) is True     # std = sqrt(3) > 1
    assert lib.checkArray(v.ctypes.data, 2.0, 100.0, 4) is False
    assert lib.checkArray(v.ctypes.data, 2.0, 3.5, 4) is True       # range 4 > 3.5


def test_job_defaults(lib):
    d = jobs.job_dict(jobs.job_defaults())
    assert d["recon_flag"] == 1 and d["size_type"] == 0 and d["resize_flag"] == 1
    assert d["n_med"] == 1.333 and d["mag"] == 85.0 and d["camera_pixel_um"] == 5.5 and d["wavelength_nm"] == 532
    assert d["criteria_std"] == 0.5 and abs(d["criteria_range"] - 3 * np.pi) < 1e-12
    assert d["qpi_method"] == 0 and d["iter_time"] == 100


def test_parse_reference_style_parameter_file(lib, tmp_path):
    # Windows folders, spaces after '=', no optional keys: the reference's own format
    text = "\n".join([
        r"SPDir=D:\mic110\SP", r"BGDir= D:\mic110\BG", r"AngDir=D:\mic110\Ang", r"SaveDir=D:\mic110\out",
        "rowPts0=0", "rowPts1=1023", "colPts0=0", "colPts1=1023",
        "ReconFlag=2", "ReconSave=1", "SizeType=1", "ResizeFlag=0",
        "Nmed=1.334", "Mag=60", "CameraPixelSize=6.5", "wavelength=561",
        "SavePhaseStack=1", "SaveAmpStack=0", "criteriaRange=9.5", "criteriaSTD=0.75"]) + "\n"
    p = tmp_path / "2.txt"
    p.write_text(text)
    d = jobs.job_dict(jobs.parse_job_file(p))
    assert d["sp_dir"] == "D:/mic110/SP" and d["bg_dir"] == "D:/mic110/BG" and d["save_dir"] == "D:/mic110/out"
    assert d["row_pts"] == [0, 1023] and d["col_pts"] == [0, 1023]
    assert (d["recon_flag"], d["recon_save"], d["size_type"], d["resize_flag"]) == (2, 1, 1, 0)
    assert (d["n_med"], d["mag"], d["camera_pixel_um"], d["wavelength_nm"]) == (1.334, 60.0, 6.5, 561.0)
    assert (d["save_phase_stack"], d["save_amp_stack"]) == (1, 0)
    assert (d["criteria_range"], d["criteria_std"]) == (9.5, 0.75)
    assert d["qpi_method"] == 0 and d["iter_time"] == 100       # compile-time defaults
    # the optional keys, round trip through the writer
    j = jobs.make_job(sp_dir=tmp_path / "a", bg_dir=tmp_path / "b", ang_dir=tmp_path / "c",
                      save_dir=tmp_path / "d", qpi_method=1, iter_time=7, criteria_std=0.25)
    q = jobs.write_job_file(tmp_path / "3.txt", j)
    assert jobs.job_dict(jobs.parse_job_file(q)) == jobs.job_dict(j)


def test_parse_errors(lib, tmp_path):
    p = tmp_path / "short.txt"
    p.write_text("SPDir=a\nBGDir=b\n")
    with pytest.raises(CtdmError) as e:
        jobs.parse_job_file(p)
    assert e.value.status == CTDM_ERR_IO and "20 needed" in str(e.value)
    j = jobs.write_job_file(tmp_path / "extra.txt", jobs.job_defaults())
    with open(j, "a") as f:
        f.write("Colour=3\n")
    with pytest.raises(CtdmError) as e:
        jobs.parse_job_file(j)
    assert e.value.status == CTDM_ERR_INVALID
    with pytest.raises(CtdmError) as e:
        jobs.parse_job_file(tmp_path / "none.txt")
    assert e.value.status == CTDM_ERR_IO


def test_job_errors_before_device_work(lib, tmp_path):
    from ctdm_gb300._lib import last_error
    empty = tmp_path / "empty"
    empty.mkdir()
    j = jobs.make_job(sp_dir=empty, bg_dir=empty, ang_dir=empty, save_dir=tmp_path / "out")
    with pytest.raises(CtdmError) as e:
        jobs.run_job(j)
    assert e.value.status == CTDM_ERR_IO and "Buffer" in str(e.value)
    j = jobs.make_job(save_dir=empty, recon_flag=2)
    with pytest.raises(CtdmError) as e:
        jobs.run_job(j)
    assert e.value.status == CTDM_ERR_IO and "phimap" in str(e.value)
    with pytest.raises(CtdmError) as e:
        jobs.run_job(jobs.make_job(qpi_method=2))
    assert e.value.status == CTDM_ERR_INVALID and "not built" in str(e.value)
    with pytest.raises(CtdmError):
        jobs.run_job(jobs.make_job(recon_flag=3))
    # mismatched sample / background sizes are refused from the headers
    sp, bg = tmp_path / "sp", tmp_path / "bg"
    sp.mkdir()
    bg.mkdir()
    dataset.write_bmp(sp / "Buffer1.bmp", np.zeros((64, 64), np.uint8))
    dataset.write_bmp(bg / "Buffer1.bmp", np.zeros((128, 128), np.uint8))
    with pytest.raises(CtdmError) as e:
        jobs.run_job(jobs.make_job(sp_dir=sp, bg_dir=bg, ang_dir=sp, save_dir=tmp_path / "o"))
    assert "Wrong size" in str(e.value)
    # scriptFileRead: 0 without a list; 1 with one, the failing job's message kept
    assert jobs.script_file_read(tmp_path / "nolist.txt") == 0
    lst = tmp_path / "JobList.txt"
    lst.write_text(str(tmp_path / "missing_job.txt") + "\n")
    assert jobs.script_file_read(lst) == 1
    assert "missing_job.txt" in last_error()
