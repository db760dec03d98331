"""JobList driver and the reference's on-disk formats, over the C ABI.

Mirrors y-h-Lin/cTDM's job entry (cTDM/HilbertTransform.cu:70-175 scriptFileRead,
:327-1230 HilbertTransform) and its files: 8-bit BMP frames read the way read_bmp
stores them (:2694-2731), per-frame ``buffer%03d.phimap`` maps (:2437-2455) and the
``3D-RI-*.rimap`` volume (:2013-2041).  Everything here calls libctdm_gb300.so; the
format functions run on the host, ``run_job`` and ``angle_from_image`` on the GPU.
"""
import ctypes
import os

import numpy as np

from ._lib import JobFile, JobResult, check, load

# The 20 ordered fields of a parameter file (cTDM/HilbertTransform.cu:96-120) and the
# JobFile member each one fills.
FIELDS = (
    ("SPDir", "sp_dir"), ("BGDir", "bg_dir"), ("AngDir", "ang_dir"), ("SaveDir", "save_dir"),
    ("rowPts0", ("row_pts", 0)), ("rowPts1", ("row_pts", 1)), ("colPts0", ("col_pts", 0)),
    ("colPts1", ("col_pts", 1)), ("ReconFlag", "recon_flag"), ("ReconSave", "recon_save"),
    ("SizeType", "size_type"), ("ResizeFlag", "resize_flag"), ("Nmed", "n_med"), ("Mag", "mag"),
    ("CameraPixelSize", "camera_pixel_um"), ("wavelength", "wavelength_nm"),
    ("SavePhaseStack", "save_phase_stack"), ("SaveAmpStack", "save_amp_stack"),
    ("criteriaRange", "criteria_range"), ("criteriaSTD", "criteria_std"),
)
OPTIONAL = (("QPI_Method", "qpi_method"), ("IterTime", "iter_time"))


def _b(path):
    return os.fsencode(str(path))


# ---- formats ------------------------------------------------------------------------
def bmp_size(path):
    """(width, height) from the BMP header (bmp_header)."""
    w, h = ctypes.c_int(), ctypes.c_int()
    check(load().ctdm_read_bmp(_b(path), ctypes.byref(w), ctypes.byref(h), None), "ctdm_read_bmp")
    return w.value, h.value


def read_bmp(path):
    """read_bmp's storage as a (height, width) uint8 array s with s[j, i] = byte j of line
    i counted from the top; for a square frame s.T is the picture (rows, columns)."""
    w, h = bmp_size(path)
    out = np.zeros((h, w), np.uint8)
    wi, hi = ctypes.c_int(), ctypes.c_int()
    check(load().ctdm_read_bmp(_b(path), ctypes.byref(wi), ctypes.byref(hi), out.ctypes.data), "ctdm_read_bmp")
    return out


def write_phimap(path, status, angle_x, angle_y, phase, amp):
    """phase, amp: (size_y, size_x) float32 maps."""
    ph = np.ascontiguousarray(phase, np.float32)
    am = np.ascontiguousarray(amp, np.float32)
    if ph.shape != am.shape or ph.ndim != 2:
        raise ValueError("phase and amp must be equal 2-D maps")
    check(load().ctdm_write_phimap(_b(path), int(bool(status)), float(angle_x), float(angle_y), ph.shape[1],
                                   ph.shape[0], ph.ctypes.data, am.ctypes.data), "ctdm_write_phimap")


def read_phimap(path):
    """dict(status, angle_x, angle_y, phase, amp) with (size_y, size_x) maps."""
    lib = load()
    st, sx, sy = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    ax, ay = ctypes.c_double(), ctypes.c_double()
    check(lib.ctdm_read_phimap(_b(path), ctypes.byref(st), ctypes.byref(ax), ctypes.byref(ay), ctypes.byref(sx),
                               ctypes.byref(sy), None, None), "ctdm_read_phimap")
    ph = np.zeros((sy.value, sx.value), np.float32)
    am = np.zeros_like(ph)
    check(lib.ctdm_read_phimap(_b(path), ctypes.byref(st), ctypes.byref(ax), ctypes.byref(ay), ctypes.byref(sx),
                               ctypes.byref(sy), ph.ctypes.data, am.ctypes.data), "ctdm_read_phimap")
    return {"status": bool(st.value), "angle_x": ax.value, "angle_y": ay.value, "phase": ph, "amp": am}


def rimap_name(r, save_mode=0):
    kind = ("Complex", "Real", "Imag")[save_mode]
    return f"3D-RI-{kind}_{r}x{r}x{r}.rimap"


def write_rimap(directory, ri, save_mode=0):
    """ri: (R, R, R) complex64 volume; returns the written path."""
    v = np.ascontiguousarray(ri, np.complex64)
    r = v.shape[0]
    if v.shape != (r, r, r):
        raise ValueError("ri must be an R^3 volume")
    check(load().ctdm_write_rimap(_b(directory), r, int(save_mode), v.ctypes.data), "ctdm_write_rimap")
    return os.path.join(str(directory), rimap_name(r, save_mode))


def read_rimap(path, r, save_mode=0):
    dt = np.complex64 if save_mode == 0 else np.float32
    return np.fromfile(path, dt).reshape(r, r, r)


def check_frame(phase, resize_flag=1, limit_std=0.5, limit_range=3 * np.pi):
    """True when the frame fails the check (checkArray on the centre half for
    resize_flag 1, on the whole map with 0.5 and 5 pi for 0)."""
    ph = np.ascontiguousarray(phase, np.float32)
    return bool(load().ctdm_check_frame(ph.ctypes.data, ph.shape[0], int(resize_flag), float(limit_std),
                                        float(limit_range)))


def angle_from_image(image, n_med=1.333, wavelength_nm=532.0, mag=85.0, camera_pixel_um=5.5):
    """AngCal_GPU on an (N, N) angle-camera picture (rows, columns): (angle, peak)."""
    img = np.ascontiguousarray(image, np.float32)
    a, pk = ctypes.c_float(), ctypes.c_long()
    check(load().ctdm_angle_from_image(img.ctypes.data, img.shape[0], float(n_med), float(wavelength_nm), float(mag),
                                       float(camera_pixel_um), ctypes.byref(a), ctypes.byref(pk)),
          "ctdm_angle_from_image")
    return a.value, pk.value


# ---- jobs ---------------------------------------------------------------------------
def job_defaults():
    j = JobFile()
    load().ctdm_job_defaults(ctypes.byref(j))
    return j


def make_job(**kw):
    """JobFile from the defaults and keyword overrides (folders as str / Path)."""
    j = job_defaults()
    for k, v in kw.items():
        if k in ("sp_dir", "bg_dir", "ang_dir", "save_dir"):
            setattr(j, k, _b(v))
        elif k in ("row_pts", "col_pts"):
            getattr(j, k)[0], getattr(j, k)[1] = int(v[0]), int(v[1])
        else:
            setattr(j, k, v)
    return j


def parse_job_file(path):
    j = JobFile()
    check(load().ctdm_parse_job_file(_b(path), ctypes.byref(j)), "ctdm_parse_job_file")
    return j


def job_dict(j):
    d = {}
    for _, member in FIELDS + OPTIONAL:
        if isinstance(member, tuple):
            d.setdefault(member[0], [0, 0])[member[1]] = getattr(j, member[0])[member[1]]
        else:
            v = getattr(j, member)
            d[member] = v.decode() if isinstance(v, bytes) else v
    return d


def write_job_file(path, job=None, optional=True, **kw):
    """Writes a parameter file with the 20 fields in order (and QPI_Method / IterTime
    when optional is true).  job: a JobFile (default: make_job(**kw))."""
    j = job if job is not None else make_job(**kw)
    lines = []
    for key, member in FIELDS:
        if isinstance(member, tuple):
            v = getattr(j, member[0])[member[1]]
        else:
            v = getattr(j, member)
            if isinstance(v, bytes):
                v = v.decode()
        lines.append(f"{key}={v}")
    if optional:
        lines += [f"{key}={getattr(j, member)}" for key, member in OPTIONAL]
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")
    return str(path)


def run_job(job):
    """Runs one job (HilbertTransform with SpeedTestFlag = 0); returns a JobResult."""
    r = JobResult()
    check(load().ctdm_run_job(ctypes.byref(job), ctypes.byref(r)), "ctdm_run_job")
    return r


def script_file_read(path):
    """scriptFileRead: 0 when the job list cannot be opened, else 1 (a failed job
    leaves its message in ctdm_last_error)."""
    return load().scriptFileRead(_b(path))
