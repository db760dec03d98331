"""Synthetic JobList datasets: seeded holograms, backgrounds and angle-camera frames
written as the 8-bit BMP folders the reference's HilbertTransform reads
(SPDir/BufferK.bmp, BGDir/BufferK.bmp, AngDir/{X,Y}/BufferK.bmp), plus the parameter
file and the job list.  No camera data is involved: every frame comes from
ctdm_gb300.phantom (FP64) and is quantised to bytes.
"""
import os
import struct

import numpy as np

from . import jobs, phantom


def write_bmp(path, image):
    """8-bit grey BMP of a (rows, columns) uint8 picture: 54-byte header, 256-entry
    grey palette, rows bottom-up padded to 4 bytes."""
    img = np.ascontiguousarray(image, np.uint8)
    h, w = img.shape
    line = (w + 3) & ~3
    data_off = 54 + 1024
    size = data_off + line * h
    hdr = b"BM" + struct.pack("<IHHI", size, 0, 0, data_off)
    hdr += struct.pack("<IiiHHIIiiII", 40, w, h, 1, 8, 0, line * h, 2835, 2835, 256, 0)
    pal = b"".join(bytes((g, g, g, 0)) for g in range(256))
    rows = bytearray()
    pad = bytes(line - w)
    for r in range(h - 1, -1, -1):
        rows += img[r].tobytes() + pad
    with open(path, "wb") as f:
        f.write(hdr + pal + bytes(rows))


def storage_picture(storage):
    """The picture whose read_bmp storage is the (N, N) array `storage` (square frames:
    read_bmp stores the picture transposed)."""
    return np.ascontiguousarray(np.asarray(storage).T)


def fringe_bins(angle, n, n_med, wavelength_nm, mag, camera_pixel_um):
    """Column offset of the angle-camera fringe whose AngCal_GPU estimate is closest to
    `angle`: AngCal_GPU returns asin(mag (1 + k) / (N pixel fm)) for a fringe k columns
    from the centre."""
    fm = n_med / (wavelength_nm * 1e-9)
    return int(np.rint(np.sin(angle) * n * camera_pixel_um * 1e-6 * fm / mag)) - 1


def angle_picture(n, kx, ky=None):
    """(N, N) uint8 fringe picture with one spectral peak at kx columns, ky rows from
    the centre (ky defaults to N/8, inside AngCal_GPU's search band)."""
    ky = n // 8 if ky is None else ky
    y, x = np.mgrid[0:n, 0:n]
    v = 127.5 * (1.0 + np.cos(2 * np.pi * (kx * x + ky * y) / n))
    return np.clip(np.rint(v), 0, 255).astype(np.uint8)


def quantise(frames, scale):
    return np.clip(np.rint(np.asarray(frames, np.float64) * scale), 0, 255).astype(np.uint8)


def make_dataset(root, n=256, frames=6, seed=0, qpi_method=0, recon_flag=1, size_type=0, resize_flag=1,
                 iter_time=2, n_med=1.333, wavelength_nm=532.0, mag=85.0, camera_pixel_um=5.5, criteria_range=1e3,
                 criteria_std=1e3, photons=1e4, na=0.6, separate_xy=True, save_phase=0, save_amp=0, carrier=None):
    """Writes root/{SP,BG,Ang,Save} and root/job.txt (one parameter file) and
    root/JobList.txt; returns a dict with the paths, the per-frame angles used to draw
    the angle pictures and the float holograms (read_bmp storage order) the driver
    reads back.  Algorithm B (qpi_method 0) filters along the storage's fast axis, so
    its default carrier lies along it, (0.25, 0) cycles per pixel; Algorithm A's
    default is the diagonal (0.125, 0.125)."""
    root = str(root)
    sp_dir, bg_dir, ang_dir, save_dir = (os.path.join(root, d) for d in ("SP", "BG", "Ang", "Save"))
    for d in (sp_dir, bg_dir, ang_dir):
        os.makedirs(d, exist_ok=True)
    if carrier is None:
        carrier = (0.25, 0.0) if qpi_method == 0 else (0.125, 0.125)
    acq = phantom.acquisition(n, n, frames, na=na, seed=seed, pixel=0.1e-6 * 256 / n, carrier=carrier,
                              photons=photons)
    rng = np.random.default_rng(seed + 17)
    bgs = [acq.background]
    for _ in range(frames - 1):
        bgs.append(phantom.holograms_from_fields(np.zeros((1, n, n), np.complex128), photons, rng, carrier)[0])
    bgs = np.stack(bgs)
    scale = 250.0 / max(float(acq.holograms.max()), float(bgs.max()))
    sp_u8, bg_u8 = quantise(acq.holograms, scale), quantise(bgs, scale)
    if separate_xy:
        os.makedirs(os.path.join(ang_dir, "X"), exist_ok=True)
        os.makedirs(os.path.join(ang_dir, "Y"), exist_ok=True)
    kxs, kys = [], []
    for k in range(frames):
        name = f"Buffer{k + 1}.bmp"
        write_bmp(os.path.join(sp_dir, name), storage_picture(sp_u8[k]))
        write_bmp(os.path.join(bg_dir, name), storage_picture(bg_u8[k]))
        kx = fringe_bins(acq.ang_x[k], n, n_med, wavelength_nm, mag, camera_pixel_um)
        ky = fringe_bins(acq.ang_y[k], n, n_med, wavelength_nm, mag, camera_pixel_um)
        kxs.append(kx)
        kys.append(ky)
        if separate_xy:
            write_bmp(os.path.join(ang_dir, "X", name), angle_picture(n, kx))
            write_bmp(os.path.join(ang_dir, "Y", name), angle_picture(n, ky))
        else:
            write_bmp(os.path.join(ang_dir, name), angle_picture(n, kx))
    job = jobs.make_job(sp_dir=sp_dir, bg_dir=bg_dir, ang_dir=ang_dir, save_dir=save_dir, row_pts=(0, n - 1),
                        col_pts=(0, n - 1), recon_flag=recon_flag, recon_save=0, size_type=size_type,
                        resize_flag=resize_flag, n_med=n_med, mag=mag, camera_pixel_um=camera_pixel_um,
                        wavelength_nm=wavelength_nm, save_phase_stack=save_phase, save_amp_stack=save_amp,
                        criteria_range=criteria_range, criteria_std=criteria_std, qpi_method=qpi_method,
                        iter_time=iter_time)
    job_path = jobs.write_job_file(os.path.join(root, "job.txt"), job)
    list_path = os.path.join(root, "JobList.txt")
    with open(list_path, "w") as f:
        f.write(job_path + "\n")
    return {"root": root, "sp_dir": sp_dir, "bg_dir": bg_dir, "ang_dir": ang_dir, "save_dir": save_dir,
            "job_file": job_path, "job_list": list_path, "job": job, "n": n, "frames": frames,
            "holograms": sp_u8.astype(np.float32), "backgrounds": bg_u8.astype(np.float32),
            "fringe_x": kxs, "fringe_y": kys, "ang_x": acq.ang_x, "ang_y": acq.ang_y}
