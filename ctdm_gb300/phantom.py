"""Seeded synthetic cTDM acquisitions (FP64 numpy).

No public dataset exists for this path; these generators stand in for the BMP
stacks the reference reads (cTDM/HilbertTransform.cu:613-771).  A phantom is a sum
of uniform ellipsoids in a medium of index n_med.  Its scattering potential
f = -k0^2 (n^2 - n_med^2) has the closed-form 3-D Fourier transform of an affine
image of the unit ball, V * 3 (sin x - x cos x) / x^3.  For each illumination
angle the first-order Rytov field is built from the Fourier diffraction relation
that the reference's mapping inverts (cTDM/Recon_kernel.cu:187-229,
cTDM/HilbertTransform.cu:1839-1862):

    DFT2(u)[nu] * dx^2 = f_hat(nu_x, nu_y, f_z - f_z0) / (i 4 pi f_z),
    f_z = sqrt(fm0^2 - (nu_x + f_x0)^2 - (nu_y + f_y0)^2),

with f_x0 = fm0 sin(AngY), f_y0 = fm0 sin(AngX) and the transpose/ifftshift
convention of CopyDataArray + cuFFT2Dshift, so that the reference algorithm maps
it back onto the phantom.  Holograms are I = I0 |exp(-i 2 pi f_R . r) + exp(u)|^2
with the carrier f_R at a quarter of Nyquist on both axes; the sign makes the
order the reference selects (rows past 600/1024 of the shifted spectrum) carry
exp(u), so the phase arg BG - arg SP equals Im u.  Poisson noise at a mean of
`photons` counts per pixel.
"""
from dataclasses import dataclass, field
from typing import List, Tuple

import numpy as np


@dataclass
class Ellipsoid:
    center: Tuple[float, float, float]   # (x, y, z) in metres, volume frame
    semi: Tuple[float, float, float]     # semi-axes (a, b, c) in metres
    n: float                             # refractive index inside
    rot: float = 0.0                     # rotation about z (radians)


@dataclass
class Acquisition:
    holograms: np.ndarray                # (A, N, N) float32, [angle, y, x]
    background: np.ndarray               # (N, N) float32
    ang_x: np.ndarray                    # (A,) float32 radians (reference AngX)
    ang_y: np.ndarray                    # (A,) float32 radians (reference AngY)
    n_holo: int
    m_crop: int
    r_vol: int
    pixel: float                         # hologram pixel (m) = reconstruction dx
    wavelength: float
    n_med: float
    ellipsoids: List[Ellipsoid] = field(default_factory=list)

    @property
    def fm0(self):
        return self.n_med / self.wavelength

    @property
    def dx(self):
        return self.pixel

    @property
    def df(self):
        return 1.0 / (self.r_vol * self.dx)

    @property
    def k2(self):
        k = 2 * np.pi * self.n_med / self.wavelength
        return k * k


def cone_angles(count, na, n_med):
    """Illumination on a circular cone with n_med sin(theta) = na, azimuths
    2 pi a / count.  Returns (AngX, AngY) in the reference's convention."""
    s = na / n_med
    phi = 2 * np.pi * np.arange(count) / count
    ang_y = np.arcsin(s * np.cos(phi))   # f_x0 = fm0 sin(AngY)
    ang_x = np.arcsin(s * np.sin(phi))   # f_y0 = fm0 sin(AngX)
    return ang_x.astype(np.float32), ang_y.astype(np.float32)


def potential_hat(ells, n_med, wavelength, kx, ky, kz):
    """Analytic 3-D FT (exp(-i 2 pi k.r)) of f = -k0^2 (n^2 - n_med^2) for nested
    ellipsoids: each ellipsoid contributes its index step over the previous
    (enclosing) one."""
    k0 = 2 * np.pi / wavelength
    out = np.zeros(np.broadcast(kx, ky, kz).shape, np.complex128)
    for idx, e in enumerate(ells):
        base = n_med if idx == 0 else ells[0].n
        df_step = -k0 * k0 * (e.n ** 2 - base ** 2)
        c, s = np.cos(e.rot), np.sin(e.rot)
        ux = c * kx + s * ky
        uy = -s * kx + c * ky
        a, b, cc = e.semi
        q = 2 * np.pi * np.sqrt((a * ux) ** 2 + (b * uy) ** 2 + (cc * kz) ** 2)
        vol = 4.0 / 3.0 * np.pi * a * b * cc
        with np.errstate(divide="ignore", invalid="ignore"):
            shape = np.where(q < 1e-6, 1.0 - q * q / 10.0, 3.0 * (np.sin(q) - q * np.cos(q)) / q ** 3)
        phase = np.exp(-2j * np.pi * (kx * e.center[0] + ky * e.center[1] + kz * e.center[2]))
        out += df_step * vol * shape * phase
    return out


def rytov_field(ells, n_med, wavelength, n, pixel, ang_x, ang_y):
    """Complex Rytov phase u on the N x N hologram grid, [y, x] layout."""
    fm0 = n_med / wavelength
    fx0 = fm0 * np.sin(float(ang_y))
    fy0 = fm0 * np.sin(float(ang_x))
    fz0 = np.sqrt(fm0 * fm0 - fx0 * fx0 - fy0 * fy0)
    dfh = 1.0 / (n * pixel)
    sgn = np.fft.fftfreq(n, 1.0 / n)           # signed bin index
    nx = sgn[None, :] * dfh                    # volume-frame x frequency (fast DFT index)
    ny = sgn[:, None] * dfh
    rad = fm0 * fm0 - (nx + fx0) ** 2 - (ny + fy0) ** 2
    ok = rad > 0
    iy, ix = np.nonzero(ok)                    # the field spectrum lives on the Ewald cap only
    kx, ky = nx[0, ix], ny[iy, 0]
    fz = np.sqrt(rad[iy, ix])
    fhat = potential_hat(ells, n_med, wavelength, kx, ky, fz - fz0)
    spec = np.zeros((n, n), np.complex128)
    spec[iy, ix] = fhat / (1j * 4 * np.pi * fz) / (pixel * pixel)
    ut_shift = np.fft.ifft2(spec)              # DFT2(u_shifted) = spec, [Ny, Nx] layout
    ut = np.fft.fftshift(ut_shift)             # undo the quadrant swap
    return ut.T                                # CopyDataArray transposes: hologram [y, x]


def intensity(u, photons, carrier=(0.125, 0.125)):
    """Mean photon counts I0 |exp(-i 2 pi f_R . r) + exp(u)|^2 of one off-axis hologram
    (float64, before the shot noise)."""
    n = u.shape[-1]
    yy, xx = np.mgrid[0:n, 0:n]
    ref = np.exp(-2j * np.pi * (carrier[0] * xx + carrier[1] * yy))
    return (photons / 2.0) * np.abs(ref + np.exp(u)) ** 2


def holograms_from_fields(fields, photons, rng, carrier=(0.125, 0.125)):
    """Off-axis holograms; carrier (cycles per pixel along x, y), by default a quarter
    of Nyquist on both axes (the 2-D window of Algorithm A); Algorithm B filters along
    x only and wants the carrier along x, e.g. (0.25, 0)."""
    return noisy(np.stack([intensity(u, photons, carrier) for u in fields]), photons, rng)


def noisy(intens, photons, rng):
    """Poisson shot noise on mean counts (angle by angle, in order, from rng)."""
    return np.stack([rng.poisson(i).astype(np.float32) if photons > 0 else i.astype(np.float32) for i in intens])


def _intensities(args):
    """Worker: mean counts of a run of angles (fields are deterministic)."""
    ells, n_med, wavelength, n, pixel, ax, ay, photons, carrier = args
    return np.stack([intensity(rytov_field(ells, n_med, wavelength, n, pixel, ax[k], ay[k]), photons, carrier)
                     for k in range(len(ax))])


def cell_phantom(rng, scale=1.0, n_cell=1.37, n_nuc=1.39, semi=(4e-6, 3e-6, 2.5e-6), nucleoli=3):
    ells = [Ellipsoid((0.0, 0.0, 0.0), tuple(s * scale for s in semi), n_cell, rot=0.3)]
    for _ in range(nucleoli):
        r = rng.uniform(0.5e-6, 1.0e-6) * scale
        lim = [max(s * scale - r, 0) * 0.5 for s in semi]
        c = tuple(rng.uniform(-l, l) for l in lim)
        ells.append(Ellipsoid(c, (r, r, r), n_nuc))
    return ells


def random_cell(rng, fov):
    """2-6 ellipsoids with RI U[1.35, 1.40] inside an envelope ellipsoid."""
    k = int(rng.integers(2, 7))
    env = (rng.uniform(0.12, 0.18) * fov, rng.uniform(0.1, 0.15) * fov, rng.uniform(0.08, 0.12) * fov)
    ells = [Ellipsoid((0.0, 0.0, 0.0), env, float(rng.uniform(1.35, 1.40)), rot=float(rng.uniform(0, np.pi)))]
    for _ in range(k - 1):
        r = rng.uniform(0.1, 0.3) * min(env)
        c = tuple(float(rng.uniform(-0.4, 0.4) * e) for e in env)
        ells.append(Ellipsoid(c, (r, r * rng.uniform(0.7, 1.0), r * rng.uniform(0.7, 1.0)),
                              float(rng.uniform(1.35, 1.40))))
    return ells


def scan_angles(count, na, n_med):
    """A one-axis scan: AngX evenly over [-asin(NA / n_med), asin(NA / n_med)], AngY = 0
    (the scan the frequency-interpolation mapping of BatchReconPOCS assumes)."""
    t = np.arcsin(na / n_med)
    return np.linspace(-t, t, count).astype(np.float32), np.zeros(count, np.float32)


def acquisition(n, r, angles, na=0.9, seed=0, pixel=0.1e-6, wavelength=532e-9, n_med=1.337,
                photons=1000.0, ells=None, scale=1.0, carrier=(0.125, 0.125), scan="cone", workers=1, **cell):
    """One tomogram: `angles` SP holograms of N x N plus one background; scan "cone"
    (illumination on a circular cone) or "line" (a one-axis AngX scan).  workers > 1
    computes the fields in that many spawned processes (the same holograms)."""
    rng = np.random.default_rng(seed)
    if ells is None:
        ells = cell_phantom(rng, scale=scale, **cell)
    ax, ay = (cone_angles if scan == "cone" else scan_angles)(angles, na, n_med)
    if workers > 1 and angles > 1:
        import concurrent.futures as cf
        import multiprocessing as mp
        runs = [c for c in np.array_split(np.arange(angles), workers) if len(c)]
        jobs = [(ells, n_med, wavelength, n, pixel, ax[c], ay[c], photons, carrier) for c in runs]
        with cf.ProcessPoolExecutor(len(jobs), mp_context=mp.get_context("spawn")) as ex:
            intens = np.concatenate(list(ex.map(_intensities, jobs)))
        holo = noisy(intens, photons, rng)
        del intens
    else:
        fields = np.stack([rytov_field(ells, n_med, wavelength, n, pixel, ax[a], ay[a]) for a in range(angles)])
        holo = holograms_from_fields(fields, photons, rng, carrier)
    bg = holograms_from_fields(np.zeros((1, n, n), np.complex128), photons, rng, carrier)[0]
    return Acquisition(holo, bg, ax, ay, n, n // 4, r, pixel, wavelength, n_med, ells)


# Workloads with the shapes of the benchmark configurations ------------------
def config_plain_small(seed=1000, angles=49):
    """49 x 256^2 holograms -> 256^3, NA 0.9, pixel 0.1 um (the plain small case)."""
    return acquisition(256, 256, angles, na=0.9, seed=seed)


def config_wrap_heavy(seed=2000, angles=121):
    """121 x 1024^2 holograms cropped to 256^2 spectra -> 256^3; RI 1.40, 10 um thick."""
    return acquisition(1024, 256, angles, na=0.9, seed=seed, n_cell=1.40, n_nuc=1.40,
                       semi=(7e-6, 5e-6, 5e-6), nucleoli=3)


def small_case(seed=7, n=64, r=64, angles=6, na=0.9, pixel=0.4e-6, photons=1000.0):
    """Tiny acquisition for parity tests: FOV 25.6 um at 0.4 um pixels."""
    return acquisition(n, r, angles, na=na, seed=seed, pixel=pixel, photons=photons)


def f2_truth(acq, r=None, chunk=16):
    """The phantom's scattering potential on the reconstruction's k-space grid, in
    the layout and scale of the measured data F2 (x fastest; signed frequency index
    ii at x = ii mod R; F2 = f_hat / dx^3, the scale the Ewald mapping gives the
    measured samples).  Every voxel is filled, so the positivity path with zero loop
    bodies turns it into the phantom's band-limited RI volume (the ground truth for
    error against the phantom).  complex64 (R, R, R) as [z][y][x]."""
    r = r or acq.r_vol
    df = 1.0 / (r * acq.dx)
    sgn = np.fft.fftfreq(r, 1.0 / r) * df
    ky, kx = np.meshgrid(sgn, sgn, indexing="ij")     # [y][x]
    out = np.empty((r, r, r), np.complex64)
    scale = 1.0 / acq.dx ** 3
    for z0 in range(0, r, chunk):
        kz = sgn[z0:z0 + chunk][:, None, None]
        out[z0:z0 + chunk] = (potential_hat(acq.ellipsoids, acq.n_med, acq.wavelength, kx[None], ky[None], kz)
                              * scale).astype(np.complex64)
    return out
