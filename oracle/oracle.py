"""ctypes wrapper around the FP64 oracle (oracle/_build/libctdm_oracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, by the smoke check and by the
CPU-baseline leg of bench.py.  The product package never imports this module.

Arrays are numpy, x-fastest like the reference: a 2-D image of width W and
height H is an (H, W) array; a volume is (R, R, R) indexed [z, y, x].
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SO = os.path.join(_HERE, "_build", "libctdm_oracle.so")
_lib = None


def build(force=False):
    """Compile the oracle with its Makefile (gcc, OpenMP)."""
    src = os.path.join(_HERE, "ctdm_oracle.c")
    if force or not os.path.exists(_SO) or os.path.getmtime(_SO) < os.path.getmtime(src):
        subprocess.check_call(["make", "-s", "-C", _HERE], stdout=subprocess.DEVNULL)
    return _SO


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(_SO)
        _lib.or_carrier_start_row.restype = ctypes.c_int
        _lib.or_goldstein_floodfill.restype = ctypes.c_int
        _lib.or_get_threads.restype = ctypes.c_int
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _c128(a):
    return np.ascontiguousarray(a, dtype=np.complex128)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


class Params(ctypes.Structure):
    _fields_ = [
        ("n", ctypes.c_int), ("m", ctypes.c_int), ("r", ctypes.c_int), ("iters", ctypes.c_int),
        ("unwrap_mode", ctypes.c_int), ("check_mode", ctypes.c_int),
        ("carrier_r", ctypes.c_int), ("carrier_c", ctypes.c_int), ("carrier_radius", ctypes.c_int),
        ("fm0", ctypes.c_double), ("df", ctypes.c_double), ("dx", ctypes.c_double),
        ("k2", ctypes.c_double), ("n_med", ctypes.c_double), ("qpi_method", ctypes.c_int),
    ]


def set_threads(n):
    lib().or_set_threads(int(n))


def get_threads():
    return lib().or_get_threads()


# ---- FFT -------------------------------------------------------------------
def fft2(a, sign=-1):
    a = _c128(a).copy()
    h, w = a.shape
    lib().or_fft2d(_p(a), w, h, int(sign))
    return a


def fft3(a, direction):
    a = _c128(a).copy()
    r = a.shape[0]
    lib().or_fft3d(_p(a), a.shape[2], a.shape[1], a.shape[0], int(direction))
    return a


def shift3d(a):
    """Octant swap of a (nz, ny, nx) complex volume (or_shift3d)."""
    a = _c128(a)
    out = np.empty_like(a)
    lib().or_shift3d(_p(a), _p(out), a.shape[2], a.shape[1], a.shape[0])
    return out


# ---- QPI -------------------------------------------------------------------
def carrier_start_row(n):
    return lib().or_carrier_start_row(int(n))


def qpi_carrier(bg):
    bg = _f32(bg)
    r, c, rad = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    lib().or_qpi_carrier(_p(bg), bg.shape[0], ctypes.byref(r), ctypes.byref(c), ctypes.byref(rad))
    return r.value, c.value, rad.value


def qpi_field(holo, m, r, c, radius):
    holo = _f32(holo)
    out = np.zeros((m, m), np.complex128)
    lib().or_qpi_field(_p(holo), holo.shape[0], int(m), int(r), int(c), int(radius), _p(out))
    return out


def qpib_center(holo):
    """Algorithm B carrier column from the column histogram of the row spectra."""
    holo = _f32(holo)
    return int(lib().or_qpib_center(_p(holo), holo.shape[0]))


def qpib_field(holo, center):
    """Algorithm B field (M x M, M = N/4) for the given carrier column."""
    holo = _f32(holo)
    m = holo.shape[0] // 4
    out = np.zeros((m, m), np.complex128)
    lib().or_qpib_field(_p(holo), holo.shape[0], int(center), _p(out))
    return out


def wrap_phase(sp, bg):
    sp, bg = _c128(sp), _c128(bg)
    ph = np.zeros(sp.shape, np.float64)
    am = np.zeros(sp.shape, np.float64)
    lib().or_wrap_phase(_p(sp), _p(bg), sp.size, _p(ph), _p(am))
    return ph, am


# ---- DCT unwrap ------------------------------------------------------------
def wrapped_laplacian(phi):
    phi = _f64(phi)
    out = np.zeros_like(phi)
    lib().or_wrapped_laplacian(_p(phi), phi.shape[1], phi.shape[0], _p(out))
    return out


def dct2d(a):
    a = _f64(a).copy()
    lib().or_dct2d(_p(a), a.shape[1], a.shape[0])
    return a


def idct2d(a, mode):
    a = _f64(a).copy()
    lib().or_idct2d(_p(a), a.shape[1], a.shape[0], int(mode))
    return a


def poisson_divide(a):
    a = _f64(a).copy()
    lib().or_poisson_divide(_p(a), a.shape[1], a.shape[0])
    return a


def dct_unwrap(phi, mode):
    phi = _f64(phi)
    out = np.zeros_like(phi)
    lib().or_dct_unwrap(_p(phi), phi.shape[1], phi.shape[0], int(mode), _p(out))
    return out


def fast_unwrap(phi):
    """Returns (unwrapped, normalised_input) -- the input is rescaled in place like
    the reference's PhaseNormalize."""
    phi = _f64(phi).copy()
    out = np.zeros_like(phi)
    lib().or_fast_unwrap(_p(phi), phi.shape[1], phi.shape[0], _p(out))
    return out, phi


# ---- Goldstein -------------------------------------------------------------
def goldstein_residues(phi):
    phi = _f32(phi)
    out = np.zeros(phi.shape, np.int8)
    lib().or_goldstein_residues(_p(phi), phi.shape[1], phi.shape[0], _p(out))
    return out


def goldstein_cuts(charges):
    charges = np.ascontiguousarray(charges, np.int8)
    out = np.zeros(charges.shape, np.uint8)
    lib().or_goldstein_cuts(_p(charges), charges.shape[1], charges.shape[0], _p(out))
    return out


def goldstein_floodfill(cuts, phi):
    cuts = np.ascontiguousarray(cuts, np.uint8)
    phi = _f32(phi)
    out = np.zeros(phi.shape, np.float32)
    ub = np.zeros(phi.shape, np.uint8)
    st = lib().or_goldstein_floodfill(_p(cuts), _p(phi), phi.shape[1], phi.shape[0], _p(out), _p(ub))
    return out, ub, st


def goldstein(phi):
    q = goldstein_residues(phi)
    cuts = goldstein_cuts(q)
    out, ub, st = goldstein_floodfill(cuts, phi)
    return q, cuts, out, st


# ---- stack / spectra / mapping / loop --------------------------------------
def resize_crop(ph, am, n2, r):
    ph, am = _f64(ph), _f64(am)
    m1 = ph.shape[1]
    po = np.zeros((r, r), np.float64)
    ao = np.zeros((r, r), np.float64)
    lib().or_resize_crop(_p(ph), _p(am), m1, ph.shape[0], int(n2), int(n2), int(r), _p(po), _p(ao))
    return po, ao


def median_check(ph, am):
    ph, am = _f64(ph), _f64(am)
    po, ao = np.zeros_like(ph), np.zeros_like(am)
    lib().or_median_check(_p(ph), _p(am), ph.shape[1], ph.shape[0], _p(po), _p(ao))
    return po, ao


def rytov_spectrum(ph, am):
    ph, am = _f64(ph), _f64(am)
    u = np.zeros(ph.shape, np.complex128)
    lib().or_rytov_spectrum(_p(ph), _p(am), ph.shape[0], _p(u))
    return u


def ewald_index(r, fm0, df, angx, angy):
    vox = np.zeros(r * r, np.int64)
    fz = np.zeros(r * r, np.float64)
    lib().or_ewald_index(int(r), ctypes.c_double(fm0), ctypes.c_double(df), ctypes.c_double(angx),
                         ctypes.c_double(angy), _p(vox), _p(fz))
    return vox, fz


def ewald_map(U, angx, angy, fm0, df, dx):
    U = _c128(U)
    na, r = U.shape[0], U.shape[1]
    F2 = np.zeros((r, r, r), np.complex128)
    C = np.zeros((r, r, r), np.uint32)
    angx, angy = _f32(angx), _f32(angy)
    lib().or_ewald_map(_p(U), _p(angx), _p(angy), na, r, ctypes.c_double(fm0), ctypes.c_double(df),
                       ctypes.c_double(dx), _p(F2), _p(C))
    return F2, C


def positivity(F2, counts, iters, k2, n_med, check_mode=0):
    F2 = _c128(F2)
    r = F2.shape[0]
    counts = np.ascontiguousarray(counts, np.uint32)
    out = np.zeros_like(F2)
    lib().or_positivity(_p(F2), _p(counts), r, int(iters), ctypes.c_double(k2), ctypes.c_double(n_med),
                        int(check_mode), _p(out))
    return out


def make_params(n, m, r, iters, fm0, df, dx, k2, n_med, unwrap_mode=0, check_mode=0, carrier=None, qpi_method=1):
    """qpi_method in the reference's numbering: 0 Algorithm B, 1 Algorithm A."""
    p = Params()
    p.qpi_method = qpi_method
    p.n, p.m, p.r, p.iters = n, m, r, iters
    p.unwrap_mode, p.check_mode = unwrap_mode, check_mode
    cr, cc, rad = carrier if carrier is not None else (-1, -1, -1)
    p.carrier_r, p.carrier_c, p.carrier_radius = cr, cc, rad
    p.fm0, p.df, p.dx, p.k2, p.n_med = fm0, df, dx, k2, n_med
    return p


def front_end(params, sp, bg, bg_per_angle=False):
    sp, bg = _f32(sp), _f32(bg)
    na = sp.shape[0]
    r = params.r
    ph = np.zeros((na, r, r), np.float64)
    am = np.zeros((na, r, r), np.float64)
    car = (ctypes.c_int * 3)()
    lib().or_front_end(ctypes.byref(params), _p(sp), _p(bg), na, int(bg_per_angle), _p(ph), _p(am), car)
    return ph, am, tuple(car)


def pipeline(params, sp, bg, angx, angy, bg_per_angle=False):
    sp, bg = _f32(sp), _f32(bg)
    angx, angy = _f32(angx), _f32(angy)
    na = sp.shape[0]
    r = params.r
    out = np.zeros((r, r, r), np.complex128)
    car = (ctypes.c_int * 3)()
    lib().or_pipeline(ctypes.byref(params), _p(sp), _p(bg), na, int(bg_per_angle), _p(angx), _p(angy),
                      _p(out), car)
    return out, tuple(car)


def tomogram(params, sp, bg, angx, angy, run_goldstein=False, want_charges=False):
    """A whole tomogram (the timed CPU baseline): the per-angle chain in parallel over
    the angles, Goldstein on every angle when run_goldstein, then the mapping and the
    loop.  Returns (volume, carrier, charges or None)."""
    sp, bg = _f32(sp), _f32(bg)
    angx, angy = _f32(angx), _f32(angy)
    na = sp.shape[0]
    r, m = params.r, params.m
    out = np.zeros((r, r, r), np.complex128)
    car = (ctypes.c_int * 3)()
    q = np.zeros((na, m, m), np.int8) if want_charges else None
    lib().or_tomogram(ctypes.byref(params), _p(sp), _p(bg), na, _p(angx), _p(angy), int(run_goldstein), _p(out),
                      _p(q) if q is not None else None, car)
    return out, tuple(car), q


# ---- job driver pieces (numpy restatements) ------------------------------------------
def angcal_peak(img):
    """AngCal_GPU (cTDM/HilbertTransform.cu:2920-2983): flat index of the first maximum
    of log10 |FFT2(img)| (quadrant-swapped, NaN/inf -> 0, cufftComplex2Real :2986-2996)
    over [int(0.53 N^2), int(0.79 N^2)).  img: (N, N) picture, x fastest."""
    img = np.asarray(img, np.float64)
    n = img.shape[0]
    spec = np.fft.fftshift(np.fft.fft2(img))
    with np.errstate(divide="ignore"):
        m = np.log10(np.abs(spec)).astype(np.float32)
    m[~np.isfinite(m)] = 0
    lo, hi = int(n * n * 0.53), int(n * n * 0.79)
    return lo + int(np.argmax(m.ravel()[lo:hi]))


def angcal_angle(peak, n, n_med, wavelength_nm, mag, camera_pixel_um):
    """The angle AngCal_GPU derives from the peak column (float32 as written, with its
    511 and 1024 read as N/2 - 1 and N)."""
    posx = peak % n
    fm = np.float32(n_med / (wavelength_nm * 1e-9))
    fx = np.float32((n // 2 - 1 - posx) * 1 / (n * camera_pixel_um * 1e-6))
    st = np.float32(np.float32(mag) * fx / fm)
    a = abs(float(np.arcsin(np.float64(st))))
    return np.float32(a if st < 0 else -a)


def check_array(values, limit_std, limit_range):
    """checkArray (cTDM/HilbertTransform.cu:3056-3092): True when the population standard
    deviation exceeds limit_std or the range exceeds limit_range."""
    v = np.asarray(values, np.float32).ravel()
    mean = float(np.sum(v.astype(np.float64))) / v.size
    std = float(np.sqrt(np.sum((v.astype(np.float64) - mean) ** 2) / v.size))
    rng = abs(np.float32(v.max()) - np.float32(v.min()))
    return bool(std > np.float32(limit_std) or rng > np.float32(limit_range))


def check_frame(phase, resize_flag, limit_std, limit_range):
    """The job loop's frame check (cTDM/HilbertTransform.cu:1087-1120): the centre half
    of the map for ResizeFlag 1, the whole map with 0.5 and 5 pi for 0."""
    ph = np.asarray(phase, np.float32)
    n = ph.shape[0]
    if resize_flag == 0:
        return check_array(ph, 0.5, 5 * np.pi)
    return check_array(ph[n // 4:3 * n // 4, n // 4:3 * n // 4], limit_std, limit_range)


# ---- frequency interpolation and ASD-POCS ------------------------------------------
class PocsParams(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int), ("tv_steps", ctypes.c_int), ("beta", ctypes.c_double),
                ("beta_red", ctypes.c_double), ("alpha", ctypes.c_double), ("alpha_red", ctypes.c_double),
                ("r_max", ctypes.c_double), ("eps_data", ctypes.c_double), ("tv_eps", ctypes.c_double)]


def pocs_params(iterations=100, tv_steps=20, beta=1.0, beta_red=0.995, alpha=0.2, alpha_red=0.95, r_max=0.95,
                eps_data=0.0, tv_eps=1e-8):
    return PocsParams(iterations, tv_steps, beta, beta_red, alpha, alpha_red, r_max, eps_data, tv_eps)


def fi_map(U, angx, fm0, df, dx):
    """Frequency-interpolation mapping of A spectra (A, R, R) for the AngX scan."""
    U = _c128(U)
    na, r = U.shape[0], U.shape[1]
    F2 = np.zeros((r, r, r), np.complex128)
    C = np.zeros((r, r, r), np.uint32)
    angx = _f32(angx)
    lib().or_fi_map(_p(U), _p(angx), na, r, ctypes.c_double(fm0), ctypes.c_double(df), ctypes.c_double(dx),
                    _p(F2), _p(C))
    return F2, C


def pocs(F2, params, k2, n_med, want_dd=True):
    """ASD-POCS from F2; returns (octant-shifted n, history (iterations, 4))."""
    F2 = _c128(F2)
    r = F2.shape[0]
    out = np.zeros_like(F2)
    hist = np.zeros((max(params.iterations, 1), 4), np.float64)
    lib().or_pocs(_p(F2), r, ctypes.byref(params), ctypes.c_double(k2), ctypes.c_double(n_med), int(want_dd),
                  _p(out), _p(hist))
    return out, hist[:params.iterations]


def bilinear(img, m2, n2):
    """bilinear (cTDM/HilbertTransform.cu:2404-2435): (N1, M1) float32 image -> (N2, M2),
    ratios (M1 - 1) / M2 and (N1 - 1) / N2, float32 arithmetic as written."""
    a = np.asarray(img, np.float32)
    n1, m1 = a.shape
    xr = np.float32(m1 - 1) / np.float32(m2)
    yr = np.float32(n1 - 1) / np.float32(n2)
    j = np.arange(m2, dtype=np.float32)
    i = np.arange(n2, dtype=np.float32)
    xs = (xr * j).astype(np.float32)
    ys = (yr * i).astype(np.float32)
    x = xs.astype(np.int64)
    y = ys.astype(np.int64)
    xd = (xs - x.astype(np.float32)).astype(np.float32)[None, :]
    yd = (ys - y.astype(np.float32)).astype(np.float32)[:, None]
    A = a[y[:, None], x[None, :]]
    B = a[y[:, None], x[None, :] + 1]
    C = a[y[:, None] + 1, x[None, :]]
    D = a[y[:, None] + 1, x[None, :] + 1]
    one = np.float32(1)
    out = A * (one - xd) * (one - yd) + B * xd * (one - yd) + C * yd * (one - xd) + D * (xd * yd)
    return out.astype(np.float32)
