"""FP64 restatement of the differentiable Fourier-domain ODT (test infrastructure only).

This is the checker for the library's ctdm_tape / ctdm_forward / ctdm_backward /
ctdm_loss_grad / ctdm_reconstruct_gradient entry points.  It is imported only by
the tests; the library never calls it.  The reference has no counterpart (it
only has the positivity loop, cTDM/Recon_kernel.cu:est_n_3D / modify_F_3D /
check_F_3D), so this module is pinned by its own finite-difference and
adjoint-identity checks instead of reference vectors.

Conventions (all arrays (R, R, R) complex128, flat index x + R y + R^2 z, i.e.
numpy shape [z, y, x]):

* A V = P F~ V, F~ the unitary 3-D DFT (numpy ``norm="ortho"``), P the sampling
  at the ascending measured-voxel indices ``idx``.
* Data y = F2[idx] / (-k^2 R^{3/2}) where F2 is the Ewald-mapped spectrum
  (cTDM/Recon_kernel.cu:EdwardSphere) -- then V = f / (-k^2) and
  n = n_med sqrt(1 + V).
* L(V) = 1/2 ||A V - y||^2 + lambda TV_eps(V),
  TV_eps = sum_voxels sqrt(|Dx V|^2 + |Dy V|^2 + |Dz V|^2 + eps^2) with forward
  differences that are zero past the last index.
* Gradients are conjugate-Wirtinger: dL/dRe V + i dL/dIm V.
"""
import numpy as np


def measured_indices(F2=None, counts=None):
    """Ascending flat indices of the measured voxels (hit mask, else F2 predicate)."""
    if counts is not None:
        return np.flatnonzero(np.asarray(counts).ravel() != 0).astype(np.uint32)
    f = np.asarray(F2).ravel()
    return np.flatnonzero((f.real != 0) & (f.imag != 0)).astype(np.uint32)


def tape_data(F2, idx, r, k2):
    return np.asarray(F2).ravel()[idx].astype(np.complex128) / (-k2 * r ** 1.5)


def forward(V, idx):
    return np.fft.fftn(np.asarray(V, np.complex128), norm="ortho").ravel()[idx]


def adjoint(g, idx, r):
    vol = np.zeros(r ** 3, np.complex128)
    vol[idx] = g
    return np.fft.ifftn(vol.reshape(r, r, r), norm="ortho")


def _diffs(V):
    V = np.asarray(V, np.complex128)
    dx = np.zeros_like(V)
    dy = np.zeros_like(V)
    dz = np.zeros_like(V)
    dx[:, :, :-1] = V[:, :, 1:] - V[:, :, :-1]
    dy[:, :-1, :] = V[:, 1:, :] - V[:, :-1, :]
    dz[:-1, :, :] = V[1:, :, :] - V[:-1, :, :]
    return dx, dy, dz


def tv(V, eps):
    dx, dy, dz = _diffs(V)
    return float(np.sum(np.sqrt(np.abs(dx) ** 2 + np.abs(dy) ** 2 + np.abs(dz) ** 2 + eps * eps)))


def tv_grad(V, eps):
    """-div(grad V / |grad V|_eps) with backward differences (adjoint of the forward ones)."""
    dx, dy, dz = _diffs(V)
    mag = np.sqrt(np.abs(dx) ** 2 + np.abs(dy) ** 2 + np.abs(dz) ** 2 + eps * eps)
    px, py, pz = dx / mag, dy / mag, dz / mag
    g = -(px + py + pz)
    g[:, :, 1:] += px[:, :, :-1]
    g[:, 1:, :] += py[:, :-1, :]
    g[1:, :, :] += pz[:-1, :, :]
    return g


def loss(V, idx, y, lam=0.0, eps=1e-4):
    r = forward(V, idx) - y
    out = 0.5 * float(np.vdot(r, r).real)
    if lam:
        out += lam * tv(V, eps)
    return out


def loss_grad(V, idx, y, lam=0.0, eps=1e-4):
    R = np.asarray(V).shape[0]
    r = forward(V, idx) - y
    g = adjoint(r, idx, R)
    L = 0.5 * float(np.vdot(r, r).real)
    if lam:
        g = g + lam * tv_grad(V, eps)
        L += lam * tv(V, eps)
    return L, g


def project_positivity(V):
    """Contrast V projected onto the positivity set of the est_n clamp: s = sqrt(1 + V)
    (principal root), s' = (max(Re s, 1), max(Im s, 0)), V' = s'^2 - 1."""
    s = np.sqrt(1.0 + np.asarray(V, np.complex128))
    s = np.maximum(s.real, 1.0) + 1j * np.maximum(s.imag, 0.0)
    return s * s - 1.0


def fista(V0, idx, y, iterations, lam=0.0, eps=1e-4, step=None, positivity=False):
    """Accelerated gradient descent in the form the library runs:
    V+ = W - tau grad L(W) (projected onto the positivity set when asked);
    W = V+ + (t_k - 1)/t_{k+1} (V+ - V).  Returns (V, losses at W)."""
    tau = step if step else 1.0 / (1.0 + 12.0 * lam / eps)
    V = np.asarray(V0, np.complex128).copy()
    W = V.copy()
    t = 1.0
    hist = []
    for _ in range(iterations):
        L, g = loss_grad(W, idx, y, lam, eps)
        hist.append(L)
        tn = 0.5 * (1.0 + np.sqrt(1.0 + 4.0 * t * t))
        Vn = W - tau * g
        if positivity:
            Vn = project_positivity(Vn)
        W = Vn + ((t - 1.0) / tn) * (Vn - V)
        V = Vn
        t = tn
    return V, np.array(hist)


def contrast_to_ri(V, n_med, clamp=False):
    """n = n_med sqrt(1 + V), optional clamp (n.re >= n_med, n.im >= 0), octant shift
    (cTDM/FFT.cu:cuFFT3Dshift)."""
    n = n_med * np.sqrt(1.0 + np.asarray(V, np.complex128))
    if clamp:
        n = np.maximum(n.real, n_med) + 1j * np.maximum(n.imag, 0.0)
    R = n.shape[0]
    return np.roll(n, (R // 2, R // 2, R // 2), axis=(0, 1, 2))
