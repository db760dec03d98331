"""GB300-native cTDM hologram -> refractive-index reconstruction.

Python host side over the C ABI of libctdm_gb300.so (include/ctdm.h).  Device
memory is passed as raw pointers; torch CUDA tensors are accepted for
convenience (torch is used for allocation and streams only).  Nothing here runs
on the CPU: every call launches the library's CUDA kernels and fails loudly when
the library is missing.
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import CtdmError, Params, check, load  # noqa: F401

CTDM_UNWRAP_REF, CTDM_UNWRAP_EXACT = 0, 1
CTDM_CHECK_REF, CTDM_CHECK_MASK = 0, 1
CTDM_METHOD_DCT, CTDM_METHOD_FAST, CTDM_METHOD_GOLDSTEIN = 0, 1, 2
CTDM_QPI_B, CTDM_QPI_A = 0, 1


def _ptr(x):
    """Device (or host) address of a torch tensor, numpy array or int."""
    if x is None:
        return None
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        return x.data_ptr()
    if isinstance(x, np.ndarray):
        return x.ctypes.data
    raise TypeError(f"cannot take the address of {type(x)}")


def _stream(stream):
    if stream is None:
        return None
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream


def default_params(**kw):
    p = Params()
    load().ctdm_params_default(ctypes.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def params_for(acq, iterations, **kw):
    """Parameters matching a ctdm_gb300.phantom.Acquisition."""
    return default_params(n_holo=acq.n_holo, m_crop=acq.m_crop, r_vol=acq.r_vol, iterations=iterations,
                          n_med=acq.n_med, wavelength=acq.wavelength, dx=acq.dx, **kw)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


class Context:
    """A device context (ctdm_ctx): workspace, tables and the last carrier."""

    def __init__(self, device=0):
        self.lib = load()
        h = ctypes.c_void_p()
        check(self.lib.ctdm_ctx_create(int(device), ctypes.byref(h)), "ctdm_ctx_create")
        self.handle = h
        self.device = device

    def close(self):
        if self.handle:
            self.lib.ctdm_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- whole path ----------------------------------------------------------
    def reconstruct_device(self, params, holo, bg, angx, angy, out, stream=None):
        angx, angy = _f32(angx), _f32(angy)
        check(self.lib.ctdm_reconstruct_device(self.handle, ctypes.byref(params), len(angx), _ptr(holo), _ptr(bg),
                                               _ptr(angx), _ptr(angy), _ptr(out), _stream(stream)),
              "ctdm_reconstruct_device")

    def reconstruct(self, params, holo, bg, angx, angy, out=None):
        """Host arrays in, host RI volume (R, R, R) complex64 out.  uint16 / uint8 holograms
        (camera counts) are uploaded as they are and converted on the GPU."""
        kind = np.asarray(holo).dtype
        fn = {np.dtype(np.uint16): ("ctdm_reconstruct_u16", np.uint16),
              np.dtype(np.uint8): ("ctdm_reconstruct_u8", np.uint8)}.get(kind, ("ctdm_reconstruct", np.float32))
        holo = np.ascontiguousarray(holo, fn[1])
        bg = np.ascontiguousarray(bg, fn[1])
        angx, angy = _f32(angx), _f32(angy)
        r = params.r_vol
        if out is None:
            out = np.empty((r, r, r), np.complex64)
        check(getattr(self.lib, fn[0])(self.handle, ctypes.byref(params), len(angx), _ptr(holo), _ptr(bg),
                                       _ptr(angx), _ptr(angy), _ptr(out)), fn[0])
        return out

    def submit(self, params, holo, bg, angx, angy, out):
        """ctdm_submit: enqueue a host-buffer reconstruction into `out` and return.  The
        arrays (numpy, or pinned torch CPU tensors for overlapped copies) must stay alive
        and `out` unread until wait(); until then only submit() may use this context."""
        def ptr_dtype(a):
            if hasattr(a, "data_ptr"):
                return a.data_ptr(), {"torch.uint16": 2, "torch.uint8": 1, "torch.float32": 4}[str(a.dtype)]
            a = np.asarray(a)
            bpc = {np.dtype(np.uint16): 2, np.dtype(np.uint8): 1, np.dtype(np.float32): 4}[a.dtype]
            assert a.flags.c_contiguous
            return a.ctypes.data, bpc
        hp, bpc = ptr_dtype(holo)
        bp, bpc_bg = ptr_dtype(bg)
        op = out.data_ptr() if hasattr(out, "data_ptr") else np.asarray(out).ctypes.data
        if bpc != bpc_bg:
            raise ValueError("holograms and background must have the same type")
        angx, angy = _f32(angx), _f32(angy)
        check(self.lib.ctdm_submit(self.handle, ctypes.byref(params), len(angx), hp, bp, bpc, _ptr(angx), _ptr(angy),
                                   op), "ctdm_submit")

    def wait(self):
        check(self.lib.ctdm_wait(self.handle), "ctdm_wait")

    def carrier(self):
        c = (ctypes.c_int * 3)()
        check(self.lib.ctdm_ctx_carrier(self.handle, c), "ctdm_ctx_carrier")
        return tuple(c)

    STAGES = ("qpi", "unwrap", "goldstein", "spectra", "ewald", "y_inverse", "x_pass", "y_forward", "z_pass",
              "x_final")

    def set_timing(self, on=True):
        check(self.lib.ctdm_ctx_set_timing(self.handle, int(on)), "ctdm_ctx_set_timing")

    def stage_times(self):
        """{stage: (ms, launches)} summed over the pipeline calls made since set_timing(True)."""
        n = len(self.STAGES)
        ms = (ctypes.c_double * n)()
        cnt = (ctypes.c_int * n)()
        check(self.lib.ctdm_ctx_stage_times(self.handle, ms, cnt, n), "ctdm_ctx_stage_times")
        return {name: (ms[i], cnt[i]) for i, name in enumerate(self.STAGES)}

    def workspace(self):
        """Device bytes this context's workspace holds now."""
        b = ctypes.c_size_t()
        check(self.lib.ctdm_ctx_workspace(self.handle, ctypes.byref(b)), "ctdm_ctx_workspace")
        return b.value

    def device_status(self):
        """Status word of the bounded device-side waits (0 = none ran out); clears it."""
        st = ctypes.c_int()
        check(self.lib.ctdm_ctx_device_status(self.handle, ctypes.byref(st)), "ctdm_ctx_device_status")
        return st.value

    def probe_wait(self, polls=0):
        """One bounded device-side wait that nothing completes (code 9 in the status
        word); returns its length in ms.  polls <= 0: the production bound."""
        ms = ctypes.c_double()
        check(self.lib.ctdm_ctx_probe_wait(self.handle, int(polls), ctypes.byref(ms)), "ctdm_ctx_probe_wait")
        return ms.value

    def buffer(self, which):
        p, n = ctypes.c_void_p(), ctypes.c_size_t()
        check(self.lib.ctdm_ctx_buffer(self.handle, int(which), ctypes.byref(p), ctypes.byref(n)), "ctdm_ctx_buffer")
        return p.value, n.value

    def read_buffer(self, which, dtype):
        """Host copy of a context buffer (see ctdm_ctx_buffer) as a flat numpy array."""
        _, n = self.buffer(which)
        out = np.empty(n // np.dtype(dtype).itemsize, dtype)
        check(self.lib.ctdm_ctx_read_buffer(self.handle, int(which), out.ctypes.data, out.nbytes),
              "ctdm_ctx_read_buffer")
        return out

    # -- stages (device pointers) ----------------------------------------------
    def qpi(self, n, m, holo, bg, phase, amp, n_angles, bg_per_angle=False, carrier=(-1, -1, -1), stream=None):
        c = (ctypes.c_int * 3)(*carrier)
        check(self.lib.ctdm_qpi(self.handle, n, m, n_angles, _ptr(holo), _ptr(bg), int(bg_per_angle), c, _ptr(phase),
                                _ptr(amp), _stream(stream)), "ctdm_qpi")
        return tuple(c)

    def qpi_b(self, n, holo, bg, phase, amp, n_angles, bg_per_angle=False, center=(-1, -1), stream=None):
        """QPI Algorithm B; returns (background carrier column, frame-1 carrier column)."""
        c = (ctypes.c_int * 2)(*center)
        check(self.lib.ctdm_qpi_b(self.handle, n, n_angles, _ptr(holo), _ptr(bg), int(bg_per_angle), c, _ptr(phase),
                                  _ptr(amp), _stream(stream)), "ctdm_qpi_b")
        return tuple(c)

    def unwrap_dct(self, phi, out, n_maps, m, mode=CTDM_UNWRAP_REF, stream=None):
        check(self.lib.ctdm_unwrap_dct(self.handle, n_maps, m, mode, _ptr(phi), _ptr(out), _stream(stream)),
              "ctdm_unwrap_dct")

    def unwrap_fast(self, phi, out, n_maps, m, stream=None):
        check(self.lib.ctdm_unwrap_fast(self.handle, n_maps, m, _ptr(phi), _ptr(out), _stream(stream)),
              "ctdm_unwrap_fast")

    def goldstein(self, phi, charges, cuts, out, n_maps, w, h, stream=None):
        st = (ctypes.c_int * n_maps)()
        rc = self.lib.ctdm_goldstein(self.handle, n_maps, w, h, _ptr(phi), _ptr(charges), _ptr(cuts), _ptr(out), st,
                                     _stream(stream))
        if rc not in (0, 5):
            check(rc, "ctdm_goldstein")
        return list(st)

    def goldstein_fill(self, cuts, phi, out, n_maps, w, h, stream=None):
        st = (ctypes.c_int * n_maps)()
        check(self.lib.ctdm_goldstein_fill(self.handle, n_maps, w, h, _ptr(cuts), _ptr(phi), _ptr(out), st,
                                           _stream(stream)), "ctdm_goldstein_fill")
        return list(st)

    def prepare_spectra(self, phase, amp, U, n_angles, m, n, r, stream=None):
        check(self.lib.ctdm_prepare_spectra(self.handle, n_angles, m, n, r, _ptr(phase), _ptr(amp), _ptr(U),
                                            _stream(stream)), "ctdm_prepare_spectra")

    def stack_spectra(self, ph, am, U, n_angles, r, stream=None):
        check(self.lib.ctdm_stack_spectra(self.handle, n_angles, r, _ptr(ph), _ptr(am), _ptr(U), _stream(stream)),
              "ctdm_stack_spectra")

    def prepare_stack(self, phase, amp, ph_out, am_out, n_angles, m, n, r, stream=None):
        check(self.lib.ctdm_prepare_stack(self.handle, n_angles, m, n, r, _ptr(phase), _ptr(amp), _ptr(ph_out),
                                          _ptr(am_out), _stream(stream)), "ctdm_prepare_stack")

    def map_ewald(self, U, angx, angy, fm0, df, dx, F2, counts=None, stream=None):
        angx, angy = _f32(angx), _f32(angy)
        r = int(round(np.sqrt(U.numel() // len(angx)))) if hasattr(U, "numel") else U.shape[-1]
        check(self.lib.ctdm_map_ewald(self.handle, len(angx), r, _ptr(U), _ptr(angx), _ptr(angy), fm0, df, dx,
                                      _ptr(F2), _ptr(counts), _stream(stream)), "ctdm_map_ewald")

    def positivity(self, F2, r, iterations, k2, n_med, out, check_mode=CTDM_CHECK_REF, counts=None, stream=None,
                   accelerated=False):
        """The positivity loop from the mapped data F2 into out (octant-shifted RI);
        accelerated=True adds Nesterov momentum to the projection step (ctdm_positivity_ex)."""
        check(self.lib.ctdm_positivity_ex(self.handle, r, iterations, check_mode, int(accelerated), k2, n_med, _ptr(F2),
                                          _ptr(counts), _ptr(out), _stream(stream)), "ctdm_positivity_ex")

    def map_fi(self, U, angx, fm0, df, dx, F2, counts=None, stream=None):
        """Frequency-interpolation mapping of the AngX scan (BatchReconPOCS's FI)."""
        angx = _f32(angx)
        r = int(round(np.sqrt(U.numel() // len(angx)))) if hasattr(U, "numel") else U.shape[-1]
        check(self.lib.ctdm_map_fi(self.handle, len(angx), r, _ptr(U), _ptr(angx), fm0, df, dx, _ptr(F2),
                                   _ptr(counts), _stream(stream)), "ctdm_map_fi")

    def pocs(self, F2, r, k2, n_med, out, params=None, history=False, stream=None, **kw):
        """ASD-POCS from F2 into out (octant-shifted RI).  params: a PocsParams (default
        pocs_params(**kw)).  Returns the (iterations, 4) history (Dp, Dd, Dg, TV step)
        when history is true."""
        p = params if params is not None else pocs_params(**kw)
        hist = np.zeros((max(p.iterations, 1), 4), np.float64) if history else None
        check(self.lib.ctdm_pocs(self.handle, int(r), ctypes.byref(p), float(k2), float(n_med), _ptr(F2), _ptr(out),
                                 _ptr(hist), _stream(stream)), "ctdm_pocs")
        return hist[:p.iterations] if history else None


def pocs_params(**kw):
    """ctdm_pocs_params with the reference's constants, overridden by keywords."""
    p = _lib.PocsParams()
    load().ctdm_pocs_defaults(ctypes.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def launch_count():
    """Kernels launched by the library in this process so far."""
    return int(load().ctdm_launch_count())


def workspace_bytes(params, n_angles):
    """Upper bound of a context's device memory for one device-buffer reconstruction."""
    b = ctypes.c_size_t()
    check(load().ctdm_workspace_bytes(ctypes.byref(params), int(n_angles), ctypes.byref(b)), "ctdm_workspace_bytes")
    return b.value


def fft(data, dims, batch=1, inverse=False, stream=None):
    """Unnormalised in-place FFT of a device buffer (dims fastest-first)."""
    d = (ctypes.c_int * len(dims))(*dims)
    check(load().ctdm_fft(_ptr(data), len(dims), d, batch, int(inverse), _stream(stream)), "ctdm_fft")


def plan_count(r):
    """FFT plan variants of the loop passes for volume side r."""
    return int(load().ctdm_plan_count(int(r)))


def autotune(r, check_mode=CTDM_CHECK_REF, device=0):
    """Tune the loop passes for side r now: (variants (x, y, z), {(pass, variant): ms}).
    Where a plane pass exists, the dict also holds ("scheme", s) for s = 0, 1, 2: one
    iteration of each loop scheme."""
    v = (ctypes.c_int * 3)()
    ms = (ctypes.c_double * 12)(*([float("nan")] * 12))
    check(load().ctdm_autotune(int(device), int(r), int(check_mode), v, ms, 12), "ctdm_autotune")
    n = plan_count(r)
    out = {(p, k): ms[3 * p + k] for p in range(3) for k in range(n)}
    for sc in range(3):
        if ms[9 + sc] == ms[9 + sc]:
            out[("scheme", sc)] = ms[9 + sc]
    return tuple(v), out


def loop_scheme(r, device=0):
    """0: x / y / z / y line passes; 1, 2: plane + z passes (two plane-pass variants)."""
    s = ctypes.c_int()
    check(load().ctdm_loop_scheme(int(device), int(r), ctypes.byref(s)), "ctdm_loop_scheme")
    return s.value


def set_loop_scheme(r, scheme, device=0):
    check(load().ctdm_set_loop_scheme(int(device), int(r), int(scheme)), "ctdm_set_loop_scheme")


def set_fill_list_capacity(capacity):
    """Shared-memory list entries of the Goldstein flood fill (0: the default)."""
    check(load().ctdm_set_fill_list_capacity(int(capacity)), "ctdm_set_fill_list_capacity")


def plans(r, device=0):
    """(variants (x, y, z), tuned) currently used for side r."""
    v = (ctypes.c_int * 3)()
    t = ctypes.c_int()
    check(load().ctdm_plans(int(device), int(r), v, ctypes.byref(t)), "ctdm_plans")
    return tuple(v), bool(t.value)


def z_tile(r, device=0):
    """Lines per packed z-pass tile of the current plan for side r (0: dense F2 reads)."""
    v = ctypes.c_int()
    check(load().ctdm_z_tile(int(device), int(r), ctypes.byref(v)), "ctdm_z_tile")
    return v.value


def set_plans(r, variants, device=0):
    v = (ctypes.c_int * 3)(*variants)
    check(load().ctdm_set_plans(int(device), int(r), v), "ctdm_set_plans")


class Batch:
    """Batched reconstruction (ctdm_batch): jobs = [(params, holo, bg, angx, angy, out), ...]
    with device tensors; plan() schedules them over `lanes` workspaces, runs them once and
    captures one CUDA graph; run() is a single graph launch."""

    def __init__(self, lanes=4, device=0):
        self.lib = load()
        h = ctypes.c_void_p()
        check(self.lib.ctdm_batch_create(int(device), int(lanes), ctypes.byref(h)), "ctdm_batch_create")
        self.handle = h
        self._keep = []

    def plan(self, jobs):
        arr = (_lib.Job * len(jobs))()
        keep = []
        for i, (params, holo, bg, angx, angy, out) in enumerate(jobs):
            ax, ay = _f32(angx), _f32(angy)
            keep += [ax, ay]
            arr[i].params = params
            arr[i].n_angles = len(ax)
            arr[i].d_holo, arr[i].d_bg = _ptr(holo), _ptr(bg)
            arr[i].h_angx, arr[i].h_angy = ax.ctypes.data, ay.ctypes.data
            arr[i].d_ri = _ptr(out)
        check(self.lib.ctdm_batch_plan(self.handle, arr, len(jobs)), "ctdm_batch_plan")
        self._keep = keep
        self.n_jobs = len(jobs)

    def run(self, stream=None):
        check(self.lib.ctdm_batch_run(self.handle, _stream(stream)), "ctdm_batch_run")

    def run_eager(self, stream=None):
        check(self.lib.ctdm_batch_run_eager(self.handle, _stream(stream)), "ctdm_batch_run_eager")

    def set_memory_limit(self, nbytes):
        """Cap the device memory the next plan may give its lanes (0: free memory alone)."""
        check(self.lib.ctdm_batch_set_memory_limit(self.handle, int(nbytes)), "ctdm_batch_set_memory_limit")

    def admission(self):
        """(lanes used, workspace bound per lane, bytes available) of the last plan."""
        n, per, avail = ctypes.c_int(), ctypes.c_size_t(), ctypes.c_size_t()
        check(self.lib.ctdm_batch_admission(self.handle, ctypes.byref(n), ctypes.byref(per), ctypes.byref(avail)),
              "ctdm_batch_admission")
        return n.value, per.value, avail.value

    def lanes(self):
        out = (ctypes.c_int * self.n_jobs)()
        check(self.lib.ctdm_batch_lanes(self.handle, out, self.n_jobs), "ctdm_batch_lanes")
        return list(out)

    def close(self):
        if self.handle:
            self.lib.ctdm_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Tape:
    """Measurement operator A = P F~ of one tomogram (ctdm_tape) with its adjoint,
    shaped like a torch.autograd.Function: forward(V) -> y, backward(dL/dy) -> dL/dV."""

    def __init__(self, F2, r, k2, counts=None, device=0):
        self.lib = load()
        h = ctypes.c_void_p()
        check(self.lib.ctdm_tape_create(int(device), int(r), _ptr(F2), _ptr(counts), float(k2), ctypes.byref(h)),
              "ctdm_tape_create")
        self.handle = h
        self.r = r

    @property
    def samples(self):
        return int(self.lib.ctdm_tape_samples(self.handle))

    def data(self):
        """(y, indices) on the host."""
        y = np.empty(self.samples, np.complex64)
        idx = np.empty(self.samples, np.uint32)
        check(self.lib.ctdm_tape_data(self.handle, y.ctypes.data, idx.ctypes.data), "ctdm_tape_data")
        return y, idx

    def forward(self, V, y, stream=None):
        check(self.lib.ctdm_forward(self.handle, _ptr(V), _ptr(y), _stream(stream)), "ctdm_forward")

    def backward(self, gy, gV, stream=None):
        check(self.lib.ctdm_backward(self.handle, _ptr(gy), _ptr(gV), _stream(stream)), "ctdm_backward")

    def loss_grad(self, V, grad, lam=0.0, eps=1e-4):
        loss = ctypes.c_double()
        check(self.lib.ctdm_loss_grad(self.handle, _ptr(V), float(lam), float(eps), _ptr(grad), ctypes.byref(loss)),
              "ctdm_loss_grad")
        return loss.value

    def reconstruct(self, V, iterations, lam=1e-3, eps=1e-4, step=0.0, record_loss=False, stream=None,
                    positivity=False):
        """FISTA on 1/2 ||A V - y||^2 + lam TV_eps(V) from V (in place); positivity=True
        projects every update onto the reference's positivity set."""
        hist = np.zeros(max(iterations, 1), np.float64) if record_loss else None
        check(self.lib.ctdm_reconstruct_gradient_ex(self.handle, int(iterations), float(lam), float(eps), float(step),
                                                    int(positivity), _ptr(V), _ptr(hist), _stream(stream)),
              "ctdm_reconstruct_gradient_ex")
        return hist

    def close(self):
        if self.handle:
            self.lib.ctdm_tape_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def contrast_to_ri(V, r, n_med, out, clamp=False, stream=None):
    check(load().ctdm_contrast_to_ri(int(r), _ptr(V), float(n_med), int(clamp), _ptr(out), _stream(stream)),
          "ctdm_contrast_to_ri")
