"""ctypes binding of libctdm_gb300.so (the C ABI declared in include/ctdm.h).

The library is built in-tree (ctdm_gb300/_build) by ctdm_gb300.build.  Loading
fails loudly when it is missing: there is no CPU or library fallback.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libctdm_gb300.so")

c_int, c_double, c_float, c_void_p, c_size_t = ctypes.c_int, ctypes.c_double, ctypes.c_float, ctypes.c_void_p, ctypes.c_size_t
c_bool = ctypes.c_bool
P_int = ctypes.POINTER(ctypes.c_int)


class Params(ctypes.Structure):
    """ctdm_params (include/ctdm.h)."""
    _fields_ = [
        ("n_holo", c_int), ("m_crop", c_int), ("r_vol", c_int), ("iterations", c_int),
        ("unwrap_mode", c_int), ("check_mode", c_int), ("unwrap_method", c_int), ("run_goldstein", c_int),
        ("bg_per_angle", c_int), ("carrier_r", c_int), ("carrier_c", c_int), ("carrier_radius", c_int),
        ("n_med", c_double), ("wavelength", c_double), ("dx", c_double), ("qpi_method", c_int),
        ("accelerated", c_int),
    ]


class Job(ctypes.Structure):
    """ctdm_job (include/ctdm.h)."""
    _fields_ = [
        ("params", Params), ("n_angles", c_int), ("d_holo", c_void_p), ("d_bg", c_void_p),
        ("h_angx", c_void_p), ("h_angy", c_void_p), ("d_ri", c_void_p),
    ]


class JobFile(ctypes.Structure):
    """ctdm_job_file (include/ctdm.h): one parameter file of a JobList."""
    _fields_ = [
        ("sp_dir", ctypes.c_char * 256), ("bg_dir", ctypes.c_char * 256), ("ang_dir", ctypes.c_char * 256),
        ("save_dir", ctypes.c_char * 256), ("row_pts", c_int * 2), ("col_pts", c_int * 2),
        ("recon_flag", c_int), ("recon_save", c_int), ("size_type", c_int), ("resize_flag", c_int),
        ("n_med", c_double), ("mag", c_double), ("camera_pixel_um", c_double), ("wavelength_nm", c_double),
        ("save_phase_stack", c_int), ("save_amp_stack", c_int), ("criteria_range", c_double),
        ("criteria_std", c_double), ("qpi_method", c_int), ("iter_time", c_int),
    ]


class PocsParams(ctypes.Structure):
    """ctdm_pocs_params (include/ctdm.h)."""
    _fields_ = [("iterations", c_int), ("tv_steps", c_int), ("beta", c_double), ("beta_red", c_double),
                ("alpha", c_double), ("alpha_red", c_double), ("r_max", c_double), ("eps_data", c_double),
                ("tv_eps", c_double)]


class JobResult(ctypes.Structure):
    """ctdm_job_result (include/ctdm.h)."""
    _fields_ = [("frames", c_int), ("rejected", c_int), ("recon_frames", c_int), ("n_holo", c_int),
                ("recon_size", c_int)]


# name -> (restype, argtypes)
_SIGS = {
    "ctdm_params_default": (None, [ctypes.POINTER(Params)]),
    "ctdm_last_error": (ctypes.c_char_p, []),
    "ctdm_version": (ctypes.c_char_p, []),
    "ctdm_ctx_create": (c_int, [c_int, ctypes.POINTER(c_void_p)]),
    "ctdm_ctx_destroy": (None, [c_void_p]),
    "ctdm_ctx_carrier": (c_int, [c_void_p, P_int]),
    "ctdm_ctx_buffer": (c_int, [c_void_p, c_int, ctypes.POINTER(c_void_p), ctypes.POINTER(c_size_t)]),
    "ctdm_ctx_read_buffer": (c_int, [c_void_p, c_int, c_void_p, c_size_t]),
    "ctdm_goldstein_fill": (c_int, [c_void_p, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, P_int, c_void_p]),
    "ctdm_ctx_set_timing": (c_int, [c_void_p, c_int]),
    "ctdm_ctx_stage_times": (c_int, [c_void_p, ctypes.POINTER(c_double), P_int, c_int]),
    "ctdm_ctx_device_status": (c_int, [c_void_p, P_int]),
    "ctdm_ctx_probe_wait": (c_int, [c_void_p, c_int, ctypes.POINTER(c_double)]),
    "ctdm_launch_count": (ctypes.c_ulonglong, []),
    "ctdm_reconstruct_device": (c_int, [c_void_p, ctypes.POINTER(Params), c_int, c_void_p, c_void_p, c_void_p,
                                        c_void_p, c_void_p, c_void_p]),
    "ctdm_reconstruct": (c_int, [c_void_p, ctypes.POINTER(Params), c_int, c_void_p, c_void_p, c_void_p, c_void_p,
                                 c_void_p]),
    "ctdm_reconstruct_u16": (c_int, [c_void_p, ctypes.POINTER(Params), c_int, c_void_p, c_void_p, c_void_p,
                                     c_void_p, c_void_p]),
    "ctdm_reconstruct_u8": (c_int, [c_void_p, ctypes.POINTER(Params), c_int, c_void_p, c_void_p, c_void_p,
                                    c_void_p, c_void_p]),
    "ctdm_submit": (c_int, [c_void_p, ctypes.POINTER(Params), c_int, c_void_p, c_void_p, c_int, c_void_p, c_void_p,
                            c_void_p]),
    "ctdm_wait": (c_int, [c_void_p]),
    "ctdm_qpi": (c_int, [c_void_p, c_int, c_int, c_int, c_void_p, c_void_p, c_int, P_int, c_void_p, c_void_p,
                         c_void_p]),
    "ctdm_qpi_b": (c_int, [c_void_p, c_int, c_int, c_void_p, c_void_p, c_int, P_int, c_void_p, c_void_p, c_void_p]),
    "extractQPI_AlgorithmA": (None, [c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_int, c_int]),
    "extractQPI_AlgorithmB": (None, [c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_int, c_int]),
    "ctdm_unwrap_dct": (c_int, [c_void_p, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p]),
    "ctdm_unwrap_fast": (c_int, [c_void_p, c_int, c_int, c_void_p, c_void_p, c_void_p]),
    "ctdm_goldstein": (c_int, [c_void_p, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p, P_int,
                               c_void_p]),
    "ctdm_prepare_spectra": (c_int, [c_void_p, c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p]),
    "ctdm_stack_spectra": (c_int, [c_void_p, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p]),
    "ctdm_prepare_stack": (c_int, [c_void_p, c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p,
                                   c_void_p]),
    "ctdm_map_ewald": (c_int, [c_void_p, c_int, c_int, c_void_p, c_void_p, c_void_p, c_double, c_double, c_double,
                               c_void_p, c_void_p, c_void_p]),
    "ctdm_positivity": (c_int, [c_void_p, c_int, c_int, c_int, c_double, c_double, c_void_p, c_void_p, c_void_p,
                                c_void_p]),
    "ctdm_positivity_ex": (c_int, [c_void_p, c_int, c_int, c_int, c_int, c_double, c_double, c_void_p, c_void_p,
                                   c_void_p, c_void_p]),
    "ctdm_fft": (c_int, [c_void_p, c_int, P_int, c_int, c_int, c_void_p]),
    "ctdm_unwrap_dct_noalloc": (c_int, [c_int, c_int, c_int, c_void_p, c_void_p, c_void_p]),
    "ctdm_tape_create": (c_int, [c_int, c_int, c_void_p, c_void_p, c_double, ctypes.POINTER(c_void_p)]),
    "ctdm_tape_destroy": (None, [c_void_p]),
    "ctdm_tape_samples": (ctypes.c_long, [c_void_p]),
    "ctdm_tape_data": (c_int, [c_void_p, c_void_p, c_void_p]),
    "ctdm_forward": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    "ctdm_backward": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    "ctdm_loss_grad": (c_int, [c_void_p, c_void_p, c_double, c_double, c_void_p, ctypes.POINTER(c_double)]),
    "ctdm_reconstruct_gradient": (c_int, [c_void_p, c_int, c_double, c_double, c_double, c_void_p, c_void_p,
                                          c_void_p]),
    "ctdm_reconstruct_gradient_ex": (c_int, [c_void_p, c_int, c_double, c_double, c_double, c_int, c_void_p,
                                             c_void_p, c_void_p]),
    "ctdm_contrast_to_ri": (c_int, [c_int, c_void_p, c_double, c_int, c_void_p, c_void_p]),
    "ctdm_batch_create": (c_int, [c_int, c_int, ctypes.POINTER(c_void_p)]),
    "ctdm_batch_destroy": (None, [c_void_p]),
    "ctdm_batch_plan": (c_int, [c_void_p, ctypes.POINTER(Job), c_int]),
    "ctdm_batch_run": (c_int, [c_void_p, c_void_p]),
    "ctdm_batch_run_eager": (c_int, [c_void_p, c_void_p]),
    "ctdm_batch_lanes": (c_int, [c_void_p, P_int, c_int]),
    "ctdm_batch_set_memory_limit": (c_int, [c_void_p, c_size_t]),
    "ctdm_batch_admission": (c_int, [c_void_p, P_int, ctypes.POINTER(c_size_t), ctypes.POINTER(c_size_t)]),
    "ctdm_workspace_bytes": (c_int, [ctypes.POINTER(Params), c_int, ctypes.POINTER(c_size_t)]),
    "ctdm_ctx_workspace": (c_int, [c_void_p, ctypes.POINTER(c_size_t)]),
    "ctdm_plan_count": (c_int, [c_int]),
    "ctdm_autotune": (c_int, [c_int, c_int, c_int, P_int, ctypes.POINTER(c_double), c_int]),
    "ctdm_z_tile": (c_int, [c_int, c_int, P_int]),
    "ctdm_plans": (c_int, [c_int, c_int, P_int, P_int]),
    "ctdm_set_plans": (c_int, [c_int, c_int, P_int]),
    "ctdm_loop_scheme": (c_int, [c_int, c_int, P_int]),
    "ctdm_set_loop_scheme": (c_int, [c_int, c_int, c_int]),
    "ctdm_set_fill_list_capacity": (c_int, [c_int]),
    "ctdm_set_recon_globals": (None, [c_int, c_double, c_double, c_double, c_double, c_int, c_int, ctypes.c_char_p]),
    "DCT_UWLS_Unwrapped": (None, [c_void_p, c_void_p, c_int, c_int]),
    "FastUnwrapping": (None, [c_void_p, c_void_p, c_int, c_int]),
    "cudaGoldsteinUnwrap2D": (None, [c_void_p, c_void_p, c_int, c_int, c_int]),
    "MedianFilter": (None, [c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_int, c_int]),
    "CopyDataArray": (None, [c_void_p, c_void_p, c_void_p, c_int, c_int, c_int, c_int]),
    "EdwardSphere": (None, [c_void_p, c_void_p, c_void_p, c_float, c_float, c_float, c_float, c_int, c_int, c_int]),
    "initial_F_and_F2": (None, [c_void_p, c_void_p, c_void_p, c_float, c_int, c_int, c_int]),
    "est_n_3D": (None, [c_void_p, c_void_p, c_float, c_float, c_int, c_int, c_int]),
    "modify_F_3D": (None, [c_void_p, c_void_p, c_float, c_float, c_int, c_int, c_int]),
    "check_F_3D": (None, [c_void_p, c_void_p, c_int, c_int, c_int]),
    "cuFFT3D": (None, [c_void_p, c_int, c_int, c_int, c_int]),
    "cuFFT2D": (None, [c_void_p, c_int, c_int, c_int]),
    "BatchRecon": (None, [c_void_p, c_void_p, c_void_p, c_void_p, c_int]),
    "ctdm_read_bmp": (c_int, [ctypes.c_char_p, P_int, P_int, c_void_p]),
    "ctdm_write_phimap": (c_int, [ctypes.c_char_p, c_int, c_double, c_double, c_int, c_int, c_void_p, c_void_p]),
    "ctdm_read_phimap": (c_int, [ctypes.c_char_p, P_int, ctypes.POINTER(c_double), ctypes.POINTER(c_double), P_int,
                                 P_int, c_void_p, c_void_p]),
    "ctdm_write_rimap": (c_int, [ctypes.c_char_p, c_int, c_int, c_void_p]),
    "ctdm_check_frame": (c_int, [c_void_p, c_int, c_int, c_double, c_double]),
    "ctdm_angle_from_image": (c_int, [c_void_p, c_int, c_double, c_double, c_double, c_double,
                                      ctypes.POINTER(c_float), ctypes.POINTER(ctypes.c_long)]),
    "ctdm_job_defaults": (None, [ctypes.POINTER(JobFile)]),
    "ctdm_parse_job_file": (c_int, [ctypes.c_char_p, ctypes.POINTER(JobFile)]),
    "ctdm_run_job": (c_int, [ctypes.POINTER(JobFile), ctypes.POINTER(JobResult)]),
    "scriptFileRead": (c_int, [ctypes.c_char_p]),
    "ctdm_map_fi": (c_int, [c_void_p, c_int, c_int, c_void_p, c_void_p, c_double, c_double, c_double, c_void_p,
                            c_void_p, c_void_p]),
    "ctdm_pocs_defaults": (None, [ctypes.POINTER(PocsParams)]),
    "ctdm_pocs": (c_int, [c_void_p, c_int, ctypes.POINTER(PocsParams), c_double, c_double, c_void_p, c_void_p,
                          c_void_p, c_void_p]),
    "BatchReconPOCS": (None, [c_void_p, c_void_p, c_void_p, c_void_p, c_int]),
    "HilbertTransform": (None, [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, P_int, P_int,
                                c_int, c_int, c_int, c_int, c_int]),
    "AngCal_GPU": (c_float, [c_void_p, c_int, c_int, c_int, c_int]),
    "checkArray": (c_bool, [c_void_p, c_float, c_float, c_int]),
}

EXPORTED = tuple(_SIGS)
_lib = None


def load(path=None):
    """Load the shared library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError(f"libctdm_gb300.so not built ({path}); run ctdm_gb300.build.build()")
    lib = ctypes.CDLL(path)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def last_error():
    return load().ctdm_last_error().decode()


class CtdmError(RuntimeError):
    def __init__(self, status, where):
        self.status = status
        super().__init__(f"{where} failed with status {status}: {last_error()}")


def check(status, where):
    if status != 0:
        raise CtdmError(status, where)
